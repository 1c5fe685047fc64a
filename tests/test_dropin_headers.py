"""The drop-in headers (include/qpesim_gb300/) in the reference's own main flow
(cpp/main.cc:97-167): ingest a Broombridge file, index the terms, set the
timestep, scale block 0 by 2^(-P/2), time_evolve_over_terms, qift,
IdentifyPhaseAmplitudes; the one-orbital pp case of the reference's end-to-end
test (cpp/time_evolution.hpp:339-367) must give probs[87] > 0.5.

Two builds of the same driver (tests/dropin/dropin_main.cc):
- against the reference's own Hamiltonian (its hamiltonian.cc with the oracle's
  yaml-cpp and doctest shims), where the reference sources are present;
- against tests/dropin/standin/, a Hamiltonian with the reference's interface
  backed by the library's own term compiler, which needs no reference sources
  and so also runs on a GPU host.
Without a GPU the driver must report the library's "no CUDA device" error as the
reference's `throw const char*`; with one it must succeed.
"""
import subprocess

import pytest

from conftest import ROOT, reference_root

REF_FILES = ["hamiltonian.cc", "hamiltonian.hpp", "types.hpp", "util.hpp", "offset_computer.hpp", "gate.hpp"]
_REF = reference_root()


def _one_orbital_pp_file(path):
    """A Broombridge file holding one spatial orbital, h_11 = 1 and no two-body
    integrals, with both spins of orbital 1 occupied in the initial state."""
    path.write_text(
        "format: {version: \"0.2\"}\n"
        "integral_sets:\n"
        "  - coulomb_repulsion: {units: hartree, value: 0.0}\n"
        "    energy_offset: {units: hartree, value: 0.0}\n"
        "    hamiltonian:\n"
        "      one_electron_integrals:\n"
        "        format: sparse\n"
        "        values:\n"
        "          - [1, 1, 1.0]\n"
        "      two_electron_integrals:\n"
        "        format: sparse\n"
        "        index_convention: mulliken\n"
        "        values: []\n"
        "    initial_state_suggestions:\n"
        "      - state:\n"
        "          label: \"|G>\"\n"
        "          superposition:\n"
        "            - [1.0, (1a)+, (1b)+, '|vacuum>']\n")
    return path


def _build(q, tmp_path, hamiltonian_dir, extra_sources):
    src = tmp_path / "src"
    src.mkdir()
    for f in ("time_evolution_over_terms.hpp", "state_vector.hpp"):
        (src / f).symlink_to(ROOT / "include" / "qpesim_gb300" / f)
    exe = tmp_path / "dropin"
    shims = ROOT / "oracle" / "ref_shims"
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-DDOCTEST_CONFIG_DISABLE", f"-I{src}", f"-I{hamiltonian_dir}",
           f"-I{shims}", f"-I{ROOT / '2022-qpesim_gb300' / 'csrc'}", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "dropin" / "dropin_main.cc"), *map(str, extra_sources), "-o", str(exe),
           f"-L{q.LIB_PATH.parent}", "-lqpe_gb300", f"-Wl,-rpath,{q.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _run_and_check(q, exe, fixture):
    r = subprocess.run([str(exe), str(fixture)], capture_output=True, text=True, timeout=120)
    if q._native.device_count() > 0:
        assert r.returncode == 0, r.stdout + r.stderr
        assert float(r.stdout.split("=")[1]) > 0.5, r.stdout
    else:
        assert r.returncode == 3 and "no CUDA device" in r.stdout, r.stdout + r.stderr
    return r.stdout


@pytest.mark.skipif(_REF is None, reason="reference sources not present")
def test_dropin_with_reference_hamiltonian(q, tmp_path):
    ref = _REF / "cpp"
    hdir = tmp_path / "ref"
    hdir.mkdir()
    for f in REF_FILES:
        (hdir / f).symlink_to(ref / f)
    exe = _build(q, tmp_path, hdir, [hdir / "hamiltonian.cc"])
    _run_and_check(q, exe, _REF / "qsharp-verify" / "broombridge" / "PP.yml")
    # the same driver on the one-orbital file this test writes
    _run_and_check(q, exe, _one_orbital_pp_file(tmp_path / "pp1.yaml"))


def test_dropin_with_standin_hamiltonian(q, tmp_path):
    """Runs everywhere; on a GPU host this is the drop-in's success path."""
    exe = _build(q, tmp_path, ROOT / "tests" / "dropin" / "standin", [])
    _run_and_check(q, exe, _one_orbital_pp_file(tmp_path / "pp1.yaml"))


@pytest.mark.gpu
def test_dropin_success_path_on_gpu(gpu, tmp_path):
    """The drop-in headers' success path on the GPU: probs[87] > 0.5."""
    exe = _build(gpu, tmp_path, ROOT / "tests" / "dropin" / "standin", [])
    out = _run_and_check(gpu, exe, _one_orbital_pp_file(tmp_path / "pp1.yaml"))
    assert "probs[87]" in out
