"""The drop-in headers compile and link against the reference's own Hamiltonian
(its hamiltonian.cc, compiled with the oracle's yaml-cpp and doctest shims), and
run the reference's PP end-to-end case: probs[87] > 0.5 on a GPU, a library error
surfaced as the reference's `throw const char*` without one. Needs the reference
sources (QPE_REFERENCE_CPP), so it is skipped where they are absent."""
import os
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

REF = Path(os.environ.get("QPE_REFERENCE_CPP", "/root/reference/cpp"))
REF_FILES = ["hamiltonian.cc", "hamiltonian.hpp", "types.hpp", "util.hpp", "offset_computer.hpp", "gate.hpp"]


@pytest.mark.skipif(not (REF / "hamiltonian.cc").exists(), reason="reference sources not present")
def test_dropin_builds_and_reports(q, tmp_path):
    for f in REF_FILES:
        (tmp_path / f).symlink_to(REF / f)
    for f in ("time_evolution_over_terms.hpp", "state_vector.hpp"):
        (tmp_path / f).symlink_to(ROOT / "include" / "qpesim_gb300" / f)
    (tmp_path / "main.cc").symlink_to(ROOT / "tests" / "dropin" / "dropin_main.cc")
    exe = tmp_path / "dropin"
    shims = ROOT / "oracle" / "ref_shims"
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-DDOCTEST_CONFIG_DISABLE", f"-I{tmp_path}", f"-I{shims}",
           f"-I{ROOT / '2022-qpesim_gb300' / 'csrc'}", f"-I{ROOT / 'include'}", str(tmp_path / "main.cc"),
           str(tmp_path / "hamiltonian.cc"), "-o", str(exe), f"-L{q.LIB_PATH.parent}", "-lqpe_gb300",
           f"-Wl,-rpath,{q.LIB_PATH.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    fixture = REF.parent / "qsharp-verify" / "broombridge" / "PP.yml"
    r = subprocess.run([str(exe), str(fixture)], capture_output=True, text=True, timeout=120)
    if q._native.device_count() > 0:
        assert r.returncode == 0, r.stdout + r.stderr
    else:
        assert r.returncode == 3 and "no CUDA device" in r.stdout, r.stdout + r.stderr
