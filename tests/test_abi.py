"""The C-ABI library loads and exports every symbol the public headers declare."""
import ctypes
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"^\s*(?:int|const char\*|void)\s+(qpe_\w+)\s*\(", text, re.M))
    return names


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert {"qpe_time_evolve_over_terms", "qpe_qift", "qpe_identify_phase_amplitudes", "qpe_rank",
            "qpe_program_create", "qpe_evolve", "qpe_ham_create"} <= names


def test_library_exports_all_declared(q):
    lib = ctypes.CDLL(str(q.LIB_PATH))
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_fails_loudly(q):
    if q._native.device_count() > 0:
        return
    import pytest
    with pytest.raises(q.QpeError) as ei:
        q.OffsetComputer.rank(5)
    assert ei.value.code == 6


def test_bf16_helpers_and_mlp_layout(q):
    import numpy as np
    import qpesim_gb300.learned_state as L
    x = np.array([1.0, -2.5, 3.14159, 1e-3, 65504.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9], np.float32)
    r = L.round_bf16(x)
    assert r[0] == 1.0 and r[1] == -2.5 and abs(r[2] - 3.140625) < 1e-7
    assert r[5] == 1.0  # halfway, ties to even
    assert r[6] == np.float32(1.0 + 2 ** -7)
    lay = L.param_layout()
    assert sum(int(np.prod(s)) for _, s in lay.values()) == 152336


def test_learned_state_helpers_on_cpu(q):
    import math

    import numpy as np
    L = q.learned_state
    s = L.register_strings(4, 2, 2)
    assert len(s) == 36 and len(set(int(x) for x in s)) == 36
    assert all(bin(int(x) & 0xF).count("1") == 2 and bin(int(x) >> 4).count("1") == 2 for x in s)
    # a Fejer peak: the ground bin is its lowest-energy local maximum, the sub-bin
    # estimate recovers the energy, and the shot count to 1e-3 Ha is finite
    n, t, E = 256, 0.05, -3.2
    phi = (-E * t / (2 * math.pi)) % 1.0
    j = np.arange(n)
    d = (j / n - phi + 0.5) % 1.0 - 0.5
    p = np.abs(np.sin(np.pi * n * d) / (n * np.sin(np.pi * d) + 1e-300)) ** 2
    p /= p.sum()
    j0 = L.ground_bin(p, t)
    assert abs(L.subbin_energy(p, j0, n, t) - E) < 1e-6
    assert L.shots_to_precision(p, j0, t, E) is not None
