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
