"""The product's host-side term compiler against the reference's (golden vectors)."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_segments, load_golden

KINDS = ("pp", "pq", "pqqp", "pqqr", "pqrs")


def _assert_segments(mine, want):
    for k in KINDS:
        a, b = mine[k], want[k]
        assert len(a) == len(b), k
        for f in ("p", "q", "r", "s"):
            assert np.array_equal(a[f], b[f]), (k, f)
        # coefficients come from libm cos / sin / exp: equal to an ulp across machines
        np.testing.assert_allclose(a["even"], b["even"], rtol=0, atol=2e-16)
        np.testing.assert_allclose(a["odd"], b["odd"], rtol=0, atol=2e-16)


@pytest.mark.parametrize("name", sorted(p.name for p in GOLDEN.glob("terms_*.npz")))
def test_compiler_matches_reference(q, name):
    z = load_golden(name)
    n, N, dt, seed = int(z["n"]), int(z["N"]), float(z["dt"]), int(z["seed"])
    h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, seed), N // 2, dt)
    _assert_segments(h.segmented_terms(), golden_segments(z))
    raw = h.PrintIndexedSegmentedHamiltonianTerms()
    for i, k in enumerate(KINDS):
        np.testing.assert_array_equal([v for _, v in raw[i]], z[k + "_raw"])


def test_coefficient_known_answers(q):
    """The reference's coefficient KATs (cpp/hamiltonian.hpp:192-313) at dt = 1."""
    h = q.Hamiltonian()
    h.SetNumOrbitals(1)
    h.SetTimestep(1.0)
    h.AddOneBodyTerm((1, 1), 1.0)
    h.IndexTerms()
    assert h.pp_term(0) == np.exp(-1j) and h.pp_term(1) == np.exp(-1j)
    h = q.Hamiltonian()
    h.SetNumOrbitals(2)
    h.SetTimestep(1.0)
    h.AddOneBodyTerm((2, 1), 1.0)
    h.IndexTerms()
    want = [np.cos(1.0), -1j * np.sin(1.0), -1j * np.sin(1.0), np.cos(1.0)]
    assert h.pq_term(1, 0, 0) == want and h.pq_term(3, 2, 0) == want
    odd = h.pq_term(1, 0, 1)
    assert odd[1] == 1j * np.sin(1.0)
    # an empty key gives the identity, a PPPP term (p, p, p, p) becomes p^ p_ p_ p^
    h = q.Hamiltonian()
    h.SetNumOrbitals(2)
    h.SetTimestep(1.0)
    h.AddTwoBodyTerm((1, 1, 1, 1), 2.0)
    h.IndexTerms()
    assert h.pqqp_term(0, 2) == np.exp(-2j)
    assert h.pq_term(1, 0, 0) == [1, 0, 0, 1]


def test_compiler_rejects_bad_input(q):
    h = q.Hamiltonian()
    with pytest.raises(q.QpeError):
        h.AddOneBodyTerm((1, 2), 1.0)  # needs p >= q
    with pytest.raises(q.QpeError):
        h.IndexTerms()  # orbital count unset
