"""Broombridge ingestion (cpp/hamiltonian.cc:8-144) in the product's native reader.

Two kinds of case, both on CPU:
- the reference's own fixture files, where the reference tree is present, against
  what the reference's IngestBroombridge produced from them (golden vectors:
  orbital and electron counts, identity, the segmented terms at dt = 1 and block 0
  with its Jordan-Wigner signs);
- files this test writes from seeded synthetic integrals, against the same
  integrals added term by term, and block 0 against a plain restatement of the
  sign rule.
"""
import math

import numpy as np
import pytest

from conftest import golden_segments, load_golden, reference_root
from test_term_compiler import _assert_segments

_REF_ROOT = reference_root()
BROOMBRIDGE = _REF_ROOT / "qsharp-verify" / "broombridge" if _REF_ROOT is not None else None
FIXTURES = {"PP": "PP.yml", "PQ": "PQ.yml", "PQQP": "PQQP.yml", "PQQR": "PQQR.yml", "PQRS": "PQRS.yml",
            "h4_sto6g_0.100": "h4_sto6g_0.100.yaml"}


@pytest.mark.parametrize("stem", sorted(FIXTURES))
def test_reference_fixture(q, stem):
    path = BROOMBRIDGE / FIXTURES[stem] if BROOMBRIDGE is not None else None
    if path is None or not path.exists():
        pytest.skip("reference fixture files not present")
    z = load_golden(f"broombridge_{stem}.npz")
    h = q.Hamiltonian()
    sv = h.IngestBroombridge(path, int(z["precision"]))
    assert h.num_orbitals() == int(z["M"]) and h.num_occupied() == int(z["e"])
    assert h.GetIdentityTerm() == float(z["identity"])
    assert np.array_equal(np.asarray(sv), z["state0"])
    h.SetTimestep(float(z["dt"]))
    h.IndexTerms()
    _assert_segments(h.segmented_terms(), golden_segments(z))


def _colex_rank(bv):
    r, order, pos = 0, 1, 0
    while bv:
        if bv & 1:
            r += math.comb(pos, order)
            order += 1
        bv >>= 1
        pos += 1
    return r


def _apply_ops(M, ops, coeff):
    """Operators applied right to left; each flips the sign once per occupied
    spin orbital below it (cpp/hamiltonian.cc:74-112)."""
    bv = 0
    for orb, spin, create in reversed(ops):
        idx = orb - 1 + (M if spin == "b" else 0)
        bv += (1 << idx) if create else -(1 << idx)
        coeff *= (-1) ** bin(bv & ((1 << idx) - 1)).count("1")
    return bv, coeff


def _write(path, ints, identity, basis):
    rows1 = "\n".join(f"          - [{p}, {q}, {v!r}]" for p, q, v in ints.one_body)
    # two_body holds AddTwoBodyTerm(i, j, k, l) arguments; the file row is [i, l, j, k]
    rows2 = "\n".join(f"          - [{i}, {l}, {j}, {k}, {v!r}]" for i, j, k, l, v in ints.two_body)
    sup = []
    for coeff, ops in basis:
        txt = ", ".join(f"({o}{sp}){'+' if c else ''}" for o, sp, c in ops)
        sup.append(f"            - [{coeff!r}, {txt}, '|vacuum>']")
    path.write_text(
        "format: {version: \"0.2\"}\n"
        "integral_sets:\n"
        "  - coulomb_repulsion: {units: hartree, value: %r}\n"
        "    energy_offset: {units: hartree, value: 0.25}\n"
        "    hamiltonian:\n"
        "      one_electron_integrals:\n"
        "        format: sparse\n"
        "        values:\n%s\n"
        "      two_electron_integrals:\n"
        "        format: sparse\n"
        "        index_convention: mulliken\n"
        "        values:\n%s\n"
        "    initial_state_suggestions:\n"
        "      - state:\n"
        "          label: \"|G>\"\n"
        "          superposition:\n%s\n" % (identity, rows1, rows2, "\n".join(sup)))


@pytest.mark.parametrize("n,seed", [(6, 1), (8, 4)])
def test_written_file_matches_term_by_term(q, tmp_path, n, seed):
    M = n // 2
    ints = q.synthetic_integrals(n, seed)
    hf = [(o, s, True) for s in "ab" for o in (1, 2)]
    # a double excitation written the reference's way: annihilate, then create
    dbl = [(3, "a", True), (3, "b", True), (2, "b", False), (2, "a", False)] + hf
    sgl = [(M, "a", True), (1, "a", False)] + hf
    basis = [(0.875, hf), (-0.25, dbl), (0.125, sgl)]
    path = tmp_path / "synthetic.yaml"
    _write(path, ints, 0.5, basis)

    h = q.Hamiltonian()
    sv = h.IngestBroombridge(path, 3)
    assert h.num_orbitals() == M and h.num_occupied() == 2
    assert h.GetIdentityTerm() == 0.5 + 0.25
    ref = q.Hamiltonian.from_integrals(ints, 2, 0.05)
    h.SetTimestep(0.05)
    h.IndexTerms()
    _assert_segments(h.segmented_terms(), ref.segmented_terms())

    want = np.zeros(sv.ld, np.complex128)
    C = math.comb(M, 2)
    for coeff, ops in basis:
        bv, c = _apply_ops(M, [(o, s, cr) for o, s, cr in ops], coeff)
        alpha, beta = bv & ((1 << M) - 1), bv >> M
        want[C * _colex_rank(alpha) + _colex_rank(beta)] = c
    assert np.array_equal(sv.block(0), want)
    assert not np.any(np.asarray(sv)[sv.ld:])
    # the case exercises the sign rule: some basis state changes sign
    assert any(_apply_ops(M, ops, 1.0)[1] == -1.0 for _, ops in basis)


def test_rejects_bad_files(q, tmp_path):
    h = q.Hamiltonian()
    with pytest.raises(q.QpeError):
        h.IngestBroombridge(tmp_path / "missing.yaml", 2)
    bad = tmp_path / "bad.yaml"
    bad.write_text("format: {version: \"0.2\"}\n")
    with pytest.raises(q.QpeError):
        q.Hamiltonian().IngestBroombridge(bad, 2)
    ints = q.synthetic_integrals(4, 0)
    # creating twice on one orbital
    _write(bad, ints, 0.0, [(1.0, [(1, "a", True), (1, "a", True)])])
    with pytest.raises(q.QpeError):
        q.Hamiltonian().IngestBroombridge(bad, 2)
