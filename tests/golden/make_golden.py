"""Generates the golden fixtures in this directory from the reference itself.

Runs oracle/_ref/libref.so (the reference's own sources compiled with the shims
of oracle/ref_shims; build it with `make -C oracle ref`) on seeded synthetic
Hamiltonians, on the reference's single-term Broombridge fixtures and on its
embedded doctests, and stores the results as small .npz / .json files:

  terms_n{n}_N{N}_s{seed}.npz   segmented terms + coefficients (the term compiler)
  evolve_*.npz                  block 0, the evolved register, the QIFT output and
                                the phase histogram of time_evolve_over_terms / qift /
                                IdentifyPhaseAmplitudes
  iqpe_*.npz                    the register before and after time_evolve_iqpe
                                (block 1 evolved in place, applyUnitary order)
  discover.npz                  run tables of the five discover*_BVs routines
  swaps.npz                     OffsetComputer rank_with_swap / rank_with_double_swap
  broombridge_*.npz             terms and block 0 from IngestBroombridge on files
  doctests.json                 outcome of each reference doctest case

Usage: python tests/golden/make_golden.py [--reference-dir /path/to/reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

EVOLVE_CASES = [
    # (n spin-orbitals, N electrons, precision P, dt, seed)
    (8, 4, 6, 0.1, 0),     # the CPU-runnable plain QPE configuration
    (8, 4, 3, 1.0, 1),
    (6, 2, 4, 0.1, 2),
    (10, 6, 3, 0.05, 3),
    (12, 6, 2, 0.05, 4),
    (4, 2, 3, 0.2, 5),
    (2, 2, 3, 0.3, 6),
    (10, 2, 2, 0.1, 7),
]
TERM_CASES = [(8, 4, 0.1, 0), (12, 6, 0.05, 3), (16, 8, 0.05, 11), (6, 2, 1.0, 5)]
IQPE_CASES = [(6, 2, 1, 0.2, 2, 4), (8, 4, 2, 0.1, 3, 3), (10, 6, 1, 0.05, 5, 2), (12, 6, 1, 0.05, 6, 1)]
SINGLE_TERM_FILES = ["PP.yml", "PQ.yml", "PQQP.yml", "PQQR.yml", "PQRS.yml", "h4_sto6g_0.100.yaml"]


def seg_arrays(seg, raw, prefix=""):
    out = {}
    for k, v in seg.items():
        out[prefix + k] = v.view(np.uint8).copy()
        out[prefix + k + "_raw"] = raw[k]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-dir", default=os.environ.get("QPE_REFERENCE_DIR"),
                    help="the reference tree (default: where the oracle's build recipe finds it)")
    a = ap.parse_args()
    import __graft_entry__ as g
    if a.reference_dir:
        refdir = Path(a.reference_dir)
    else:
        src = g.load_oracle().reference_cpp()
        if src is None:
            raise SystemExit("the reference sources are not present: pass --reference-dir")
        refdir = src.parent
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), f"REF={refdir / 'cpp'}", "ref"], check=True)
    q = g.load_package()
    O = g.load_oracle()
    ref = O.Reference()

    for n, N, dt, seed in TERM_CASES:
        it = q.synthetic_integrals(n, seed)
        h = ref.hamiltonian(n // 2, N // 2, it.one_body, it.two_body, dt)
        seg, raw = ref.segments(h)
        np.savez_compressed(HERE / f"terms_n{n}_N{N}_s{seed}.npz", n=n, N=N, dt=dt, seed=seed, **seg_arrays(seg, raw))
        ref.destroy(h)

    for n, N, P, dt, seed in EVOLVE_CASES:
        M, e = n // 2, N // 2
        it = q.synthetic_integrals(n, seed)
        h = ref.hamiltonian(M, e, it.one_body, it.two_body, dt)
        seg, raw = ref.segments(h)
        C = ref.nchoosek(M, e)
        state = np.zeros((1 << P) * C * C, np.complex128)
        state[0] = 2.0 ** (-P / 2)
        block0 = state[: C * C].copy()
        ref.time_evolve(h, P, state)
        evolved = state.copy()
        ref.qift(P, M, e, state)
        probs = ref.identify_phase_amplitudes(P, M, e, state)
        np.savez_compressed(HERE / f"evolve_n{n}_N{N}_P{P}_s{seed}.npz", n=n, N=N, P=P, dt=dt, seed=seed,
                            block0=block0, evolved=evolved, qift=state, probs=probs, **seg_arrays(seg, raw))
        ref.destroy(h)

    # time_evolve_iqpe: block 1 (a seeded random state) evolved in place.
    for n, N, P, dt, seed, apps in IQPE_CASES:
        M, e = n // 2, N // 2
        it = q.synthetic_integrals(n, seed)
        h = ref.hamiltonian(M, e, it.one_body, it.two_body, dt)
        seg, raw = ref.segments(h)
        C = ref.nchoosek(M, e)
        rng = np.random.default_rng(seed)
        state = np.zeros((1 << P) * C * C, np.complex128)
        state[0] = 1.0
        state[C * C:2 * C * C] = rng.standard_normal(C * C) + 1j * rng.standard_normal(C * C)
        state[C * C:2 * C * C] /= np.linalg.norm(state[C * C:2 * C * C])
        before = state.copy()
        ref.time_evolve_iqpe(h, P, state, apps)
        np.savez_compressed(HERE / f"iqpe_n{n}_N{N}_P{P}_a{apps}_s{seed}.npz", n=n, N=N, P=P, dt=dt, seed=seed,
                            applications=apps, before=before, after=state, **seg_arrays(seg, raw))
        ref.destroy(h)

    # discover tables
    rows, tabs = [], []
    for M, e in [(4, 2), (5, 2), (6, 3), (7, 3), (8, 4)]:
        combos = [(0, (0, q, 0, 0)) for q in range(M)]
        combos += [(1, (p, 0, r, 0)) for p in range(M) for r in range(p + 1, M)]
        combos += [(2, (p, 0, r, 0)) for p in range(M) for r in range(M) if p != r]
        combos += [(3, (p, q_, r, 0)) for p in range(M) for r in range(p + 1, M) for q_ in range(M) if q_ not in (p, r)]
        combos += [(4, (p, q_, r, s)) for p in range(M) for q_ in range(M) for r in range(M) for s in range(M)
                   if len({p, q_, r, s}) == 4 and p < q_ and s < r and p < s]
        for kind, (p, q_, r, s) in combos:
            ni, o1, o2, pa = ref.discover(kind, M, e, p, q_, r, s)
            rows.append((kind, M, e, p, q_, r, s, len(ni)))
            tabs.append(np.stack([ni, o1, o2, pa.astype(np.uint64)], 1) if len(ni) else np.zeros((0, 4), np.uint64))
    np.savez_compressed(HERE / "discover.npz", rows=np.array(rows, np.int64),
                        tables=np.concatenate(tabs, 0) if tabs else np.zeros((0, 4), np.uint64))

    # OffsetComputer incremental ranks: the reference's test shapes (n = 15 single
    # swaps, n = 20 double swaps with an even number of ones among the four bits).
    rng = np.random.default_rng(2022)
    sw_bv, sw_q, sw_out = [], [], []
    for n, count in ((15, 5), (20, 5)):
        for _ in range(count):
            bv = int(rng.integers(0, 1 << n))
            qs = [(i, j, 0xFFFFFFFF, 0xFFFFFFFF) for i in range(n) for j in range(n)]
            if n == 20:
                qs += [(i, j, k, l) for i in range(n) for j in range(i + 1, n) for k in range(j + 1, n)
                       for l in range(k + 1, n) if sum((bv >> x) & 1 for x in (i, j, k, l)) in (0, 2, 4)][::7]
            qs = np.array(qs, np.uint32)
            sw_bv.append((n, bv, len(qs)))
            sw_q.append(qs)
            sw_out.append(ref.rank_with_swaps(n, bv, qs))
    ranks_bv = rng.integers(0, 1 << 24, size=2000).astype(np.uint64)
    np.savez_compressed(HERE / "swaps.npz", heads=np.array(sw_bv, np.int64), queries=np.concatenate(sw_q),
                        ranks=np.concatenate(sw_out), rank_bv=ranks_bv,
                        rank_out=np.array([ref.rank(int(b)) for b in ranks_bv], np.int64))

    # Broombridge: the reference's own ingestion on its fixtures.
    bdir = refdir / "qsharp-verify" / "broombridge"
    for name in SINGLE_TERM_FILES:
        h, M, e, ident, s0 = ref.broombridge(bdir / name, 3, 1.0)
        seg, raw = ref.segments(h)
        np.savez_compressed(HERE / f"broombridge_{Path(name).stem}.npz", M=M, e=e, identity=ident, precision=3,
                            dt=1.0, state0=s0, **seg_arrays(seg, raw))
        ref.destroy(h)

    # Doctests, each in its own process (some abort on the reference's asserts).
    results = {}
    names = ["offset computing test: swap one zero-one pair", "offset computing test: swap one one-one or zero-zero pair",
             "offset computing test: double swaps", "Simple 1D Gate Application", "Hadamard",
             "Simple Controlled 1D Gate Application", "QIFT", "PP term verification", "PQ term verification",
             "PQQP term verification", "PQQR term verification", "PQRS term verification"]
    for nm in names:
        code = ("import sys; sys.path.insert(0, %r); from oracle import Reference; import json; "
                "r = Reference(); d = r.run_doctests(%r); print(json.dumps({k: list(v) for k, v in d.items() if k == %r}))"
                % (str(ROOT / "oracle"), nm, nm))
        p = subprocess.run([sys.executable, "-c", code], cwd=refdir / "cpp", capture_output=True, text=True)
        if p.returncode == 0:
            d = json.loads(p.stdout.strip().splitlines()[-1])
            checks, failed = d[nm]
            results[nm] = {"checks": checks, "failed": failed, "aborted": False}
        else:
            results[nm] = {"checks": None, "failed": None, "aborted": True,
                           "message": (p.stderr.strip().splitlines() or [""])[-1][-200:].replace(str(refdir) + "/", "")}
    (HERE / "doctests.json").write_text(json.dumps(results, indent=1) + "\n")
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
