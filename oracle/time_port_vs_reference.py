"""Times the oracle (the CPU restatement that bench.py's reference arm runs on a
GPU host) against the reference itself, compiled from its own sources by this
directory's Makefile (`make ref`: _ref/libref_fast.so, -O3 -march=native
-funroll-loops -fopenmp), on the same Hamiltonian and the same powers.

TEST INFRASTRUCTURE ONLY. It needs the reference sources (to build _ref/), so it
runs where they are present, not on a GPU host.

Usage: python oracle/time_port_vs_reference.py [--threads 1] [--sizes 12,16,20]

For each size (n spin orbitals, N = n / 2, seeded synthetic integrals, dt 0.05,
first order, one step per power: the reference's own mode) it times the same
number of controlled powers from the Hartree-Fock start in both, best of three,
and prints one JSON line per size with both rates in amplitude updates per second
and their ratio.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent


def _synthetic():
    spec = importlib.util.spec_from_file_location("qpe_workload_synthetic", ROOT / "2022-qpesim_gb300" / "synthetic.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod  # dataclasses look their module up while the class is built
    spec.loader.exec_module(mod)
    return mod


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=1)
    ap.add_argument("--sizes", default="12,16,20")
    ap.add_argument("--powers", type=int, default=0, help="powers timed per size (0: about 2 s of work)")
    a = ap.parse_args()
    os.environ["OMP_NUM_THREADS"] = str(a.threads)
    sys.path.insert(0, str(HERE))
    import oracle as O  # noqa: E402
    O.build(ref=True)
    orc = O.Oracle(fast=True)
    orc.set_threads(a.threads)
    ref = O.Reference(fast=True)
    syn = _synthetic()
    for n in (int(x) for x in a.sizes.split(",")):
        M, e, dt = n // 2, n // 4, 0.05
        ints = syn.synthetic_integrals(n, 0)
        seg = orc.segmented_terms(M, e, dt, ints.one_body, ints.two_body)
        touches = orc.touches_per_power(M, e, e, seg)
        C = int(orc.nchoosek(M, e))
        # enough powers for about 2 s of the oracle's work, within the register
        state = np.zeros(2 * C * C, np.complex128)
        state[0] = 1.0
        t0 = time.perf_counter()
        orc.time_evolve(M, e, e, 1, seg, state)
        one = time.perf_counter() - t0
        npow = a.powers or max(1, min(255, int(2.0 / max(one, 1e-9))))
        P = max(1, int(np.ceil(np.log2(npow + 1))))
        h = ref.hamiltonian(M, e, ints.one_body, ints.two_body, dt)
        best_o, best_r = float("inf"), float("inf")
        for _ in range(3):
            st = np.zeros((1 << P) * C * C, np.complex128)
            st[0] = 2.0 ** (-P / 2)
            t0 = time.perf_counter()
            orc.time_evolve(M, e, e, P, seg, st, first=1, last=1 + npow)
            best_o = min(best_o, (time.perf_counter() - t0) / npow)
            st = np.zeros((1 << P) * C * C, np.complex128)
            st[0] = 2.0 ** (-P / 2)
            best_r = min(best_r, ref.time_steps(h, P, st, npow))
        ref.destroy(h)
        print(json.dumps({"n": n, "electrons": 2 * e, "threads": a.threads, "powers": npow,
                          "touches_per_power": touches, "oracle_touches_per_s": touches / best_o,
                          "reference_touches_per_s": touches / best_r, "oracle_over_reference": best_r / best_o}),
              flush=True)


if __name__ == "__main__":
    main()
