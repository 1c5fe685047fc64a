"""Benchmark of the QPE hot path on GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

One step is one full QPE run of the workload: the controlled evolution of all
2^P - 1 powers, the QIFT and the phase histogram. The metric is amplitude-term
updates per second (a pair update counts 2, a diagonal phase 1, the same
definition for every arm). `value` is timed with CUDA events on the library's
stream with the register resident in HBM; `e2e` repeats the step through host
buffers (block 0 copied in from page-locked memory, the whole register and the
histogram copied back) inside the timed region. L2 is flushed between steps.

--impl reference runs the CPU restatement of the reference (oracle/, all host
threads) on a bounded sample of the same workload and prints its own line.
Under torchrun (N > 1) every rank runs an independent replica (the path does not
shard); rank 0 prints, with the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
import __graft_entry__ as graft  # noqa: E402



def load_synthetic():
    """The workloads' integral generator (2022-qpesim_gb300/synthetic.py, numpy
    only), loaded from its file on its own, so that the reference arm draws the
    same integrals without importing the package or loading its library."""
    name = "qpe_workload_synthetic"
    mod = sys.modules.get(name)
    if mod is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location(name, ROOT / "2022-qpesim_gb300" / "synthetic.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return mod

WORKLOADS = {
    # Plain QPE in FP64: n = 16, N = 8, 10 ancilla qubits (the default workload).
    "plain-n16": dict(n=16, N=8, P=10, dt=0.05, order=2, steps=4, dtype="c128", seed=0,
                      desc="Plain QPE, FP64: n=16 spin-orbitals, N=8, 10 ancilla qubits, complex128, 2nd-order "
                           "Trotter dt=0.05, 4 steps per power, Hartree-Fock start"),
    # The reference's own CPU-runnable case: n = 8, N = 4, 6 ancilla qubits (a parity case).
    "plain-n8": dict(n=8, N=4, P=6, dt=0.1, order=1, steps=1, dtype="c128", seed=0,
                     desc="Plain QPE, FP64: n=8, N=4, 6 ancilla qubits, 1st-order Trotter dt=0.1"),
}
# The batching form: 256 Hamiltonians of n = 12..20.
WORKLOADS["batched-256"] = dict(batch=True, count=256, sizes=(12, 14, 16, 18, 20), P=6, dt=0.05, order=1, steps=1,
                                dtype="c64", seed=2024, check_c128=True,
                                desc="Batching form: 256 seeded Hamiltonians, n uniform in {12,14,16,18,20}, N=n/2 "
                                     "(odd N split ceil/floor over the spins), 6 ancilla qubits, complex64 with FP64 "
                                     "coefficients and histograms, 1st-order Trotter dt=0.05, Hartree-Fock starts, "
                                     "one graph launch per step")
# The precision form: one n = 24, N = 12 instance in complex64.
WORKLOADS["precision-n24"] = dict(n=24, N=12, P=8, dt=0.05, order=1, steps=1, dtype="c64", seed=0, check_c128=True,
                                  desc="Precision form: n=24, N=12 (853,776 amplitudes per block in the reference's "
                                       "Na=Nb layout), 8 ancilla qubits, complex64 state with FP64 coefficients, "
                                       "block norms and histogram, 1st-order Trotter dt=0.05, Hartree-Fock start; "
                                       "error stated against a complex128 run of the same program")
# A 32-instance draw of the batching form's distribution: the case the batched
# kernels are profiled on (same shapes per class, fewer members per launch).
WORKLOADS["batched-32"] = dict(WORKLOADS["batched-256"], count=32,
                               desc="Batching form, 32-instance draw (profiling case): n uniform in "
                                    "{12,14,16,18,20}, N=n/2, 6 ancilla qubits, complex64, dt=0.05")
# The learned initial-state form: n = 20, N = 10.
WORKLOADS["learned-n20"] = dict(learned=True, n=20, N=10, P=10, P_data=8, dt=0.05, tau=1e-3, train=512, held_out=64,
                                train_steps=3000, batch=65536, lr=1e-3, seed=31337, dtype="c64",
                                desc="Learned initial state: n=20, N=10 (63,504 amplitudes per block in the "
                                     "reference's Na=Nb layout), 10 ancilla qubits for evaluation; MLP (20 occupation "
                                     "bits + 2 diagonal-energy features of the string under its Hamiltonian) -> 3 x 256 "
                                     "GELU -> (log|a|, phase), BF16 tensor-core training on the post-selected ground "
                                     "projections of 512 seeded Hamiltonians (QPE with 8 ancilla qubits from each "
                                     "Hamiltonian's lowest-diagonal determinant, complex64), evaluated on 64 held-out "
                                     "seeds against Hartree-Fock")
# A small draw of the same form (n=12) for quick checks of the pipeline.
WORKLOADS["learned-n12"] = dict(WORKLOADS["learned-n20"], n=12, N=6, P=8, train=64, held_out=16, train_steps=600,
                                batch=8192, desc="Learned initial state, small check: n=12, N=6, 64 training and "
                                                 "16 held-out seeds, 8 ancilla qubits")
DEFAULT_WORKLOAD = "plain-n16"

# DRAM bytes per launch of the dominant kernel (dram__bytes_read.sum +
# dram__bytes_write.sum) from the ncu captures summarised under profiles/.
MEASURED_TRAFFIC = {
    "plain-n16": (25_823_744, "k_resident_lean with update-unit windows, cluster of 16: one launch runs every "
                              "power; the capture of a 2-power launch read the block, the program and the warp "
                              "programs of the column-pair windows once (25.8 MB, then L2-resident) and wrote "
                              "nothing back to DRAM, the snapshots staying in L2 (ncu capture of the same kernel, "
                              "small case)"),
    "precision-n24": (3_810_000, "k_pass MIX launch, one tile per CTA, pass image in shared memory: DRAM reads "
                                 "of a cold-cache ncu capture at P = 3 (3.79-3.82 MB; the 6.8 MB working block is "
                                 "the same at any P, and a MIX pass touches its column pairs, about half of it)"),
    "batched-256": (16_650_000, "k_pass MIX launch: 2.08 MB for the 32-instance draw (cold-cache ncu capture), "
                                "scaled by the 8x members per launch"),
}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


DATA_NOTE = ("synthetic: seeded integrals (h_pq ~ N(0,1) exp(-|p-q|/2), (pq|rs) ~ N(0,0.1^2) "
             "exp(-(|p-q|+|r-s|)/3)), Hartree-Fock start, one replica per rank")


def workload_config(args, w, touches_per_power, ws):
    """The `config` object of a single-instance workload, identical in both arms."""
    M, na, P = w["n"] // 2, w["N"] // 2, w["P"]
    npow = (1 << P) - 1
    if getattr(args, "powers", 0):
        npow = min(npow, args.powers)
    cfg = {"workload": args.workload, "description": w["desc"], "n_spin_orbitals": w["n"], "electrons": w["N"],
           "precision": P, "dt": w["dt"], "trotter_order": w["order"], "steps_per_power": w["steps"],
           "state": w["dtype"], "amps_per_block": math.comb(M, na) ** 2, "blocks": 1 << P,
           "touches_per_power": int(touches_per_power), "touches_per_step": int(touches_per_power) * npow,
           "l2": "flushed before every timed step (256 MiB write)", "parallelism": f"replicas x{ws}"}
    if getattr(args, "powers", 0):
        cfg["powers_evolved"] = npow
    if getattr(args, "precision", 0):
        cfg["precision_override"] = args.precision
    return cfg


def measure_fp64_peak(N, ctx):
    """The device's FP64 FMA throughput in TFLOP/s, measured live by the library's
    probe (qpe_measure_fp64_peak: 8 independent FMA chains per thread, 4 CTAs of
    256 threads per SM, CUDA events)."""
    import ctypes
    v = ctypes.c_double()
    N.check(N.lib().qpe_measure_fp64_peak(ctx, ctypes.byref(v)))
    return v.value


GB300_SMS = 152  # the SMs of one GB300 (the only target)


def roofline_single(w, achieved, peak, peak_kind, kernel, touches_step, ev_s, fp64_peak, cluster_sms=0,
                    num_sms=GB300_SMS):
    """Roofline object of a single-instance workload. achieved is the algorithmic
    HBM figure (2 * sizeof(amplitude) per touch over the evolution time); `bound`
    names the resource that limits the dominant kernel, as measured."""
    r = {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
         "peak_source": peak_kind, "peak_note": f"{peak_kind} HBM copy bandwidth (MEASURED_PEAKS.json hbm_gbs)",
         "kernel": kernel}
    if w["dtype"] == "c128":
        ops = touches_step * 6 / ev_s / 1e12  # 6 FP64 DMUL / DADD per touch, no FMA (reference rounding)
        r["bound"] = "latency"
        r["bound_note"] = ("pass latency: every controlled power is a chain of dependent passes (a cluster "
                           "barrier each) whose terms are chains of dependent FP64 operations on one block "
                           "held in the cluster's shared memory; DRAM moves only the snapshots (traffic below), "
                           "and FP64 issue is a small fraction of the live-measured peak (fp64)")
        r["fp64"] = {"achieved_tflops": ops, "peak_fma_tflops": fp64_peak,
                     "frac_of_fma_peak": ops / fp64_peak if fp64_peak else None,
                     "frac_of_issue_rate": 2 * ops / fp64_peak if fp64_peak else None,
                     "frac_of_cluster_issue_rate": (2 * ops / (fp64_peak * cluster_sms / num_sms)
                                                    if fp64_peak and cluster_sms else None),
                     "cluster_sms": cluster_sms,
                     "ops_per_touch": 6,
                     "peak_method": "measured live in this run by qpe_measure_fp64_peak (an FMA counts 2 FLOP; "
                                    "the path issues DMUL and DADD, so its ceiling is half the FMA FLOP/s: "
                                    "frac_of_issue_rate)"}
    else:
        r["bound"] = "latency"
        r["bound_note"] = ("L2 latency: the complex64 working block stays in L2 across the passes, so the "
                           "tile passes wait on L2 round trips; the algorithmic HBM figure is a ceiling "
                           "reference, not the binding resource")
    return r


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("LOCAL_RANK", "0"), "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        finally:
            os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": float(rows[0][2]) if rows else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def setup_dist(backend="nccl"):
    """Replicas: one process per GPU (RANK / LOCAL_RANK / WORLD_SIZE from the
    launcher); the only collectives are the timing barrier and the max of the
    per-rank times. backend "gloo" runs the same host logic on CPU."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return rank, ws, local
    return 0, 1, 0


def reduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def build_problem(q, w, seed_offset=0):
    ints = q.synthetic_integrals(w["n"], w["seed"] + seed_offset)
    # A second-order step applies two half steps: coefficients at dt / 2.
    t = w["dt"] / 2 if w["order"] == 2 else w["dt"]
    h = q.Hamiltonian.from_integrals(ints, w["N"] // 2, t)
    return h, h.segmented_terms()


def oracle_terms(orc, w, n, n_alpha, seed):
    """The workload's segmented terms from the oracle's own term compiler (the
    reference's, restated in oracle/terms_oracle.cc): seeded synthetic integrals,
    coefficients at dt (first order) or dt / 2 (each sweep of a second-order step)."""
    ints = load_synthetic().synthetic_integrals(n, seed)
    t = w["dt"] / 2 if w["order"] == 2 else w["dt"]
    return orc.segmented_terms(n // 2, n_alpha, t, ints.one_body, ints.two_body)


def thread_choices():
    n = os.cpu_count() or 1
    return sorted({1, 2, 4, 8, n} & set(range(1, n + 1)))


def choose_threads(orc, run_powers, trial_powers=2):
    """The host thread count the CPU evolution runs fastest with: every count in
    thread_choices() times `trial_powers` controlled powers (run_powers(k) evolves
    k powers); returns (threads, seconds per power at that count)."""
    best = None
    for th in thread_choices():
        orc.set_threads(th)
        t0 = time.perf_counter()
        run_powers(trial_powers)
        per = (time.perf_counter() - t0) / trial_powers
        if best is None or per < best[1]:
            best = (th, per)
    orc.set_threads(best[0])
    return best


def cpu_baseline(orc, w, seg, budget_s=15.0):
    """The oracle (CPU restatement of the reference, liborc_fast.so) on a bounded
    sample of the workload: as many controlled powers as fit in about budget_s,
    at the fastest host thread count. Returns (touches/s, threads, sample dict)."""
    M, e, P = w["n"] // 2, w["N"] // 2, w["P"]
    C2 = math.comb(M, e) ** 2
    touches = orc.touches_per_power(M, e, e, seg, w["order"], w["steps"])
    total = (1 << P) - 1
    state = np.zeros((1 << P) * C2, np.complex128)
    state[0] = 2 ** (-P / 2)

    def run_powers(k):
        orc.time_evolve(M, e, e, P, seg, state, order=w["order"], steps=w["steps"], first=1, last=1 + k)

    threads, per_power = choose_threads(orc, run_powers)
    npow = int(max(1, min(total, budget_s / max(per_power, 1e-9))))
    t0 = time.perf_counter()
    run_powers(npow)
    el = time.perf_counter() - t0
    return touches * npow / el, threads, {
        "powers_sampled": npow, "powers_total": total, "seconds": el, "threads": threads,
        "thread_choices": thread_choices(), "touches_per_power": touches,
        "what": f"{npow} of {total} controlled powers of the same workload from the Hartree-Fock start "
                f"({el:.1f} s, {threads} thread(s), fastest of {thread_choices()}); QIFT excluded"}


def run_ours(args, w, rank, ws, local):
    q = graft.load_package()
    N = q._native
    h, seg = build_problem(q, w, seed_offset=rank)
    M, e, P = w["n"] // 2, w["N"] // 2, w["P"]
    dtype = np.complex128 if w["dtype"] == "c128" else np.complex64
    prog = q.Program(seg, M, e, e, trotter_order=w["order"], steps=w["steps"], device=local)
    st = q.DeviceState(M, e, e, P, dtype=dtype, device=local)
    npow = (1 << P) - 1
    if args.powers:  # profiling runs: the first `powers` controlled powers only
        npow = min(npow, args.powers)
    touches_step = prog.touches_per_power * npow
    block0 = q.hf_block0(st.c_alpha, st.c_beta, P, dtype)
    ctx = N.context(local)
    timer = N.Timer(local)
    lib = N.lib()

    def evolve():
        st.evolve(prog, 1, 1 + npow, strategy=args.strategy, cluster_size=args.cluster,
                  replicas=getattr(args, "replicas", 0))

    def step():
        evolve()
        st.qift()
        return st.phase_probs()

    st.upload(block0)
    for _ in range(args.warmup):
        st.upload(block0)
        step()
    barrier(ws)
    clocks = Clocks()
    clocks.start()
    total_ms, evolve_ms = 0.0, 0.0
    for _ in range(args.steps):
        st.upload(block0)
        N.check(lib.qpe_flush_l2(ctx))
        timer.record(0)
        evolve()
        timer.record(1)
        st.qift()
        probs = st.phase_probs()
        timer.record(2)
        total_ms += timer.elapsed_ms(0, 2)
        evolve_ms += timer.elapsed_ms(0, 1)
    clk = clocks.stop()
    total_ms = reduce_max(total_ms, ws)
    barrier(ws)

    # End to end through host buffers: block 0 in from page-locked memory, the
    # whole register and the histogram back.
    pin_in = N.PinnedBuffer(st.ld, dtype)
    pin_in.array[:] = block0
    pin_out = N.PinnedBuffer(st.size, dtype)
    probs_host = np.zeros(1 << P)
    e2e_ms = 0.0
    for _ in range(args.steps):
        N.check(lib.qpe_flush_l2(ctx))
        timer.record(3)
        st.upload(pin_in.array)
        evolve()
        st.qift()
        probs_host[:] = st.phase_probs()
        st.download(out=pin_out.array)
        timer.record(4)
        e2e_ms += timer.elapsed_ms(3, 4)
    e2e_ms = reduce_max(e2e_ms, ws)

    ms_step = total_ms / args.steps
    value = touches_step * ws / (ms_step / 1e3)
    e2e_value = touches_step * ws / (e2e_ms / args.steps / 1e3)
    # Roofline of the dominant kernel family (the tile-pass kernels of the
    # evolution): algorithmic bytes 2 * sizeof(amplitude) per update.
    bpt = 32 if w["dtype"] == "c128" else 16
    ev_s = evolve_ms / args.steps / 1e3
    achieved = touches_step * bpt / ev_s / 1e9
    peak, peak_kind = peaks()
    info = prog.info
    strat, kc = st.last_strategy()
    nrep = st.last_replicas()
    fp64_peak = measure_fp64_peak(N, ctx) if w["dtype"] == "c128" else None
    if strat == 3:
        kernel = "k_pass (evolution tile passes, one launch per pass)"
        launches = args.steps * (npow * (info["num_passes_per_power"] + 2) + 1 + 2 + 1)
    else:
        kname = {4: "k_resident_group", 6: "k_resident_lean", 7: "k_resident_lean"}.get(strat, "k_resident")
        extra = {5: ", column pairs by four-warp groups",
                 7: ", column-pair passes as windows of independent update units"}.get(strat, "")
        if nrep > 1:
            extra += f", {nrep} replica clusters splitting the row and column passes"
        kernel = f"{kname} (whole evolution in one launch, cluster of {kc} CTA(s){extra})"
        launches = args.steps * (1 + 2)
    strategy_name = {1: "resident (one CTA)", 2: f"cluster of {kc} CTAs", 3: "tiled passes",
                     4: f"cluster of {kc} CTAs, four-warp tile groups",
                     5: f"cluster of {kc} CTAs, column-pair tiles by four-warp groups",
                     6: f"cluster of {kc} CTAs, every tile by a three-warp group",
                     7: f"cluster of {kc} CTAs, three-warp groups, column-pair passes as windows of "
                        f"independent update units" + (f", {nrep} replica clusters" if nrep > 1 else "")}.get(strat, "?")
    line = {
        "metric": "amplitude-term updates/s per Trotter step",
        "value": value,
        "unit": "touches/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if w["dtype"] == "c128" else "f32",
        "data": DATA_NOTE,
        "config": workload_config(args, w, prog.touches_per_power, ws),
        "kernel_strategy": strategy_name,
        "roofline": roofline_single(w, achieved, peak, peak_kind, kernel, touches_step, ev_s, fp64_peak,
                                    cluster_sms=kc * nrep if strat in (2, 4, 5, 6, 7) else (1 if strat == 1 else 0)),
        "e2e": {"value": e2e_value, "unit": "touches/s",
                "h2d_bytes_per_step": int(st.ld * dtype().itemsize),
                "d2h_bytes_per_step": int(st.size * dtype().itemsize + (1 << P) * 8)},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if args.workload in MEASURED_TRAFFIC:
        line["roofline"]["traffic"], line["roofline"]["traffic_note"] = MEASURED_TRAFFIC[args.workload]
    if w.get("check_c128") and not args.powers:
        line["precision_check"] = precision_check(q, w, seg, st, prog, block0, local)
    if rank == 0 and not args.no_cpu_baseline:
        orc = graft.load_oracle().Oracle(fast=True)
        rate, threads, sample = cpu_baseline(orc, w, seg)
        line["cpu_baseline"] = {"value": rate, "unit": "touches/s", "cores": threads, "kind": "port",
                                "sample": sample["what"], "powers_sampled": sample["powers_sampled"],
                                "powers_total": sample["powers_total"]}
    return line


def precision_check(q, w, seg, st, prog, block0, device):
    """The complex64 register against a complex128 run of the same program (after
    the timed steps, outside the timing): amplitude error after the evolution, the
    phase histogram after the QIFT, and the phase / energy estimates read from
    each (FP64 readout on both)."""
    M, e, P = w["n"] // 2, w["N"] // 2, w["P"]
    ref = q.DeviceState(M, e, e, P, dtype=np.complex128, device=device)
    ref.upload(block0.astype(np.complex128))
    ref.evolve(prog)
    st.upload(block0)
    st.evolve(prog)
    norms64, norms128 = st.block_norms(), ref.block_norms()
    a64 = st.download().astype(np.complex128)
    a128 = ref.download()
    amp_err = float(np.max(np.abs(a64 - a128)))
    rel_l2 = float(np.linalg.norm(a64 - a128) / np.linalg.norm(a128))
    del a64, a128
    st.qift()
    ref.qift()
    p64, p128 = st.phase_probs(), ref.phase_probs()
    ph64, ph128 = q.subbin_phase(p64), q.subbin_phase(p128)
    return {"against": "complex128 run of the same program on the GPU (bit-identical to the FP64 oracle "
                       "at the parity sizes)",
            "max_abs_amplitude_error": amp_err, "relative_l2_error": rel_l2,
            "max_block_norm_drift_c64": float(np.max(np.abs(norms64 - norms64[0]))),
            "max_block_norm_drift_c128": float(np.max(np.abs(norms128 - norms128[0]))),
            "histogram_l1_error": float(np.sum(np.abs(p64 - p128))),
            "argmax_bin": [int(np.argmax(p64)), int(np.argmax(p128))],
            "reference_phase_estimate": [q.reference_phase(p64), q.reference_phase(p128)],
            "subbin_phase_estimate": [ph64, ph128], "subbin_phase_error": abs(ph64 - ph128),
            "energy_error_ha": abs(q.phase_to_energy(ph64, w["dt"]) - q.phase_to_energy(ph128, w["dt"]))}


def batch_instances(w, rank=0):
    """(n, N, seed) of every instance of a batched workload."""
    rng = np.random.default_rng(w["seed"] + 7919 * rank)
    ns = rng.choice(w["sizes"], size=w["count"])
    return [(int(n), int(n) // 2, w["seed"] + 1000 * rank + i) for i, n in enumerate(ns)]


def build_batch_terms(q, w, rank=0):
    """(n, n_alpha, n_beta, segmented terms) of every instance, from the package's
    term compiler (the GPU arm)."""
    out = []
    for n, Nel, seed in batch_instances(w, rank):
        h = q.Hamiltonian.from_integrals(q.synthetic_integrals(n, seed), (Nel + 1) // 2, w["dt"])
        out.append((n, (Nel + 1) // 2, Nel // 2, h.segmented_terms()))
    return out


def build_batch_terms_oracle(orc, w, rank=0):
    """The same instances' terms from the oracle's own term compiler (the
    reference arm; bit-identical to the package's)."""
    return [(n, (Nel + 1) // 2, Nel // 2, oracle_terms(orc, w, n, (Nel + 1) // 2, seed))
            for n, Nel, seed in batch_instances(w, rank)]


def batch_config(args, w, terms, touches_per_step, ws):
    """The `config` object of a batched workload, identical in both arms."""
    sizes = {}
    for n, *_ in terms:
        sizes[str(n)] = sizes.get(str(n), 0) + 1
    return {"workload": args.workload, "description": w["desc"], "instances": len(terms),
            "instances_per_n": dict(sorted(sizes.items(), key=lambda kv: int(kv[0]))), "precision": w["P"],
            "dt": w["dt"], "trotter_order": w["order"], "steps_per_power": w["steps"], "state": w["dtype"],
            "touches_per_step": int(touches_per_step), "l2": "flushed before every timed step (256 MiB write)",
            "parallelism": f"replicas x{ws}"}


def cpu_baseline_batch(orc, w, terms, budget_s=20.0):
    """The oracle on a bounded sample of the batch: one instance of each size, the
    powers that fit in its share of the budget at its fastest host thread count;
    the batch's CPU time is the sum over its instances at those per-size rates.
    Returns (touches/s, max threads used, sample dict)."""
    P = w["P"]
    total = (1 << P) - 1
    rate, cores, parts = {}, {}, []
    sizes = sorted({t[0] for t in terms})
    touches_of = {}
    for n, na, nb, seg in terms:
        key = (n, na, nb, id(seg))
        touches_of[key] = orc.touches_per_power(n // 2, na, nb, seg, w["order"], w["steps"])
    sampled = 0
    for n in sizes:
        n_, na, nb, seg = next(t for t in terms if t[0] == n)
        M = n // 2
        touches = touches_of[(n_, na, nb, id(seg))]
        ld = math.comb(M, na) * math.comb(M, nb)
        state = np.zeros((1 << P) * ld, np.complex128)
        state[0] = 2 ** (-P / 2)

        def run_powers(k):
            orc.time_evolve(M, na, nb, P, seg, state, order=w["order"], steps=w["steps"], first=1, last=1 + k)

        th, per = choose_threads(orc, run_powers, trial_powers=1)
        npow = int(max(1, min(total, budget_s / len(sizes) / max(per, 1e-9))))
        t0 = time.perf_counter()
        run_powers(npow)
        el = time.perf_counter() - t0
        rate[n] = touches * npow / el
        cores[n] = th
        sampled += npow
        parts.append(f"n={n}: {npow} powers, {th} thread(s), {rate[n] / 1e6:.0f} M/s")
    total_t, total_touch = 0.0, 0
    for n, na, nb, seg in terms:
        tp = touches_of[(n, na, nb, id(seg))] * total
        total_touch += tp
        total_t += tp / rate[n]
    return total_touch / total_t, max(cores.values()), {
        "what": "one instance per size, one at a time, fastest of " + str(thread_choices()) + " threads: " +
                "; ".join(parts), "powers_sampled": sampled, "powers_total": total * len(terms),
        "touches_per_step": total_touch}


def batch_phase_check(q, progs, P, b0, probs64, device):
    """Every instance's eigenphase from the complex64 batch against a complex128
    batch of the same programs (the plain FP64 path: bit-identical to the oracle
    per instance), after the timed steps. Phases are the sub-bin estimates of the
    histograms, in turns (fractions of 2 pi)."""
    ref = q.Batch(progs, P, dtype=np.complex128, device=device)
    for i, a in enumerate(b0):
        ref.upload(i, a.astype(np.complex128))
    ref.run()
    d = []
    same_bin = 0
    for i in range(len(progs)):
        p128 = ref.phase_probs(i)
        p64 = probs64[i]
        same_bin += int(np.argmax(p64) == np.argmax(p128))
        dp = abs(q.subbin_phase(p64) - q.subbin_phase(p128))
        d.append(min(dp, 1.0 - dp))
    d = np.array(d)
    return {"against": "complex128 batch of the same programs on the GPU (the plain FP64 path)",
            "instances": len(progs), "same_argmax_bin": same_bin,
            "max_phase_error_turns": float(d.max()), "max_phase_error_rad": float(2 * np.pi * d.max()),
            "median_phase_error_rad": float(2 * np.pi * np.median(d))}


def run_batch(args, w, rank, ws, local):
    q = graft.load_package()
    N = q._native
    P = w["P"]
    dtype = np.complex64 if w["dtype"] == "c64" else np.complex128
    terms = build_batch_terms(q, w, rank)
    progs = [q.Program(seg, n // 2, na, nb, trotter_order=w["order"], steps=w["steps"], device=local)
             for n, na, nb, seg in terms]
    bt = q.Batch(progs, P, dtype=dtype, device=local)
    bt.tune()
    info = bt.info
    timer = N.Timer(local)
    lib = N.lib()
    ctx = N.context(local)
    b0 = [q.hf_block0(math.comb(n // 2, na), math.comb(n // 2, nb), P, dtype) for n, na, nb, _ in terms]

    def upload_all(src):
        for i, a in enumerate(src):
            bt.upload(i, a)

    for _ in range(args.warmup):
        upload_all(b0)
        bt.run()
    info = bt.info  # the launch count is known once the graph exists
    barrier(ws)
    clocks = Clocks()
    clocks.start()
    total_ms = 0.0
    for _ in range(args.steps):
        upload_all(b0)
        N.check(lib.qpe_flush_l2(ctx))
        timer.record(0)
        bt.run(synchronize=False)
        timer.record(1)
        total_ms += timer.elapsed_ms(0, 1)
    clk = clocks.stop()
    total_ms = reduce_max(total_ms, ws)
    barrier(ws)
    # End to end: block 0 of every instance in from page-locked memory, every
    # histogram back.
    pins = []
    for a in b0:
        pb = N.PinnedBuffer(a.size, dtype)
        pb.array[:] = a
        pins.append(pb)
    probs = np.zeros((len(terms), 1 << P))
    e2e_ms = 0.0
    for _ in range(args.steps):
        N.check(lib.qpe_flush_l2(ctx))
        timer.record(2)
        upload_all([p.array for p in pins])
        bt.run(synchronize=False)
        for i in range(len(terms)):
            probs[i] = bt.phase_probs(i)
        timer.record(3)
        e2e_ms += timer.elapsed_ms(2, 3)
    e2e_ms = reduce_max(e2e_ms, ws)
    touches = info["touches_per_run"]
    ms_step = total_ms / args.steps
    value = touches * ws / (ms_step / 1e3)
    peak, peak_kind = peaks()
    achieved = touches * 16 / (ms_step / 1e3) / 1e9
    line = {
        "metric": "amplitude-term updates/s per Trotter step", "value": value, "unit": "touches/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": DATA_NOTE.replace(
            "Hartree-Fock start", "one seed per instance, Hartree-Fock starts"),
        "config": batch_config(args, w, terms, touches, ws),
        "classes": info["classes"],
        "roofline": {"bound": "latency", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": peak_kind,
                     "peak_note": f"{peak_kind} HBM copy bandwidth (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": "k_pass (batched tile passes), 16 algorithmic bytes per touch over the whole run",
                     "bound_note": "every class's complex64 working blocks stay in L2 across the passes; the tile "
                                   "passes wait on L2 round trips and per-pass launches, so the algorithmic HBM "
                                   "figure is a ceiling reference, not the binding resource"},
        "e2e": {"value": touches * ws / (e2e_ms / args.steps / 1e3), "unit": "touches/s",
                "h2d_bytes_per_step": int(sum(a.nbytes for a in b0)),
                "d2h_bytes_per_step": int(probs.nbytes)},
        "gpu_launches": int(info["launches_per_run"]) * args.steps,
        "clocks": clk,
    }
    if args.workload in MEASURED_TRAFFIC:
        line["roofline"]["traffic"], line["roofline"]["traffic_note"] = MEASURED_TRAFFIC[args.workload]
    # throughput per instance size: each class (one size) timed alone by the autotuner
    per_size = {}
    for c in bt.classes():
        ms = c["ms_per_power"]
        per_size[str(2 * c["num_orbitals"])] = {
            "instances": c["members"], "electrons": c["n_alpha"] + c["n_beta"],
            "touches_per_power": c["touches_per_power"], "ms_per_power_alone": ms,
            "touches_per_s_alone": c["touches_per_power"] / (ms / 1e3) if ms > 0 else None,
            "tile": {"lines": c["tile_lines"], "warps_per_cta": c["warps_per_cta"]}}
    line["per_size"] = per_size
    if w.get("check_c128") and w["dtype"] == "c64":
        line["precision_check"] = batch_phase_check(q, progs, P, b0, probs, local)
    if rank == 0 and not args.no_cpu_baseline:
        r, cores, sample = cpu_baseline_batch(graft.load_oracle().Oracle(fast=True), w, terms)
        line["cpu_baseline"] = {"value": r, "unit": "touches/s", "cores": cores, "kind": "port",
                                "sample": sample["what"], "powers_sampled": sample["powers_sampled"],
                                "powers_total": sample["powers_total"]}
    return line


def run_reference(args, w, rank, ws):
    """The reference arm: the CPU restatement of the reference's path (oracle/,
    liborc_fast.so) on the host cores, at its fastest thread count, on the same
    workload. It loads neither the package nor its library: the integrals come
    from the workload generator's file, the terms from the oracle's own term
    compiler and the touch counts from the oracle's run tables. Every step is a
    bounded sample of the workload (the first controlled powers from the
    Hartree-Fock start, sized so that the steps end within a few minutes);
    ms_per_step is the sample's own time."""
    if rank != 0:
        return None
    if w.get("learned"):
        return {"impl": "reference", "unavailable": "the reference has no learned initial state (Hartree-Fock "
                                                    "only); the Hartree-Fock arm is part of this workload's own line"}
    orc = graft.load_oracle().Oracle(fast=True)
    per_step_s = max(2.0, 60.0 / max(args.steps, 1))
    if w.get("batch"):
        terms = build_batch_terms_oracle(orc, w)
        r, cores, sample = cpu_baseline_batch(orc, w, terms, budget_s=2.0)  # warm-up and thread choice
        rates, secs = [], []
        for _ in range(args.steps):
            r, cores, sample = cpu_baseline_batch(orc, w, terms, budget_s=per_step_s)
            rates.append(r)
            secs.append(per_step_s)
        value = statistics.median(rates)
        touches = sample["touches_per_step"]
        cfg = batch_config(args, w, terms, touches, ws)
        what = sample["what"]
        sampled, total = sample["powers_sampled"], sample["powers_total"]
    else:
        seg = oracle_terms(orc, w, w["n"], w["N"] // 2, w["seed"])
        cpu_baseline(orc, w, seg, budget_s=1.0)  # warm-up
        rates, secs = [], []
        for _ in range(args.steps):
            r, cores, sample = cpu_baseline(orc, w, seg, budget_s=per_step_s)
            rates.append(r)
            secs.append(sample["seconds"])
        value = statistics.median(rates)
        cfg = workload_config(args, w, sample["touches_per_power"], ws)
        touches = cfg["touches_per_step"]
        what = sample["what"]
        sampled, total = sample["powers_sampled"], sample["powers_total"]
    ms_step = statistics.median(secs) * 1e3
    return {"metric": "amplitude-term updates/s per Trotter step", "value": value, "unit": "touches/s",
            "impl": "reference", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (the same integrals as the GPU arm, from the same generator)",
            "config": cfg,
            "sample_per_step": {"powers_sampled": sampled, "powers_total": total,
                                "extrapolated_ms_per_full_step": touches / value * 1e3,
                                "note": "each step evolves a bounded sample of the workload's controlled powers; "
                                        "value is the sample's throughput, ms_per_step the sample's time"},
            "cpu_baseline": {"value": value, "unit": "touches/s", "cores": cores, "kind": "port",
                             "sample": what + "; CPU restatement of the reference (oracle/qpe_oracle.cc, "
                                              "oracle/terms_oracle.cc), complex128 (the reference has no complex64 "
                                              "path); the reference's own build needs its sources, which a GPU host does not have"},
            "e2e": {"value": value, "unit": "touches/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_learned(args, w, rank, ws, local):
    """The learned-state form end to end.

    1. Training data from the simulator itself: a batched QPE run (complex64,
       P_data ancilla qubits) of every training Hamiltonian from its determinant
       of lowest diagonal energy; the histogram's lowest-energy peak picks the
       ground bin and that block of the QIFT'd register, normalised, is the
       post-selected ground projection.
    2. BF16 training of the model on the tensor cores.
    3. The learned start of every held-out Hamiltonian, chosen without the
       answer: the model proposes its state and cuts of it to its m largest
       amplitudes (learned_candidates); the lowest variational energy among them
       (one short GPU evolution each, all in one batched launch) is the learned
       start, which is run if its energy is below Hartree-Fock's; Hartree-Fock
       stays the fallback whenever the proposal loses.
    4. One batched QPE run (P ancilla qubits) per held-out Hamiltonian from four
       starts: Hartree-Fock, the learned start, the lowest-diagonal determinant
       (a classical reference that needs no training) and the model's uncut
       proposal. The ground bin is the lowest-energy peak over the four
       histograms; success is each start's mass in that bin +- 1; the overlap is
       with the post-selected ground projection of the start with the largest
       success; the time to 1e-3 Ha is the textbook QPE cost
       (qpe_time_to_precision) at the measured GPU time per controlled power."""
    q = graft.load_package()
    N = q._native
    L = q.learned_state
    M, na, nb = w["n"] // 2, w["N"] // 2, w["N"] - w["N"] // 2
    dt, Pd, P, tau = w["dt"], w["P_data"], w["P"], w["tau"]
    strings = L.register_strings(M, na, nb)
    ld = len(strings)
    timer = N.Timer(local)

    def hams(seeds, t):
        return [q.Hamiltonian.from_integrals(q.synthetic_integrals(w["n"], s), na, t) for s in seeds]

    base = w["seed"] + 100000 * rank
    train_seeds = [base + i for i in range(w["train"])]
    eval_seeds = [base + 50000 + i for i in range(w["held_out"])]
    t0 = time.perf_counter()
    # 1. post-selected ground projections of the training Hamiltonians
    th = hams(train_seeds, dt)
    progs = [q.Program(h.segmented_terms(), M, na, nb, device=local) for h in th]
    tfeats = [L.diagonal_features(h, strings) for h in th]
    bt = q.Batch(progs, Pd, dtype=np.complex64, device=local)
    for i, h in enumerate(th):
        bt.upload(i, (L.lowest_diagonal_state(h, strings) * 2.0 ** (-Pd / 2)).astype(np.complex64))
    timer.record(0)
    bt.run()
    timer.record(1)
    data_ms = timer.elapsed_ms(0, 1)
    la, ph, wt = [], [], []
    for i in range(len(progs)):
        j0 = L.ground_bin(bt.phase_probs(i), dt)
        a, b, c = L.state_targets(bt.download(i, first=j0 * ld, count=ld))
        la.append(a)
        ph.append(b)
        wt.append(c)
    del bt, progs
    data_s = time.perf_counter() - t0
    # 2. training on the tensor cores
    model = L.AmplitudeMLP(w["n"], batch=w["batch"], seed=w["seed"], device=local, n_feat=L.N_DIAG_FEATURES)
    model.set_data(np.concatenate([strings] * len(th)), np.concatenate(la), np.concatenate(ph), np.concatenate(wt),
                   np.concatenate(tfeats))
    model.train(20, lr=w["lr"], seed=1)  # warm-up
    t1 = time.perf_counter()
    losses = model.train(w["train_steps"], lr=w["lr"], seed=2)
    train_s = time.perf_counter() - t1
    tflops = model.tensor_flops_per_step() * w["train_steps"] / train_s / 1e12
    # 3. the starts of every held-out Hamiltonian and the choice without the answer
    eh = hams(eval_seeds, dt)
    eprogs = [q.Program(h.segmented_terms(), M, na, nb, device=local) for h in eh]
    ptau = [q.Program(h.segmented_terms(), M, na, nb, device=local) for h in hams(eval_seeds, tau)]
    H = len(eh)
    t2 = time.perf_counter()
    psi_hf = np.zeros(ld, np.complex128)
    psi_hf[0] = 1.0
    diags = [L.lowest_diagonal_state(h, strings) for h in eh]
    fulls, cands, owner, flat = [], [], [], []
    for i, h in enumerate(eh):
        full = L.proposed_state(model, strings, L.diagonal_features(h, strings))
        fulls.append(full)
        c = L.learned_candidates(full)
        cands.append(c)
        for x in [psi_hf, diags[i]] + c:
            owner.append(i)
            flat.append(x)
    ev_flat = L.variational_energies([ptau[o] for o in owner], flat, tau, device=local)
    choose_s = (time.perf_counter() - t2) / H
    starts, evar, picked = [], [], []
    pos = 0
    for i in range(H):
        k = len(cands[i])
        e_hf, e_dg, e_c = ev_flat[pos], ev_flat[pos + 1], ev_flat[pos + 2:pos + 2 + k]
        pos += 2 + k
        sel = int(np.argmin(e_c))
        picked.append(0 if sel == 0 else L.CANDIDATE_TRUNCATIONS[sel - 1])
        starts.append((psi_hf, cands[i][sel], diags[i], fulls[i]))
        evar.append((float(e_hf), float(e_c[sel]), float(e_dg), float(e_c[0])))
    # 4. QPE from the four starts in one batched launch
    names = ("hf", "learned", "diagonal", "learned_full")
    ns = len(names)
    bt = q.Batch(eprogs * ns, P, dtype=np.complex64, device=local)
    scale = 2.0 ** (-P / 2)

    def upload_starts():
        for k in range(ns):
            for i in range(H):
                bt.upload(k * H + i, (starts[i][k] * scale).astype(np.complex64))

    upload_starts()
    bt.run()  # warm-up of the graph
    upload_starts()
    timer.record(2)
    bt.run()
    timer.record(3)
    eval_ms = timer.elapsed_ms(2, 3)
    sec_per_power = eval_ms / 1e3 / (ns * H * ((1 << P) - 1))  # one instance's power, batched
    rows = []
    for i in range(H):
        hists = [bt.phase_probs(k * H + i) for k in range(ns)]
        j0 = L.shared_ground_bin(hists, dt)
        succ = [L.window_mass(p, j0) for p in hists]
        best = int(np.argmax(succ))
        g = bt.download(best * H + i, first=j0 * ld, count=ld).astype(np.complex128)
        g /= np.linalg.norm(g)
        ov = [float(abs(np.vdot(g, starts[i][k])) ** 2) for k in range(ns)]
        tt = [L.qpe_time_to_precision(sc, sec_per_power, dt)[0] for sc in succ]
        use_l = evar[i][1] < evar[i][0]
        r = {f"{nm}_{key}": v for key, vals in (("overlap", ov), ("success", succ), ("time_s", tt),
                                                ("energy_var", evar[i])) for nm, v in zip(names, vals)}
        r["learned_chosen"] = use_l
        r["chosen_time_s"] = tt[1] if use_l else tt[0]
        r["chosen_no_slower"] = tt[0] is None or (r["chosen_time_s"] is not None and r["chosen_time_s"] <= tt[0])
        rows.append(r)
    del bt

    def med(key):
        v = [r[key] for r in rows if r[key] is not None]
        return statistics.median(v) if v else None

    gain = [r["hf_time_s"] / r["chosen_time_s"] for r in rows if r["hf_time_s"] and r["chosen_time_s"]]
    value = med("chosen_time_s")
    peaks_d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    bf16_peak = float(peaks_d.get("bf16_tflops", 1900.0))
    bits = L.qpe_time_to_precision(0.5, sec_per_power, dt)[2]
    return {
        "metric": "time to 1e-3 Ha QPE, learned (Hartree-Fock fallback) vs Hartree-Fock", "value": value, "unit": "s",
        "n_gpus": ws, "steps": 1, "warmup": 1, "ms_per_step": eval_ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 model, complex64 register",
        "data": f"synthetic: seeded integrals, {w['train']} training and {w['held_out']} held-out seeds",
        "config": {"workload": args.workload, "description": w["desc"], "train_hamiltonians": w["train"],
                   "held_out": w["held_out"], "precision": P, "precision_data": Pd, "dt": dt, "tau": tau,
                   "train_steps": w["train_steps"], "batch": w["batch"], "lr": w["lr"]},
        "learned": {"median_time_hf_s": med("hf_time_s"), "median_time_learned_s": med("learned_time_s"),
                    "median_time_diagonal_s": med("diagonal_time_s"), "median_time_chosen_s": value,
                    "median_speedup_chosen_over_hf": statistics.median(gain) if gain else None,
                    "median_overlap_hf": med("hf_overlap"), "median_overlap_learned": med("learned_overlap"),
                    "median_overlap_diagonal": med("diagonal_overlap"),
                    "median_overlap_learned_full": med("learned_full_overlap"),
                    "median_success_hf": med("hf_success"), "median_success_learned": med("learned_success"),
                    "median_success_diagonal": med("diagonal_success"),
                    "median_success_learned_full": med("learned_full_success"),
                    "learned_cut_picked": {str(m): int(sum(1 for x in picked if x == m)) for m in sorted(set(picked))},
                    "learned_chosen": int(sum(r["learned_chosen"] for r in rows)), "held_out": len(rows),
                    "learned_beats_hf_success": int(sum(r["learned_success"] > r["hf_success"] for r in rows)),
                    "learned_beats_diagonal_success": int(sum(r["learned_success"] > r["diagonal_success"]
                                                              for r in rows)),
                    "chosen_no_slower_than_hf": int(sum(r["chosen_no_slower"] for r in rows)),
                    "qpe_bits_for_1e-3_ha": bits, "gpu_seconds_per_power": sec_per_power,
                    "choice_seconds_per_hamiltonian": choose_s,
                    "loss_first": float(losses[:10].mean()), "loss_last": float(losses[-10:].mean()),
                    "data_generation_s": data_s, "data_qpe_gpu_ms": data_ms, "training_s": train_s},
        "roofline": {"bound": "latency", "achieved": tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                     "frac": tflops / bf16_peak, "traffic": None,
                     "kernel": "k_gemm (tcgen05 BF16, a training step of 11 GEMMs of a 150k-parameter model plus "
                               "elementwise kernels)",
                     "bound_note": "each GEMM of the small model is a few microseconds of tensor work; a step is "
                                   "bound by its chain of dependent launches"},
        "target": "the ground bin shared by the four starts' histograms; overlap with the post-selected ground "
                  "projection of the start with the largest success; time from the textbook QPE cost model",
    }


FORMS = ("precision-n24", "batched-256")


def run_forms(args, rank, ws, local):
    """The precision and batching forms, run after the headline workload in the
    same command, each with its own line (value, e2e, roofline, cpu_baseline,
    precision_check; per_size for the batch). They time min(steps, 5) steps after
    3 warm-up steps, so that the default run stays within minutes."""
    out = {}
    for name in FORMS:
        a = argparse.Namespace(**vars(args))
        a.workload, a.steps, a.warmup = name, min(args.steps, 5), 3
        a.strategy, a.cluster, a.powers, a.precision = 0, 0, 0, 0
        fw = dict(WORKLOADS[name])
        out[name] = run_batch(a, fw, rank, ws, local) if fw.get("batch") else run_ours(a, fw, rank, ws, local)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--strategy", type=int, default=0,
                    help="0 auto, 1 one-CTA resident, 2 cluster, 3 tiled, 4 cluster with four-warp groups, "
                         "5 cluster with column pairs by four-warp groups, 6 cluster of three-warp groups, "
                         "7 as 6 with column-pair passes as windows of update units")
    ap.add_argument("--cluster", type=int, default=0, help="CTAs per cluster for --strategy 2 (0: smallest)")
    ap.add_argument("--replicas", type=int, default=0,
                    help="replica clusters for --strategy 7 (0 or 1: one; the autotuner picks them with --strategy 0)")
    ap.add_argument("--powers", type=int, default=0,
                    help="evolve only the first K controlled powers (profiling runs; not a workload's figure)")
    ap.add_argument("--precision", type=int, default=0,
                    help="override the ancilla count (profiling runs on a smaller register; not a workload's figure)")
    ap.add_argument("--no-forms", action="store_true",
                    help="with the default workload, skip the nested precision and batching forms")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    rank, ws, local = setup_dist() if args.impl == "ours" else (int(os.environ.get("RANK", "0")),
                                                                 int(os.environ.get("WORLD_SIZE", "1")), 0)
    w = dict(WORKLOADS[args.workload])
    if args.precision:
        w["P"] = args.precision
    if args.impl == "reference":
        line = run_reference(args, w, rank, ws)
    elif w.get("learned"):
        line = run_learned(args, w, rank, ws, local)
    elif w.get("batch"):
        line = run_batch(args, w, rank, ws, local)
    else:
        line = run_ours(args, w, rank, ws, local)
        if (args.workload == DEFAULT_WORKLOAD and not args.no_forms and not args.powers and not args.precision
                and not args.strategy):
            line["forms"] = run_forms(args, rank, ws, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if ws > 1 and args.impl == "ours":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
