"""The multi-GPU form is replicas only: every rank runs an independent instance
(its own seeds), and the bench's only collectives are a barrier around the timed
region and the maximum of the per-rank times. This runs that host logic with
two gloo ranks on CPU."""
import os
import subprocess
import sys
import textwrap

from conftest import ROOT

SCRIPT = textwrap.dedent("""
    import json, os, sys
    sys.path.insert(0, {root!r})
    import bench
    rank, ws, local = bench.setup_dist("gloo")
    bench.barrier(ws)
    t = bench.reduce_max(10.0 + rank, ws)
    w = bench.WORKLOADS["batched-32"]
    inst = bench.batch_instances(w, rank)
    print(json.dumps({{"rank": rank, "ws": ws, "max": t, "seeds": [s for _, _, s in inst][:4],
                      "sizes": [n for n, _, _ in inst][:4]}}), flush=True)
    import torch.distributed as dist
    dist.destroy_process_group()
""")


def test_two_gloo_replicas(tmp_path):
    script = tmp_path / "replica.py"
    script.write_text(SCRIPT.format(root=str(ROOT)))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT="29541", WORLD_SIZE="2")
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=240)
        assert p.returncode == 0, err[-2000:]
        outs.append(out.strip().splitlines()[-1])
    import json
    a, b = (json.loads(o) for o in outs)
    assert a["ws"] == b["ws"] == 2
    assert a["max"] == b["max"] == 11.0            # max over ranks
    assert set(a["seeds"]).isdisjoint(b["seeds"])  # independent instances per replica
