"""Multi-rank helpers on CPU with gloo, world size 2: sharding covers every solve once,
timings reduce to the max over ranks, and ensemble work summed over ranks equals the
single-process total (the oracle stands in for the GPU solve on CPU)."""
import os
import socket
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


SCRIPT = textwrap.dedent("""
    import os, sys, json
    sys.path.insert(0, {root!r}); sys.path.insert(0, os.path.join({root!r}, "chorus-mhd_gb300"))
    from chorus_mhd import dist, ensemble
    world, rank, local = dist.init("gloo")
    specs = ensemble.draw(count=10, lo=4, hi=8, seed=5)
    mine = dist.shard(list(range(len(specs))), world, rank)
    dof = sum(specs[i].nx * specs[i].ny * specs[i].N ** 2 for i in mine)
    total = dist.sum_over_ranks(world, float(dof))
    t = dist.max_over_ranks(world, float(rank + 1))
    dist.barrier(world)
    with open(os.path.join({out!r}, "rank%d.json" % rank), "w") as f:
        json.dump(dict(rank=rank, mine=mine, total=total, tmax=t), f)
""")


@pytest.mark.timeout(300)
def test_two_rank_sharding_and_reductions(tmp_path):
    script = tmp_path / "w.py"
    script.write_text(SCRIPT.format(root=ROOT, out=str(tmp_path)))
    port = _free_port()
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(script)]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=280)
    assert r.returncode == 0, r.stderr[-2000:]
    import json
    outs = [json.loads((tmp_path / ("rank%d.json" % k)).read_text()) for k in range(2)]
    assert len(outs) == 2
    allmine = sorted(sum((o["mine"] for o in outs), []))
    assert allmine == list(range(10))
    from chorus_mhd import ensemble
    specs = ensemble.draw(count=10, lo=4, hi=8, seed=5)
    expect = sum(s.nx * s.ny * s.N ** 2 for s in specs)
    assert all(o["total"] == expect for o in outs)
    assert all(o["tmax"] == 2.0 for o in outs)
