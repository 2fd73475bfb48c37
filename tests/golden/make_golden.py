"""Generate tests/golden/*.npz from the oracle (run on x86-64 with the committed oracle).

Each fixture holds the case spec, sha256 digests of the integer maps, the state after
set-up and after `steps` full time steps of iterations.f90:19-87, and the diagnostic
norms (iterations.f90:39-76).  Large states are stored as per-variable L2 norms plus a
strided sample so the fixtures stay small.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "chorus-mhd_gb300"))

import oracle  # noqa: E402
from chorus_mhd import meshgen  # noqa: E402

CASES = {
    "ot_8x8_N4_uniform": (dict(problem="orszag_tang", nx=8, ny=8, N=4), 20),
    "ot_6x6_N3_jitter": (dict(problem="orszag_tang", nx=6, ny=6, N=3, jitter=0.15, seed=2), 12),
    "ot_4x5_N6_jitter": (dict(problem="orszag_tang", nx=4, ny=5, N=6, jitter=0.1, seed=3), 10),
    "ot_5x5_N4_fivestage": (dict(problem="orszag_tang", nx=5, ny=5, N=4, jitter=0.1, seed=4, k_stage=5), 6),
    "ot_6x6_N4_viscous_resistive": (dict(problem="orszag_tang", nx=6, ny=6, N=4, jitter=0.1, seed=5, mu=0.01,
                                         eta0=0.02), 8),
    "alfven_6x5_N4": (dict(problem="alfven", nx=6, ny=5, N=4), 10),
    "rotor_64x64_N3_jitter": (dict(problem="rotor", nx=64, ny=64, N=3, jitter=0.1, seed=6), 5),
}
FULL_LIMIT = 20000  # store the full state below this many doubles
MAPS = ["IF2C", "IC2F", "IF2V", "IBFINTER", "IBFREE", "CYC2FPAIR"]


def summarize(Q):
    q = np.asarray(Q).reshape(-1, 9)
    out = {"norms": np.sqrt((q * q).sum(axis=0)), "sums": q.sum(axis=0)}
    if Q.size <= FULL_LIMIT:
        out["full"] = np.array(Q)
    else:
        out["sample_idx"] = np.arange(0, Q.size, 997, dtype=np.int64)
        out["sample"] = np.array(Q)[out["sample_idx"]]
    return out


def generate(name, spec, steps, tmp):
    d = meshgen.write_case(meshgen.CaseSpec(**spec), os.path.join(tmp, name))
    o = oracle.Oracle(d)
    maps = {m: hashlib.sha256(np.ascontiguousarray(o.array(m)).tobytes()).hexdigest() for m in MAPS}
    q0 = summarize(o.array("Q"))
    diags = []
    for _ in range(steps):
        r = o.step()
        if r is not None:
            diags.append((o.geti("iter"),) + r)
    q1 = summarize(o.array("Q"))
    rec = {"spec": json.dumps(spec), "steps": steps, "maps": json.dumps(maps), "dt": o.getd("dt"),
           "ctime": o.getd("ctime"), "diag": np.array(diags, dtype=np.float64)}
    for k, v in q0.items():
        rec["q0_" + k] = v
    for k, v in q1.items():
        rec["q1_" + k] = v
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    o.close()


def main():
    tmp = tempfile.mkdtemp()
    for name, (spec, steps) in CASES.items():
        generate(name, spec, steps, tmp)
        print("wrote", name)


if __name__ == "__main__":
    main()
