"""Long-horizon fixtures: the oracle run over each workload's stated number of steps.

    python tests/golden/make_long_golden.py [name ...] [--threads T]

The three single-solve workloads of the metric, run from their initial data for the
number of time steps each is quoted at (the loop of iterations.f90:19-87):

* ``ot_64x64_N4_1000steps``   Orszag-Tang, periodic 64x64 uniform mesh, N = 4, 1000 steps;
* ``rotor_256x256_N4_500steps`` MHD rotor, [0,1]^2 256x256 mesh jittered by +-0.1h (seed 1),
  FREE boundaries, gamma = 1.4, N = 4, 500 steps;
* ``ot_512x512_N5_200steps``  Orszag-Tang, periodic 512x512 mesh jittered by +-0.15h (seed 1),
  N = 5, 200 steps.

A state of these sizes (4.7 to 472 MB) cannot be committed, so each checkpoint keeps

* the per-variable L2 norms and sums of Q (exact up to the summation's rounding);
* a count sketch of Q: K buckets, element i added with sign s(i) into bucket b(i), where
  b and s come from a fixed integer hash of the element index.  The sketch is linear, so
  sketch(Q_a) - sketch(Q_b) = sketch(Q_a - Q_b), and the bucket norm of that difference is
  an unbiased estimate of ||Q_a - Q_b||^2 with relative standard deviation <= sqrt(2/K)
  (K = 2048: 3% in the squared norm, 1.6% in the norm).  A comparison against the fixture
  therefore measures the relative L2 error of the WHOLE state, not of a sample;
* a strided sample of Q at the last checkpoint.

and the run keeps the diagnostic norms of every tenth step (iterations.f90:39-76).  The
oracle is the plain-C restatement compiled with -ffp-contract=off on x86-64; these files
were generated by it with every core of the machine (OpenMP gives the same bits for any
thread count).
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (ROOT, os.path.join(ROOT, "chorus-mhd_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

SKETCH_K = 2048
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)

# name: (case spec, steps, checkpoint interval)
LONG_CASES = {
    "ot_64x64_N4_1000steps": (dict(problem="orszag_tang", nx=64, ny=64, N=4, jitter=0.0, seed=0), 1000, 100),
    "rotor_256x256_N4_500steps": (dict(problem="rotor", nx=256, ny=256, N=4, jitter=0.1, seed=1), 500, 50),
    "ot_512x512_N5_200steps": (dict(problem="orszag_tang", nx=512, ny=512, N=5, jitter=0.15, seed=1), 200, 20),
}


def _hash(idx: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser of the element index (uint64 arithmetic wraps modulo 2^64)."""
    with np.errstate(over="ignore"):
        z = idx.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def sketch(Q, k: int = SKETCH_K, chunk: int = 1 << 22) -> np.ndarray:
    """Count sketch of the flat array Q (k buckets, sign from the top hash bit)."""
    q = np.asarray(Q, np.float64).reshape(-1)
    out = np.zeros(k, np.float64)
    for a in range(0, q.size, chunk):
        b = min(q.size, a + chunk)
        h = _hash(np.arange(a, b, dtype=np.uint64))
        bucket = (h % np.uint64(k)).astype(np.intp)
        sign = np.where((h >> np.uint64(63)) != 0, -1.0, 1.0)
        out += np.bincount(bucket, weights=sign * q[a:b], minlength=k)
    return out


def summary(Q) -> dict:
    q = np.asarray(Q, np.float64).reshape(-1, 9)
    return {"norms": np.sqrt((q * q).sum(axis=0)), "sums": q.sum(axis=0), "sketch": sketch(Q)}


def sketch_rel_l2(sk_a, sk_b, norms_b) -> float:
    """Estimated ||Q_a - Q_b|| / ||Q_b|| from two sketches and Q_b's per-variable norms."""
    nb = float(np.sqrt((np.asarray(norms_b) ** 2).sum()))
    return float(np.linalg.norm(np.asarray(sk_a) - np.asarray(sk_b)) / (nb if nb > 0 else 1.0))


def sample_index(size: int, count: int = 4096) -> np.ndarray:
    return np.arange(0, size, max(1, size // count), dtype=np.int64)[:count]


def load(name: str) -> dict:
    """The fixture as a dict of arrays (the spec decoded)."""
    with np.load(os.path.join(HERE, name + ".npz")) as z:
        d = {k: z[k] for k in z.files}
    d["spec"] = json.loads(str(d["spec"]))
    return d


def generate(name: str, tmp: str, threads: int) -> None:
    import oracle
    from chorus_mhd import meshgen
    spec, steps, every = LONG_CASES[name]
    d = meshgen.write_case(meshgen.CaseSpec(**spec), os.path.join(tmp, name))
    o = oracle.Oracle(d, threads=threads)
    Q = o.array("Q")
    cps, norms, sums, sks, ctimes, diags = [], [], [], [], [], []

    def checkpoint(it):
        s = summary(Q)
        cps.append(it)
        norms.append(s["norms"])
        sums.append(s["sums"])
        sks.append(s["sketch"])
        ctimes.append(o.getd("ctime"))

    t0 = time.time()
    checkpoint(0)
    for it in range(1, steps + 1):
        r = o.step()
        if r is not None:
            diags.append((o.geti("iter"), o.getd("ctime"), r[0], r[1], o.getd("eigvmax_g"), o.getd("epsilon0")))
        if it % every == 0:
            checkpoint(it)
            print("%s: step %d / %d  %.0f s" % (name, it, steps, time.time() - t0), flush=True)
    idx = sample_index(Q.size)
    rec = {"spec": json.dumps(spec), "steps": steps, "dt": o.getd("dt"), "checkpoints": np.array(cps, np.int64),
           "ctime": np.array(ctimes), "norms": np.array(norms), "sums": np.array(sums), "sketch": np.array(sks),
           "sketch_k": SKETCH_K, "diag": np.array(diags, np.float64), "sample_idx": idx,
           "sample": np.array(Q[idx]), "generator": "oracle/chorus_oracle.c, gcc -O2 -ffp-contract=off, x86-64",
           "oracle_seconds": time.time() - t0, "threads": threads}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
    o.close()


def main(argv) -> None:
    threads = os.cpu_count() or 1
    names = []
    i = 0
    while i < len(argv):
        if argv[i] == "--threads":
            threads = int(argv[i + 1])
            i += 2
            continue
        names.append(argv[i])
        i += 1
    tmp = tempfile.mkdtemp(prefix="chorus_long_")
    for name in names or list(LONG_CASES):
        generate(name, tmp, threads)
        print("wrote", name, flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
