"""How far two correct FP64 evaluations of the same scheme drift apart over a long run.

    python tests/golden/oracle_sensitivity.py NAME [--threads T] [--perturb-ulp SEED] [--record]

Builds a second copy of the oracle that differs from the committed one only in its
floating-point contraction (gcc -ffp-contract=fast, plus -mfma on x86-64: a*b+c becomes
one fused multiply-add, as an aarch64 build of the reference would compute it), runs the
long-horizon case NAME of make_long_golden.py over its stated number of steps, and prints
at every checkpoint the relative L2 distance between this run and the committed fixture
(the -ffp-contract=off oracle), estimated from the fixture's count sketch.  Both runs are
the same algorithm in the same order; they differ by one rounding here and there, so the
printed curve is the scheme's own amplification of round-off on that case -- the floor
below which no FP64 implementation that is not bit-identical to the reference can stay.

With --perturb-ulp the committed oracle itself runs instead, from its initial state with
every value moved by one unit in the last place up or down (seeded signs): the growth of
a one-ulp perturbation of the state under the scheme, with no difference in arithmetic.

--record keeps the curve in tests/golden/NAME_sensitivity.npz (key "contracted" or
"ulp<SEED>": rows of checkpoint, estimated relative L2), beside the fixture it measures.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for _p in (ROOT, os.path.join(ROOT, "chorus-mhd_gb300"), HERE):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import make_long_golden as LG  # noqa: E402


def build_contracted() -> str:
    import oracle
    out = os.path.join(oracle.BUILD, "liborc_fma.so")
    os.makedirs(oracle.BUILD, exist_ok=True)
    flags = ["-ffp-contract=fast"] + (["-mfma"] if platform.machine() in ("x86_64", "AMD64") else [])
    cmd = ["gcc", "-O2", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", "-std=c99", "-w"] + flags + \
          ["-o", out, oracle.SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return out


def main(argv) -> None:
    name = argv[0]
    threads = int(argv[argv.index("--threads") + 1]) if "--threads" in argv else (os.cpu_count() or 1)
    import oracle
    perturb = "--perturb-ulp" in argv
    if not perturb:
        oracle.LIB = build_contracted()  # this process loads the contracted copy only
        oracle._lib = None
    from chorus_mhd import meshgen
    fx = LG.load(name)
    d = meshgen.write_case(meshgen.CaseSpec(**fx["spec"]), tempfile.mkdtemp(prefix="sens_"))
    o = oracle.Oracle(d, threads=threads)
    Q = o.array("Q")
    if perturb:
        seed = int(argv[argv.index("--perturb-ulp") + 1])
        up = np.random.default_rng(seed).integers(0, 2, Q.size).astype(bool)
        Q[:] = np.where(up, np.nextafter(Q, np.inf), np.nextafter(Q, -np.inf))
    curve = []
    t0 = time.time()
    what = "one-ulp perturbed initial state" if perturb else "oracle with FMA contraction"
    print("%s, %s vs the fixture: step, est. rel L2, sample rel L2" % (name, what), flush=True)
    for k, it in enumerate(fx["checkpoints"]):
        while o.geti("iter") < it:
            o.step()
        err = LG.sketch_rel_l2(LG.sketch(Q), fx["sketch"][k], fx["norms"][k])
        curve.append((float(it), err))
        line = "  %5d  %.3e" % (it, err)
        if k == len(fx["checkpoints"]) - 1:
            idx = fx["sample_idx"]
            line += "  %.3e" % (np.linalg.norm(Q[idx] - fx["sample"]) / np.linalg.norm(fx["sample"]))
        print(line + "   (%.0f s)" % (time.time() - t0), flush=True)
    o.close()
    if "--record" in argv:
        path = os.path.join(HERE, name + "_sensitivity.npz")
        rec = {}
        if os.path.exists(path):
            with np.load(path) as z:
                rec = {k: z[k] for k in z.files}
        key = "ulp%d" % int(argv[argv.index("--perturb-ulp") + 1]) if perturb else "contracted"
        rec[key] = np.array(curve)
        np.savez_compressed(path, **rec)


if __name__ == "__main__":
    main(sys.argv[1:])
