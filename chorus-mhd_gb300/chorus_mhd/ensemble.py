"""Seeded mixed-size, mixed-order ensembles of independent solves.

The batched configuration: `count` solves whose cells per side are drawn log-uniform on
[lo, hi], order p uniform on {2,3,4,5} (N = p + 1 in {3,4,5,6}), problem uniform among
Orszag-Tang, rotor and the circularly polarised Alfven wave.  Rotor solves need about
192 solution points per side to resolve the 0.015-wide taper of the initial rotor (the
reference scheme blows up below that: 32^2 and 40^2 at N=3 go non-finite within 20 steps),
so a rotor draw's side is raised to at least ceil(192/N).
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import meshgen

PROBLEMS = ["orszag_tang", "rotor", "alfven"]
ROTOR_MIN_POINTS = 192


def draw(count: int = 256, lo: int = 32, hi: int = 256, seed: int = 2024, jitter: float = 0.1,
         problems=tuple(PROBLEMS)):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        side = int(math.floor(math.exp(rng.uniform(math.log(lo), math.log(hi + 1)))))
        side = max(lo, min(hi, side))
        N = int(rng.integers(3, 7))
        prob = problems[int(rng.integers(0, len(problems)))]
        if prob == "rotor":
            side = max(side, int(math.ceil(ROTOR_MIN_POINTS / N)))
        specs.append(meshgen.CaseSpec(nx=side, ny=side, N=N, problem=prob,
                                      jitter=jitter if prob != "alfven" else 0.0, seed=seed + i))
    return specs


def write_all(specs, root: str):
    dirs = []
    for i, sp in enumerate(specs):
        d = os.path.join(root, "solve%03d" % i)
        meshgen.write_case(sp, d)
        dirs.append(d)
    return dirs
