"""Regenerate the golden fixtures from the reference itself.

For every small parity workload this builds the unmodified reference sources
into a checker (oracle/ref/build_ref.py), runs it from the seeded initial
state for the workload's step count, and stores its output -- every hot-path
field in tag order, the four neighbour relations as CSR, the bucket index of
every particle, the final time and dt -- as tests/golden/<workload>.npz.

Needs the reference sources (present only where the fixtures are made):

    python tests/golden/make_golden.py [workload ...]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "sph-dem_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle", "ref"))

from sphdem import cases  # noqa: E402
from sphdem.state import read_output  # noqa: E402

import build_ref  # noqa: E402

WORKLOADS = ["dambreak2d_small", "dambreak2d_monaghan_small", "dem_small", "sediment3d_small",
             "dambreak2d_own_small", "dambreak2d_cg_varh_small", "sediment3d_reinit_small",
             "sediment3d_block_small", "dambreak2d_flow_small", "sediment3d_flow_small"]


def make(name: str) -> str:
    case = cases.workload(name)
    build_ref.build(case)
    out = read_output(build_ref.run(case))
    arrays = {"meta_nsteps": np.int64(case.nsteps), "meta_n": np.int64(case.n),
              "time": np.float64(out["time"]), "dt": np.float64(out["dt"]),
              "cells": out["cells"]}
    for k, v in out["fields"].items():
        arrays["field_" + k] = v
    if "output_vars" in out:
        arrays["output_vars"] = out["output_vars"]
    for k, (offs, idx) in out["pairs"].items():
        arrays["pairs_" + k + "_offs"] = offs
        arrays["pairs_" + k + "_idx"] = idx
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    return path


if __name__ == "__main__":
    for w in sys.argv[1:] or WORKLOADS:
        print(make(w))
