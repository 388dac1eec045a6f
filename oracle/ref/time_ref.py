"""Time the reference checker against the oracle port (test infrastructure).

The bench's CPU baseline and its reference arm run the oracle port
(``oracle/port``), because the reference's sources are not present where
the bench runs.  This recipe shows how the port's speed compares with the
reference's own hot path on the same seeded case: it compiles the checker
with ``build_ref.build`` (the unmodified reference sources, -O2
-ffp-contract=off, as the port is built) and times, on one core each, the
same number of steps from the same initial state.  Setup (list building at
creation) is outside both timed regions.

    python oracle/ref/time_ref.py [workload ...]
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "sph-dem_gb300"))

import build_ref  # noqa: E402
from oracle.port_api import OracleSim  # noqa: E402
from sphdem import cases  # noqa: E402
from sphdem.state import write_state  # noqa: E402

STEPS = {"sediment3d_small": 60, "dambreak2d_small": 400}


def time_reference(case: cases.Case, steps: int) -> float:
    """particle-steps/s of the reference checker's timed step loop."""
    exe = build_ref.build(case)
    d = os.path.dirname(exe)
    state, out = os.path.join(d, "init.state"), os.path.join(d, "timing.bin")
    write_state(state, case.particles, case.events)
    res = subprocess.run([exe, state, out, str(steps), "1"], capture_output=True, text=True, check=True)
    m = re.search(r"particle_steps_per_s=([0-9.eE+-]+)", res.stderr)
    if not m:
        raise RuntimeError("no timing in the checker's output: " + res.stderr[-2000:])
    return float(m.group(1))


def time_port(case: cases.Case, steps: int) -> float:
    """particle-steps/s of the oracle port's step loop."""
    sim = OracleSim(case.cfg, case.particles)
    t0 = time.perf_counter()
    sim.step(steps)
    return sim.n * steps / (time.perf_counter() - t0)


def main(names):
    for name in names:
        case = cases.workload(name)
        steps = STEPS.get(name, case.nsteps)
        ref = time_reference(case, steps)
        port = time_port(case, steps)
        print(f"{name}: {case.n} particles, {steps} steps, one core: reference checker {ref:.4g}, "
              f"oracle port {port:.4g} particle-steps/s (port / reference {port / ref:.2f})", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or list(STEPS))
