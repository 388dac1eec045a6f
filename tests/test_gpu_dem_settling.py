"""DEM-only granular settling at its full size (-m gpu): 50,000 polydisperse
spheres (radius 1 mm x U[0.9, 1.1], density 2500) on a jittered lattice in a
walled 0.1 x 0.1 x 0.3 m box, linear spring-dashpot normal contacts
(k = 1e4 N/m, restitution 0.5), gravity, dt = 1e-5 s, 2000 steps; the
contact law of sph.h:1676-1706 with demNormal LINEAR (sph.h:1513-1515).

Both paths run the same 2000 steps from the same input.  A DEM-only
handle has no FP32 pair pass (the contact law is FP64 on both paths), so
the mixed handle runs the FP64 phases and the two runs agree bit for bit.
Every 500 steps:

- the contact relation of each precision equals the exact pair set of the
  FP64 path on the same positions (two fresh handles, one per precision,
  made from the mixed run's state and rebuilt twice), and both put every
  sphere in the same reference bucket;
- the mixed run's difference from the FP64 run is printed: max |dr| / R,
  max |dv| / max |v|, max |df| / max |f|.  The spheres fall freely until
  step ~1350 and then land on the floor.

The reference has one global sphere radius (sph.h:1685); the polydisperse
form (overlap = R_a + R_b - r) is pinned to the oracle on the small
polydisperse case (dem_small_poly in tests/test_gpu_parity.py), whose
oracle carries the same per-particle radius change.
"""
import numpy as np
import pytest

from sphdem import capi, cases

pytestmark = pytest.mark.gpu

NSTEPS = 2000
EVERY = 500


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def _exact_relations(lib, case, state):
    """Contact pairs and buckets of a mixed and an FP64 handle built from the
    same state (positions, velocities, radii), each rebuilt twice."""
    ps = {k: np.array(state[k]) for k in ("r", "v", "vhat", "mass", "dens", "h", "radius", "iam")}
    out = []
    for prec in (cases.PREC_MIXED, cases.PREC_FP64):
        sim = capi.Simulation(lib, case.cfg, ps, precision=prec)
        sim.rebuild()
        sim.rebuild()
        out.append((sim.pairs(capi.PAIRS_DEM), sim.cell_ids()))
        sim.close()
    return out


def test_dem_settling_50k_mixed_vs_fp64(lib):
    case = cases.dem_settling3d()
    assert case.n == 50_000 and case.notes["polydisperse"]
    R = case.cfg["dem_radius"]
    mixed = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    fp64 = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    rows = []
    try:
        for k in range(NSTEPS // EVERY):
            mixed.step(EVERY)
            fp64.step(EVERY)
            a, b = mixed.get(), fp64.get()
            e_r = float(np.abs(a["r"] - b["r"]).max() / R)
            e_v = float(np.abs(a["v"] - b["v"]).max() / np.abs(b["v"]).max())
            e_f = float(np.abs(a["f"] - b["f"]).max() / np.abs(b["f"]).max())
            (pm, cm), (pf, cf) = _exact_relations(lib, case, a)
            assert np.array_equal(pm[0], pf[0]) and np.array_equal(pm[1], pf[1]), \
                f"step {EVERY * (k + 1)}: contact relations differ"
            assert np.array_equal(cm, cf), f"step {EVERY * (k + 1)}: buckets differ"
            rows.append((EVERY * (k + 1), e_r, e_v, e_f, int(pm[1].size)))
    finally:
        mixed.close()
        fp64.close()
    for s, e_r, e_v, e_f, npairs in rows:
        print(f"step {s}: max|dr|/R {e_r:.2e}  max|dv|/max|v| {e_v:.2e}  max|df|/max|f| {e_f:.2e}  "
              f"contact pairs {npairs}")
    for s, e_r, e_v, e_f, _ in rows:
        assert e_r == 0.0 and e_v == 0.0 and e_f == 0.0, f"step {s}: {e_r} {e_v} {e_f}"
