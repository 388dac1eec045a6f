"""The seeded synthetic workloads behind the bench line and the GPU tests
(sphdem.cases): their sizes and composition as the bench reports them, and
determinism (the same arrays on every call), on the CPU."""
import numpy as np

from sphdem import cases


def _counts(case):
    iam = case.particles["iam"]
    return {"fluid": int(np.sum(iam == cases.SPH)),
            "boundary": int(np.sum((iam == cases.SPH_BOUNDARY) | (iam == cases.BOUNDARY))),
            "dem": int(np.sum(iam == cases.DEM))}


def test_coupled_sedimentation_at_full_size():
    case = cases.workload("sediment3d")
    assert case.n == 1_080_400
    assert _counts(case) == {"fluid": 1_024_000, "boundary": 6_400, "dem": 50_000}
    cfg = case.cfg
    assert cfg["ndim"] == 3 and list(cfg["periodic"][:3]) == [1, 1, 0]
    assert np.allclose(np.array(cfg["rmax"]) - np.array(cfg["rmin"]), [0.2, 0.2, 0.4])
    assert cfg["flags"] & cases.F_LIQ_DEM and cfg["flags"] & cases.F_VAR_H_CORRECTION
    assert abs(cfg["dem_radius"] - 0.5 * cfg["psep"]) <= 1e-15


def test_other_configurations_at_full_size():
    dem = cases.workload("dem_settling3d")
    assert dem.n == 50_000 and _counts(dem)["dem"] == 50_000
    rad = dem.particles["radius"]
    assert rad.min() >= 0.9e-3 * (1 - 1e-12) and rad.max() <= 1.1e-3 * (1 + 1e-12) and rad.std() > 0
    dam = cases.workload("dambreak2d")
    assert dam.n == 23_018 and _counts(dam)["fluid"] == 20_000
    adj = cases.workload("sediment3d_adjoint")
    assert adj.n == 107_675 and _counts(adj) == {"fluid": 98_568, "boundary": 4_107, "dem": 5_000}


def test_ensemble_of_dam_breaks():
    members = cases.dambreak_ensemble()
    n = [m.n for m in members]
    assert len(members) == 256
    assert sum(n) == 3_781_140 and min(n) == 2_872 and max(n) == 44_697


def test_workloads_are_deterministic():
    for name in ("sediment3d_small", "dambreak2d_small", "dem_small_poly", "sediment3d_adjoint"):
        a, b = cases.workload(name), cases.workload(name)
        assert a.cfg == b.cfg
        for k, v in a.particles.items():
            np.testing.assert_array_equal(v, b.particles[k], err_msg=f"{name}: {k}")
