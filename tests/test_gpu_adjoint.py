"""Adjoint of the DEM step (sphdem_adjoint_forward / _backward) against FP64
central finite differences through the C ABI (-m gpu).

Loss: mean final DEM height plus the summed squared final vhat.  Gradients
w.r.t. the spring constant k, the dashpot coefficient gamma (hence the
restitution), and the initial positions along seeded random directions,
each compared with a central difference of relative step 1e-6; tolerance
1e-3 relative.
"""
import copy

import numpy as np
import pytest

from sphdem import capi, cases

pytestmark = pytest.mark.gpu

NSTEPS, KCKPT = 60, 10
RTOL = 1e-3


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def loss_and_seed(sim):
    a = sim.get()
    dem = a["iam"] == cases.DEM
    z = a["r"][:, 2]
    L = z[dem].mean() + (a["vhat"][dem] ** 2).sum()
    dr = np.zeros((sim.n, 3))
    dr[dem, 2] = 1.0 / dem.sum()
    dvh = np.zeros((sim.n, 3))
    dvh[dem] = 2.0 * a["vhat"][dem]
    return L, dr, dvh


def run_loss(lib, case, precision, cfg=None, r=None):
    parts = copy.deepcopy(case.particles)
    if r is not None:
        parts["r"] = r
    sim = capi.Simulation(lib, cfg or case.cfg, parts, precision=precision)
    sim.step(NSTEPS)
    L, _, _ = loss_and_seed(sim)
    sim.close()
    return L


@pytest.mark.parametrize("precision", [cases.PREC_FP64, cases.PREC_MIXED])
def test_dem_adjoint_vs_central_differences(lib, precision):
    case = cases.workload("dem_small")
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=precision)
    sim.adjoint_forward(NSTEPS, KCKPT)
    L0, dr, dvh = loss_and_seed(sim)
    grads, dr0, dv0, dvh0 = sim.adjoint_backward(dL_dr=dr, dL_dvhat=dvh)
    # the handle is back at the final state
    L1, _, _ = loss_and_seed(sim)
    assert L1 == L0
    sim.close()
    assert grads.valid & capi.GRAD_DEM_GAMMA and grads.valid & capi.GRAD_POSITIONS

    for name in ("dem_k", "dem_gamma"):
        base = case.cfg[name]
        eps = 1e-6 * base
        cp, cm = dict(case.cfg), dict(case.cfg)
        cp[name] = base + eps
        cm[name] = base - eps
        fd = (run_loss(lib, case, precision, cfg=cp) - run_loss(lib, case, precision, cfg=cm)) / (2 * eps)
        ad = getattr(grads, name)
        print(name, "adjoint", ad, "fd", fd)
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-12), f"{name}: adjoint {ad} fd {fd}"

    rng = np.random.default_rng(4)
    r0 = np.asarray(case.particles["r"], dtype=np.float64)
    scale = np.abs(r0).max()
    for k in range(4):
        u = rng.normal(size=r0.shape)
        u /= np.linalg.norm(u)
        eps = 1e-6 * scale
        fd = (run_loss(lib, case, precision, r=r0 + eps * u) - run_loss(lib, case, precision, r=r0 - eps * u)) / (2 * eps)
        ad = float((dr0 * u).sum())
        print("direction", k, "adjoint", ad, "fd", fd)
        assert abs(ad - fd) <= RTOL * max(abs(fd), 1e-9), f"direction {k}: adjoint {ad} fd {fd}"


def test_adjoint_rejects_fluid(lib):
    case = cases.workload("dambreak2d_small")
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    with pytest.raises(capi.SphDemError, match="UNSUPPORTED"):
        sim.adjoint_forward(4, 2)
    sim.close()
