"""Adjoint of the step (sphdem_adjoint_forward / _backward) against FP64
central finite differences through the C ABI (-m gpu).

DEM step: loss = mean final DEM height plus the summed squared final vhat;
gradients w.r.t. the spring constant k, the dashpot coefficient gamma
(hence the restitution), and the initial positions along seeded random
directions.  Fluid step: see the dam-break section below.  Each gradient is
compared with a central difference of relative step 1e-6; tolerance 1e-3
relative.
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


# ---------------------------------------------------------------------------
# Fluid step (dam break: SPH + fixed SPH-boundary particles, artificial
# viscosity).  Loss: mean final fluid height + kinetic energy of the fluid
# (through v) + summed squared fluid vhat.  Gradients w.r.t. alpha (the
# artificial viscosity coefficient) and the initial positions / vhat along
# seeded random directions, against FP64 central differences.

SPH_STEPS, SPH_K = 40, 7      # 7 does not divide 40: a short last segment


def moving_dambreak():
    """The small dam break with a seeded velocity field on the fluid.  At rest
    every pair sits exactly on the artificial-viscosity switch (vdr = 0,
    sph.h:633-646), where the loss has a kink in vhat and a central
    difference averages the two one-sided slopes."""
    case = cases.workload("dambreak2d_small")
    fl = np.asarray(case.particles["iam"]) == cases.SPH
    v = np.zeros((case.n, 3))
    v[fl, :2] = np.random.default_rng(7).normal(0.0, 0.05, size=(fl.sum(), 2))
    case.particles["v"] = v
    case.particles["vhat"] = v.copy()
    return case


def sph_loss_and_seed(sim):
    a = sim.get()
    fl = a["iam"] == cases.SPH
    m = a["mass"][:, None]
    L = (a["r"][fl, 1].mean() + 0.5 * (m[fl] * a["v"][fl] ** 2).sum()
         + (a["vhat"][fl] ** 2).sum())
    dr = np.zeros((sim.n, 3))
    dr[fl, 1] = 1.0 / fl.sum()
    dv = np.zeros((sim.n, 3))
    dv[fl] = m[fl] * a["v"][fl]
    dvh = np.zeros((sim.n, 3))
    dvh[fl] = 2.0 * a["vhat"][fl]
    return L, dr, dv, dvh


def sph_run_loss(lib, case, cfg=None, r=None, vhat=None):
    parts = copy.deepcopy(case.particles)
    if r is not None:
        parts["r"] = r
    if vhat is not None:
        parts["vhat"] = vhat
    sim = capi.Simulation(lib, cfg or case.cfg, parts, precision=cases.PREC_FP64)
    sim.step(SPH_STEPS)
    L = sph_loss_and_seed(sim)[0]
    sim.close()
    return L


@pytest.mark.parametrize("precision", [cases.PREC_FP64, cases.PREC_MIXED])
def test_sph_adjoint_vs_central_differences(lib, precision):
    case = moving_dambreak()
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=precision)
    sim.adjoint_forward(SPH_STEPS, SPH_K)
    L0, dr, dv, dvh = sph_loss_and_seed(sim)
    grads, dr0, dv0, dvh0 = sim.adjoint_backward(dL_dr=dr, dL_dv=dv, dL_dvhat=dvh)
    assert sph_loss_and_seed(sim)[0] == L0      # back at the final state
    sim.close()
    assert grads.valid & capi.GRAD_VISCOSITY and grads.valid & capi.GRAD_POSITIONS
    assert not grads.valid & capi.GRAD_DEM_K

    # FP64 finite differences for both precisions: the mixed path's FP32
    # pair sums are too noisy for a difference quotient of step 1e-6
    base = case.cfg["alpha_artificial"]
    eps = 1e-6 * base
    cp, cm = dict(case.cfg), dict(case.cfg)
    cp["alpha_artificial"] = base + eps
    cm["alpha_artificial"] = base - eps
    fd = (sph_run_loss(lib, case, cfg=cp) - sph_run_loss(lib, case, cfg=cm)) / (2 * eps)
    print("alpha adjoint", grads.viscosity, "fd", fd)
    assert abs(grads.viscosity - fd) <= RTOL * abs(fd), f"alpha: adjoint {grads.viscosity} fd {fd}"

    rng = np.random.default_rng(4)
    r0 = np.asarray(case.particles["r"], dtype=np.float64).copy()
    scale = np.abs(r0).max()
    for k in range(3):
        u = rng.normal(size=r0.shape)
        u[:, 2] = 0.0
        u /= np.linalg.norm(u)
        eps = 1e-6 * scale
        fd = (sph_run_loss(lib, case, r=r0 + eps * u) - sph_run_loss(lib, case, r=r0 - eps * u)) / (2 * eps)
        ad = float((dr0 * u).sum())
        print("r direction", k, "adjoint", ad, "fd", fd)
        assert abs(ad - fd) <= RTOL * abs(fd), f"r direction {k}: adjoint {ad} fd {fd}"

    vh0 = np.asarray(case.particles["vhat"], dtype=np.float64).copy()
    u = rng.normal(size=vh0.shape)
    u[:, 2] = 0.0
    u /= np.linalg.norm(u)
    eps = 1e-4
    fd = (sph_run_loss(lib, case, vhat=vh0 + eps * u) - sph_run_loss(lib, case, vhat=vh0 - eps * u)) / (2 * eps)
    ad = float((dvh0 * u).sum())
    print("vhat direction adjoint", ad, "fd", fd)
    assert abs(ad - fd) <= RTOL * abs(fd), f"vhat direction: adjoint {ad} fd {fd}"
    # v0 enters the loss only through v1 = v0 + dt sum f
    fl = np.asarray(case.particles["iam"]) == cases.SPH
    assert np.allclose(dv0[fl], dv[fl], rtol=0, atol=0)


# ---------------------------------------------------------------------------
# Coupled SPH-DEM step (periodic x/y box, fluid over three fixed boundary
# layers, DEM spheres in the top half; Morris viscosity, porosity, Shepard
# sums, two-way Di Felice drag, contacts, a DEM floor wall).  Loss: mean final
# DEM height + the squared kinetic energy of the fluid.  Gradients w.r.t. the
# viscosity, the drag scale, k, gamma (restitution) and the initial DEM
# positions along seeded random directions, against FP64 central
# differences.

CPL_STEPS, CPL_K = 30, 7


def moving_coupled():
    """The small coupled case with seeded velocities on fluid and DEM, so that
    the drag law works away from zero slip (where its Jacobian is that of the
    Stokes limit, which the adjoint does not take)."""
    case = cases.workload("sediment3d_adjoint_small")
    iam = np.asarray(case.particles["iam"])
    rng = np.random.default_rng(9)
    # pair the DEM spheres up with a 2% overlap, so that contacts (k, gamma)
    # act from the first step
    idx = np.flatnonzero(iam == cases.DEM)
    R = case.cfg["dem_radius"]
    r = np.asarray(case.particles["r"], dtype=np.float64).copy()
    for a, b in zip(idx[0::2], idx[1::2]):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        r[b] = r[a] + 1.98 * R * u
    case.particles["r"] = r
    v = np.zeros((case.n, 3))
    fl, dem = iam == cases.SPH, iam == cases.DEM
    v[fl] = rng.normal(0.0, 0.02, size=(fl.sum(), 3))
    v[dem] = rng.normal(0.0, 0.05, size=(dem.sum(), 3))
    case.particles["v"] = v
    case.particles["vhat"] = v.copy()
    return case


def cpl_loss_and_seed(sim):
    a = sim.get()
    fl, dem = a["iam"] == cases.SPH, a["iam"] == cases.DEM
    m = a["mass"][:, None]
    ke = 0.5 * (m[fl] * a["v"][fl] ** 2).sum()
    L = a["r"][dem, 2].mean() + ke * ke
    dr = np.zeros((sim.n, 3))
    dr[dem, 2] = 1.0 / dem.sum()
    dv = np.zeros((sim.n, 3))
    dv[fl] = 2.0 * ke * m[fl] * a["v"][fl]
    return L, dr, dv


def cpl_run_loss(lib, case, cfg=None, r=None):
    parts = copy.deepcopy(case.particles)
    if r is not None:
        parts["r"] = r
    sim = capi.Simulation(lib, cfg or case.cfg, parts, precision=cases.PREC_FP64)
    sim.step(CPL_STEPS)
    L = cpl_loss_and_seed(sim)[0]
    sim.close()
    return L


@pytest.mark.parametrize("precision", [cases.PREC_FP64, cases.PREC_MIXED])
def test_coupled_adjoint_vs_central_differences(lib, precision):
    case = moving_coupled()
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=precision)
    sim.adjoint_forward(CPL_STEPS, CPL_K)
    L0, dr, dv = cpl_loss_and_seed(sim)
    grads, dr0, dv0, dvh0 = sim.adjoint_backward(dL_dr=dr, dL_dv=dv)
    assert cpl_loss_and_seed(sim)[0] == L0
    sim.close()
    want = (capi.GRAD_DEM_K | capi.GRAD_DEM_GAMMA | capi.GRAD_VISCOSITY | capi.GRAD_DRAG_SCALE
            | capi.GRAD_POSITIONS)
    assert grads.valid & want == want

    # FP64 differences for both precisions.  Steps: 1e-6 relative on k and
    # gamma; 1e-4 on the viscosity and the drag scale, whose effect on this
    # short run is small enough that a 1e-6 step would sit in the roundoff of
    # the loss (the central difference is O(step^2) accurate in both).
    for name, attr, rel in (("dem_k", "dem_k", 1e-6), ("dem_gamma", "dem_gamma", 1e-6),
                            ("viscosity", "viscosity", 1e-4), ("drag_scale", "drag_scale", 1e-4)):
        base = case.cfg.get(name, 1.0)
        eps = rel * base
        cp, cm = dict(case.cfg), dict(case.cfg)
        cp[name] = base + eps
        cm[name] = base - eps
        fd = (cpl_run_loss(lib, case, cfg=cp) - cpl_run_loss(lib, case, cfg=cm)) / (2 * eps)
        ad = getattr(grads, attr)
        print(name, "adjoint", ad, "fd", fd)
        assert abs(ad - fd) <= RTOL * abs(fd), f"{name}: adjoint {ad} fd {fd}"

    rng = np.random.default_rng(4)
    r0 = np.asarray(case.particles["r"], dtype=np.float64).copy()
    dem = np.asarray(case.particles["iam"]) == cases.DEM
    scale = np.abs(r0).max()
    for k in range(4):
        u = np.zeros_like(r0)
        u[dem] = rng.normal(size=(dem.sum(), 3))
        u /= np.linalg.norm(u)
        eps = 1e-6 * scale
        fd = (cpl_run_loss(lib, case, r=r0 + eps * u) - cpl_run_loss(lib, case, r=r0 - eps * u)) / (2 * eps)
        ad = float((dr0 * u).sum())
        print("DEM direction", k, "adjoint", ad, "fd", fd)
        assert abs(ad - fd) <= RTOL * abs(fd), f"DEM direction {k}: adjoint {ad} fd {fd}"


def moving_coupled_varh():
    """moving_coupled() with VAR_H_CORRECTION: h follows the density
    (h = 1.5 (m / rho)^(1/3)) and the gradients carry 1/Omega."""
    base = moving_coupled()
    case = cases.workload("sediment3d_adjoint_varh_small")
    for k in ("r", "v", "vhat"):
        case.particles[k] = base.particles[k].copy()
    return case


def test_coupled_varh_adjoint_vs_central_differences(lib):
    """The coupled adjoint under VAR_H_CORRECTION (mixed-precision handles)
    against FP64 central differences: the four scalars, DEM positions and
    fluid positions (whose pair terms carry the h and Omega derivatives)."""
    case = moving_coupled_varh()
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    sim.adjoint_forward(CPL_STEPS, CPL_K)
    L0, dr, dv = cpl_loss_and_seed(sim)
    grads, dr0, _, _ = sim.adjoint_backward(dL_dr=dr, dL_dv=dv)
    sim.close()
    want = (capi.GRAD_DEM_K | capi.GRAD_DEM_GAMMA | capi.GRAD_VISCOSITY | capi.GRAD_DRAG_SCALE
            | capi.GRAD_POSITIONS)
    assert grads.valid & want == want
    for name, rel in (("dem_k", 1e-6), ("dem_gamma", 1e-6), ("viscosity", 1e-4), ("drag_scale", 1e-4)):
        base = case.cfg.get(name, 1.0)
        eps = rel * base
        cp, cm = dict(case.cfg), dict(case.cfg)
        cp[name], cm[name] = base + eps, base - eps
        fd = (cpl_run_loss(lib, case, cfg=cp) - cpl_run_loss(lib, case, cfg=cm)) / (2 * eps)
        ad = getattr(grads, name)
        print("varh", name, "adjoint", ad, "fd", fd)
        assert abs(ad - fd) <= RTOL * abs(fd), f"{name}: adjoint {ad} fd {fd}"
    rng = np.random.default_rng(11)
    r0 = np.asarray(case.particles["r"], dtype=np.float64).copy()
    iam = np.asarray(case.particles["iam"])
    scale = np.abs(r0).max()
    smooth = 0
    for kind, mask in (("DEM", iam == cases.DEM), ("fluid", iam == cases.SPH)):
        for k in range(4):
            u = np.zeros_like(r0)
            u[mask] = rng.normal(size=(mask.sum(), 3))
            u /= np.linalg.norm(u)
            ad = float((dr0 * u).sum())
            fds = []
            for e in (1e-6, 0.25e-6):
                eps = e * scale
                fds.append((cpl_run_loss(lib, case, r=r0 + eps * u) - cpl_run_loss(lib, case, r=r0 - eps * u))
                           / (2 * eps))
            print("varh", kind, "direction", k, "adjoint", ad, "fd", fds)
            if abs(fds[0] - fds[1]) > RTOL * abs(fds[1]):
                continue      # a discontinuity of the step inside the bracket
            smooth += 1
            assert abs(ad - fds[1]) <= RTOL * abs(fds[1]), f"{kind} direction {k}: adjoint {ad} fd {fds}"
    assert smooth >= 6


def test_coupled_forward_taps_equal_scanned_tables(lib, monkeypatch):
    """Mixed handles take the reverse sweep's coupling, FPI and contact tables
    from the forward passes that evaluate those pairs (k_couple, k_dem_end);
    scanning for them after each phase, as FP64 handles do, gives the same
    gradients (the tables differ only in entry order and in zero-weight
    pairs beyond the coupling radius)."""
    case = moving_coupled()
    out = {}
    for scan in (False, True):
        if scan:
            monkeypatch.setenv("SPHDEM_ADJ_SCAN_TAPS", "1")
        else:
            monkeypatch.delenv("SPHDEM_ADJ_SCAN_TAPS", raising=False)
        sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
        sim.adjoint_forward(CPL_STEPS, CPL_K)
        L0, dr, dv = cpl_loss_and_seed(sim)
        grads, dr0, dv0, _ = sim.adjoint_backward(dL_dr=dr, dL_dv=dv)
        sim.close()
        out[scan] = (grads, dr0, dv0)
    (g1, r1, v1), (g2, r2, v2) = out[False], out[True]
    for name in ("dem_k", "dem_gamma", "viscosity", "drag_scale"):
        a, b = getattr(g1, name), getattr(g2, name)
        print(name, a, b)
        assert abs(a - b) <= 1e-6 * abs(b), f"{name}: forward taps {a}, scanned {b}"
    for x, y in ((r1, r2), (v1, v2)):
        assert np.abs(x - y).max() <= 1e-6 * np.abs(y).max()


@pytest.mark.parametrize("family", ["fluid", "coupled"])
def test_tape_store_equals_checkpoint_replay(lib, family):
    """Keeping every checkpoint segment's tape from the forward pass
    (sphdem_adjoint_set_tape_memory) gives the gradients of the classic form,
    which keeps one segment's tape and replays the others from their
    checkpoints; a second backward pass after the store was reused for a
    replay still gives them."""
    if family == "fluid":
        case, steps, K, prec = moving_dambreak(), SPH_STEPS, SPH_K, cases.PREC_FP64
        seed = lambda sim: dict(zip(("dL_dr", "dL_dv", "dL_dvhat"), sph_loss_and_seed(sim)[1:]))
    else:
        case, steps, K, prec = moving_coupled(), CPL_STEPS, CPL_K, cases.PREC_MIXED
        seed = lambda sim: dict(zip(("dL_dr", "dL_dv"), cpl_loss_and_seed(sim)[1:]))
    out = []
    for mem in (0, 1 << 36):
        sim = capi.Simulation(lib, case.cfg, case.particles, precision=prec)
        sim.adjoint_set_tape_memory(mem)
        sim.adjoint_forward(steps, K)
        sd = seed(sim)
        out.append(sim.adjoint_backward(**sd))
        if mem:
            out.append(sim.adjoint_backward(**sd))
        sim.close()
    g0, r0 = out[0][0], out[0][1]
    for g, r, *_ in out[1:]:
        for name in ("dem_k", "dem_gamma", "viscosity", "drag_scale"):
            a, b = getattr(g, name), getattr(g0, name)
            assert abs(a - b) <= 1e-6 * max(abs(b), 1e-300), f"{name}: {a} vs {b}"
        assert np.abs(r - r0).max() <= 1e-6 * np.abs(r0).max()


def test_adjoint_rejects_unsupported_fluid(lib):
    # damBreak's own options (Monaghan viscosity, anticlumping, h following
    # density) are outside the fluid adjoint
    case = cases.workload("dambreak2d_monaghan_small")
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    with pytest.raises(capi.SphDemError, match="UNSUPPORTED"):
        sim.adjoint_forward(4, 2)
    sim.close()


# ---------------------------------------------------------------------------
# The differentiated coupled workload at its own size: 100k fluid + 5k DEM
# (sediment3d_adjoint: periodic x/y, three fixed floor layers, constant h),
# loss = mean final DEM height + (fluid kinetic energy)^2, gradients w.r.t.
# the viscosity, the drag scale, the restitution (through the dashpot
# coefficient gamma(e)) and all initial DEM positions along 32 seeded random
# directions, against FP64 central differences.  The run is CFG4_STEPS steps
# with a checkpoint every CFG4_K: the flow separates two runs whose inputs
# differ in one bit by a decade every ~60 steps (tests/test_gpu_precision.py),
# so differences over the full 500 steps leave the linear regime.

CFG4_STEPS, CFG4_K = 20, 10


def cfg4_case(var_h=False):
    case = cases.workload("sediment3d_adjoint_varh" if var_h else "sediment3d_adjoint")
    iam = np.asarray(case.particles["iam"])
    rng = np.random.default_rng(10)
    # spheres in touching pairs (2 % overlap), so that the contacts act from
    # the first step, as in moving_coupled()
    idx = np.flatnonzero(iam == cases.DEM)
    R = case.cfg["dem_radius"]
    r = np.asarray(case.particles["r"], dtype=np.float64).copy()
    for a, b in zip(idx[0::2], idx[1::2]):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        r[b] = r[a] + 1.98 * R * u
    case.particles["r"] = r
    v = np.zeros((case.n, 3))
    fl, dem = iam == cases.SPH, iam == cases.DEM
    v[fl] = rng.normal(0.0, 0.02, size=(fl.sum(), 3))
    v[dem] = rng.normal(0.0, 0.05, size=(dem.sum(), 3))
    case.particles["v"] = v
    case.particles["vhat"] = v.copy()
    return case


def cfg4_loss(lib, case, cfg=None, r=None):
    parts = copy.deepcopy(case.particles)
    if r is not None:
        parts["r"] = r
    sim = capi.Simulation(lib, cfg or case.cfg, parts, precision=cases.PREC_FP64)
    sim.step(CFG4_STEPS)
    L = cpl_loss_and_seed(sim)[0]
    sim.close()
    return L


@pytest.mark.parametrize("var_h", [False, True], ids=["const_h", "var_h"])
def test_config4_coupled_adjoint_vs_central_differences(lib, var_h):
    """var_h: the coupled configuration's VAR_H_CORRECTION (mixed handles)."""
    case = cfg4_case(var_h)
    assert case.notes["n_dem"] == 5000 and case.notes["n_fluid"] > 98000
    grads = {}
    for prec in ((cases.PREC_MIXED,) if var_h else (cases.PREC_FP64, cases.PREC_MIXED)):
        sim = capi.Simulation(lib, case.cfg, case.particles, precision=prec)
        sim.adjoint_forward(CFG4_STEPS, CFG4_K)
        L0, dr, dv = cpl_loss_and_seed(sim)
        g, dr0, _, _ = sim.adjoint_backward(dL_dr=dr, dL_dv=dv)
        sim.close()
        grads[prec] = (g, dr0)

    # restitution e -> gamma(e) with the reduced mass the case used
    e0 = 0.5
    k = case.cfg["dem_k"]
    m_red = 0.5 * case.cfg["dem_vol"] * case.cfg["dem_dens"]
    de = 1e-6 * e0
    dgam_de = (cases.dem_gamma_from_restitution(k, m_red, e0 + de)
               - cases.dem_gamma_from_restitution(k, m_red, e0 - de)) / (2 * de)
    fds = {}
    for name, rel in (("viscosity", 1e-4), ("drag_scale", 1e-4)):
        base = case.cfg.get(name, 1.0)
        eps = rel * base
        cp, cm = dict(case.cfg), dict(case.cfg)
        cp[name], cm[name] = base + eps, base - eps
        fds[name] = (cfg4_loss(lib, case, cfg=cp) - cfg4_loss(lib, case, cfg=cm)) / (2 * eps)
    cp, cm = dict(case.cfg), dict(case.cfg)
    cp["dem_gamma"] = cases.dem_gamma_from_restitution(k, m_red, e0 + de)
    cm["dem_gamma"] = cases.dem_gamma_from_restitution(k, m_red, e0 - de)
    fds["restitution"] = (cfg4_loss(lib, case, cfg=cp) - cfg4_loss(lib, case, cfg=cm)) / (2 * de)

    rng = np.random.default_rng(4)
    r0 = np.asarray(case.particles["r"], dtype=np.float64).copy()
    dem = np.asarray(case.particles["iam"]) == cases.DEM
    scale = np.abs(r0).max()
    dirs, fd_dirs = [], []
    for _ in range(32):
        u = np.zeros_like(r0)
        u[dem] = rng.normal(size=(dem.sum(), 3))
        u /= np.linalg.norm(u)
        eps = 1e-6 * scale
        dirs.append(u)
        fd_dirs.append((cfg4_loss(lib, case, r=r0 + eps * u) - cfg4_loss(lib, case, r=r0 - eps * u)) / (2 * eps))

    # A direction whose difference bracket contains a discontinuity of the
    # step -- a sphere crossing a DEM bucket face, where the reference's
    # asymmetric coupling rule (dataLL.cpp:1154-1190) admits or drops pairs
    # at nonzero W, or a contact opening -- has no derivative to compare.
    # Such a bracket shows as a difference that changes with the step: the
    # test recomputes any direction that disagrees with the adjoint at a
    # quarter of the step, and counts it as a discontinuity when the two
    # differences disagree with each other.
    fd_quarter = {}

    def quarter(k):
        if k not in fd_quarter:
            eps = 0.25e-6 * scale
            u = dirs[k]
            fd_quarter[k] = (cfg4_loss(lib, case, r=r0 + eps * u) - cfg4_loss(lib, case, r=r0 - eps * u)) / (2 * eps)
        return fd_quarter[k]

    for prec, (g, dr0) in grads.items():
        label = "fp64" if prec == cases.PREC_FP64 else "mixed"
        ad = {"viscosity": g.viscosity, "drag_scale": g.drag_scale, "restitution": g.dem_gamma * dgam_de}
        for name, fd in fds.items():
            print(label, name, "adjoint", ad[name], "fd", fd)
            assert abs(ad[name] - fd) <= RTOL * abs(fd), f"{label} {name}: adjoint {ad[name]} fd {fd}"
        smooth, jumps = [], []
        for k, (u, fd) in enumerate(zip(dirs, fd_dirs)):
            a = float((dr0 * u).sum())
            rel = abs(a - fd) / abs(fd)
            if rel > RTOL:
                fq = quarter(k)
                if abs(fq - fd) > RTOL * abs(fd):
                    jumps.append(k)
                    print(label, f"direction {k}: difference {fd:.6e} at the step, {fq:.6e} at a quarter "
                                 f"(a discontinuity in the bracket), adjoint {a:.6e}")
                    continue
            smooth.append(rel)
            assert rel <= RTOL, f"{label} direction {k}: adjoint {a} fd {fd}"
        print(label, f"{len(smooth)} smooth DEM position directions of 32: worst relative difference "
                     f"{max(smooth):.2e}; {len(jumps)} with a discontinuity in the bracket")
        assert len(smooth) >= 24
