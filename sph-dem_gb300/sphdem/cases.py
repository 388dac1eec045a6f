"""Seeded synthetic case generators for the SPH-DEM hot path.

Each generator returns a :class:`Case`: a configuration dictionary whose keys
are the members of ``SphDemConfig`` (``include/sphdem.h``) and a particle set
in structure-of-arrays form.  The same ``Case`` feeds the CUDA library, the
CPU oracle and, for small sizes, the reference build that pins the oracle, so
all three start from bit-identical inputs.

The geometry follows the reference's own case set-ups:

* ``dambreak2d`` -- water column in a tank with three walls of fixed
  ``sphBoundary`` particles (lattice as damBreak/setup.cpp:65-79, wall layers
  as misc.cpp:382-420 / sediment3D/setup.cpp:59-93).
* ``dem_settling3d`` -- DEM spheres on a jittered lattice in a walled box; the
  walls are the planar-wall hook of sediment3D/customSim.cpp:67-81.
* ``sediment3d`` -- the sediment3D lattice (sediment3D/setup.cpp:65-108,
  staggered odd layers, one layer of ``boundary`` particles at k=0) with DEM
  spheres seeded uniformly in the top half, rejecting overlaps.

Particle type codes are ``iamTypes`` (particle.h:17).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# iamTypes, particle.h:17
SPH, SPH_BOUNDARY, IMMOVABLE, BOUNDARY, GHOST = 0, 1, 2, 3, 4
DEM, DEM_BOUNDARY, IMMERSED_DEM = 11, 12, 13

VISC_NONE, VISC_ARTIFICIAL, VISC_MONAGHAN, VISC_MORRIS = 0, 1, 2, 3

F_CONST_H = 1 << 0
F_NO_ANTICLUMPING = 1 << 1
F_VAR_H_CORRECTION = 1 << 2
F_LIQ_DEM = 1 << 3
F_FIXED_DT = 1 << 4
F_CORRECTED_GRADIENT = 1 << 6
F_DEM_BLOCK = 1 << 7

PREC_FP64, PREC_MIXED = 0, 1

REF_PI = 3.14159265  # the PI constant every reference customConstants.h defines


@dataclass
class Case:
    name: str
    cfg: dict
    particles: dict
    nsteps: int
    notes: dict = field(default_factory=dict)
    # insertions and deletions after a step's last hook: {"step": s,
    # "insert": particle block} or {"step": s, "delete": tag-order indices}
    events: list = field(default_factory=list)

    @property
    def n(self) -> int:
        return int(self.particles["iam"].shape[0])

    @property
    def n_inserted(self) -> int:
        return sum(int(e["insert"]["iam"].shape[0]) for e in self.events if "insert" in e)


def _base_cfg(ndim: int) -> dict:
    return dict(
        ndim=ndim, visc_model=VISC_NONE, flags=0, precision=PREC_FP64,
        periodic=[0, 0, 0], n_walls=0, pi=REF_PI,
        rmin=[0.0, 0.0, 0.0], rmax=[0.0, 0.0, 0.0],
        domain_min=[0.0, 0.0, 0.0], domain_max=[0.0, 0.0, 0.0],
        hfac=1.3, psep=0.0, h=0.0, dens=1000.0, refd=1000.0,
        gamma=7.0, prb=0.0, spsound=0.0, viscosity=1e-6,
        alpha_artificial=0.0, bfac=1.0, maxdt=0.0, damptime=0.0,
        dem_radius=0.0, dem_dens=2500.0, dem_k=0.0, dem_gamma=0.0,
        dem_search_radius=0.0, dem_vol=0.0, coupling_radius=0.0,
        dem_timestep=1e30, liq_dem_timestep=1e30,
        time_drop_particle=1e30, freeze_dem_until=-1.0, drag_scale=1.0,
        reinit_dens_every=0, reinit_dens_at=0,
        gravity_sph=[0.0, 0.0, 0.0], gravity_dem=[0.0, 0.0, 0.0],
        walls=[],
    )


def _empty_particles(n: int) -> dict:
    return dict(
        iam=np.zeros(n, np.int32), tag=np.arange(1, n + 1, dtype=np.int32),
        concave=np.ones(n, np.uint8),
        r=np.zeros((n, 3)), v=np.zeros((n, 3)), mass=np.zeros(n),
        dens=np.zeros(n), h=np.zeros(n), radius=np.zeros(n),
        norm1=np.zeros((n, 3)), norm2=np.zeros((n, 3)), norm3=np.zeros((n, 3)),
    )


def _concat(parts: list[dict]) -> dict:
    out = {}
    for k in parts[0]:
        out[k] = np.concatenate([p[k] for p in parts], axis=0)
    out["tag"] = np.arange(1, out["iam"].shape[0] + 1, dtype=np.int32)
    return out


def _domain_with_margin(rmin, rmax, periodic, ndim):
    """procDomain as sediment3D/setup.cpp:114-125 sets it: 25% margin on
    non-periodic axes, exact extents on periodic ones."""
    lo, hi = [0.0] * 3, [0.0] * 3
    for j in range(ndim):
        ext = rmax[j] - rmin[j]
        lo[j] = rmin[j] if periodic[j] else rmin[j] - 0.25 * ext
        hi[j] = rmax[j] if periodic[j] else rmax[j] + 0.25 * ext
    return lo, hi


def dem_gamma_from_restitution(k: float, m_reduced: float, e: float) -> float:
    """Dashpot coefficient of a linear spring-dashpot giving restitution e
    for reduced mass m_reduced: gamma = -2 ln(e) sqrt(k m / (pi^2 + ln^2 e))."""
    le = math.log(e)
    return -2.0 * le * math.sqrt(k * m_reduced / (math.pi ** 2 + le * le))


# --------------------------------------------------------------------------
# 2D dam break
# --------------------------------------------------------------------------
def dambreak2d(dx: float = 0.01, width: float = 1.0, height: float = 2.0,
               tank=(4.0, 3.0), seed: int = 1, jitter: float = 0.01,
               nsteps: int = 1000, layers: int = 3,
               visc_model: int = VISC_ARTIFICIAL, const_h: bool = True,
               anticlumping: bool = False, viscosity: float = 1e-6,
               var_h: bool = False, corrected_gradient: bool = False,
               reinit_every: int = 0, reinit_at: int = 0, fixed_dt: bool = True) -> Case:
    """Weakly-compressible 2D dam break: a width x height water column at rest
    in a tank[0] x tank[1] tank with three walls of `layers` fixed
    sphBoundary layers.  Wendland C2, h = 1.3 dx (CONST_H), Tait EOS
    gamma = 7, rho0 = 1000, c0 = 10 sqrt(2 g height), artificial viscosity
    alpha = 0.1, gravity -9.81, dt = 0.25 h / c0.  Options: VAR_H_CORRECTION,
    CORRECTED_GRADIENT, and the density re-initialisation of start() every
    `reinit_every` steps and at step `reinit_at` (0: never); fixed_dt=False
    lets dt follow the reference's time-step conditions."""
    ndim = 2
    rho0 = 1000.0
    c0 = 10.0 * math.sqrt(2.0 * 9.81 * height)
    h = 1.3 * dx
    cfg = _base_cfg(ndim)
    cfg.update(
        visc_model=visc_model,
        flags=(F_CONST_H if const_h else 0) | (0 if anticlumping else F_NO_ANTICLUMPING)
        | (F_VAR_H_CORRECTION if var_h else 0) | (F_CORRECTED_GRADIENT if corrected_gradient else 0)
        | (F_FIXED_DT if fixed_dt else 0),
        reinit_dens_every=reinit_every, reinit_dens_at=reinit_at,
        rmin=[0.0, 0.0, 0.0], rmax=[tank[0], tank[1], 0.0],
        hfac=1.3, psep=dx, h=h, dens=rho0, refd=rho0, gamma=7.0,
        spsound=c0, prb=c0 * c0 * rho0 / 7.0, viscosity=viscosity,
        alpha_artificial=0.1, bfac=1.0, maxdt=0.25 * h / c0,
        gravity_sph=[0.0, -9.81, 0.0],
        # DEM constants are unused without LIQ_DEM but keep the grids sane.
        dem_radius=0.5 * dx, dem_search_radius=0.5 * dx, coupling_radius=2.0 * h,
    )
    cfg["domain_min"], cfg["domain_max"] = _domain_with_margin(
        cfg["rmin"], cfg["rmax"], cfg["periodic"], ndim)

    nxt = int(round(tank[0] / dx))
    nyt = int(round(tank[1] / dx))
    nxw = int(round(width / dx))
    nyw = int(round(height / dx))
    mass = dx * dx * rho0

    # walls: bottom (with corners) then left and right
    pts = []
    for k in range(layers):
        y = -(k + 0.5) * dx
        for i in range(-layers, nxt + layers):
            pts.append(((i + 0.5) * dx, y))
    for k in range(layers):
        for j in range(nyt):
            pts.append((-(k + 0.5) * dx, (j + 0.5) * dx))
            pts.append((tank[0] + (k + 0.5) * dx, (j + 0.5) * dx))
    nb = len(pts)
    wall = _empty_particles(nb)
    wall["r"][:, :2] = np.array(pts)
    wall["iam"][:] = SPH_BOUNDARY

    rng = np.random.default_rng(seed)
    ii, jj = np.meshgrid(np.arange(nxw), np.arange(nyw), indexing="ij")
    nf = nxw * nyw
    fluid = _empty_particles(nf)
    fluid["r"][:, 0] = (ii.ravel() + 0.5) * dx
    fluid["r"][:, 1] = (jj.ravel() + 0.5) * dx
    fluid["r"][:, :2] += rng.uniform(-jitter * dx, jitter * dx, size=(nf, 2))
    fluid["iam"][:] = SPH

    ps = _concat([wall, fluid])
    ps["mass"][:] = mass
    ps["dens"][:] = rho0
    ps["h"][:] = h
    return Case("dambreak2d", cfg, ps, nsteps,
                notes=dict(n_fluid=nf, n_boundary=nb, dx=dx, dt=cfg["maxdt"],
                           viscosity_form="VISC_ARTIFICIAL alpha=0.1"))


# --------------------------------------------------------------------------
# 3D DEM settling
# --------------------------------------------------------------------------
def dem_settling3d(lattice=(25, 25, 80), box=(0.1, 0.1, 0.3), radius: float = 1e-3,
                   spread: float = 0.1, rho_s: float = 2500.0, k: float = 1e4,
                   restitution: float = 0.5, dt: float = 1e-5, seed: int = 2,
                   nsteps: int = 2000, vel_amp: float = 0.0) -> Case:
    """DEM-only granular settling: spheres of radius radius*U[1-spread,1+spread]
    on a jittered non-overlapping lattice in a walled box, linear
    spring-dashpot normal contacts (no tangential force), gravity -9.81."""
    ndim = 3
    n = int(np.prod(lattice))
    rng = np.random.default_rng(seed)
    rad = radius * rng.uniform(1.0 - spread, 1.0 + spread, size=n) if spread > 0 \
        else np.full(n, radius)
    rmax_p = radius * (1.0 + spread)
    sp = [box[d] / lattice[d] for d in range(3)]
    amp = 0.25 * (min(sp) - 2.0 * rmax_p)
    if amp < 0:
        raise ValueError("lattice too dense for the largest sphere")
    ii, jj, kk = np.meshgrid(*[np.arange(m) for m in lattice], indexing="ij")
    ps = _empty_particles(n)
    ps["r"][:, 0] = (ii.ravel() + 0.5) * sp[0]
    ps["r"][:, 1] = (jj.ravel() + 0.5) * sp[1]
    ps["r"][:, 2] = (kk.ravel() + 0.5) * sp[2]
    ps["r"] += rng.uniform(-amp, amp, size=(n, 3))
    if vel_amp > 0:
        ps["v"][:] = rng.uniform(-vel_amp, vel_amp, size=(n, 3))
    ps["iam"][:] = DEM
    ps["radius"][:] = rad
    ps["mass"][:] = (4.0 / 3.0) * REF_PI * rad ** 3 * rho_s
    ps["dens"][:] = rho_s
    ps["h"][:] = rmax_p  # p.h = DEM_SEARCH_RADIUS (misc.cpp:95,147)

    m_nom = (4.0 / 3.0) * REF_PI * radius ** 3 * rho_s
    gamma = dem_gamma_from_restitution(k, 0.5 * m_nom, restitution)
    cfg = _base_cfg(ndim)
    cfg.update(
        flags=F_LIQ_DEM | F_CONST_H | F_NO_ANTICLUMPING | F_FIXED_DT,
        rmin=[0.0, 0.0, 0.0], rmax=list(box), hfac=1.5,
        psep=2.0 * rmax_p, h=rmax_p, dens=1000.0, refd=1000.0, gamma=7.0,
        spsound=10.0, prb=100.0 * 1000.0 / 7.0, viscosity=1e-6,
        maxdt=dt, dem_radius=radius, dem_dens=rho_s, dem_k=k, dem_gamma=gamma,
        dem_search_radius=rmax_p, dem_vol=(4.0 / 3.0) * REF_PI * radius ** 3,
        coupling_radius=2.0 * rmax_p,
        gravity_dem=[0.0, 0.0, -9.81],
    )
    walls = []
    for d in range(3):
        n_lo = [0.0, 0.0, 0.0]
        n_lo[d] = 1.0
        n_hi = [0.0, 0.0, 0.0]
        n_hi[d] = -1.0
        p_hi = [0.0, 0.0, 0.0]
        p_hi[d] = box[d]
        walls.append(dict(point=[0.0, 0.0, 0.0], normal=n_lo))
        walls.append(dict(point=p_hi, normal=n_hi))
    cfg["walls"] = walls
    cfg["n_walls"] = len(walls)
    cfg["domain_min"], cfg["domain_max"] = _domain_with_margin(
        cfg["rmin"], cfg["rmax"], cfg["periodic"], ndim)
    _dem_timesteps(cfg)
    return Case("dem_settling3d", cfg, ps, nsteps,
                notes=dict(n_dem=n, restitution=restitution, dem_gamma=gamma,
                           polydisperse=spread > 0, dt=dt))


def _dem_timesteps(cfg: dict) -> None:
    """DEM_TIMESTEP and LIQ_DEM_TIMESTEP exactly as demConstants.h:6, 19."""
    pi = cfg["pi"]
    vol = (4.0 / 3.0) * pi * cfg["dem_radius"] ** 3
    mass = vol * cfg["dem_dens"]
    mr = 0.5 * mass
    k, g = cfg["dem_k"], cfg["dem_gamma"]
    arg = k / mr - (0.5 * g / mr) ** 2 if mr > 0 else 0.0
    cfg["dem_timestep"] = (1.0 / 50.0) * pi / math.sqrt(arg) if arg > 0 else 1e30
    visc = cfg["viscosity"]
    if visc > 0 and cfg["dem_radius"] > 0:
        cfg["liq_dem_timestep"] = (1.0 / 5.0) * vol * cfg["dem_dens"] / (
            6.0 * pi * visc * cfg["dens"] * cfg["dem_radius"])


# --------------------------------------------------------------------------
# 3D coupled SPH-DEM sedimentation
# --------------------------------------------------------------------------
def sediment3d(nx: int = 80, L: float = 0.2, height: float = 0.4,
               n_dem: int = 50000, dem_radius_factor: float = 0.5,
               rho_s: float = 2500.0, k: float = 1e4, restitution: float = 0.5,
               viscosity: float = 1e-6, seed: int = 3, nsteps: int = 1000,
               dt: float | None = None, floor: str = "boundary", var_h: bool = True,
               dem_top_margin: float | None = None, reinit_every: int = 0,
               dem_block: bool = False) -> Case:
    """Coupled SPH-DEM sedimentation in a periodic-x/y box L x L x height with
    a bottom wall.  Fluid lattice as sediment3D/setup.cpp:65-108 (staggered
    odd layers, one `boundary` layer at k=0), h = 1.5 dx, Morris viscosity
    (kinematic `viscosity`), VAR_H_CORRECTION, porosity-weighted Tait EOS,
    Di Felice drag.  DEM spheres of radius dem_radius_factor*dx seeded
    uniformly in the top half with overlap rejection (periodic in x, y).

    floor="sphb3" makes the floor three fixed sphBoundary layers (k = 0..2)
    instead of the repulsive boundary layer, and var_h=False gives constant
    h without VAR_H_CORRECTION: the coupled form the adjoint covers.
    dem_top_margin keeps the DEM centres that far below the free surface
    (default R): spheres at the surface see about half a kernel of fluid, the
    0.5 threshold of calcFPI's Shepard normalisation (sph.h:1759-1760).
    reinit_every > 0 re-initialises the fluid density every that many steps
    (sediment3D's REINIT_DENS_EVERY_N_STEPS); dem_block moves the DEM
    particles as one block under their mean force (sediment3D's DEM_BLOCK)."""
    ndim = 3
    psep = L / nx
    nz = int(round(height / psep))
    h = 1.5 * psep
    rho0 = 1000.0
    vmax = 2.0 * math.sqrt(2.0 * 9.81 * height)
    c0 = 10.0 * vmax
    R = dem_radius_factor * psep
    vol_d = (4.0 / 3.0) * REF_PI * R ** 3
    porosity_est = 1.0 - n_dem * vol_d / (L * L * 0.5 * height)
    rc = 1.999 * h / porosity_est ** (1.0 / 3.0)

    # fluid + boundary lattice
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(nx), np.arange(nz + 1),
                             indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    nf = ii.size
    ps = _empty_particles(nf)
    odd = (kk % 2) == 1
    ps["r"][:, 0] = np.where(odd, ii * psep, (ii + 0.5) * psep)
    ps["r"][:, 1] = np.where(odd, jj * psep, (jj + 0.5) * psep)
    ps["r"][:, 2] = kk * psep
    if floor == "sphb3":
        bnd = kk <= 2
        ps["iam"][:] = np.where(bnd, SPH_BOUNDARY, SPH).astype(np.int32)
    else:
        bnd = kk <= 0
        ps["iam"][:] = np.where(bnd, BOUNDARY, SPH).astype(np.int32)
        ps["norm1"][bnd] = (0.0, 0.0, 1.0)
        ps["norm3"][bnd] = (0.0, 1.0, 0.0)
    ps["mass"][:] = psep ** 3 * rho0
    ps["dens"][:] = rho0
    ps["h"][:] = 1.5 * (psep ** 3) ** (1.0 / 3.0)
    ps["h"][:] = 1.5 * np.power(ps["mass"] / ps["dens"], 1.0 / 3.0)

    # DEM: uniform in the top half, periodic overlap rejection on a hash grid
    rng = np.random.default_rng(seed)
    zlo, zhi = 0.5 * height + R, height - (R if dem_top_margin is None else max(R, dem_top_margin))
    cell = 2.0 * R
    ncx = max(1, int(L / cell))
    grid: dict = {}
    pos = np.zeros((n_dem, 3))
    count = 0
    tries = 0
    while count < n_dem:
        tries += 1
        if tries > 200 * n_dem:
            raise RuntimeError("could not place DEM particles")
        p = np.array([rng.uniform(0.0, L), rng.uniform(0.0, L), rng.uniform(zlo, zhi)])
        cx, cy, cz = int(p[0] / L * ncx) % ncx, int(p[1] / L * ncx) % ncx, int(p[2] / cell)
        ok = True
        for ox in (-1, 0, 1):
            for oy in (-1, 0, 1):
                for oz in (-1, 0, 1):
                    for q in grid.get(((cx + ox) % ncx, (cy + oy) % ncx, cz + oz), ()):
                        d = p - pos[q]
                        d[0] -= L * round(d[0] / L)
                        d[1] -= L * round(d[1] / L)
                        if d @ d < (2.0 * R) ** 2:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            pos[count] = p
            grid.setdefault((cx, cy, cz), []).append(count)
            count += 1
    dem = _empty_particles(n_dem)
    dem["r"][:] = pos
    dem["iam"][:] = DEM
    dem["radius"][:] = R
    dem["mass"][:] = vol_d * rho_s
    dem["dens"][:] = rho_s
    dem["h"][:] = R  # p.h = DEM_SEARCH_RADIUS
    ps = _concat([ps, dem])

    m_d = vol_d * rho_s
    gamma_d = dem_gamma_from_restitution(k, 0.5 * m_d, restitution)
    cfg = _base_cfg(ndim)
    cfg.update(
        visc_model=VISC_MORRIS,
        flags=((F_LIQ_DEM | F_VAR_H_CORRECTION | F_NO_ANTICLUMPING | F_FIXED_DT) if var_h
               else (F_LIQ_DEM | F_CONST_H | F_NO_ANTICLUMPING | F_FIXED_DT))
        | (F_DEM_BLOCK if dem_block else 0),
        periodic=[1, 1, 0], reinit_dens_every=reinit_every,
        rmin=[0.0, 0.0, 0.0], rmax=[L, L, height],
        hfac=1.5, psep=psep, h=h, dens=rho0, refd=rho0, gamma=7.0,
        spsound=c0, prb=c0 * c0 * rho0 / 7.0, viscosity=viscosity,
        bfac=1.0, maxdt=dt if dt is not None else 0.25 * h / c0,
        dem_radius=R, dem_dens=rho_s, dem_k=k, dem_gamma=gamma_d,
        dem_search_radius=R, dem_vol=vol_d, coupling_radius=rc,
        gravity_sph=[0.0, 0.0, -9.81], gravity_dem=[0.0, 0.0, -9.81],
        walls=[dict(point=[0.0, 0.0, 0.0], normal=[0.0, 0.0, 1.0])], n_walls=1,
    )
    cfg["domain_min"], cfg["domain_max"] = _domain_with_margin(
        cfg["rmin"], cfg["rmax"], cfg["periodic"], ndim)
    _dem_timesteps(cfg)
    n_sph = int((ps["iam"] == SPH).sum())
    return Case("sediment3d", cfg, ps, nsteps,
                notes=dict(n_fluid=n_sph, n_boundary=int(bnd.sum()), n_dem=n_dem,
                           dem_radius=R, porosity_est=porosity_est,
                           coupling_radius=rc, viscosity_kinematic=viscosity,
                           dt=cfg["maxdt"], dem_gamma=gamma_d))


# --------------------------------------------------------------------------
# named workloads
# --------------------------------------------------------------------------
def dambreak_ensemble(n_instances: int = 256, seed: int = 5, n_min: int = 2000, n_max: int = 40000,
                      h_min: float = 1.0, h_max: float = 2.5, width: float = 1.0) -> list:
    """Batched-ensemble workload: independent 2D dam breaks whose fluid
    particle counts are log-uniform in [n_min, n_max] (set through dx) and
    whose column heights are uniform in [h_min, h_max]; one seeded draw."""
    rng = np.random.default_rng(seed)
    n_target = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_instances))
    heights = rng.uniform(h_min, h_max, n_instances)
    out = []
    for k in range(n_instances):
        dx = math.sqrt(width * heights[k] / n_target[k])
        out.append(dambreak2d(dx=dx, width=width, height=float(heights[k]), seed=seed + 1 + k))
    return out


def advance(sim, case: Case, nsteps: int | None = None, start: int = 0) -> None:
    """Step `sim` (anything with step / insert / mark_for_deletion: a
    capi.Simulation, the oracle) through steps start+1 .. start+nsteps of the
    case, applying its insertions and deletions after the steps they follow,
    as a case's afterEnd hook would."""
    end = start + (case.nsteps if nsteps is None else nsteps)
    s = start
    for t in sorted({e["step"] for e in case.events if start < e["step"] <= end}):
        sim.step(t - s)
        s = t
        for e in case.events:
            if e["step"] == t:
                if "insert" in e:
                    sim.insert(e["insert"])
                else:
                    sim.mark_for_deletion(e["delete"])
    if end > s:
        sim.step(end - s)


def dambreak2d_flow(dx: float = 0.05, nsteps: int = 30, seed: int = 7) -> Case:
    """The small dam break with particles leaving and entering between steps:
    after step 8 every 13th fluid particle is marked for deletion; after step
    12 a row of fluid particles enters above the column, falling at 1 m/s
    (taking the freed slots); after step 20 every 17th fluid particle more
    and two wall particles go; after step 22 five more rows enter (more than
    the free slots, so the last ones are appended)."""
    case = dambreak2d(dx=dx, nsteps=nsteps, seed=seed)
    ps = case.particles
    fluid = np.nonzero(ps["iam"] == SPH)[0]
    k = fluid - fluid[0]
    rng = np.random.default_rng(seed + 100)
    rho0, nx = case.cfg["dens"], int(round(1.0 / dx))
    top = float(ps["r"][fluid, 1].max())

    def rows(y0: float, nrows: int) -> dict:
        ii, jj = np.meshgrid(np.arange(nx), np.arange(nrows), indexing="ij")
        m = nx * nrows
        blk = _empty_particles(m)
        blk["r"][:, 0] = (ii.ravel() + 0.5) * dx
        blk["r"][:, 1] = y0 + jj.ravel() * dx
        blk["r"][:, :2] += rng.uniform(-0.01 * dx, 0.01 * dx, size=(m, 2))
        blk["v"][:, 1] = -1.0
        blk["iam"][:] = SPH
        blk["mass"][:] = dx * dx * rho0
        blk["dens"][:] = rho0
        blk["h"][:] = 1.3 * dx
        return blk

    del1 = fluid[k % 13 == 0]
    del2 = np.concatenate([fluid[(k % 17 == 5) & (k % 13 != 0)], [0, 1]])
    case.events = [{"step": 8, "delete": del1}, {"step": 12, "insert": rows(top + dx, 1)},
                   {"step": 20, "delete": del2}, {"step": 22, "insert": rows(top + 2 * dx, 5)}]
    case.notes["events"] = "8: -%d, 12: +%d, 20: -%d, 22: +%d" % (del1.size, nx, del2.size, 5 * nx)
    return case


def sediment3d_flow(nsteps: int = 16) -> Case:
    """The small coupled sedimentation box with particles leaving and
    entering between steps: after step 4 five DEM spheres enter near the top
    (a sphere inflow) and every 40th fluid particle is marked for deletion;
    after step 9 two of the new spheres and one of the first ones leave and
    three more fluid particles enter."""
    case = sediment3d(nx=10, L=0.04, height=0.08, n_dem=100, nsteps=nsteps, seed=8)
    ps, c = case.particles, case.cfg
    R, L = case.notes["dem_radius"], c["rmax"][0]
    fluid = np.nonzero(ps["iam"] == SPH)[0]
    dem = np.nonzero(ps["iam"] == DEM)[0]

    def spheres(xyz):
        m = len(xyz)
        blk = _empty_particles(m)
        blk["r"][:] = np.asarray(xyz, float)
        blk["iam"][:] = DEM
        blk["mass"][:] = c["dem_vol"] * c["dem_dens"]
        blk["dens"][:] = c["dem_dens"]
        blk["h"][:] = R
        blk["radius"][:] = R
        blk["v"][:, 2] = -0.05
        return blk

    def droplets(xyz):
        m = len(xyz)
        blk = _empty_particles(m)
        blk["r"][:] = np.asarray(xyz, float)
        blk["iam"][:] = SPH
        blk["mass"][:] = ps["mass"][fluid[0]]
        blk["dens"][:] = c["dens"]
        blk["h"][:] = c["h"]
        return blk

    # five free places near the top: clear of the seeded spheres by 1.1 diameters
    old = ps["r"][dem]
    chosen = []
    for zt in (0.072, 0.066, 0.060):
        for fy in (0.5, 0.2, 0.8):
            for fx in (0.15, 0.32, 0.49, 0.66, 0.83):
                p = np.array([L * fx, L * fy, zt])
                near = np.vstack([old] + [np.array(chosen)] if chosen else [old]) - p
                near[:, :2] -= L * np.round(near[:, :2] / L)
                if len(chosen) < 5 and np.linalg.norm(near, axis=1).min() > 2.2 * R:
                    chosen.append(p)
    new1 = spheres(chosen)
    new2 = droplets([[L * 0.3, L * 0.31, 0.05], [L * 0.6, L * 0.62, 0.05], [L * 0.45, L * 0.77, 0.05]])
    n0 = case.n
    case.events = [{"step": 4, "insert": new1}, {"step": 4, "delete": fluid[::40]},
                   {"step": 9, "delete": np.array([n0 + 1, n0 + 3, dem[7]])}, {"step": 9, "insert": new2}]
    case.notes["events"] = "4: +5 DEM, -%d fluid; 9: -3 DEM, +3 fluid" % fluid[::40].size
    return case


def workload(name: str, **kw) -> Case:
    """The five configurations at full size, plus the small variants used as
    golden-fixture and parity cases."""
    table = {
        # full-size configurations
        "dambreak2d": lambda: dambreak2d(),
        "dem_settling3d": lambda: dem_settling3d(),
        "sediment3d": lambda: sediment3d(),
        # differentiated coupled workload: 100k fluid, 5k DEM, in the form the
        # adjoint covers (three fixed sphBoundary floor layers, constant h)
        "sediment3d_adjoint": lambda: sediment3d(nx=37, n_dem=5000, nsteps=500, seed=4, floor="sphb3",
                                                 var_h=False),
        # the same with the coupled configuration's VAR_H_CORRECTION
        "sediment3d_adjoint_varh": lambda: sediment3d(nx=37, n_dem=5000, nsteps=500, seed=4, floor="sphb3",
                                                      var_h=True),
        # small parity cases (seconds on one CPU core)
        "dambreak2d_small": lambda: dambreak2d(dx=0.05, nsteps=40),
        # damBreak's own options: Monaghan viscosity (nu = 1e-2), anticlumping,
        # smoothing length following density
        "dambreak2d_monaghan_small": lambda: dambreak2d(dx=0.05, nsteps=40,
                                                        visc_model=VISC_MONAGHAN,
                                                        anticlumping=True, const_h=False,
                                                        viscosity=1e-2),
        # damBreak's customConstants.h as written: the above plus
        # CORRECTED_GRADIENT and density re-initialisation every step
        "dambreak2d_own_small": lambda: dambreak2d(dx=0.05, nsteps=30, visc_model=VISC_MONAGHAN,
                                                   anticlumping=True, const_h=False, viscosity=1e-2,
                                                   corrected_gradient=True, reinit_every=1,
                                                   fixed_dt=False),
        # the corrected gradient under VAR_H_CORRECTION, re-initialisation
        # every 7 steps and at step 3
        "dambreak2d_cg_varh_small": lambda: dambreak2d(dx=0.05, nsteps=20, const_h=False, var_h=True,
                                                       corrected_gradient=True, reinit_every=7,
                                                       reinit_at=3, seed=5, fixed_dt=False),
        "dem_small": lambda: dem_settling3d(lattice=(6, 6, 10), box=(0.0138, 0.0138, 0.023),
                                            spread=0.0, nsteps=600, vel_amp=0.3),
        "dem_small_poly": lambda: dem_settling3d(lattice=(6, 6, 10), box=(0.0144, 0.0144, 0.024),
                                                 nsteps=600, vel_amp=0.3),
        "sediment3d_small": lambda: sediment3d(nx=10, L=0.04, height=0.08, n_dem=100,
                                               nsteps=20),
        # particles deleted and inserted between steps (insertNewParticle,
        # markForDeletion)
        "dambreak2d_flow_small": lambda: dambreak2d_flow(),
        # coupled, with DEM spheres and fluid particles entering and leaving
        "sediment3d_flow_small": lambda: sediment3d_flow(),
        # coupled, DEM moving as one block under the mean DEM force
        "sediment3d_block_small": lambda: sediment3d(nx=10, L=0.04, height=0.08, n_dem=100, nsteps=20,
                                                     dem_block=True, seed=6),
        # coupled, periodic: density re-initialisation every 4 steps (the
        # surface particles' h grows by ~1/3, so the box is 8.75 h_max wide)
        "sediment3d_reinit_small": lambda: sediment3d(nx=15, L=0.06, height=0.05, n_dem=100, nsteps=12,
                                                      reinit_every=4),
        "sediment3d_adjoint_small": lambda: sediment3d(nx=10, L=0.04, height=0.08, n_dem=60, nsteps=30,
                                                       floor="sphb3", var_h=False, viscosity=1e-4),
        # the same with sediment3D's VAR_H_CORRECTION (h following density)
        "sediment3d_adjoint_varh_small": lambda: sediment3d(nx=10, L=0.04, height=0.08, n_dem=60, nsteps=30,
                                                            floor="sphb3", var_h=True, viscosity=1e-4),
    }
    if name not in table:
        raise KeyError(f"unknown workload {name!r}; known: {sorted(table)}")
    case = table[name]()
    case.name = name
    return case
