"""CUDA path against the CPU oracle through the C ABI (-m gpu).

Bar: neighbour relations and reference bucket indices bit-exact; FP64
fields within 1e-9 of each field's scale after the workload's full step
count (the only differences are FMA contraction and integer powers in place
of pow()); the oracle itself is pinned to the reference by
tests/test_oracle_golden.py.
"""
import numpy as np
import pytest

from sphdem import capi, cases
from sphdem.state import pair_set
from oracle.port_api import OracleSim

pytestmark = pytest.mark.gpu

WORKLOADS = ["dambreak2d_small", "dambreak2d_monaghan_small", "dem_small", "dem_small_poly",
             "sediment3d_small", "dambreak2d_own_small", "dambreak2d_cg_varh_small",
             "sediment3d_reinit_small", "sediment3d_block_small", "dambreak2d_flow_small",
             "sediment3d_flow_small"]
FIELDS = ["r", "v", "vhat", "v0", "vhat0", "f", "fp", "fv", "fb", "dens", "dddt", "h",
          "press", "pdr2", "porosity", "dporositydt", "grad_porosity", "shep_sum", "fdrag",
          "fvel", "omega"]
FP64_RTOL = 1e-9


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def field_floor(cfg, k):
    """Pressure is PRB*((rho/rho0)^7-1): near rest it cancels, so its scale is PRB."""
    if k == "press":
        return cfg["prb"]
    if k == "pdr2":
        return cfg["prb"] / cfg["dens"] ** 2
    return 1e-300


def compare(gpu, ora, fields, rtol, label, cfg=None):
    """Fields of the live particles (deleted slots keep stale values)."""
    worst = {}
    fails = []
    live = ora["iam"] >= 0
    assert np.array_equal(gpu["iam"] >= 0, live), f"{label}: live sets differ"
    for k in fields:
        a, b = gpu[k][live], ora[k][live]
        scale = max(np.abs(b).max(), field_floor(cfg, k) if cfg else 1e-300)
        err = np.abs(a - b).max()
        worst[k] = err / scale
        if err > rtol * scale:
            fails.append(f"{k} err {err:.3e} scale {scale:.3e}")
    print(label, {k: f"{v:.1e}" for k, v in worst.items()})
    assert not fails, f"{label}: " + "; ".join(fails)
    return worst


@pytest.mark.parametrize("name", WORKLOADS)
def test_fp64_step_by_step_phases(lib, name):
    """Phase-level API (sphdem_phase) matches the oracle after one step."""
    case = cases.workload(name)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    ora = OracleSim(case.cfg, case.particles)
    for p in range(7):
        sim.phase(p)
        ora.phase(p)
    compare(sim.get(), ora.get(), FIELDS, 1e-11, name + "@1", case.cfg)
    g1, g2 = sim.globals(), ora.globals()
    assert g1.time == pytest.approx(g2.time, rel=1e-15)
    assert g1.sph_step == g2.sph_step == 1


@pytest.mark.parametrize("name", WORKLOADS)
def test_fp64_full_run_fields_pairs_cells(lib, name):
    case = cases.workload(name)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64,
                          capacity=case.n + case.n_inserted)
    ora = OracleSim(case.cfg, case.particles)
    cases.advance(sim, case)
    cases.advance(ora, case)
    assert sim.n == ora.n
    compare(sim.get(), ora.get(), FIELDS, FP64_RTOL, name, case.cfg)
    g1, g2 = sim.globals(), ora.globals()
    # equal under FIXED_DT; adaptive dt is a minimum over the forces
    assert g1.dt == pytest.approx(g2.dt, rel=1e-12) and g1.n_deleted == g2.n_deleted
    if case.cfg["flags"] & cases.F_FIXED_DT:
        assert g1.dt == g2.dt
    assert g1.new_dt == pytest.approx(g2.new_dt, rel=1e-9)
    sim.rebuild()
    ora.rebuild()
    for kind, kname in capi.PAIR_KIND_NAMES.items():
        a = pair_set(*sim.pairs(kind))
        b = pair_set(*ora.pairs(kind))
        assert np.array_equal(a, b), f"{name}:{kname}: gpu {a.size} oracle {b.size}"
    live = ora.get()["iam"] >= 0
    assert np.array_equal(sim.cell_ids()[live], ora.cells()[live])


# ---------------------------------------------------------------------------
# mixed precision: FP32 pair math on cell-relative offsets, FP64 integration
MIXED_WORKLOADS = ["dambreak2d_small", "dambreak2d_monaghan_small", "dem_small", "sediment3d_small",
                   "sediment3d_reinit_small", "sediment3d_block_small", "dambreak2d_flow_small",
                   "sediment3d_flow_small", "dambreak2d_own_small", "dambreak2d_cg_varh_small"]
# stated tolerances over the workloads' full step counts: density to 1e-5 of
# its value, positions to 1e-6 of the largest coordinate, accelerations to
# 1e-3 of the largest acceleration magnitude
MIXED_TOL = {"dens": 1e-5, "r": 1e-6, "f": 1e-3}
# damBreak's own constants: the corrected gradient multiplies each pair's
# gradient by the inverse moment matrix, whose condition number at particles
# of the free surface (few neighbours) amplifies the FP32 rounding of the pair
# offsets; with density re-initialisation every step (a summation over those
# positions) the run keeps the mixed-precision bar of 1e-4 on density, not 1e-5
MIXED_TOL_BY_CASE = {"dambreak2d_own_small": {"dens": 1e-4, "r": 1e-5, "f": 1e-3}}


@pytest.mark.parametrize("name", MIXED_WORKLOADS)
def test_mixed_pair_lists_exact(lib, name):
    """The FP32-built neighbour lists equal the reference's FP64 pair set."""
    case = cases.workload(name)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED,
                          capacity=case.n + case.n_inserted)
    ora = OracleSim(case.cfg, case.particles)
    n = min(case.nsteps, 24)
    cases.advance(sim, case, n)
    cases.advance(ora, case, n)
    # compare at the oracle's positions: load them into the GPU, rebuild both
    buf = ora.get()
    sim.set(buf, capi.FIELD_R | capi.FIELD_H)
    sim.rebuild()
    ora.rebuild()
    for kind in (capi.PAIRS_SPH, capi.PAIRS_DEM, capi.PAIRS_COUPLE_SD, capi.PAIRS_COUPLE_DS):
        a = pair_set(*sim.pairs(kind))
        b = pair_set(*ora.pairs(kind))
        assert np.array_equal(a, b), f"{name}:{capi.PAIR_KIND_NAMES[kind]}: {a.size} vs {b.size}"


@pytest.mark.parametrize("name", MIXED_WORKLOADS)
def test_mixed_fields_within_tolerance(lib, name):
    case = cases.workload(name)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED,
                          capacity=case.n + case.n_inserted)
    ora = OracleSim(case.cfg, case.particles)
    cases.advance(sim, case)
    cases.advance(ora, case)
    a, b = sim.get(), ora.get()
    live = b["iam"] >= 0
    assert np.array_equal(a["iam"] >= 0, live)
    a = {k: a[k][live] for k in ("dens", "r", "f")}
    b = {k: b[k][live] for k in ("dens", "r", "f")}
    errs = {
        "dens": np.abs(a["dens"] - b["dens"]).max() / np.abs(b["dens"]).max(),
        "r": np.abs(a["r"] - b["r"]).max() / np.abs(b["r"]).max(),
        "f": np.abs(a["f"] - b["f"]).max() / max(np.abs(b["f"]).max(), 1e-300),
    }
    print(name, "mixed vs oracle", {k: f"{v:.2e}" for k, v in errs.items()})
    for k, tol in MIXED_TOL_BY_CASE.get(name, MIXED_TOL).items():
        assert errs[k] <= tol, f"{name}: {k} {errs[k]:.3e} > {tol}"


# ---------------------------------------------------------------------------
# CORRECTED_GRADIENT and density re-initialisation
def test_reinit_graph_and_phase_paths_agree(lib):
    """Steps through the graph cache (re-initialising and plain steps have
    their own graphs) equal the phase-by-phase path, across the steps where
    the re-initialisation switches on and off."""
    case = cases.workload("dambreak2d_cg_varh_small")
    a = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    b = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    a.step(15)
    for _ in range(15):
        for p in range(7):
            b.phase(p)
    assert a.globals().sph_step == b.globals().sph_step == 15
    compare(a.get(), b.get(), ["r", "v", "dens", "h", "f"], 1e-13, "graph vs phases")


def test_corrected_gradient_and_reinit_restrictions(lib):
    """CORRECTED_GRADIENT runs on both paths but not with LIQ_DEM (the
    reference's calcFPI would take a DEM particle's invM, which calcInvM never
    sets); a batch takes no handle that re-initialises the density."""
    case = cases.workload("dambreak2d_own_small")
    cpl = cases.workload("sediment3d_small")
    cfg = dict(cpl.cfg)
    cfg["flags"] |= cases.F_CORRECTED_GRADIENT
    for prec in (cases.PREC_MIXED, cases.PREC_FP64):
        with pytest.raises(capi.SphDemError):
            capi.Simulation(lib, cfg, cpl.particles, precision=prec)
    cfg = dict(case.cfg)
    cfg["flags"] &= ~cases.F_CORRECTED_GRADIENT
    sim = capi.Simulation(lib, cfg, case.particles, precision=cases.PREC_FP64)
    with pytest.raises(capi.SphDemError):
        capi.Batch(lib, [sim])


@pytest.mark.parametrize("name", ["sediment3d_small", "dambreak2d_small", "dambreak2d_own_small"])
def test_staged_force_pass_equals_plain_loads(lib, name, monkeypatch):
    """The force and continuity passes with their neighbour records staged in
    shared memory by bulk copies (SPHDEM_FORCE_TILE=1) give bit for bit the
    results of the same passes reading every record through L1 (the
    default)."""
    case = cases.workload(name)
    out = []
    for tile in ("1", "0"):
        monkeypatch.setenv("SPHDEM_FORCE_TILE", tile)
        sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
        for _ in range(4):
            for p in range(7):
                sim.phase(p)
        out.append(sim.get(capi.FIELD_F | capi.FIELD_R | capi.FIELD_DENS))
        sim.close()
    for k in ("f", "r", "dens"):
        if name.startswith("sediment"):
            # the coupled step's Shepard scatter sums with atomics: rounding
            scale = np.abs(out[1][k]).max()
            assert np.abs(out[0][k] - out[1][k]).max() <= 1e-6 * scale, k
        else:
            np.testing.assert_array_equal(out[0][k], out[1][k], err_msg=k)
