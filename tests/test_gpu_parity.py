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
             "sediment3d_small"]
FIELDS = ["r", "v", "vhat", "v0", "vhat0", "f", "fp", "fv", "fb", "dens", "dddt", "h",
          "press", "pdr2", "porosity", "dporositydt", "grad_porosity", "shep_sum", "fdrag",
          "fvel", "omega"]
FP64_RTOL = 1e-9


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def compare(gpu, ora, fields, rtol, label):
    worst = {}
    for k in fields:
        a, b = gpu[k], ora[k]
        scale = np.abs(b).max()
        err = np.abs(a - b).max()
        worst[k] = err / scale if scale > 0 else err
        assert err <= rtol * max(scale, 1e-300), f"{label}: {k} err {err:.3e} scale {scale:.3e}"
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
    compare(sim.get(), ora.get(), FIELDS, 1e-11, name + "@1")
    g1, g2 = sim.globals(), ora.globals()
    assert g1.time == pytest.approx(g2.time, rel=1e-15)
    assert g1.sph_step == g2.sph_step == 1


@pytest.mark.parametrize("name", WORKLOADS)
def test_fp64_full_run_fields_pairs_cells(lib, name):
    case = cases.workload(name)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    ora = OracleSim(case.cfg, case.particles)
    sim.step(case.nsteps)
    ora.step(case.nsteps)
    compare(sim.get(), ora.get(), FIELDS, FP64_RTOL, name)
    g1, g2 = sim.globals(), ora.globals()
    assert g1.dt == g2.dt and g1.n_deleted == g2.n_deleted
    assert g1.new_dt == pytest.approx(g2.new_dt, rel=1e-9)
    sim.rebuild()
    ora.rebuild()
    for kind, kname in capi.PAIR_KIND_NAMES.items():
        a = pair_set(*sim.pairs(kind))
        b = pair_set(*ora.pairs(kind))
        assert np.array_equal(a, b), f"{name}:{kname}: gpu {a.size} oracle {b.size}"
    assert np.array_equal(sim.cell_ids(), ora.cells())
