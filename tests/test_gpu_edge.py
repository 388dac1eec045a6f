"""Edge cases of the step (-m gpu), each against the CPU oracle: an empty
input, a lone particle, coincident particles, particles exactly on bucket
faces, and a list that outgrows its depth (an error, never a dropped pair)."""
import numpy as np
import pytest

from sphdem import capi, cases
from sphdem.state import pair_set
from oracle.port_api import OracleSim

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def _fluid(case, xy):
    dx = case.cfg["psep"]
    m = len(xy)
    blk = cases._empty_particles(m)
    blk["r"][:, :2] = np.asarray(xy, float)
    blk["iam"][:] = cases.SPH
    blk["mass"][:] = dx * dx * case.cfg["dens"]
    blk["dens"][:] = case.cfg["dens"]
    blk["h"][:] = case.cfg["h"]
    return blk


def _compare(lib, cfg, ps, steps, precision, rtol):
    sim = capi.Simulation(lib, cfg, ps, precision=precision)
    ora = OracleSim(cfg, ps)
    sim.step(steps)
    ora.step(steps)
    a, b = sim.get(), ora.get()
    for k in ("r", "v", "dens", "f"):
        assert np.isfinite(a[k]).all(), k
        scale = max(np.abs(b[k]).max(), 1e-30)
        assert np.abs(a[k] - b[k]).max() <= rtol * scale, k
    return sim, ora


def test_empty_input_is_rejected(lib):
    case = cases.workload("dambreak2d_small")
    empty = {k: v[:0] for k, v in case.particles.items()}
    with pytest.raises(capi.SphDemError, match="INVALID"):
        capi.Simulation(lib, case.cfg, empty)


@pytest.mark.parametrize("precision", [cases.PREC_FP64, cases.PREC_MIXED])
def test_lone_particle_falls_freely(lib, precision):
    case = cases.workload("dambreak2d_small")
    ps = _fluid(case, [[2.0, 1.5]])
    sim, ora = _compare(lib, case.cfg, ps, 10, precision, 1e-12)
    a = sim.get()
    assert a["dens"][0] == case.cfg["dens"]   # no neighbours: the continuity sum is empty
    assert a["v"][0, 1] < 0.0                 # gravity only


@pytest.mark.parametrize("precision", [cases.PREC_FP64, cases.PREC_MIXED])
def test_coincident_particles(lib, precision):
    """r = 0 between two particles: the gradient is zero there (gradW skips
    q = 0, sph.h:324), no NaN."""
    case = cases.workload("dambreak2d_small")
    ps = _fluid(case, [[2.0, 1.5], [2.0, 1.5], [2.03, 1.5]])
    _compare(lib, case.cfg, ps, 5, precision, 1e-9 if precision == cases.PREC_FP64 else 1e-4)


def test_particles_on_bucket_faces(lib):
    """Particles exactly on SPH bucket faces (integer multiples of the bucket
    size from the grid origin): the same buckets and pair set as the oracle."""
    case = cases.workload("dambreak2d_small")
    cfg = case.cfg
    w = 2.0 * cfg["h"]                     # bucket size at the first rebuild (search radius = h)
    x0, y0 = cfg["domain_min"][0], cfg["domain_min"][1]
    kx = np.arange(int((1.0 - x0) / w), int((1.6 - x0) / w))
    ky = np.arange(int((0.5 - y0) / w), int((1.0 - y0) / w))
    xy = [[x0 + i * w, y0 + j * w] for i in kx for j in ky]
    xy += [[x0 + i * w + 0.5 * cfg["psep"], y0 + j * w] for i in kx for j in ky]
    ps = _fluid(case, xy)
    sim = capi.Simulation(lib, cfg, ps, precision=cases.PREC_FP64)
    ora = OracleSim(cfg, ps)
    assert np.array_equal(sim.cell_ids(), ora.cells())
    a = pair_set(*sim.pairs(capi.PAIRS_SPH))
    b = pair_set(*ora.pairs(capi.PAIRS_SPH))
    assert a.size > 0 and np.array_equal(a, b)
    mx = capi.Simulation(lib, cfg, ps, precision=cases.PREC_MIXED)
    assert np.array_equal(pair_set(*mx.pairs(capi.PAIRS_SPH)), b)


def test_list_depth_overflow_is_an_error(lib):
    """Mixed precision sizes its lists at creation; squeezing the particles
    together afterwards must stop the step with CAPACITY, not drop pairs."""
    case = cases.workload("dambreak2d_small")
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    buf = sim.get(capi.FIELD_R | capi.FIELD_IAM)
    fluid = buf["iam"] == cases.SPH
    r = buf["r"].copy()
    c = r[fluid].mean(axis=0)
    r[fluid] = c + 0.25 * (r[fluid] - c)   # four times denser in each direction
    buf["r"][...] = r
    sim.set(buf, capi.FIELD_R)
    with pytest.raises(capi.SphDemError, match="CAPACITY"):
        sim.step(1)
