"""Particle insertion and deletion through the C ABI (-m gpu):
sphdem_insert_particles (CdataLL::insertNewParticle, dataLL.cpp:238-261) and
sphdem_mark_for_deletion (CdataLL::markForDeletion, dataLL.cpp:263-266).
The scheduled run against the oracle and the reference's golden is in
test_gpu_parity.py (workload dambreak2d_flow_small); these are the edge cases.
"""
import numpy as np
import pytest

from sphdem import capi, cases
from oracle.port_api import OracleSim

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def _fluid_block(case, xy, v=(0.0, -1.0)):
    dx = case.cfg["psep"]
    m = len(xy)
    blk = {k: np.zeros((m, 3)) for k in ("r", "v")}
    blk["r"][:, :2] = xy
    blk["v"][:, :2] = v
    blk["iam"] = np.zeros(m, np.int32)
    blk["mass"] = np.full(m, dx * dx * case.cfg["dens"])
    blk["dens"] = np.full(m, case.cfg["dens"])
    blk["h"] = np.full(m, case.cfg["h"])
    return blk


def test_capacity_and_index_errors(lib):
    case = cases.workload("dambreak2d_small")
    sim = capi.Simulation(lib, case.cfg, case.particles, capacity=case.n + 3)
    # more than the capacity: nothing inserted
    with pytest.raises(capi.SphDemError, match="CAPACITY"):
        sim.insert(_fluid_block(case, [[0.5, 2.1]] * 4))
    assert sim.n == case.n
    # an empty insertion is a no-op
    assert sim.insert(_fluid_block(case, np.zeros((0, 2)))).size == 0
    # deletion indices: out of range, then of an already deleted particle
    with pytest.raises(capi.SphDemError, match="INVALID"):
        sim.mark_for_deletion([case.n])
    sim.mark_for_deletion([5])
    sim.rebuild()
    assert sim.get()["iam"][5] == -1
    with pytest.raises(capi.SphDemError, match="INVALID"):
        sim.mark_for_deletion([5])
    # the freed slot is taken first, then the ones past the end
    idx = sim.insert(_fluid_block(case, [[0.5, 2.1], [0.6, 2.1], [0.7, 2.1]]))
    assert list(idx) == [5, case.n, case.n + 1]
    assert sim.n == case.n + 2
    sim.step(3)
    g = sim.get()
    assert (g["iam"] >= 0).all() and np.isfinite(g["r"]).all()


def test_marked_particles_stay_until_the_next_reset(lib):
    """A marked particle takes part in the step as usual until the middle
    phase's reset removes it -- the phase-level path against the oracle."""
    case = cases.workload("dambreak2d_small")
    sim = capi.Simulation(lib, case.cfg, case.particles)
    ora = OracleSim(case.cfg, case.particles)
    sim.step(2)
    ora.step(2)
    marked = np.arange(400, 420)
    sim.mark_for_deletion(marked)
    ora.mark_for_deletion(marked)
    for p in range(3):          # before-start hook, start, before-middle hook
        sim.phase(p)
        ora.phase(p)
    a, b = sim.get(), ora.get()
    assert (a["iam"][marked] >= 0).all() and (b["iam"][marked] >= 0).all()
    np.testing.assert_allclose(a["r"], b["r"], rtol=0, atol=1e-12)
    sim.phase(capi.PHASE_MIDDLE)
    ora.phase(capi.PHASE_MIDDLE)
    a, b = sim.get(), ora.get()
    assert (a["iam"][marked] == -1).all() and (b["iam"][marked] == -1).all()
    live = b["iam"] >= 0
    np.testing.assert_allclose(a["f"][live], b["f"][live], rtol=0, atol=1e-9 * np.abs(b["f"][live]).max())


def test_out_of_domain_slot_is_reused(lib):
    """A particle lost from the binning domain frees its slot too."""
    case = cases.workload("dambreak2d_small")
    p = {k: v.copy() for k, v in case.particles.items()}
    far = int(np.nonzero(p["iam"] == 0)[0][-1])
    p["r"][far, 1] = 100.0          # outside the domain: deleted by the first reset
    sim = capi.Simulation(lib, case.cfg, p, capacity=case.n + 1)
    assert sim.globals().n_deleted == 1
    assert sim.get()["iam"][far] == -1
    idx = sim.insert(_fluid_block(case, [[0.5, 2.1]]))
    assert list(idx) == [far]
    sim.step(2)
    assert sim.get()["iam"][far] == 0


def test_batch_recaptures_after_insertion(lib):
    case = cases.workload("dambreak2d_small")
    sims = [capi.Simulation(lib, case.cfg, case.particles, capacity=case.n + 8) for _ in range(2)]
    ref = capi.Simulation(lib, case.cfg, case.particles, capacity=case.n + 8)
    b = capi.Batch(lib, sims)
    b.step(2)
    ref.step(2)
    blk = _fluid_block(case, [[0.5, 2.1], [0.55, 2.1]])
    sims[0].insert(blk)
    ref.insert(blk)
    b.step(3)
    ref.step(3)
    a, r = sims[0].get(), ref.get()
    assert a.n == r.n == case.n + 2
    np.testing.assert_array_equal(a["r"], r["r"])
    assert sims[1].n == case.n
