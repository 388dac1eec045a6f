"""Allocation-free bucket-index export (sphdem_cell_ids_noalloc) through the
C ABI, against the allocating entry point sphdem_cell_ids (-m gpu).

Integer output, so the bar is equality.  Collected last on purpose: it must
hold after every other test has used the device, and alone in a fresh
process.
"""
import numpy as np
import pytest

from sphdem import capi, cases

pytestmark = pytest.mark.gpu

NOALLOC_MAX = 262144  # SPHDEM_CELL_IDS_NOALLOC_MAX in include/sphdem.h


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


@pytest.mark.parametrize("name,precision", [("sediment3d_small", cases.PREC_MIXED),
                                            ("sediment3d_small", cases.PREC_FP64),
                                            ("dambreak2d_small", cases.PREC_FP64)])
def test_noalloc_matches_cell_ids(lib, name, precision):
    case = cases.workload(name)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=precision)
    try:
        sim.step(3)
        ref = sim.cell_ids()
        first = sim.cell_ids_noalloc()
        second = sim.cell_ids_noalloc()
        np.testing.assert_array_equal(first, ref)
        np.testing.assert_array_equal(second, ref)
        # after the state moves on, the shared array holds the new indices
        sim.step(2)
        np.testing.assert_array_equal(sim.cell_ids_noalloc(), sim.cell_ids())
    finally:
        sim.close()


def test_noalloc_rejects_large(lib):
    case = cases.sediment3d(nx=40, L=0.1, height=0.4, n_dem=12500, seed=3, nsteps=2)
    assert case.n > NOALLOC_MAX
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    try:
        with pytest.raises(capi.SphDemError, match="CAPACITY"):
            sim.cell_ids_noalloc()
        # the handle stays usable
        assert sim.cell_ids().shape == (case.n, 3)
    finally:
        sim.close()
