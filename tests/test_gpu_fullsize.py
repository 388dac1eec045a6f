"""Size-independent properties at the full coupled sedimentation workload
(1,080,400 particles: 1,024,000 fluid, 6,400 boundary, 50,000 DEM; -m gpu).

The oracle does not finish this size in seconds, so parity at this size rests
on properties that hold at any size, checked against the FP64 path (which the
small workloads pin to the oracle field by field):

- after mixed-precision steps, the FP32-built neighbour lists equal the exact
  pair sets of the reference predicate evaluated in FP64 on the same
  positions, for all four relations (fluid, DEM contacts, fluid -> DEM,
  DEM -> fluid);
- both paths put every particle in the same reference bucket.
"""
import numpy as np
import pytest

from sphdem import capi, cases

pytestmark = pytest.mark.gpu

NSTEPS = 5


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def test_full_size_lists_and_buckets_exact(lib):
    case = cases.sediment3d(seed=3)
    assert case.n == 1_080_400
    mixed = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    mixed.step(NSTEPS)
    fp64 = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    fp64.set(mixed.get(capi.FIELD_R | capi.FIELD_H), capi.FIELD_R | capi.FIELD_H)
    # The periodic ghost widths of a rebuild come from the largest h per
    # slot at the rebuild before it (dataLL.cpp:522-582, 688-693), so two
    # rebuilds on the same positions and h give both handles the same widths.
    for _ in range(2):
        mixed.rebuild()
        fp64.rebuild()
    try:
        for kind, kname in capi.PAIR_KIND_NAMES.items():
            oa, ia = mixed.pairs(kind)
            ob, ib = fp64.pairs(kind)
            assert np.array_equal(oa, ob), f"{kname}: neighbour counts differ"
            assert np.array_equal(ia, ib), f"{kname}: neighbour sets differ"
            print(f"{kname}: {ia.size} pairs")
        assert np.array_equal(mixed.cell_ids(), fp64.cell_ids())
    finally:
        mixed.close()
        fp64.close()
