"""sphdem_get_fields_async / sphdem_fields_wait (-m gpu): fields copied while
the following steps run equal the ones sphdem_get_fields returns after each
step."""
import numpy as np
import pytest

from sphdem import capi, cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


@pytest.mark.parametrize("pinned", [True, False])
def test_async_copies_match_sync(lib, pinned):
    # a workload without atomics in its step, so that two runs agree bit for bit
    case = cases.workload("dambreak2d_monaghan_small")
    a = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    b = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    mask = capi.FIELD_R | capi.FIELD_DENS | capi.FIELD_V
    bufs = [capi.ParticleBuffers(a.n, pinned=lib if pinned else None, fields=("r", "dens", "v")) for _ in range(5)]
    want = []
    for k in range(5):
        a.step(1)
        a.get_async(mask, bufs[k])     # up to five transfers queued behind the steps
        b.step(1)
        want.append(b.get(mask))
    a.fields_wait()
    for k in range(5):
        for f in ("r", "dens", "v"):
            np.testing.assert_array_equal(bufs[k][f], want[k][f], err_msg=f"step {k + 1} {f}")
