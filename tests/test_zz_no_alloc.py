"""Allocation-free bucket-index export (sphdem_cell_ids_noalloc) through the
C ABI, against the allocating entry point sphdem_cell_ids (-m gpu).

Integer output, so the bar is equality.  Collected last on purpose: it must
hold after every other test has used the device, and alone in a fresh
process.
"""
import ctypes as C
import os
import subprocess
import sys

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


def _free_device_bytes() -> int:
    """cudaMemGetInfo's free bytes, through the CUDA runtime libsphdem.so loads."""
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def test_noalloc_takes_no_device_memory(lib):
    """After the first call (which may load the module, and with it the static
    array, on the device), further calls leave the device's free memory as it
    was: the entry point allocates nothing."""
    case = cases.workload("sediment3d_small")
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
    try:
        sim.step(2)
        first = sim.cell_ids_noalloc()
        free0 = _free_device_bytes()
        for _ in range(5):
            again = sim.cell_ids_noalloc()
            np.testing.assert_array_equal(again, first)
        assert _free_device_bytes() == free0
    finally:
        sim.close()


FRESH = r"""
import sys
sys.path[:0] = {paths!r}
import numpy as np
from sphdem import capi, cases
lib = capi.Library()
case = cases.workload("sediment3d_small")
sim = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_MIXED)
sim.step(3)
a = sim.cell_ids_noalloc()
b = sim.cell_ids_noalloc()
ref = sim.cell_ids()
assert (a == ref).all() and (b == ref).all()
sim.close()
print("fresh-process noalloc ok")
"""


def test_noalloc_first_call_in_fresh_process(lib, repo_root):
    """The entry point as the first device export of a process that has run
    nothing else: two calls in a row, then the allocating export."""
    paths = [os.path.join(repo_root, "sph-dem_gb300"), repo_root]
    res = subprocess.run([sys.executable, "-c", FRESH.format(paths=paths)], capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-4000:]
    assert "fresh-process noalloc ok" in res.stdout


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
