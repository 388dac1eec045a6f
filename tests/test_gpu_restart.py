"""Restart through the reference's file formats (-m gpu): a run saved at an
output step (restart pair + Globals + Domain, sphdem.io_vtk.save_simulation)
and loaded into a new handle continues as the uninterrupted run does.

The exact form (Float64 points plus f, dddt, fdrag and the energy rates)
continues to 1e-12 of each field's scale in FP64; mixed-precision coupled
runs differ between any two runs at FP32 rounding level (the FP32 Shepard
scatter's atomics add in a varying order, which moves the drag), so their
bar is 1e-6.  The reference's own
form (Float32 points, no f or dddt, as its writer stores them) is checked to
load and step, staying within 1e-2 of the particle spacing of the
uninterrupted run after 5 steps (the first step restarts the predictor
from f = 0, as a restart of the reference does).
"""
import numpy as np
import pytest

from sphdem import capi, cases, io_vtk

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


@pytest.mark.parametrize("name,precision", [("dambreak2d_small", cases.PREC_FP64),
                                            ("dambreak2d_small", cases.PREC_MIXED),
                                            ("sediment3d_small", cases.PREC_FP64),
                                            ("sediment3d_small", cases.PREC_MIXED)])
def test_exact_restart_continues_the_run(lib, tmp_path, name, precision):
    case = cases.workload(name)
    a = capi.Simulation(lib, case.cfg, case.particles, precision=precision)
    try:
        a.step(10)
        base = str(tmp_path / "run")
        pvtu = io_vtk.save_simulation(a, base, 1, exact=True)
        b = io_vtk.load_simulation(lib, case.cfg, pvtu, precision=precision, globals_path=base + "Globals0.dat")
        try:
            ga, gb = a.globals(), b.globals()
            assert (ga.time, ga.dt, ga.sph_step) == (gb.time, gb.dt, gb.sph_step)
            a.step(10)
            b.step(10)
            x, y = a.get(), b.get()
            tol = 1e-12 if precision == cases.PREC_FP64 or name.startswith("dambreak") else 1e-6
            for k in ("r", "v", "vhat", "dens", "f", "u"):
                scale = max(np.abs(x[k]).max(), 1e-300)
                err = np.abs(x[k] - y[k]).max()
                assert err <= tol * scale, f"{name}:{k} err {err:.3e} scale {scale:.3e}"
            assert a.globals().time == b.globals().time
        finally:
            b.close()
    finally:
        a.close()


def test_reference_form_restart_loads_and_steps(lib, tmp_path):
    case = cases.workload("dambreak2d_small")
    a = capi.Simulation(lib, case.cfg, case.particles, precision=cases.PREC_FP64)
    try:
        a.step(5)
        pvtu = io_vtk.save_simulation(a, str(tmp_path / "ref"), 0, exact=False)
        d = io_vtk.read_restart(pvtu)
        assert d["points_type"] == "Float32" and "f" not in d["arrays"]
        b = io_vtk.load_simulation(lib, case.cfg, pvtu, precision=cases.PREC_FP64)
        try:
            b.step(5)
            x = b.get()
            assert np.isfinite(x["r"]).all() and np.isfinite(x["dens"]).all()
            a.step(5)
            ref = a.get()["r"]
            assert np.abs(x["r"] - ref).max() < 1e-2 * case.cfg["psep"]
        finally:
            b.close()
    finally:
        a.close()
