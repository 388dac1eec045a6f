"""The reference's on-disk formats (sphdem.io_vtk): VTK XML restart files,
Globals and Domain files.

Round trips run everywhere.  Where the reference's own shipped restart and
Globals files are present, they are decoded and checked against the numbers
VTK itself wrote into them (each array's RangeMin / RangeMax, the point
count) and against their structure (unique tags, valid particle types).
"""
import os

import numpy as np
import pytest

from oracle.refroot import REF_ROOT as REF
from sphdem import cases, io_vtk

SHIPPED = ["singleDEM", "singleDEM3D", "singleDEMdrop3d"]


@pytest.mark.parametrize("name", ["dambreak2d_small", "sediment3d_small"])
@pytest.mark.parametrize("exact", [False, True])
def test_restart_round_trip(tmp_path, name, exact):
    case = cases.workload(name)
    nd = case.cfg["ndim"]
    ps = {k: np.asarray(v) for k, v in case.particles.items()}
    rng = np.random.default_rng(1)
    n = case.n
    ps["tag"] = np.arange(1, n + 1, dtype=np.int32)
    ps["v"] = rng.normal(size=(n, 3))
    ps["vhat"] = rng.normal(size=(n, 3))
    ps["u"] = rng.normal(size=n)
    ps["e_visc"] = rng.normal(size=n)
    ps["f"] = rng.normal(size=(n, 3))
    ps["dddt"] = rng.normal(size=n)
    if nd == 2:
        for k in ("r", "v", "vhat", "f", "norm1", "norm2", "norm3"):
            ps[k][:, 2] = 0.0
    base = str(tmp_path / "case")
    path = io_vtk.write_restart(base, 7, ps, nd, exact=exact)
    assert path.endswith("Restart0000007.pvtu") and os.path.exists(base + "Restart0000007_0.vtu")
    back = io_vtk.particles_from_restart(io_vtk.read_restart(path), nd)
    want_r = ps["r"] if exact else ps["r"].astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(back["r"][:, :nd], want_r[:, :nd])
    for k in ("v", "vhat", "mass", "dens", "h", "u", "e_visc", "iam", "tag"):
        np.testing.assert_array_equal(np.asarray(back[k]).reshape(n, -1)[:, :nd if np.ndim(ps[k]) == 2 else 1],
                                      np.asarray(ps[k]).reshape(n, -1)[:, :nd if np.ndim(ps[k]) == 2 else 1])
    if exact:
        np.testing.assert_array_equal(back["f"][:, :nd], ps["f"][:, :nd])
        np.testing.assert_array_equal(back["dddt"], ps["dddt"])
    else:
        assert "f" not in back and "dddt" not in back
    # a piece read on its own carries the same arrays
    piece = io_vtk.read_vtu(base + "Restart0000007_0.vtu")
    assert piece["n"] == n and piece["points_type"] == ("Float64" if exact else "Float32")


def test_encode_decode_many_blocks():
    a = np.random.default_rng(2).normal(size=(70000, 3))   # > one 32 KiB block
    txt = io_vtk.encode_array(a, "Float64")
    np.testing.assert_array_equal(io_vtk.decode_array(txt, "Float64", 3, True), a)


def test_globals_and_domain_round_trip(tmp_path):
    ov = {"lin_mom": [1.5, -2.25, 0.0], "ang_mom": 0.125, "e_ke": 3.0, "e_elast": 4.5, "e_elast_exact": 4.4,
          "ed_elast_dt": -0.5, "e_visc_f": 0.25, "ed_visc_f_dt": -0.01, "e_ff": 0.0, "ed_ff_dt": 0.0,
          "e_visc_b": 0.0, "e_b_force": 0.0, "e_total": 7.75, "max_v": 1.25, "max_f": 9.81, "max_ff": 0.0,
          "rms_ff": 0.0, "ave_dens": 1000.5, "var_dens": 0.03, "ave_dens_from_mass": 0.2, "n": 1418, "n_sph": 800}
    p = str(tmp_path / "caseGlobals0.dat")
    io_vtk.append_globals(p, 0, 0, 0.0, ov, dt=1e-4)
    io_vtk.append_globals(p, 1, 40, 0.0052, ov, dt=1e-4)
    rows = io_vtk.read_globals(p)
    assert len(rows) == 2 and rows[1]["SPHStep"] == 40 and rows[1]["Time"] == 0.0052
    assert rows[1]["linMomY"] == -2.25 and rows[1]["n"] == 1418 and rows[1]["custom"] == [1e-4]
    assert open(p).readline().startswith("# OutStep SPHStep Time linMomX")
    d = str(tmp_path / "caseDomain.dat")
    io_vtk.write_domain(d, 2, [0.0, 4.0, -0.1, 3.0])
    dom = io_vtk.read_domain(d, 2)
    assert dom["proc_domain"] == [0.0, 4.0, -0.1, 3.0] and dom["neighbours"][4] == -1


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference's shipped files are not present")
@pytest.mark.parametrize("case_dir", SHIPPED)
def test_reads_reference_restart_files(case_dir):
    pvtu = os.path.join(REF, case_dir, "initDataRestart0000000.pvtu")
    d = io_vtk.read_restart(pvtu)
    piece = os.path.join(REF, case_dir, "initDataRestart0000000_0.vtu")
    ranges = io_vtk.array_ranges(piece)
    assert d["n"] > 0 and d["points"].shape == (d["n"], 3)
    for name, a in d["arrays"].items():
        if name not in ranges:
            continue
        lo, hi = ranges[name]
        m = np.linalg.norm(a, axis=1) if a.ndim == 2 else a.astype(np.float64)
        assert m.min() == pytest.approx(lo, rel=1e-8, abs=1e-12), name
        assert m.max() == pytest.approx(hi, rel=1e-8, abs=1e-12), name
    pts = np.linalg.norm(d["points"], axis=1)
    # the points array carries its own range attributes (the first unnamed array)
    tags = d["arrays"]["tag"]
    assert np.unique(tags).size == d["n"]
    assert set(np.unique(d["arrays"]["iam"])) <= {0, 1, 2, 3, 4, 5, 11, 12, 13}
    ps = io_vtk.particles_from_restart(d, 3)
    assert np.all(np.diff(ps["tag"]) > 0) and np.isfinite(pts).all()


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference's shipped files are not present")
def test_reads_reference_globals_files():
    for d in ("damBreak", "singleDEM", "singleDEM3D", "singleDEMdrop3d", "2dMicro"):
        rows = io_vtk.read_globals(os.path.join(REF, d, "initDataGlobals0.dat"))
        assert len(rows) == 1 and rows[0]["OutStep"] == 0 and rows[0]["SPHStep"] == 0 and rows[0]["Time"] == 0
    dom = io_vtk.read_domain(os.path.join(REF, "damBreak", "initDataDomain.dat"), 2)
    assert dom["rank"] == 0 and len(dom["proc_domain"]) == 4
