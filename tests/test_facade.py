"""The C++ façade of the plug-in surface: case directories compile against
it (-m "not gpu") and a case's host hooks driving the device phases give the
same state as the device's built-in hooks (-m gpu)."""
import os
import struct
import subprocess
import sys

import numpy as np
import pytest

from oracle.refroot import REF_ROOT
from sphdem import capi, cases, state

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FACADE = os.path.join(REPO, "sph-dem_gb300", "facade")
sys.path.insert(0, FACADE)
from build_case import build_case  # noqa: E402

LIB = os.path.join(REPO, "sph-dem_gb300", "libsphdem.so")


def _need_lib():
    if not os.path.exists(LIB):
        import __graft_entry__
        __graft_entry__.build()


def test_example_case_builds(tmp_path):
    _need_lib()
    out = build_case(os.path.join(FACADE, "example_sediment"), str(tmp_path / "run_example"))
    assert os.path.exists(out)


def test_example_constants_in_step(tmp_path):
    sys.path.insert(0, os.path.join(FACADE, "example_sediment"))
    import make_constants
    with open(os.path.join(FACADE, "example_sediment", "customConstants.h")) as fh:
        assert fh.read() == make_constants.constants()


REF_CASE = os.path.join(REF_ROOT, "sediment3D")


@pytest.mark.skipif(not os.path.isdir(REF_CASE), reason="reference sources not present")
def test_reference_case_sources_build_unchanged(tmp_path):
    """The reference's own sediment3D hooks and output code, unmodified."""
    _need_lib()
    out = build_case(REF_CASE, str(tmp_path / "run_sediment3D"))
    assert os.path.exists(out)


@pytest.mark.skipif(not os.path.isdir(REF_CASE), reason="reference sources not present")
@pytest.mark.parametrize("name,option", [("cell3D", "SPH-DEM coupling variant"),
                                         ("porosityJump", "SPH-DEM coupling variant"),
                                         ("solitonPeriodic", "viscosity or boundary variant"),
                                         ("couette", "Wendland C2 kernel only")])
def test_reference_cases_with_options_the_device_lacks_do_not_build(tmp_path, name, option):
    """Reference case directories that compile against the reference's own
    headers but ask for step options the device path does not implement
    (cell3D and porosityJump: LIQ_DEM_SEPARATE_DRAGS, LIQ_DEM_VARIABLE_TIMESTEP;
    solitonPeriodic: a boundary variant; couette: a kernel other than
    Wendland C2) stop at compile time with the reason, instead of stepping
    differently from the reference."""
    _need_lib()
    with pytest.raises(RuntimeError, match=option):
        build_case(os.path.join(REF_ROOT, name), str(tmp_path / f"run_{name}"))


ORACLE_ABI = os.path.join(REPO, "tests", "facade_oracle", "sphdem_oracle_abi.cpp")
PORT_SRC = os.path.join(REPO, "oracle", "port", "sphdem_oracle.cpp")


@pytest.mark.skipif(not os.path.isdir(REF_CASE), reason="reference sources not present")
def test_reference_case_hooks_run_unchanged(tmp_path):
    """The reference's own sediment3D customSim.cpp / customOutput.cpp,
    unmodified, run end to end through the façade: the host mirror pulled and
    pushed around every hook, the case's constants as the configuration, the
    step loop of run.cpp.  The test runs where the reference's sources are
    present, on the CPU: the step phases come from the CPU oracle port through
    the same C ABI (tests/facade_oracle links it in place of the device
    library).  After
    four steps (adaptive dt) the state equals the oracle port's with its
    built-in hooks, which are sediment3D's: gravity on the fluid before the
    middle phase; gravity on the spheres, the floor wall and freezing
    (before TIME_DROP_PARTICLE) before the end phase; freezing after it."""
    libdir = tmp_path / "oracle_abi"
    libdir.mkdir()
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    "-I" + os.path.join(REPO, "include"), ORACLE_ABI, PORT_SRC, "-o", str(libdir / "libsphdem.so")],
                   check=True, capture_output=True, text=True)
    exe = build_case(REF_CASE, str(tmp_path / "run_sediment3D"), libdir=str(libdir))

    # the configuration the case's constants give (a one-particle run dumps it)
    probe = cases.dambreak2d(dx=0.1, nsteps=1)
    one = {k: np.asarray(v)[:1] for k, v in probe.particles.items()}
    one["r"] = np.array([[1e-3, 1e-3, 1e-3]])
    state.write_state(str(tmp_path / "one.spdm"), one)
    cfg_path = tmp_path / "cfg.bin"
    res = subprocess.run([exe, str(tmp_path / "one.spdm"), "0", str(tmp_path / "one.bin"), "--dump-config",
                          str(cfg_path)], capture_output=True, text=True, timeout=120, cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    cfg = capi.SphDemConfig.from_buffer_copy(cfg_path.read_bytes())
    assert cfg.ndim == 3 and cfg.flags & cases.F_LIQ_DEM and cfg.flags & cases.F_VAR_H_CORRECTION

    # a sedimentation state inside the case's box: fluid lattice on the case's
    # spacing over a repulsive floor layer, spheres of the case's radius
    L, height = cfg.rmax[0] - cfg.rmin[0], cfg.rmax[2] - cfg.rmin[2]
    nx = int(round(L / cfg.psep))
    gen = cases.sediment3d(nx=nx, L=L, height=height, n_dem=150, dem_radius_factor=cfg.dem_radius / cfg.psep,
                           rho_s=cfg.dem_dens, viscosity=cfg.viscosity, seed=12, nsteps=4)
    parts = {k: np.array(v) for k, v in gen.particles.items()}
    parts["h"][parts["iam"] == cases.DEM] = cfg.dem_search_radius
    init = tmp_path / "init.spdm"
    state.write_state(str(init), parts)
    nsteps = 4
    final = tmp_path / "final.bin"
    # the case's output code writes its own files into the working directory
    res = subprocess.run([exe, str(init), str(nsteps), str(final)], capture_output=True, text=True, timeout=600,
                         cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    a = read_final(str(final))

    # the oracle port with the built-in hooks
    import ctypes as C
    from oracle import port_api
    hooks = capi.SphDemConfig.from_buffer_copy(cfg_path.read_bytes())
    hooks.gravity_sph = capi.D3(0.0, 0.0, -9.81)
    hooks.gravity_dem = capi.D3(0.0, 0.0, -9.81)
    hooks.n_walls = 1
    hooks.walls[0].point = capi.D3(cfg.rmin[0], cfg.rmin[1], cfg.rmin[2])
    hooks.walls[0].normal = capi.D3(0.0, 0.0, 1.0)
    hooks.freeze_dem_until = cfg.time_drop_particle
    lib = port_api.lib()
    buf = capi.ParticleBuffers(len(parts["iam"]), parts)
    h = C.c_void_p()
    assert lib.oracle_create(C.byref(hooks), buf.ref(), C.byref(h)) == 0, lib.oracle_last_error()
    try:
        assert lib.oracle_step(h, nsteps) == 0, lib.oracle_last_error()
        out = capi.ParticleBuffers(len(parts["iam"]))
        lib.oracle_get(h, out.ref())
    finally:
        lib.oracle_destroy(h)
    fl = parts["iam"] == cases.SPH
    assert np.abs(out["vhat"][fl]).max() > 0.0          # the fluid moved under gravity
    for k in ("r", "v", "vhat", "f", "dens", "h"):
        scale = max(np.abs(out[k]).max(), 1e-300)
        err = np.abs(a[k] - out[k]).max() / scale
        print("reference sediment3D hooks vs built-in hooks", k, err)
        assert err <= 1e-12, f"{k}: {err:.3e}"


def read_final(path):
    with open(path, "rb") as fh:
        buf = fh.read()
    assert buf[:8] == b"SPDMFAC1"
    (n,) = struct.unpack_from("<q", buf, 8)
    rec = np.frombuffer(buf, "<f8", 14 * n, 16).reshape(n, 14)
    return {"r": rec[:, 0:3], "v": rec[:, 3:6], "vhat": rec[:, 6:9], "f": rec[:, 9:12],
            "dens": rec[:, 12], "h": rec[:, 13]}


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_case_hooks_match_device_hooks(tmp_path, precision):
    import __graft_entry__
    __graft_entry__.build()
    exe = build_case(os.path.join(FACADE, "example_sediment"), str(tmp_path / "run_example"))
    case = cases.workload("sediment3d_small")
    init = tmp_path / "init.spdm"
    state.write_state(str(init), case.particles)
    final = tmp_path / "final.bin"
    nsteps = 5
    args = [exe, str(init), str(nsteps), str(final), "--fixed-dt"] + (["--mixed"] if precision == "mixed" else [])
    res = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    a = read_final(str(final))
    lib = capi.Library()
    prec = cases.PREC_MIXED if precision == "mixed" else cases.PREC_FP64
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=prec)
    sim.step(nsteps)
    b = sim.get()
    sim.close()
    # same arithmetic on the host as in the device hooks; only the order of
    # the force sums (FP32 atomics in the mixed coupling) may differ
    tol = 1e-12 if precision == "fp64" else 1e-6
    for k in ("r", "vhat", "dens"):
        scale = np.abs(b[k]).max()
        err = np.abs(a[k] - b[k]).max() / scale
        print(precision, k, err)
        assert err <= tol, f"{k}: {err}"


HOOK_H = """#ifndef CUSTOMSIM_H
#define CUSTOMSIM_H
#include "customConstants.h"
#include "customSimBase.h"
#include "dataLL.h"
#include "sph.h"
#include "vect.h"
class CcustomSim : public CcustomSimBase {
   public:
    CcustomSim(CdataLL *_data, double _time) : CcustomSimBase(_data, _time) {}
    void beforeMiddle(double newTime);
    void beforeEnd(double newTime);
    void afterEnd(double newTime);
};
#endif
"""

# after the second step: every 50th fluid particle is marked for deletion and
# three spheres are inserted, through the reference's own CdataLL calls
HOOK_CPP = """
void CcustomSim::afterEnd(double newTime) {
    static int step = 0;
    if (++step != 2) return;
    particleContainer &ps = *data->getParticles();
    int k = 0;
    for (size_t i = 0; i < ps.size(); i++)
        if (ps[i].iam == sph && (k++ % 50) == 0) data->markForDeletion(ps[i]);
    for (int j = 0; j < 3; j++) {
        Cparticle p;
        p.iam = dem;
        p.r = vect(0.01 * (j + 1), 0.02, 0.072);
        p.mass = DEM_VOL * DEM_DENS;
        p.dens = DEM_DENS;
        p.h = DEM_RADIUS;
        p.radius = DEM_RADIUS;
        data->insertNewParticle(p);
    }
}
"""


@pytest.mark.gpu
def test_case_hook_insertion_and_deletion(tmp_path):
    """insertNewParticle / markForDeletion in a case hook, through the
    façade, against the same changes made through the C ABI."""
    import shutil
    import __graft_entry__
    __graft_entry__.build()
    src = os.path.join(FACADE, "example_sediment")
    case_dir = tmp_path / "case"
    shutil.copytree(src, case_dir, ignore=shutil.ignore_patterns("__pycache__"))
    (case_dir / "customSim.h").write_text(HOOK_H)
    with open(case_dir / "customSim.cpp", "a") as fh:
        fh.write(HOOK_CPP)
    exe = build_case(str(case_dir), str(tmp_path / "run_case"))
    case = cases.workload("sediment3d_small")
    init = tmp_path / "init.spdm"
    state.write_state(str(init), case.particles)
    final = tmp_path / "final.bin"
    res = subprocess.run([exe, str(init), "5", str(final), "--fixed-dt"], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    a = read_final(str(final))

    lib = capi.Library()
    sim = capi.Simulation(lib, case.cfg, case.particles, capacity=case.n + 256)
    sim.step(2)
    fluid = np.nonzero(case.particles["iam"] == cases.SPH)[0]
    sim.mark_for_deletion(fluid[::50])
    R = case.cfg["dem_radius"]
    blk = {"iam": np.full(3, cases.DEM, np.int32), "r": np.array([[0.01 * (j + 1), 0.02, 0.072] for j in range(3)]),
           "mass": np.full(3, case.cfg["dem_vol"] * case.cfg["dem_dens"]), "dens": np.full(3, case.cfg["dem_dens"]),
           "h": np.full(3, R), "radius": np.full(3, R)}
    idx = sim.insert(blk)
    assert list(idx) == [case.n, case.n + 1, case.n + 2]   # no slot is free before the next rebuild
    sim.step(3)
    b = sim.get()
    live = b["iam"] >= 0
    assert (~live).sum() == fluid[::50].size
    assert a["r"].shape[0] == b.n
    for k in ("r", "vhat", "dens"):
        scale = np.abs(b[k][live]).max()
        err = np.abs(a[k][live] - b[k][live]).max() / scale
        assert err <= 1e-12, f"{k}: {err}"


# ---------------------------------------------------------------------------
# restart files through the façade's C++ reader and writer (Cio_data_vtk)
VTK_TOOL = r"""
#include <cstdio>
#include <cstring>
#include <fstream>
#include "io_data_vtk.h"
/* vtk_tool <in.vtu> <out fields bin> <out piece.vtu> <float64 points 0/1> */
int main(int argc, char **argv) {
    particleContainer ps;
    if (!Cio_data_vtk::readPiece(argv[1], ps)) return 1;
    std::ofstream out(argv[2], std::ios::binary);
    for (const Cparticle &p : ps) {
        double rec[16] = {0};
        for (int d = 0; d < NDIM; d++) {
            rec[d] = p.r[d];
            rec[3 + d] = p.v[d];
            rec[6 + d] = p.vhat[d];
            rec[9 + d] = p.norm1[d];
        }
        rec[12] = p.mass;
        rec[13] = p.dens;
        rec[14] = p.h;
        rec[15] = p.iam + 1000.0 * p.tag;
        out.write(reinterpret_cast<const char *>(rec), sizeof rec);
    }
    return Cio_data_vtk::writePiece(argv[3], ps, std::atoi(argv[4]) != 0) ? 0 : 2;
}
"""


def _facade_tool(tmp_path, ndim, name, source):
    """A small program over the façade's I/O (io_data_vtk.cpp) for NDIM = ndim."""
    d = tmp_path / f"{name}{ndim}"
    d.mkdir(exist_ok=True)
    # the constants every case defines that the I/O headers read
    box = ", ".join(["0.0"] * ndim), ", ".join(["1.0"] * ndim)
    (d / "customConstants.h").write_text(f"#ifndef CC_H\n#define CC_H\nconst int NDIM = {ndim};\n"
                                         f"const double RMIN[NDIM] = {{{box[0]}}};\n"
                                         f"const double RMAX[NDIM] = {{{box[1]}}};\n#endif\n")
    (d / f"{name}.cpp").write_text(source)
    sys.path.insert(0, FACADE)
    from build_case import zlib_flags
    exe = str(d / name)
    res = subprocess.run(["g++", "-std=gnu++17", "-O1", f"-I{d}", f"-I{os.path.join(FACADE, 'include')}",
                          str(d / f"{name}.cpp"), os.path.join(FACADE, "io_data_vtk.cpp"), "-o", exe,
                          *zlib_flags()], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return exe


def _vtk_tool(tmp_path, ndim):
    return _facade_tool(tmp_path, ndim, "vtk_tool", VTK_TOOL)


@pytest.mark.parametrize("name", ["dambreak2d_small", "sediment3d_small"])
@pytest.mark.parametrize("exact", [False, True])
def test_cpp_restart_reader_and_writer(tmp_path, name, exact):
    """A restart piece written by sphdem.io_vtk reads back through the C++
    reader field for field, and the C++ writer's piece reads back through
    sphdem.io_vtk (Float32 points as the reference writes them, Float64 for
    the exact form)."""
    from sphdem import io_vtk
    case = cases.workload(name)
    nd = case.cfg["ndim"]
    ps = {k: np.asarray(v) for k, v in case.particles.items()}
    n = case.n
    rng = np.random.default_rng(2)
    ps["tag"] = np.arange(1, n + 1, dtype=np.int32)
    ps["v"] = np.zeros((n, 3))
    ps["v"][:, :nd] = rng.normal(size=(n, nd))
    ps["vhat"] = ps["v"] * 0.5
    io_vtk.write_restart(str(tmp_path / "case"), 0, ps, nd, exact=exact)
    exe = _vtk_tool(tmp_path, nd)
    fields, back = tmp_path / "fields.bin", tmp_path / "back.vtu"
    res = subprocess.run([exe, str(tmp_path / "caseRestart0000000_0.vtu"), str(fields), str(back),
                          "1" if exact else "0"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr[-2000:]
    rec = np.fromfile(str(fields), "<f8").reshape(n, 16)
    r_want = ps["r"][:, :nd] if exact else ps["r"][:, :nd].astype(np.float32).astype(np.float64)
    np.testing.assert_array_equal(rec[:, 0:nd], r_want)
    np.testing.assert_array_equal(rec[:, 3:3 + nd], ps["v"][:, :nd])
    np.testing.assert_array_equal(rec[:, 6:6 + nd], ps["vhat"][:, :nd])
    np.testing.assert_array_equal(rec[:, 9:9 + nd], np.asarray(ps["norm1"])[:, :nd])
    np.testing.assert_array_equal(rec[:, 12], ps["mass"])
    np.testing.assert_array_equal(rec[:, 13], ps["dens"])
    np.testing.assert_array_equal(rec[:, 14], ps["h"])
    np.testing.assert_array_equal(rec[:, 15], ps["iam"] + 1000.0 * ps["tag"])
    d = io_vtk.read_vtu(str(back))
    assert d["n"] == n and d["points_type"] == ("Float64" if exact else "Float32")
    np.testing.assert_array_equal(d["points"][:, :nd], r_want)
    for k in ("dens", "h", "mass"):
        np.testing.assert_array_equal(d["arrays"][k], ps[k])
    np.testing.assert_array_equal(d["arrays"]["tag"], ps["tag"])
    np.testing.assert_array_equal(d["arrays"]["v"][:, :nd], ps["v"][:, :nd])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "singleDEM3D")), reason="reference files not present")
def test_cpp_reader_on_the_reference_restart_files(tmp_path):
    """The restart piece the reference shipped (written by VTK) reads through
    the C++ reader as it reads through sphdem.io_vtk."""
    from sphdem import io_vtk
    import glob
    pieces = sorted(glob.glob(os.path.join(REF_ROOT, "singleDEM3D", "*Restart*_0.vtu")))
    if not pieces:
        pytest.skip("no restart piece shipped")
    exe = _vtk_tool(tmp_path, 3)
    fields, back = tmp_path / "fields.bin", tmp_path / "back.vtu"
    res = subprocess.run([exe, pieces[0], str(fields), str(back), "0"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr[-2000:]
    d = io_vtk.read_vtu(pieces[0])
    rec = np.fromfile(str(fields), "<f8").reshape(d["n"], 16)
    np.testing.assert_array_equal(rec[:, 0:3], d["points"])
    np.testing.assert_array_equal(rec[:, 13], d["arrays"]["dens"])
    np.testing.assert_array_equal(rec[:, 15], d["arrays"]["iam"] + 1000.0 * d["arrays"]["tag"])


@pytest.mark.gpu
def test_case_runs_from_a_restart_piece(tmp_path):
    """run_facade started from the restart piece a case's setup writes
    (<base>Restart0000000_0.vtu, Float64 points) gives the state the SPDMST01
    start gives, and its own final restart reads back."""
    import __graft_entry__
    from sphdem import io_vtk
    __graft_entry__.build()
    exe = build_case(os.path.join(FACADE, "example_sediment"), str(tmp_path / "run_example"))
    case = cases.workload("sediment3d_small")
    ps = dict(case.particles)
    ps["tag"] = np.arange(1, case.n + 1, dtype=np.int32)
    pvtu = io_vtk.write_restart(str(tmp_path / "init"), 0, ps, 3, exact=True)
    spdm = tmp_path / "init.spdm"
    state.write_state(str(spdm), case.particles)
    outs = []
    for src in (str(spdm), str(tmp_path / "initRestart0000000_0.vtu"), pvtu):
        final = tmp_path / f"final{len(outs)}.bin"
        res = subprocess.run([exe, src, "4", str(final), "--fixed-dt", "--restart-out", str(tmp_path / "out")],
                             capture_output=True, text=True, timeout=300)
        assert res.returncode == 0, res.stderr[-2000:]
        outs.append(read_final(str(final)))
    # the FP64 Shepard scatter sums with atomics, so two runs of the coupled
    # step agree to rounding, not bit for bit
    for o in outs[1:]:
        for k in ("r", "vhat", "dens"):
            scale = np.abs(outs[0][k]).max()
            assert np.abs(o[k] - outs[0][k]).max() <= 1e-12 * scale, k
    d = io_vtk.read_vtu(str(tmp_path / "outRestart0000004_0.vtu"))
    np.testing.assert_array_equal(d["points"], outs[-1]["r"])


def _oracle_abi(libdir):
    """The oracle-backed C-ABI library of tests/facade_oracle in libdir."""
    os.makedirs(libdir, exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    "-I" + os.path.join(REPO, "include"), ORACLE_ABI, PORT_SRC, "-o",
                    os.path.join(libdir, "libsphdem.so")], check=True, capture_output=True, text=True)
    return str(libdir)


def test_run_loop_of_the_reference_command_line(tmp_path):
    """run_case <inbase> <intimestep> <outbase>, run.cpp's own command line
    and loop (run.cpp:16-164), on the CPU through the oracle-backed C ABI.
    From the Domain file and restart a case's setup writes, the loop steps
    the example case's hooks until time passes MAXTIME (fixed dt = MAXTIME /
    OUTSTEP) and writes, every MAXTIME / OUTSTEP of simulated time, an output
    piece and a Globals row, and every RESTART_EVERY_N_STEPS (5) output steps
    a restart and a Domain file.  The state it writes at an output step
    equals the fixed-step command's after as many steps; the Globals row
    carries that step's count, time and output-step quantities.  Started
    again from the restart of output step 5 (its Globals row gives time and
    step count), the loop continues the output steps, overwriting the rows
    after step 5 of the same Globals file as CioGlobals does."""
    from sphdem import io_vtk
    lib = _oracle_abi(str(tmp_path / "oracle_abi"))
    exe = build_case(os.path.join(FACADE, "example_sediment"), str(tmp_path / "run_example"), libdir=lib)
    case = cases.workload("sediment3d_small")
    ps = dict(case.particles)
    ps["tag"] = np.arange(1, case.n + 1, dtype=np.int32)
    io_vtk.write_restart(str(tmp_path / "init"), 0, ps, 3, exact=True)
    # the domain the case's constants give, so both command lines bin alike
    res = subprocess.run([exe, str(tmp_path / "initRestart0000000_0.vtu"), "0", str(tmp_path / "probe.bin"),
                          "--dump-config", str(tmp_path / "cfg.bin")], capture_output=True, text=True, timeout=120,
                         cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    cfg = capi.SphDemConfig.from_buffer_copy((tmp_path / "cfg.bin").read_bytes())
    dom = [x for d in range(3) for x in (cfg.domain_min[d], cfg.domain_max[d])]
    io_vtk.write_domain(str(tmp_path / "initDomain0.dat"), 3, dom)

    res = subprocess.run([exe, "init", "0", "out", "--fixed-dt"], capture_output=True, text=True, timeout=600,
                         cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    rows = io_vtk.read_globals(str(tmp_path / "outGlobals0.dat"))
    dt = cfg.maxdt
    maxtime = dt * 10  # the example case: OUTSTEP 10, MAXTIME = 10 maxdt
    assert [int(r["OutStep"]) for r in rows] == list(range(1, len(rows) + 1))
    assert len(rows) >= 8
    steps = [int(r["SPHStep"]) for r in rows]
    assert steps == sorted(steps) and len(set(steps)) == len(steps)
    for r in rows:
        assert abs(r["Time"] - r["SPHStep"] * dt) <= 1e-9 * dt * r["SPHStep"]
        assert int(r["n"]) == case.n
    # the loop ended on time > MAXTIME, as run.cpp's does
    assert rows[-1]["Time"] > maxtime and rows[-2]["Time"] <= maxtime
    for k in range(1, len(rows) + 1):
        assert (tmp_path / f"out{k:07d}_0.vtu").exists() and (tmp_path / f"out{k:07d}.pvtu").exists()
    assert (tmp_path / "outRestart0000005_0.vtu").exists() and not (tmp_path / "outRestart0000004_0.vtu").exists()
    assert io_vtk.read_domain(str(tmp_path / "outDomain0.dat"), 3)["proc_domain"] == dom

    # output step 5 against the fixed-step command after as many steps
    row5 = rows[4]
    n5 = int(row5["SPHStep"])
    final = tmp_path / "final.bin"
    res = subprocess.run([exe, str(tmp_path / "initRestart0000000_0.vtu"), str(n5), str(final), "--fixed-dt"],
                         capture_output=True, text=True, timeout=600, cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    a = read_final(str(final))
    d = io_vtk.read_vtu(str(tmp_path / "outRestart0000005_0.vtu"))
    for k in ("v", "vhat"):
        np.testing.assert_array_equal(d["arrays"][k], a[k])
    for k in ("dens", "h"):
        np.testing.assert_array_equal(d["arrays"][k], a[k])
    np.testing.assert_array_equal(d["points"], a["r"].astype(np.float32).astype(np.float64))
    # the row's output-step quantities are the oracle's calcOutputVars of that state
    iam, m, vh = d["arrays"]["iam"], d["arrays"]["mass"], d["arrays"]["vhat"]
    ke = 0.5 * float(np.sum(m[iam == cases.SPH] * np.sum(vh[iam == cases.SPH] ** 2, axis=1)))
    assert abs(row5["KE"] - ke) <= 1e-12 * ke
    assert int(row5["nSph"]) == int(np.sum(iam == cases.SPH))

    # continued from output step 5 into the same files
    res = subprocess.run([exe, "out", "5", "out", "--fixed-dt"], capture_output=True, text=True, timeout=600,
                         cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    again = io_vtk.read_globals(str(tmp_path / "outGlobals0.dat"))
    assert [int(r["OutStep"]) for r in again] == list(range(1, len(again) + 1))
    assert again[:5] == rows[:5]
    # time and step count carry on from the row of step 5
    assert int(again[5]["SPHStep"]) > n5
    for r in again[5:]:
        assert abs(r["Time"] - r["SPHStep"] * dt) <= 1e-9 * dt * r["SPHStep"]


GD_TOOL = r"""
#include <cstdio>
#include <cstdlib>
#include "io_data_vtk.h"
/* gd_tool <inbase> <outbase>: prints the Domain file of inbase (rank,
 * procDomain, procNeighbrs); writes Globals rows 1, 2, 3 and then 2 again
 * under outbase and prints what readGlobals(2) reads back */
int main(int argc, char **argv) {
    CglobalVars g;
    Cio_data_vtk in(argv[1], &g);
    if (!in.readDomain(0, &g)) return 1;
    std::printf("%d", g.mpiRank);
    for (int i = 0; i < 2 * NDIM; i++) std::printf(" %.17g", g.procDomain[i]);
    for (int k = 0; k < SPHDEM_FACADE_NEIGHBOURS; k++) std::printf(" %d", g.procNeighbrs[k]);
    std::printf("\n");
    Cio_data_vtk out(argv[2], &g);
    for (int step : {1, 2, 3, 2}) {
        g.sphStep = 10 * step + (step == 2 ? 7 : 0);
        g.time = 0.1 * step + 1e-13;
        g.eKE = 1.0 / 3.0 * step;
        g.n = 100 + step;
        g.custom[0] = -step;
        out.writeGlobals(step, &g);
    }
    CglobalVars r;
    out.readGlobals(2, &r);
    std::printf("%d %.17g %.17g %d\n", r.sphStep, r.time, r.eKE, r.n);
    if (argc > 3) {  /* a Globals file written elsewhere: its row 2 */
        CglobalVars q;
        Cio_data_vtk other(argv[3], &q);
        other.readGlobals(2, &q);
        std::printf("%d %.17g %.17g %d\n", q.sphStep, q.time, q.eKE, q.n);
    }
    return 0;
}
"""


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF_ROOT, "damBreak", "initDataGlobals0.dat")),
                    reason="reference files not present")
def test_cpp_globals_and_domain_files_in_the_reference_layout(tmp_path):
    """The façade's C++ Globals and Domain files against the files the
    reference wrote for damBreak (2D): the Globals header line is the
    reference's own, and its Domain line (rank, procDomain[4], procNeighbrs[9],
    ioDomain.cpp:3-23) reads back value for value.  Rows written for steps 1,
    2, 3 and then 2 again leave rows 1 and 2, as CioGlobals's
    openAndSeekToStep(outStep - 1) places the write (ioGlobals.cpp:48-73,
    111-139), and readGlobals(2) reads row 2 back to full precision."""
    from sphdem import io_vtk
    ref_dir = os.path.join(REF_ROOT, "damBreak")
    # one process: the single-rank line of the Domain file, under the rank's name
    line = open(os.path.join(ref_dir, "initDataDomain.dat")).readline()
    (tmp_path / "initDomain0.dat").write_text(line)
    exe = _facade_tool(tmp_path, 2, "gd_tool", GD_TOOL)
    # rows written by the Python writer, read back by the C++ reader
    ov = {"lin_mom": [0.0, 0.0, 0.0], "ang_mom": 0.0, "e_ke": 0.0, "e_b_force": 0.0, "e_elast": 0.0,
          "e_elast_exact": 0.0, "e_visc_f": 0.0, "e_visc_b": 0.0, "e_ff": 0.0, "e_total": 0.0, "max_v": 0.0,
          "ave_dens": 0.0, "var_dens": 0.0, "ave_dens_from_mass": 0.0, "n": 0, "n_sph": 0, "max_f": 0.0,
          "max_ff": 0.0, "rms_ff": 0.0, "ed_elast_dt": 0.0, "ed_visc_f_dt": 0.0, "ed_ff_dt": 0.0}
    for k in (1, 2, 3):
        io_vtk.append_globals(str(tmp_path / "pyGlobals0.dat"), k, 5 * k, 0.7 * k + 1e-14,
                              dict(ov, e_ke=1.0 / 7.0 * k, n=200 + k))
    res = subprocess.run([exe, str(tmp_path / "init"), str(tmp_path / "out"), str(tmp_path / "py")],
                         capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stderr
    dom, back, py = res.stdout.splitlines()
    step, time, eke, n = py.split()
    assert (int(step), float(time), float(eke), int(n)) == (10, 1.4 + 1e-14, 2.0 / 7.0, 202)
    want = line.split()
    got = dom.split()
    assert int(got[0]) == int(want[0])
    assert [float(x) for x in got[1:5]] == [float(x) for x in want[1:5]]
    nb = [int(x) for x in want[5:14]]
    nb[4] = -1  # the process itself (ioDomain.cpp:14-15)
    assert [int(x) for x in got[5:14]] == nb

    ours = open(tmp_path / "outGlobals0.dat").read().splitlines()
    theirs = open(os.path.join(ref_dir, "initDataGlobals0.dat")).read().splitlines()
    assert ours[0] == theirs[0]
    rows = io_vtk.read_globals(str(tmp_path / "outGlobals0.dat"))
    assert [int(r["OutStep"]) for r in rows] == [1, 2]
    assert rows[1]["SPHStep"] == 27 and rows[1]["custom"][0] == -2.0
    step, time, eke, n = back.split()
    assert (int(step), float(time), float(eke), int(n)) == (27, 0.2 + 1e-13, 2.0 / 3.0, 102)


NEIGHBOUR_OUTPUT = r"""
#include <fstream>
#include <iomanip>

#include "customOutput.h"
#include "dataLL.impl.h"
#include "sph.h"
#include "sphIncompress.h"

namespace {
struct Tally {
    double mass = 0;
};
inline void addMass(Cparticle &p, CglobalVars &, Tally &t) { t.mass += p.mass; }
inline void countPair(Cparticle &, Cparticle &, CglobalVars &g) { g.custom[0] += 1.0; }
inline void countGroup(Cparticle &, vector<Cparticle *> &nb, CglobalVars &g) { g.custom[1] += nb.size(); }
inline void countAt(Cparticle &, vector<Cparticle *> &nb, CglobalVars &g) { g.custom[2] += nb.size(); }
inline void countUsing(Cparticle &, vector<Cparticle *> &nb, CglobalVars &g) { g.custom[3] += nb.size(); }
inline void countAgain(Cparticle &, vector<Cparticle *> &nb, CglobalVars &g) { g.custom[4] += nb.size(); }
inline void countSD(Cparticle &p, vector<Cparticle *> &nb, CglobalVars &g) {
    g.custom[5] += nb.size();
    for (Cparticle *pn : nb) g.custom[7] = std::max(g.custom[7], len(p.r - pn->r));
}
inline void countDS(Cparticle &, vector<Cparticle *> &nb, CglobalVars &g) { g.custom[6] += nb.size(); }
inline void mark2(Cparticle &p, CglobalVars &, double a, double b) { p.colour = a + b; }
inline void mark3(Cparticle &p, CglobalVars &, double a, double b, double c) { p.tmp = a + b + c; }
}  // namespace

/* the SPH density summation over neighbour groups with periodic images, then
 * the other CdataLL forms, each tallied into the globals */
void CcustomOutput::calcOutput(int outstep, CcustomSim *, Cio_data_vtk *io) {
    CglobalVars &g = data->globals;
    for (int k = 0; k < 8; k++) g.custom[k] = 0;
    data->neighboursGroup<Nsph::calcDensity, Nsph::ifSphOrSphBoundary>();
    particleContainer &ps = *data->getParticles();
    {
        std::ofstream out((io->filename + ".dens").c_str(), std::ios::binary);
        for (Cparticle &p : ps) {
            const double rec[7] = {p.r[0], p.r[1], p.r[2], p.mass, p.h, p.dens, (double)p.iam};
            out.write(reinterpret_cast<const char *>(rec), sizeof rec);
        }
    }
    data->neighbours<countPair, Nsph::ifSphOrSphBoundary>();
    data->neighboursGroup<countGroup, Nsph::ifSphOrSphBoundary>();
    Tally t;
    data->traverse<Tally, addMass, Nsph::ifSph>(t);
    data->traverse<mark2, Nsph::ifSph>(1.0, 2.0);
    data->traverse<mark3, Nsph::ifSph>(1.0, 2.0, 3.0);
    data->neighboursGroupAtRadius<countAt, Nsph::ifSph>(0.005);
    vector<Cparticle> qs(ps.begin(), ps.begin() + 50);
    data->neighboursUsing<countUsing>(qs);
    data->neighboursGroupCoupling<countSD, Nsph::ifSphOrSphBoundary>();
    data->neighboursGroupCoupling<countDS, Nsph::ifDem>();
    data->reset();
    data->neighboursGroup<countAgain, Nsph::ifSphOrSphBoundary>();
    double colour = 0, tmp = 0;
    for (Cparticle &p : ps)
        if (p.iam == sph) {
            colour = p.colour;
            tmp = p.tmp;
            break;
        }
    std::ofstream s((io->filename + ".stats").c_str());
    s << std::setprecision(17) << g.custom[0] << ' ' << g.custom[1] << ' ' << t.mass << ' ' << data->numParticles()
      << ' ' << colour << ' ' << tmp << ' ' << g.custom[2] << ' ' << g.custom[3] << ' ' << g.custom[4] << ' '
      << g.custom[5] << ' ' << g.custom[6] << ' ' << g.custom[7] << '\n';
}
"""


def test_neighbour_forms_with_periodic_images(tmp_path):
    """The façade's neighbour forms on the CPU through the oracle-backed C
    ABI, with a case whose output code uses them (the example case's
    constants and hooks: periodic x and y).  Over neighbour groups,
    Nsph::calcDensity (sph.h:1149-1190) gives the SPH density summation with
    each neighbour at its nearest periodic image, as the reference's ghost
    copies place it; it matches a brute-force minimum-image summation.  The
    pair, group, at-radius and external-query forms count the pairs a
    brute-force search counts; the traverse forms with a state object and
    with two and three constants reach every particle; reset() keeps the
    lists."""
    lib = _oracle_abi(str(tmp_path / "oracle_abi"))
    case_dir = tmp_path / "case"
    case_dir.mkdir()
    src = os.path.join(FACADE, "example_sediment")
    for f in ("customConstants.h", "customSim.h", "customSim.cpp", "customOutput.h"):
        (case_dir / f).write_text(open(os.path.join(src, f)).read())
    (case_dir / "customOutput.cpp").write_text(NEIGHBOUR_OUTPUT)
    exe = build_case(str(case_dir), str(tmp_path / "run_case"), libdir=lib)
    case = cases.workload("sediment3d_small")
    init = tmp_path / "init.spdm"
    state.write_state(str(init), case.particles)
    out = tmp_path / "final.bin"
    res = subprocess.run([exe, str(init), "10", str(out), "--fixed-dt"], capture_output=True, text=True,
                         timeout=600, cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    rec = np.fromfile(str(out) + ".dens", dtype="<f8").reshape(-1, 7)
    r, m, h, dens, iam = rec[:, 0:3], rec[:, 3], rec[:, 4], rec[:, 5], rec[:, 6].astype(int)
    cfg = case.cfg
    L = np.array(cfg["rmax"]) - np.array(cfg["rmin"])
    per = np.array(cfg["periodic"], bool)
    n = len(m)
    fluid = (iam == cases.SPH) | (iam == cases.SPH_BOUNDARY)
    nondem = iam != cases.DEM
    # nearest images, as the reference places its ghosts: RMIN - RMAX + r or RMAX - RMIN + r
    rmin, rmax = np.array(cfg["rmin"]), np.array(cfg["rmax"])
    d = r[:, None, :] - r[None, :, :]
    img = np.broadcast_to(r[None, :, :], d.shape).copy()
    for a in range(3):
        if per[a]:
            hi, lo = d[:, :, a] > 0.5 * L[a], d[:, :, a] < -0.5 * L[a]
            img[:, :, a] = np.where(hi, (rmax[a] - rmin[a]) + r[None, :, a], img[:, :, a])
            img[:, :, a] = np.where(lo, (rmin[a] - rmax[a]) + r[None, :, a], img[:, :, a])
    dx = r[:, None, :] - img
    d2 = (dx[:, :, 0] * dx[:, :, 0] + dx[:, :, 1] * dx[:, :, 1]) + dx[:, :, 2] * dx[:, :, 2]
    lim2 = (2.0 * np.maximum(h[:, None], h[None, :])) ** 2
    off = ~np.eye(n, dtype=bool)
    crossing = (np.abs(r[:, None, :] - r[None, :, :]) > 0.5 * L).any(axis=2) & (d2 <= lim2) & off
    assert crossing[fluid][:, nondem].sum() > 0  # the summation does use periodic images

    def wendland(q, hh):
        c = 21.0 / (256.0 * cfg["pi"])  # the case's PI (3.14159265 in the reference's cases)
        return np.where(q <= 2.0, c * (2.0 - q) ** 4 * (1.0 + 2.0 * q), 0.0) / hh ** 3

    pair = (d2 <= lim2) & off & nondem[None, :] & fluid[None, :]
    q = np.sqrt(d2) / h[:, None]
    want = m * wendland(0.0, h) + np.sum(np.where(pair, m[None, :] * wendland(q, h[:, None]), 0.0), axis=1)
    err = np.abs(dens[fluid] - want[fluid]).max() / np.abs(want[fluid]).max()
    assert err <= 1e-12, err

    stats = open(str(out) + ".stats").read().split()
    pairs, groups, mass_sph, count, colour, tmp, at_r, using, again, sd, ds, sd_max = (float(x) for x in stats)
    # ties at exactly 2 max(h) may fall either way: bracket the brute-force counts
    tie = np.abs(d2 - lim2) <= 1e-12 * lim2
    grp = off & nondem[None, :] & fluid[:, None]
    lo_n, hi_n = (grp & (d2 <= lim2) & ~tie).sum(), (grp & ((d2 <= lim2) | tie)).sum()
    assert lo_n <= groups <= hi_n and pairs == groups and again == groups
    assert abs(mass_sph - m[iam == cases.SPH].sum()) <= 1e-12 * mass_sph
    assert int(count) == n and colour == 3.0 and tmp == 6.0
    sphq = iam == cases.SPH
    at = off & nondem[None, :] & sphq[:, None] & (d2 <= 0.005 ** 2)
    assert at.sum() - (np.abs(d2 - 0.005 ** 2) <= 1e-12 * 0.005 ** 2).sum() <= at_r <= at.sum() + (np.abs(d2 - 0.005 ** 2) <= 1e-12 * 0.005 ** 2).sum()
    # external queries: copies of the first 50 particles find their originals too
    rel = np.where(iam[:50, None] == cases.DEM, iam[None, :] == cases.DEM, iam[None, :] != cases.DEM)
    u_lo = (rel & (d2[:50] <= lim2[:50]) & ~tie[:50]).sum()
    u_hi = (rel & ((d2[:50] <= lim2[:50]) | tie[:50])).sum()
    assert u_lo <= using <= u_hi
    # coupling groups: the port's two coupling relations at the same state
    # (the example hooks are the port's built-in ones), partners at their
    # nearest image within the coupling radius
    import ctypes as C
    from oracle import port_api
    pcfg = capi.config_struct(case.cfg)
    port = port_api.lib()
    pbuf = capi.ParticleBuffers(case.n, case.particles)
    ph = C.c_void_p()
    assert port.oracle_create(C.byref(pcfg), pbuf.ref(), C.byref(ph)) == 0, port.oracle_last_error()
    try:
        assert port.oracle_step(ph, 10) == 0
        tot = []
        for kind in (2, 3):
            offs = (C.c_int64 * (n + 1))()
            npairs = C.c_int64(0)
            assert port.oracle_pairs(ph, kind, offs, None, 0, C.byref(npairs)) == 0
            tot.append(npairs.value)
        chk = capi.ParticleBuffers(case.n)
        port.oracle_get(ph, chk.ref())
    finally:
        port.oracle_destroy(ph)
    np.testing.assert_array_equal(chk["r"], r)  # the same state
    assert (sd, ds) == (tot[0], tot[1]) and sd > 0 and ds > 0
    assert sd_max < cfg["coupling_radius"]


def test_case_with_mirror_ghosts_is_refused_at_start(tmp_path):
    """A case whose GHOST[] asks for mirror boundaries (dataLL.cpp:667-686),
    which the device path does not implement, builds but stops at start-up
    with the reason."""
    lib = _oracle_abi(str(tmp_path / "oracle_abi"))
    case_dir = tmp_path / "case"
    case_dir.mkdir()
    src = os.path.join(FACADE, "example_sediment")
    for f in ("customSim.h", "customSim.cpp", "customOutput.h", "customOutput.cpp"):
        (case_dir / f).write_text(open(os.path.join(src, f)).read())
    consts = open(os.path.join(src, "customConstants.h")).read()
    assert "const int GHOST[2*NDIM] = {0, 0, 0, 0, 0, 0};" in consts
    (case_dir / "customConstants.h").write_text(
        consts.replace("const int GHOST[2*NDIM] = {0, 0, 0, 0, 0, 0};", "const int GHOST[2*NDIM] = {0, 0, 0, 0, 1, 0};"))
    exe = build_case(str(case_dir), str(tmp_path / "run_case"), libdir=lib)
    case = cases.workload("sediment3d_small")
    init = tmp_path / "init.spdm"
    state.write_state(str(init), case.particles)
    res = subprocess.run([exe, str(init), "1", str(tmp_path / "final.bin")], capture_output=True, text=True,
                         timeout=120, cwd=str(tmp_path))
    assert res.returncode != 0 and "GHOST[] mirror boundaries" in res.stderr, res.stderr


def test_case_hook_insertion_and_deletion_on_the_oracle(tmp_path):
    """insertNewParticle / markForDeletion in a case hook through the façade,
    on the CPU through the oracle-backed C ABI, against the same changes made
    directly on the oracle port (the device form of this test runs with -m
    gpu)."""
    import ctypes as C
    import shutil
    from oracle import port_api
    lib = _oracle_abi(str(tmp_path / "oracle_abi"))
    src = os.path.join(FACADE, "example_sediment")
    case_dir = tmp_path / "case"
    shutil.copytree(src, case_dir, ignore=shutil.ignore_patterns("__pycache__"))
    (case_dir / "customSim.h").write_text(HOOK_H)
    with open(case_dir / "customSim.cpp", "a") as fh:
        fh.write(HOOK_CPP)
    exe = build_case(str(case_dir), str(tmp_path / "run_case"), libdir=lib)
    case = cases.workload("sediment3d_small")
    init = tmp_path / "init.spdm"
    state.write_state(str(init), case.particles)
    final = tmp_path / "final.bin"
    res = subprocess.run([exe, str(init), "5", str(final), "--fixed-dt", "--dump-config", str(tmp_path / "cfg.bin")],
                         capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    a = read_final(str(final))

    cfg = capi.SphDemConfig.from_buffer_copy((tmp_path / "cfg.bin").read_bytes())
    # the example case's hooks as the port's built-in ones
    cfg.gravity_sph = capi.D3(0.0, 0.0, -9.81)
    cfg.gravity_dem = capi.D3(0.0, 0.0, -9.81)
    cfg.n_walls = 1
    cfg.walls[0].point = capi.D3(cfg.rmin[0], cfg.rmin[1], cfg.rmin[2])
    cfg.walls[0].normal = capi.D3(0.0, 0.0, 1.0)
    port = port_api.lib()
    buf = capi.ParticleBuffers(case.n, case.particles)
    h = C.c_void_p()
    assert port.oracle_create(C.byref(cfg), buf.ref(), C.byref(h)) == 0, port.oracle_last_error()
    try:
        assert port.oracle_step(h, 2) == 0
        fluid = np.nonzero(case.particles["iam"] == cases.SPH)[0][::50].astype(np.int64)
        assert port.oracle_mark_for_deletion(h, fluid.ctypes.data_as(C.POINTER(C.c_int64)), len(fluid)) == 0
        R = cfg.dem_radius
        blk = {"iam": np.full(3, cases.DEM, np.int32),
               "r": np.array([[0.01 * (j + 1), 0.02, 0.072] for j in range(3)]),
               "mass": np.full(3, cfg.dem_vol * cfg.dem_dens), "dens": np.full(3, cfg.dem_dens),
               "h": np.full(3, R), "radius": np.full(3, R)}
        ins = capi.ParticleBuffers(3, blk)
        idx = (C.c_int64 * 3)()
        assert port.oracle_insert(h, ins.ref(), idx) == 0, port.oracle_last_error()
        assert list(idx) == [case.n, case.n + 1, case.n + 2]
        assert port.oracle_step(h, 3) == 0
        out = capi.ParticleBuffers(case.n + 3)
        port.oracle_get(h, out.ref())
    finally:
        port.oracle_destroy(h)
    live = out["iam"] >= 0
    assert (~live).sum() == fluid.size and a["r"].shape[0] == case.n + 3
    for k in ("r", "vhat", "dens"):
        np.testing.assert_array_equal(a[k][live], out[k][live], err_msg=k)


def _constants_2d(case, outstep=10):
    """customConstants.h of a 2D fluid case (no LIQ_DEM) from a workload of
    sphdem.cases: the dam break's constants in the reference's form."""
    c = case.cfg
    r = lambda v: repr(float(v))  # noqa: E731
    assert c["ndim"] == 2 and not c["flags"] & cases.F_LIQ_DEM
    flags = c["flags"]
    lines = ["#ifndef CUSTOMCONSTANTS_H", "#define CUSTOMCONSTANTS_H", "#include <cmath>", "#define _2D_",
             "#define NDIM 2", "#define WENDLAND", "#define VISC_ARTIFICIAL"]
    if flags & 1:
        lines.append("#define CONST_H")
    if flags & 2:
        lines.append("#define NO_ANTICLUMPING")
    lines += [
        f"const double PI = {r(c['pi'])};",
        f"const double RMIN[NDIM] = {{{r(c['rmin'][0])}, {r(c['rmin'][1])}}};",
        f"const double RMAX[NDIM] = {{{r(c['rmax'][0])}, {r(c['rmax'][1])}}};",
        "const int PERIODIC[NDIM] = {0, 0};", "const int GHOST[2*NDIM] = {0, 0, 0, 0};",
        "const double DENS_DROP[NDIM] = {0.0, 0.0};",
        f"const double PSEP = {r(c['psep'])};", f"const double HFAC = {r(c['hfac'])};",
        f"const double H = {r(c['h'])};", f"const double DENS = {r(c['dens'])};",
        f"const double REFD = {r(c['refd'])};", f"const double GAMMA = {r(c['gamma'])};",
        f"const double PRB = {r(c['prb'])};", f"const double SPSOUND = {r(c['spsound'])};",
        f"const double VISCOSITY = {r(c['viscosity'])};",
        f"const double ALPHA_ARTIFICIAL = {r(c['alpha_artificial'])};", f"const double BFAC = {r(c['bfac'])};",
        f"const int OUTSTEP = {outstep};", f"const double MAXTIME = {r(c['maxdt'])} * OUTSTEP;",
        "const int RESTART_EVERY_N_STEPS = 5;", f"const double DAMPTIME = {r(c['damptime'])};",
        f"const int MAX_NUM_PARTICLES_PER_CPU = {case.n + 16};",
        "const int REINIT_DENS_EVERY_N_STEPS = 50000000;", "const int REINIT_DENS_AT_N_STEPS = 50000000;",
        "#endif", ""]
    return "\n".join(lines)


CASE_2D_SIM_H = """#ifndef CUSTOMSIM_H
#define CUSTOMSIM_H
#include "customConstants.h"
#include "customSimBase.h"
#include "dataLL.h"
#include "sph.h"
class CcustomSim : public CcustomSimBase {
   public:
    CcustomSim(CdataLL *_data, double _time) : CcustomSimBase(_data, _time) {}
    void beforeMiddle(double newTime);
};
#endif
"""
CASE_2D_SIM_CPP = """#include "customSim.h"
#include "dataLL.impl.h"
namespace {
inline void gravity(Cparticle &p, CglobalVars &g) { p.f[1] -= 9.81; }
}
void CcustomSim::beforeMiddle(double newTime) { data->traverse<gravity, Nsph::ifSph>(); }
"""
CASE_2D_OUT_H = """#ifndef CUSTOMOUTPUT_H
#define CUSTOMOUTPUT_H
#include "customOutputBase.h"
#include "customSim.h"
class CcustomOutput : public CcustomOutputBase {
   public:
    CcustomOutput(CdataLL *_data) : CcustomOutputBase(_data) {}
    void calcOutput(int outstep, CcustomSim *custSim, Cio_data_vtk *io) {}
};
#endif
"""


def test_2d_fluid_case_through_the_facade_on_the_oracle(tmp_path):
    """A 2D fluid case without LIQ_DEM (the dam break's configuration:
    Wendland C2, artificial viscosity, CONST_H, walls of boundary particles)
    built against the façade and stepped through its hooks (gravity on the
    fluid before the middle phase) on the CPU oracle, against the oracle
    port with the same gravity as its built-in hook: equal bit for bit."""
    import ctypes as C
    from oracle import port_api
    lib = _oracle_abi(str(tmp_path / "oracle_abi"))
    case = cases.workload("dambreak2d_small")
    case_dir = tmp_path / "case"
    case_dir.mkdir()
    (case_dir / "customConstants.h").write_text(_constants_2d(case))
    (case_dir / "customSim.h").write_text(CASE_2D_SIM_H)
    (case_dir / "customSim.cpp").write_text(CASE_2D_SIM_CPP)
    (case_dir / "customOutput.h").write_text(CASE_2D_OUT_H)
    exe = build_case(str(case_dir), str(tmp_path / "run_case"), libdir=lib)
    init = tmp_path / "init.spdm"
    state.write_state(str(init), case.particles)
    nsteps = 20
    final = tmp_path / "final.bin"
    res = subprocess.run([exe, str(init), str(nsteps), str(final), "--fixed-dt", "--dump-config",
                          str(tmp_path / "cfg.bin")], capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert res.returncode == 0, res.stderr[-2000:]
    a = read_final(str(final))
    cfg = capi.SphDemConfig.from_buffer_copy((tmp_path / "cfg.bin").read_bytes())
    assert cfg.ndim == 2 and cfg.visc_model == cases.VISC_ARTIFICIAL
    for k in ("domain_min", "domain_max"):
        assert list(getattr(cfg, k))[:2] == list(case.cfg[k])[:2], k
    cfg.gravity_sph = capi.D3(0.0, -9.81, 0.0)
    port = port_api.lib()
    buf = capi.ParticleBuffers(case.n, case.particles)
    h = C.c_void_p()
    assert port.oracle_create(C.byref(cfg), buf.ref(), C.byref(h)) == 0, port.oracle_last_error()
    try:
        assert port.oracle_step(h, nsteps) == 0
        out = capi.ParticleBuffers(case.n)
        port.oracle_get(h, out.ref())
    finally:
        port.oracle_destroy(h)
    assert np.abs(out["vhat"]).max() > 0.0
    for k in ("r", "v", "vhat", "f", "dens", "h"):
        np.testing.assert_array_equal(a[k][:, :2] if a[k].ndim == 2 else a[k],
                                      out[k][:, :2] if out[k].ndim == 2 else out[k], err_msg=k)


@pytest.mark.parametrize("macro,reason", [
    ("LUBRICATION", "DEM contact law"),
    ("SMOOTHED_VISC_VELOCITY", "velocity smoothing"),
    ("LIQ_DEM_SEPARATE_DRAGS", "SPH-DEM coupling variant"),
    ("LIQ_DEM_VARIABLE_TIMESTEP", "SPH-DEM coupling variant"),
    ("FIXED_DEM", "FIXED_DEM / NO_DEM_CONTACTS"),
    ("VAR_H_CORRECTION2", "SPH step variant"),
    ("MORRIS_SPH_BOUNDARY", "viscosity or boundary variant"),
])
def test_constants_bridge_refuses_options_the_device_lacks(tmp_path, macro, reason):
    """sphdem_case_config.h stops the build of a case that defines a step
    option of the reference the device path does not implement."""
    src = tmp_path / "probe.cpp"
    src.write_text(f'#define {macro}\n#include "sphdem_case_config.h"\nint main() {{ return 0; }}\n')
    res = subprocess.run(["g++", "-std=gnu++17", "-fsyntax-only",
                          "-I" + os.path.join(FACADE, "example_sediment"), "-I" + os.path.join(FACADE, "include"),
                          str(src)], capture_output=True, text=True)
    assert res.returncode != 0 and reason in res.stderr, res.stderr[-1500:]


def test_constants_bridge_accepts_the_example_case(tmp_path):
    src = tmp_path / "probe.cpp"
    src.write_text('#include "sphdem_case_config.h"\nint main() { return sphdem_case_unsupported() ? 1 : 0; }\n')
    res = subprocess.run(["g++", "-std=gnu++17", "-fsyntax-only",
                          "-I" + os.path.join(FACADE, "example_sediment"), "-I" + os.path.join(FACADE, "include"),
                          str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-1500:]
