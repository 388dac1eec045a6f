"""Error behaviour of the C ABI that needs no GPU: every entry point answers a
null handle or a bad argument with a status code (never a crash), and the
reason for a failed sphdem_create / sphdem_batch_create is readable through
the *_last_error functions with a null handle.

The reference has no status codes: it prints to cerr and exits
(dataLL.cpp:207-211).  All calls here return before any CUDA call, except
the last test, which runs only where no CUDA device is visible.
"""
import ctypes as C
import os

import numpy as np
import pytest

from sphdem import capi, cases

INVALID, CUDA = 1, 2
H = C.c_void_p


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(capi.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    return capi.Library()


def _text(fn, h=None) -> str:
    buf = C.create_string_buffer(1024)
    assert fn(h, buf, len(buf)) == 0
    return buf.value.decode()


def _create(lib, cfg, parts, capacity=None, precision=None):
    s = capi.config_struct(cfg, precision)
    init = capi.ParticleBuffers(int(parts["iam"].shape[0]), parts)
    h = H()
    rc = lib.lib.sphdem_create(C.byref(s), init.ref(), capacity or init.n, C.byref(h))
    return rc, h, _text(lib.lib.sphdem_last_error)


def test_create_rejects_bad_configurations_with_text(lib):
    dam = cases.workload("dambreak2d_small")
    sed = cases.workload("sediment3d_small")
    rc = lib.lib.sphdem_create(None, None, 10, C.byref(H()))
    assert rc == INVALID
    assert "null config or particles" in _text(lib.lib.sphdem_last_error)
    assert lib.lib.sphdem_create(None, None, 10, None) == INVALID

    def bad(case, msg, capacity=None, precision=None, **edit):
        cfg = dict(case.cfg, **edit.pop("cfg", {}))
        parts = {k: np.array(v) for k, v in case.particles.items()}
        for k, f in edit.items():
            f(parts[k])
        rc, h, text = _create(lib, cfg, parts, capacity, precision)
        assert rc == INVALID and not h.value, (rc, text)
        assert msg in text, text

    bad(dam, "ndim must be 1, 2 or 3", cfg={"ndim": 4})
    bad(dam, "capacity smaller than the particle count", capacity=dam.n - 1)
    bad(dam, "h and maxdt must be positive", cfg={"maxdt": 0.0})
    bad(dam, "unknown precision", precision=7)
    bad(dam, "empty binning domain", cfg={"domain_max": dam.cfg["domain_min"]})

    def nan_first(r):
        r[0, 0] = np.nan

    def zero_mass(m):
        m[3] = 0.0

    bad(dam, "non-finite position", r=nan_first)
    bad(dam, "h, mass and dens must be positive", mass=zero_mass)
    flags = sed.cfg["flags"]
    bad(sed, "CORRECTED_GRADIENT is not combined with LIQ_DEM", cfg={"flags": flags | (1 << 6)})
    bad(dam, "DEM_BLOCK needs LIQ_DEM", cfg={"flags": dam.cfg["flags"] | (1 << 7)})
    bad(sed, "LIQ_DEM needs dem_search_radius and coupling_radius", cfg={"coupling_radius": 0.0})
    # mixed coupling packs DEM bucket indices into 10 bits per axis
    wide = [m + 2000.0 * sed.cfg["dem_search_radius"] for m in sed.cfg["domain_max"]]
    bad(sed, "outside [-512, 511]", precision=cases.PREC_MIXED, cfg={"domain_max": wide})


def test_null_handle_everywhere(lib):
    L = lib.lib
    i64, i32, dbl = C.c_int64(0), (C.c_int32 * 8)(), C.c_double(0)
    parts = capi.SphDemParticles()
    calls = {
        "destroy": lambda: L.sphdem_destroy(None),
        "phase": lambda: L.sphdem_phase(None, capi.PHASE_START),
        "step": lambda: L.sphdem_step(None, 1),
        "get_fields": lambda: L.sphdem_get_fields(None, capi.FIELD_ALL, C.byref(parts)),
        "set_fields": lambda: L.sphdem_set_fields(None, capi.FIELD_ALL, C.byref(parts)),
        "get_fields_async": lambda: L.sphdem_get_fields_async(None, capi.FIELD_ALL, C.byref(parts)),
        "fields_wait": lambda: L.sphdem_fields_wait(None),
        "get_globals": lambda: L.sphdem_get_globals(None, C.byref(capi.SphDemGlobals())),
        "set_globals": lambda: L.sphdem_set_globals(None, C.byref(capi.SphDemGlobals())),
        "get_stats": lambda: L.sphdem_get_stats(None, C.byref(capi.SphDemStats())),
        "insert": lambda: L.sphdem_insert_particles(None, C.byref(parts), None),
        "mark": lambda: L.sphdem_mark_for_deletion(None, None, 0),
        "rebuild": lambda: L.sphdem_rebuild(None),
        "pairs": lambda: L.sphdem_pairs(None, 0, None, None, 0, C.byref(i64)),
        "output_vars": lambda: L.sphdem_output_vars(None, C.byref(capi.SphDemOutputVars())),
        "cell_ids": lambda: L.sphdem_cell_ids(None, i32),
        "cell_ids_noalloc": lambda: L.sphdem_cell_ids_noalloc(None, i32),
        "adjoint_forward": lambda: L.sphdem_adjoint_forward(None, 10, 5),
        "adjoint_set_tape_memory": lambda: L.sphdem_adjoint_set_tape_memory(None, 0),
        "adjoint_backward": lambda: L.sphdem_adjoint_backward(None, None, None, None,
                                                              C.byref(capi.SphDemGrads()), None, None, None),
        "kernel_times_reset": lambda: L.sphdem_kernel_times_reset(None, 1),
        "kernel_times": lambda: L.sphdem_kernel_times(None, C.create_string_buffer(64), 64, C.byref(dbl),
                                                      C.byref(i64), 1, C.byref(C.c_int(0))),
        "time_steps": lambda: L.sphdem_time_steps(None, 1, C.byref(dbl)),
        "batch_destroy": lambda: L.sphdem_batch_destroy(None),
        "batch_step": lambda: L.sphdem_batch_step(None, 1),
        "batch_time_steps": lambda: L.sphdem_batch_time_steps(None, 1, C.byref(dbl)),
        "batch_tune": lambda: L.sphdem_batch_tune(None, 1, None),
    }
    got = {k: f() for k, f in calls.items()}
    assert all(rc == INVALID for rc in got.values()), got
    # a text buffer is required
    assert L.sphdem_last_error(None, None, 16) == INVALID
    assert L.sphdem_batch_last_error(None, C.create_string_buffer(4), 0) == INVALID


def test_batch_create_rejects_bad_members_with_text(lib):
    L = lib.lib
    out = H()
    assert L.sphdem_batch_create(None, 2, C.byref(out)) == INVALID
    assert "no members" in _text(L.sphdem_batch_last_error)
    members = (H * 2)(None, None)
    assert L.sphdem_batch_create(members, 0, C.byref(out)) == INVALID
    assert "no members" in _text(L.sphdem_batch_last_error)
    assert L.sphdem_batch_create(members, 2, C.byref(out)) == INVALID
    assert "member 0 is a null handle" in _text(L.sphdem_batch_last_error)
    assert not out.value
    with pytest.raises(capi.SphDemError, match="no members"):
        capi.Batch(lib, [])


def _cuda_devices() -> int:
    try:
        rt = C.CDLL("libcudart.so.13")
    except OSError:
        return 0
    n = C.c_int(0)
    return n.value if rt.cudaGetDeviceCount(C.byref(n)) == 0 else 0


def test_create_without_a_device_fails_loudly(lib):
    """A valid configuration where no CUDA device is visible: sphdem_create
    returns SPHDEM_ERR_CUDA with the runtime's reason, and the Python
    wrapper raises (there is no CPU fallback)."""
    if _cuda_devices() > 0:
        pytest.skip("a CUDA device is visible")
    case = cases.workload("dambreak2d_small")
    rc, h, text = _create(lib, case.cfg, case.particles)
    assert rc == CUDA and not h.value
    assert "cuda" in text.lower() and text != "no handle", text
    with pytest.raises(capi.SphDemError, match="sphdem_create: CUDA"):
        capi.Simulation(lib, case.cfg, case.particles)
