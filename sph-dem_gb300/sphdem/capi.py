"""ctypes view of the C ABI in include/sphdem.h.

`SphDemConfig` / `SphDemParticles` mirror the C structs member for member;
`config_struct` fills one from a case configuration dictionary and
`ParticleBuffers` owns numpy arrays behind a `SphDemParticles`.  `Library`
loads ``libsphdem.so`` (the CUDA implementation) and raises on any non-zero
status with the library's own error text.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "libsphdem.so")

OK = 0
ERR_NAMES = {1: "INVALID", 2: "CUDA", 3: "CAPACITY", 4: "OUT_OF_RANGE",
             5: "NOT_FINITE", 6: "UNSUPPORTED", 7: "TIMEOUT"}

HOOK_BEFORE_START, PHASE_START, HOOK_BEFORE_MIDDLE, PHASE_MIDDLE = 0, 1, 2, 3
HOOK_BEFORE_END, PHASE_END, HOOK_AFTER_END = 4, 5, 6
PAIRS_SPH, PAIRS_DEM, PAIRS_COUPLE_SD, PAIRS_COUPLE_DS = 0, 1, 2, 3
PAIR_KIND_NAMES = {PAIRS_SPH: "sph", PAIRS_DEM: "dem",
                   PAIRS_COUPLE_SD: "couple_sd", PAIRS_COUPLE_DS: "couple_ds"}

FIELD_ALL = 0xFFFFFFFF
FIELD_R, FIELD_V, FIELD_VHAT, FIELD_MASS = 1 << 0, 1 << 1, 1 << 2, 1 << 3
FIELD_DENS, FIELD_H, FIELD_F, FIELD_DDDT = 1 << 4, 1 << 5, 1 << 6, 1 << 7
FIELD_PRESS, FIELD_COUPLING, FIELD_OMEGA, FIELD_V0, FIELD_IAM = 1 << 8, 1 << 9, 1 << 10, 1 << 11, 1 << 12
FIELD_ENERGY, FIELD_NORMALS, FIELD_RADIUS = 1 << 13, 1 << 14, 1 << 15

D3 = C.c_double * 3
I3 = C.c_int32 * 3


class SphDemWall(C.Structure):
    _fields_ = [("point", D3), ("normal", D3)]


class SphDemConfig(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("visc_model", C.c_int32), ("flags", C.c_uint32),
        ("precision", C.c_int32), ("periodic", I3), ("n_walls", C.c_int32),
        ("pi", C.c_double), ("rmin", D3), ("rmax", D3),
        ("domain_min", D3), ("domain_max", D3),
        ("hfac", C.c_double), ("psep", C.c_double), ("h", C.c_double),
        ("dens", C.c_double), ("refd", C.c_double),
        ("gamma", C.c_double), ("prb", C.c_double), ("spsound", C.c_double),
        ("viscosity", C.c_double), ("alpha_artificial", C.c_double), ("bfac", C.c_double),
        ("maxdt", C.c_double), ("damptime", C.c_double),
        ("dem_radius", C.c_double), ("dem_dens", C.c_double),
        ("dem_k", C.c_double), ("dem_gamma", C.c_double),
        ("dem_search_radius", C.c_double), ("dem_vol", C.c_double),
        ("coupling_radius", C.c_double), ("dem_timestep", C.c_double),
        ("liq_dem_timestep", C.c_double), ("time_drop_particle", C.c_double),
        ("freeze_dem_until", C.c_double),
        ("gravity_sph", D3), ("gravity_dem", D3),
        ("walls", SphDemWall * 6),
        ("drag_scale", C.c_double),
        ("reinit_dens_every", C.c_int32), ("reinit_dens_at", C.c_int32),
    ]


P_I32 = C.POINTER(C.c_int32)
P_U8 = C.POINTER(C.c_uint8)
P_F64 = C.POINTER(C.c_double)


class SphDemParticles(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("iam", P_I32), ("tag", P_I32), ("concave", P_U8),
        ("r", P_F64), ("v", P_F64), ("vhat", P_F64),
        ("mass", P_F64), ("dens", P_F64), ("h", P_F64), ("radius", P_F64),
        ("norm1", P_F64), ("norm2", P_F64), ("norm3", P_F64),
        ("f", P_F64), ("fp", P_F64), ("fv", P_F64), ("fb", P_F64),
        ("dddt", P_F64), ("press", P_F64), ("pdr2", P_F64),
        ("porosity", P_F64), ("dporositydt", P_F64), ("shep_sum", P_F64), ("omega", P_F64),
        ("fdrag", P_F64), ("fvel", P_F64), ("grad_porosity", P_F64),
        ("v0", P_F64), ("vhat0", P_F64),
        ("u", P_F64), ("dudt", P_F64), ("e_visc", P_F64), ("de_visc_dt", P_F64),
    ]


class SphDemGlobals(C.Structure):
    _fields_ = [("time", C.c_double), ("dt", C.c_double), ("new_dt", C.c_double),
                ("maxdt", C.c_double), ("dem_dt", C.c_double),
                ("sph_step", C.c_int64), ("n_deleted", C.c_int64)]


GRAD_DEM_K, GRAD_DEM_GAMMA, GRAD_POSITIONS, GRAD_VISCOSITY, GRAD_DRAG_SCALE = 1, 2, 4, 8, 16


class SphDemGrads(C.Structure):
    _fields_ = [("dem_k", C.c_double), ("dem_gamma", C.c_double), ("viscosity", C.c_double),
                ("drag_scale", C.c_double), ("valid", C.c_uint32)]


class SphDemOutputVars(C.Structure):
    _fields_ = [("lin_mom", C.c_double * 3), ("ang_mom", C.c_double),
                ("e_ke", C.c_double), ("e_elast", C.c_double), ("e_elast_exact", C.c_double),
                ("ed_elast_dt", C.c_double), ("e_visc_f", C.c_double), ("ed_visc_f_dt", C.c_double),
                ("e_ff", C.c_double), ("ed_ff_dt", C.c_double), ("e_visc_b", C.c_double),
                ("e_b_force", C.c_double), ("e_total", C.c_double), ("max_v", C.c_double),
                ("max_f", C.c_double), ("max_ff", C.c_double), ("rms_ff", C.c_double),
                ("ave_dens", C.c_double), ("var_dens", C.c_double), ("ave_dens_from_mass", C.c_double),
                ("n", C.c_int64), ("n_sph", C.c_int64)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["lin_mom"] = list(self.lin_mom)
        return d


class SphDemStats(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("n_alive", C.c_int64), ("n_list_pairs", C.c_int64),
                ("list_depth", C.c_int64), ("n_sph_cells", C.c_int64), ("n_dem_cells", C.c_int64),
                ("h_max", C.c_double), ("search_radius", C.c_double),
                ("n_band_candidates", C.c_int64), ("band_queue_capacity", C.c_int64)]


VEC_FIELDS = ("r", "v", "vhat", "norm1", "norm2", "norm3", "f", "fp", "fv", "fb",
              "fdrag", "fvel", "grad_porosity", "v0", "vhat0")
SCA_FIELDS = ("mass", "dens", "h", "radius", "dddt", "press", "pdr2", "porosity",
              "dporositydt", "shep_sum", "omega", "u", "dudt", "e_visc", "de_visc_dt")


def config_struct(cfg: dict, precision: int | None = None) -> SphDemConfig:
    s = SphDemConfig()
    for name, ctype in SphDemConfig._fields_:
        if name == "walls":
            for i, w in enumerate(cfg.get("walls", [])[:6]):
                s.walls[i].point = D3(*w["point"])
                s.walls[i].normal = D3(*w["normal"])
            continue
        if name == "drag_scale":
            val = cfg.get(name, 1.0)
        elif name in ("reinit_dens_every", "reinit_dens_at"):
            val = cfg.get(name, 0)
        else:
            val = cfg[name]
        if ctype in (D3, I3):
            setattr(s, name, ctype(*val))
        else:
            setattr(s, name, val)
    if precision is not None:
        s.precision = precision
    return s


class ParticleBuffers:
    """numpy storage behind a SphDemParticles (all fields allocated).

    With `pinned` (a Library), the field arrays live in page-locked host
    memory from sphdem_alloc_host, so get/set_fields run at link bandwidth."""

    def __init__(self, n: int, init: dict | None = None, pinned: "Library | None" = None,
                 fields: tuple | None = None):
        self.n = n
        self._pinned = []
        self._lib = pinned
        self.arrays: dict[str, np.ndarray] = {
            "iam": np.zeros(n, np.int32), "tag": np.arange(1, n + 1, dtype=np.int32),
            "concave": np.ones(n, np.uint8),
        }
        for k in VEC_FIELDS:
            if fields is not None and k not in fields:
                continue
            self.arrays[k] = self._alloc((n, 3))
        for k in SCA_FIELDS:
            if fields is not None and k not in fields:
                continue
            self.arrays[k] = self._alloc((n,))
        if init is not None:
            for k, v in init.items():
                if k in self.arrays:
                    self.arrays[k][...] = v
            if "vhat" not in init and "v" in init:
                self.arrays["vhat"][...] = init["v"]
        self.struct = SphDemParticles()
        self.struct.n = n
        for name, ctype in SphDemParticles._fields_:
            if name == "n" or name not in self.arrays:
                continue
            a = self.arrays[name]
            setattr(self.struct, name, a.ctypes.data_as(ctype))

    def _alloc(self, shape):
        if self._lib is None:
            return np.zeros(shape, np.float64)
        nbytes = int(np.prod(shape)) * 8
        p = C.c_void_p()
        if self._lib.lib.sphdem_alloc_host(nbytes, C.byref(p)) != 0:
            raise SphDemError("sphdem_alloc_host failed")
        self._pinned.append(p)
        buf = (C.c_double * int(np.prod(shape))).from_address(p.value)
        a = np.frombuffer(buf, np.float64).reshape(shape)
        a[...] = 0.0
        return a

    def __del__(self):
        for p in getattr(self, "_pinned", []):
            try:
                self._lib.lib.sphdem_free_host(p)
            except Exception:
                pass

    def __getitem__(self, k):
        return self.arrays[k]

    def ref(self):
        return C.byref(self.struct)


class SphDemError(RuntimeError):
    pass


class Library:
    """Thin loader of libsphdem.so with checked calls."""

    def __init__(self, path: str | None = None):
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise SphDemError(f"CUDA library not built: {path} (run __graft_entry__.build())")
        self.lib = C.CDLL(path)
        L = self.lib
        H = C.c_void_p
        L.sphdem_create.argtypes = [C.POINTER(SphDemConfig), C.POINTER(SphDemParticles),
                                    C.c_int64, C.POINTER(H)]
        L.sphdem_destroy.argtypes = [H]
        L.sphdem_phase.argtypes = [H, C.c_int]
        L.sphdem_step.argtypes = [H, C.c_int]
        L.sphdem_get_fields.argtypes = [H, C.c_uint32, C.POINTER(SphDemParticles)]
        L.sphdem_set_fields.argtypes = [H, C.c_uint32, C.POINTER(SphDemParticles)]
        L.sphdem_get_globals.argtypes = [H, C.POINTER(SphDemGlobals)]
        L.sphdem_set_globals.argtypes = [H, C.POINTER(SphDemGlobals)]
        L.sphdem_rebuild.argtypes = [H]
        L.sphdem_get_fields_async.argtypes = [H, C.c_uint32, C.POINTER(SphDemParticles)]
        L.sphdem_fields_wait.argtypes = [H]
        L.sphdem_insert_particles.argtypes = [H, C.POINTER(SphDemParticles), C.POINTER(C.c_int64)]
        L.sphdem_mark_for_deletion.argtypes = [H, C.POINTER(C.c_int64), C.c_int64]
        L.sphdem_pairs.argtypes = [H, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                   C.c_int64, C.POINTER(C.c_int64)]
        L.sphdem_cell_ids.argtypes = [H, C.POINTER(C.c_int32)]
        L.sphdem_cell_ids_noalloc.argtypes = [H, C.POINTER(C.c_int32)]
        D = C.POINTER(C.c_double)
        L.sphdem_adjoint_forward.argtypes = [H, C.c_int, C.c_int]
        L.sphdem_adjoint_set_tape_memory.argtypes = [H, C.c_int64]
        L.sphdem_output_vars.argtypes = [H, C.POINTER(SphDemOutputVars)]
        L.sphdem_adjoint_backward.argtypes = [H, D, D, D, C.POINTER(SphDemGrads), D, D, D]
        L.sphdem_batch_create.argtypes = [C.POINTER(H), C.c_int, C.POINTER(H)]
        L.sphdem_batch_destroy.argtypes = [H]
        L.sphdem_batch_step.argtypes = [H, C.c_int]
        L.sphdem_batch_time_steps.argtypes = [H, C.c_int, C.POINTER(C.c_double)]
        L.sphdem_batch_tune.argtypes = [H, C.c_int, C.POINTER(C.c_int)]
        L.sphdem_batch_last_error.argtypes = [H, C.c_char_p, C.c_size_t]
        L.sphdem_kernel_times.argtypes = [H, C.c_char_p, C.c_size_t, C.POINTER(C.c_double),
                                          C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int)]
        L.sphdem_kernel_times_reset.argtypes = [H, C.c_int]
        L.sphdem_time_steps.argtypes = [H, C.c_int, C.POINTER(C.c_double)]
        L.sphdem_last_error.argtypes = [H, C.c_char_p, C.c_size_t]
        L.sphdem_version.restype = C.c_char_p
        L.sphdem_get_stats.argtypes = [H, C.POINTER(SphDemStats)]
        L.sphdem_alloc_host.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
        L.sphdem_free_host.argtypes = [C.c_void_p]

    def check(self, rc: int, h=None, what: str = ""):
        if rc != OK:
            buf = C.create_string_buffer(2048)
            self.lib.sphdem_last_error(h, buf, 2048)
            raise SphDemError(f"{what}: {ERR_NAMES.get(rc, rc)}: {buf.value.decode(errors='replace')}")


class Simulation:
    """One handle of the CUDA library, driven with numpy arrays."""

    def __init__(self, lib: Library, cfg: dict, particles: dict, precision: int = 0,
                 capacity: int | None = None):
        self.L = lib
        self.n = int(particles["iam"].shape[0])
        self.cfg_struct = config_struct(cfg, precision)
        init = ParticleBuffers(self.n, particles)
        self.h = C.c_void_p()
        rc = lib.lib.sphdem_create(C.byref(self.cfg_struct), init.ref(),
                                   capacity or self.n, C.byref(self.h))
        lib.check(rc, None, "sphdem_create")

    def close(self):
        if self.h:
            self.L.lib.sphdem_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n: int = 1):
        self.L.check(self.L.lib.sphdem_step(self.h, n), self.h, "sphdem_step")

    def phase(self, p: int):
        self.L.check(self.L.lib.sphdem_phase(self.h, p), self.h, "sphdem_phase")

    def rebuild(self):
        self.L.check(self.L.lib.sphdem_rebuild(self.h), self.h, "sphdem_rebuild")

    def get_async(self, mask: int, out: "ParticleBuffers") -> "ParticleBuffers":
        """sphdem_get_fields_async: `out` is filled once fields_wait() returns."""
        self.L.check(self.L.lib.sphdem_get_fields_async(self.h, mask, out.ref()), self.h, "get_fields_async")
        return out

    def fields_wait(self):
        self.L.check(self.L.lib.sphdem_fields_wait(self.h), self.h, "fields_wait")

    def insert(self, particles: dict) -> np.ndarray:
        """sphdem_insert_particles: the tag-order index each new particle took."""
        k = int(particles["iam"].shape[0])
        buf = ParticleBuffers(k, particles)
        out = np.zeros(max(k, 1), np.int64)
        self.L.check(self.L.lib.sphdem_insert_particles(self.h, buf.ref(), out.ctypes.data_as(C.POINTER(C.c_int64))),
                     self.h, "sphdem_insert_particles")
        out = out[:k]
        if k:
            self.n = max(self.n, int(out.max()) + 1)
        return out

    def mark_for_deletion(self, idx):
        idx = np.ascontiguousarray(idx, np.int64).reshape(-1)
        self.L.check(self.L.lib.sphdem_mark_for_deletion(self.h, idx.ctypes.data_as(C.POINTER(C.c_int64)),
                                                         int(idx.size)),
                     self.h, "sphdem_mark_for_deletion")

    def get(self, mask: int = FIELD_ALL, out: ParticleBuffers | None = None) -> ParticleBuffers:
        out = out or ParticleBuffers(self.n)
        self.L.check(self.L.lib.sphdem_get_fields(self.h, mask, out.ref()), self.h, "get_fields")
        return out

    def set(self, buf: ParticleBuffers, mask: int):
        self.L.check(self.L.lib.sphdem_set_fields(self.h, mask, buf.ref()), self.h, "set_fields")

    def globals(self) -> SphDemGlobals:
        g = SphDemGlobals()
        self.L.check(self.L.lib.sphdem_get_globals(self.h, C.byref(g)), self.h, "get_globals")
        return g

    def set_globals(self, g: SphDemGlobals):
        self.L.check(self.L.lib.sphdem_set_globals(self.h, C.byref(g)), self.h, "set_globals")

    def stats(self) -> SphDemStats:
        st = SphDemStats()
        self.L.check(self.L.lib.sphdem_get_stats(self.h, C.byref(st)), self.h, "get_stats")
        return st

    def pairs(self, kind: int):
        offs = np.zeros(self.n + 1, np.int64)
        npairs = C.c_int64(0)
        self.L.check(self.L.lib.sphdem_pairs(self.h, kind, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                             None, 0, C.byref(npairs)), self.h, "pairs")
        idx = np.zeros(max(1, npairs.value), np.int32)
        self.L.check(self.L.lib.sphdem_pairs(self.h, kind, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                             idx.ctypes.data_as(C.POINTER(C.c_int32)), idx.size,
                                             C.byref(npairs)), self.h, "pairs")
        return offs, idx[: npairs.value]

    def cell_ids(self) -> np.ndarray:
        cells = np.zeros((self.n, 3), np.int32)
        self.L.check(self.L.lib.sphdem_cell_ids(self.h, cells.ctypes.data_as(C.POINTER(C.c_int32))),
                     self.h, "cell_ids")
        return cells

    def cell_ids_noalloc(self) -> np.ndarray:
        """cell_ids through the allocation-free entry point (static device
        staging array of SPHDEM_CELL_IDS_NOALLOC_MAX particles)."""
        cells = np.zeros((self.n, 3), np.int32)
        self.L.check(self.L.lib.sphdem_cell_ids_noalloc(self.h, cells.ctypes.data_as(C.POINTER(C.c_int32))),
                     self.h, "cell_ids_noalloc")
        return cells

    def time_steps(self, n: int) -> float:
        ms = C.c_double(0)
        self.L.check(self.L.lib.sphdem_time_steps(self.h, n, C.byref(ms)), self.h, "time_steps")
        return ms.value

    def output_vars(self) -> dict:
        """calcOutputVars of the current state (sphdem_output_vars)."""
        o = SphDemOutputVars()
        self.L.check(self.L.lib.sphdem_output_vars(self.h, C.byref(o)), self.h, "output_vars")
        return o.as_dict()

    def adjoint_set_tape_memory(self, nbytes: int):
        """Device memory for the tapes of checkpoint segments kept from the
        forward pass (0: one segment's; < 0: half of the free memory)."""
        self.L.check(self.L.lib.sphdem_adjoint_set_tape_memory(self.h, int(nbytes)), self.h, "set_tape_memory")

    def adjoint_forward(self, nsteps: int, ckpt_every: int):
        self.L.check(self.L.lib.sphdem_adjoint_forward(self.h, nsteps, ckpt_every), self.h, "adjoint_forward")

    def adjoint_backward(self, dL_dr=None, dL_dv=None, dL_dvhat=None):
        """Adjoint of the final state (tag order, (n, 3) arrays or None) ->
        (SphDemGrads, dL/dr0, dL/dv0, dL/dvhat0)."""
        def arg(x):
            if x is None:
                return None
            x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.n, 3)
            return x.ctypes.data_as(C.POINTER(C.c_double))
        keep = [np.ascontiguousarray(x, dtype=np.float64).reshape(self.n, 3) if x is not None else None
                for x in (dL_dr, dL_dv, dL_dvhat)]
        outs = [np.zeros((self.n, 3)) for _ in range(3)]
        g = SphDemGrads()
        self.L.check(self.L.lib.sphdem_adjoint_backward(
            self.h, *[arg(x) for x in keep], C.byref(g),
            *[o.ctypes.data_as(C.POINTER(C.c_double)) for o in outs]), self.h, "adjoint_backward")
        return g, outs[0], outs[1], outs[2]

    def kernel_times_reset(self, enable: bool = True):
        self.L.check(self.L.lib.sphdem_kernel_times_reset(self.h, int(enable)), self.h, "kt_reset")

    def kernel_times(self) -> dict:
        names = C.create_string_buffer(16384)
        ms = (C.c_double * 128)()
        cnt = (C.c_int64 * 128)()
        nk = C.c_int(0)
        self.L.check(self.L.lib.sphdem_kernel_times(self.h, names, 16384, ms, cnt, 128, C.byref(nk)),
                     self.h, "kernel_times")
        keys = names.value.decode().split("\n")
        return {keys[i]: (ms[i], cnt[i]) for i in range(nk.value)}


class Batch:
    """Many Simulations stepped by one CUDA graph per step
    (sphdem_batch_*).  Keep the member Simulations alive while the batch
    exists; close the batch first."""

    def __init__(self, lib: "Library", sims):
        self.L = lib
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[s.h.value for s in self.sims])
        h = C.c_void_p()
        rc = lib.lib.sphdem_batch_create(arr, len(self.sims), C.byref(h))
        self.h = h
        self._check(rc, "sphdem_batch_create")

    def _check(self, rc, what):
        if rc:
            buf = C.create_string_buffer(1024)
            self.L.lib.sphdem_batch_last_error(self.h, buf, len(buf))
            raise SphDemError(f"{what}: {ERR_NAMES.get(rc, rc)}: {buf.value.decode(errors='replace')}")

    def step(self, n: int = 1):
        self._check(self.L.lib.sphdem_batch_step(self.h, n), "sphdem_batch_step")

    def time_steps(self, n: int) -> float:
        ms = C.c_double(0)
        self._check(self.L.lib.sphdem_batch_time_steps(self.h, n, C.byref(ms)), "sphdem_batch_time_steps")
        return ms.value

    def tune(self, steps_per_trial: int = 3):
        """sphdem_batch_tune: per member (block size, grid divisor, staged tiles)."""
        chosen = (C.c_int * (3 * len(self.sims)))()
        self._check(self.L.lib.sphdem_batch_tune(self.h, steps_per_trial, chosen), "sphdem_batch_tune")
        return [(chosen[3 * i], chosen[3 * i + 1], chosen[3 * i + 2]) for i in range(len(self.sims))]

    def close(self):
        if getattr(self, "h", None):
            self.L.lib.sphdem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

