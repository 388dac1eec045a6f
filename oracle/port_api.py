"""ctypes driver of the CPU oracle port -- test infrastructure only.

The same SphDemConfig / SphDemParticles structs as the CUDA library's C ABI
are passed, so a test feeds both with identical inputs.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "sph-dem_gb300"))

from sphdem.capi import (ParticleBuffers, SphDemConfig, SphDemGlobals,  # noqa: E402
                         SphDemOutputVars, SphDemParticles, config_struct)

from . import build_oracle  # noqa: E402

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(build_oracle.build())
        H = C.c_void_p
        L.oracle_create.argtypes = [C.POINTER(SphDemConfig), C.POINTER(SphDemParticles), C.POINTER(H)]
        L.oracle_destroy.argtypes = [H]
        L.oracle_step.argtypes = [H, C.c_int]
        L.oracle_phase.argtypes = [H, C.c_int]
        L.oracle_rebuild.argtypes = [H]
        L.oracle_insert.argtypes = [H, C.POINTER(SphDemParticles), C.POINTER(C.c_int64)]
        L.oracle_mark_for_deletion.argtypes = [H, C.POINTER(C.c_int64), C.c_int64]
        L.oracle_get.argtypes = [H, C.POINTER(SphDemParticles)]
        L.oracle_pairs.argtypes = [H, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                   C.c_int64, C.POINTER(C.c_int64)]
        L.oracle_cells.argtypes = [H, C.POINTER(C.c_int32)]
        L.oracle_globals.argtypes = [H, C.POINTER(SphDemGlobals)]
        L.oracle_output_vars.argtypes = [H, C.POINTER(SphDemOutputVars)]
        L.oracle_last_error.restype = C.c_char_p
        _LIB = L
    return _LIB


class OracleSim:
    def __init__(self, cfg: dict, particles: dict):
        self.L = lib()
        self.n = int(particles["iam"].shape[0])
        self.cfg = config_struct(cfg)
        init = ParticleBuffers(self.n, particles)
        self.h = C.c_void_p()
        rc = self.L.oracle_create(C.byref(self.cfg), init.ref(), C.byref(self.h))
        if rc:
            raise RuntimeError("oracle_create: " + self.L.oracle_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def step(self, n=1):
        rc = self.L.oracle_step(self.h, n)
        if rc:
            raise RuntimeError("oracle_step: " + self.L.oracle_last_error().decode())

    def phase(self, p):
        rc = self.L.oracle_phase(self.h, p)
        if rc:
            raise RuntimeError("oracle_phase: " + self.L.oracle_last_error().decode())

    def rebuild(self):
        rc = self.L.oracle_rebuild(self.h)
        if rc:
            raise RuntimeError("oracle_rebuild: " + self.L.oracle_last_error().decode())

    def insert(self, particles: dict) -> np.ndarray:
        k = int(particles["iam"].shape[0])
        buf = ParticleBuffers(k, particles)
        out = np.zeros(max(k, 1), np.int64)
        self.L.oracle_insert(self.h, buf.ref(), out.ctypes.data_as(C.POINTER(C.c_int64)))
        out = out[:k]
        if k:
            self.n = max(self.n, int(out.max()) + 1)
        return out

    def mark_for_deletion(self, idx):
        idx = np.ascontiguousarray(idx, np.int64).reshape(-1)
        rc = self.L.oracle_mark_for_deletion(self.h, idx.ctypes.data_as(C.POINTER(C.c_int64)), int(idx.size))
        if rc:
            raise RuntimeError("oracle_mark_for_deletion: " + self.L.oracle_last_error().decode())

    def get(self) -> ParticleBuffers:
        out = ParticleBuffers(self.n)
        self.L.oracle_get(self.h, out.ref())
        return out

    def pairs(self, kind):
        offs = np.zeros(self.n + 1, np.int64)
        npairs = C.c_int64(0)
        self.L.oracle_pairs(self.h, kind, offs.ctypes.data_as(C.POINTER(C.c_int64)), None, 0,
                            C.byref(npairs))
        idx = np.zeros(max(1, npairs.value), np.int32)
        self.L.oracle_pairs(self.h, kind, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                            idx.ctypes.data_as(C.POINTER(C.c_int32)), idx.size, C.byref(npairs))
        return offs, idx[: npairs.value]

    def cells(self):
        c = np.zeros((self.n, 3), np.int32)
        self.L.oracle_cells(self.h, c.ctypes.data_as(C.POINTER(C.c_int32)))
        return c

    def globals(self):
        g = SphDemGlobals()
        self.L.oracle_globals(self.h, C.byref(g))
        return g

    def output_vars(self) -> dict:
        o = SphDemOutputVars()
        self.L.oracle_output_vars(self.h, C.byref(o))
        return o.as_dict()
