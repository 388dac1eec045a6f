"""Binary particle-state files shared by the reference driver, the CPU oracle
and the tests.

Input state (``SPDMST01``): the initial particles of a case, in tag order,
optionally followed by a schedule of insertions and deletions (``SPDMEV01``:
per event its step, kind 1 = insert a particle block / 2 = mark tag-order
indices for deletion, and the payload), applied after the step's last hook.
Output state (``SPDMOUT1``): per-particle fields in tag order, the neighbour
relations as CSR over tag order (rows sorted ascending), the bucket index of
every particle and the final time / dt.
"""
from __future__ import annotations

import struct

import numpy as np

IN_MAGIC = b"SPDMST01"
EV_MAGIC = b"SPDMEV01"
OUT_MAGIC = b"SPDMOUT1"


def _write_block(fh, ps: dict, with_tag: bool) -> None:
    fh.write(np.ascontiguousarray(ps["iam"], "<i4").tobytes())
    if with_tag:
        fh.write(np.ascontiguousarray(ps["tag"], "<i4").tobytes())
    fh.write(np.ascontiguousarray(ps["concave"], "<i4").tobytes())
    for k in ("r", "v"):
        fh.write(np.ascontiguousarray(ps[k], "<f8").tobytes())
    for k in ("mass", "dens", "h", "radius"):
        fh.write(np.ascontiguousarray(ps[k], "<f8").tobytes())
    for k in ("norm1", "norm2", "norm3"):
        fh.write(np.ascontiguousarray(ps[k], "<f8").tobytes())


def write_state(path, ps: dict, events=()) -> None:
    """events: dicts {"step": s, "insert": particle block} or
    {"step": s, "delete": tag-order indices}."""
    n = ps["iam"].shape[0]
    with open(path, "wb") as fh:
        fh.write(IN_MAGIC)
        fh.write(struct.pack("<q", n))
        _write_block(fh, ps, True)
        if events:
            fh.write(EV_MAGIC)
            fh.write(struct.pack("<q", len(events)))
            for ev in events:
                if "insert" in ev:
                    blk = ev["insert"]
                    fh.write(struct.pack("<qqq", ev["step"], 1, blk["iam"].shape[0]))
                    _write_block(fh, blk, False)
                else:
                    idx = np.ascontiguousarray(ev["delete"], "<i8")
                    fh.write(struct.pack("<qqq", ev["step"], 2, idx.shape[0]))
                    fh.write(idx.tobytes())


def read_output(path) -> dict:
    with open(path, "rb") as fh:
        buf = fh.read()
    if buf[:8] != OUT_MAGIC:
        raise ValueError(f"{path}: not an SPDMOUT1 file")
    off = 8
    (n,) = struct.unpack_from("<q", buf, off)
    off += 8
    (nf,) = struct.unpack_from("<q", buf, off)
    off += 8
    out = {"n": n, "fields": {}, "pairs": {}}
    for _ in range(nf):
        name = buf[off:off + 16].rstrip(b"\0").decode()
        off += 16
        (nc,) = struct.unpack_from("<q", buf, off)
        off += 8
        a = np.frombuffer(buf, "<f8", n * nc, off).copy()
        off += 8 * n * nc
        out["fields"][name] = a.reshape(n, nc) if nc > 1 else a
    (nk,) = struct.unpack_from("<q", buf, off)
    off += 8
    for _ in range(nk):
        name = buf[off:off + 16].rstrip(b"\0").decode()
        off += 16
        (npairs,) = struct.unpack_from("<q", buf, off)
        off += 8
        offs = np.frombuffer(buf, "<i8", n + 1, off).copy()
        off += 8 * (n + 1)
        idx = np.frombuffer(buf, "<i4", npairs, off).copy()
        off += 4 * npairs
        out["pairs"][name] = (offs, idx)
    out["cells"] = np.frombuffer(buf, "<i4", 3 * n, off).copy().reshape(n, 3)
    off += 12 * n
    out["time"], out["dt"] = struct.unpack_from("<dd", buf, off)
    off += 16
    if off + 8 <= len(buf):
        (nov,) = struct.unpack_from("<q", buf, off)
        off += 8
        out["output_vars"] = np.frombuffer(buf, "<f8", nov, off).copy()
    return out


def pair_set(offs: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """Pairs (a, b) as one int64 key a*2^32+b, sorted -- for exact set checks."""
    n = offs.shape[0] - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(offs))
    keys = (rows << 32) | idx.astype(np.int64)
    return np.sort(keys)
