"""The reference's on-disk formats without VTK.

- Restart files: VTK XML UnstructuredGrid pieces (`<base>Restart%07d_<rank>.vtu`)
  and their parallel index (`<base>Restart%07d.pvtu`), binary appended as
  base64 with the vtkZLibDataCompressor block header, as
  Cio_data_vtk::writeRestart / readRestart use them (io_data_vtk.cpp:15-226,
  231-411).  The point arrays are the reference's, in its order: dens, h,
  eBForce, eViscF, eViscB, eFF, u, mass, colour, iam, tag, v, vhat, vort,
  norm1, norm2 (, norm3); positions are the points (Float32, as VTK writes
  them for the reference).  `exact=True` writes Float64 points and adds the
  arrays a restart needs to continue bit for bit (f, dddt, fdrag, the
  calcEnergies rates); the reference's reader ignores arrays it does not ask
  for, and this reader accepts files without them.
- Globals files (`<base>Globals<rank>.dat`): one text line per output step in
  the column order of CioGlobals::myWriteLine (ioGlobals.cpp:18, 39-46); the
  wall-time columns are written as 0, the time step as the first custom
  column.
- Domain files (`<base>Domain.dat`): rank, procDomain[2*NDIM],
  procNeighbrs[3^NDIM] (CioDomain::writeDomain, ioDomain.cpp:26-40).
"""
from __future__ import annotations

import base64
import os
import re
import struct
import xml.etree.ElementTree as ET
import zlib

import numpy as np

# --------------------------------------------------------------------------
# data arrays

_NP = {"Float32": "<f4", "Float64": "<f8", "Int32": "<i4", "Int64": "<i8", "UInt8": "u1", "UInt32": "<u4",
       "Int8": "i1", "UInt64": "<u8"}
BLOCK = 32768


def _b64_len(nbytes: int) -> int:
    return 4 * ((nbytes + 2) // 3)


def decode_array(text: str, vtk_type: str, ncomp: int, compressed: bool, header_type: str = "UInt32"):
    """One `format="binary"` DataArray body -> numpy array (n, ncomp) or (n,)."""
    s = "".join(text.split())
    hb = 8 if header_type == "UInt64" else 4
    hfmt = "<Q" if hb == 8 else "<I"
    if compressed:
        first = base64.b64decode(s[:_b64_len(hb)])
        nblocks = struct.unpack_from(hfmt, first)[0]
        hbytes = (3 + nblocks) * hb
        hlen = _b64_len(hbytes)
        head = base64.b64decode(s[:hlen])
        vals = struct.unpack_from("<" + ("Q" if hb == 8 else "I") * (3 + nblocks), head)
        csizes = vals[3:]
        data = base64.b64decode(s[hlen:]) if nblocks else b""
        raw, off = bytearray(), 0
        for cs in csizes:
            raw += zlib.decompress(data[off:off + cs])
            off += cs
        raw = bytes(raw)
    else:
        first = base64.b64decode(s[:_b64_len(hb)])
        nbytes = struct.unpack_from(hfmt, first)[0]
        allb = base64.b64decode(s)
        raw = allb[hb:hb + nbytes]
    a = np.frombuffer(raw, _NP[vtk_type]).copy()
    return a.reshape(-1, ncomp) if ncomp > 1 else a


def encode_array(a: np.ndarray, vtk_type: str) -> str:
    """numpy array -> zlib-compressed base64 body with the VTK block header."""
    raw = np.ascontiguousarray(a, dtype=_NP[vtk_type]).tobytes()
    blocks = [raw[i:i + BLOCK] for i in range(0, len(raw), BLOCK)] or []
    comp = [zlib.compress(b) for b in blocks]
    last = len(blocks[-1]) if blocks else 0
    head = struct.pack("<" + "I" * (3 + len(comp)), len(comp), BLOCK, last, *[len(c) for c in comp])
    return base64.b64encode(head).decode() + base64.b64encode(b"".join(comp)).decode()


def _range(a: np.ndarray):
    if a.size == 0:
        return 1e299, -1e299
    m = np.linalg.norm(a, axis=1) if a.ndim == 2 else a
    return float(m.min()), float(m.max())


# --------------------------------------------------------------------------
# .vtu / .pvtu

def read_vtu(path: str) -> dict:
    """A VTK XML UnstructuredGrid piece -> {"points": (n, 3) float64,
    "arrays": {name: array}, "types": {name: vtk type}}."""
    root = ET.parse(path).getroot()
    compressed = root.get("compressor") == "vtkZLibDataCompressor"
    header_type = root.get("header_type", "UInt32")
    piece = root.find("UnstructuredGrid/Piece")
    n = int(piece.get("NumberOfPoints"))

    def body(da):
        ncomp = int(da.get("NumberOfComponents", "1"))
        t = da.get("type")
        if da.get("format") == "ascii":
            a = np.array((da.text or "").split(), dtype=_NP[t])
            return a.reshape(-1, ncomp) if ncomp > 1 else a
        return decode_array(da.text or "", t, ncomp, compressed, header_type)

    out = {"n": n, "arrays": {}, "types": {}}
    pd = piece.find("PointData")
    for da in (pd if pd is not None else []):
        out["arrays"][da.get("Name")] = body(da)
        out["types"][da.get("Name")] = da.get("type")
    pts = body(piece.find("Points/DataArray"))
    out["points"] = pts.reshape(n, 3).astype(np.float64)
    out["points_type"] = piece.find("Points/DataArray").get("type")
    return out


def read_pvtu(path: str) -> dict:
    """A parallel index and all its pieces, concatenated in piece order."""
    root = ET.parse(path).getroot()
    base = os.path.dirname(os.path.abspath(path))
    pieces = [read_vtu(os.path.join(base, p.get("Source"))) for p in root.iter("Piece")]
    names = list(pieces[0]["arrays"])
    out = {"n": sum(p["n"] for p in pieces),
           "points": np.concatenate([p["points"] for p in pieces]),
           "arrays": {k: np.concatenate([p["arrays"][k] for p in pieces]) for k in names},
           "types": pieces[0]["types"], "points_type": pieces[0]["points_type"]}
    return out


def read_restart(path: str) -> dict:
    return read_pvtu(path) if path.endswith(".pvtu") else read_vtu(path)


def _data_array(name, a, vtk_type, indent):
    ncomp = a.shape[1] if a.ndim == 2 else 1
    lo, hi = _range(a)
    attrs = f'type="{vtk_type}"' + (f' Name="{name}"' if name else "")
    if ncomp > 1:
        attrs += f' NumberOfComponents="{ncomp}"'
    attrs += f' format="binary" RangeMin="{lo:.17g}" RangeMax="{hi:.17g}"'
    return f"{indent}<DataArray {attrs}>\n{indent}  {encode_array(a, vtk_type)}\n{indent}</DataArray>\n"


def write_vtu(path: str, points: np.ndarray, arrays: list, points_type: str = "Float32") -> None:
    """arrays: [(name, array, vtk type)] in file order."""
    n = points.shape[0]
    ind = "        "
    s = ['<?xml version="1.0"?>\n',
         '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian" '
         'compressor="vtkZLibDataCompressor">\n',
         "  <UnstructuredGrid>\n",
         f'    <Piece NumberOfPoints="{n}" NumberOfCells="0">\n',
         '      <PointData Scalars="iam" Vectors="v" Normals="norm1">\n']
    for name, a, t in arrays:
        s.append(_data_array(name, np.asarray(a), t, ind))
    s.append("      </PointData>\n      <Points>\n")
    s.append(_data_array(None, np.asarray(points, dtype=np.float64).reshape(n, 3), points_type, ind))
    s.append("      </Points>\n      <Cells>\n")
    for nm, t in (("connectivity", "Int32"), ("offsets", "Int32"), ("types", "UInt8")):
        s.append(_data_array(nm, np.zeros(0), t, ind))
    s.append("      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n")
    with open(path, "w") as fh:
        fh.write("".join(s))


def write_pvtu(path: str, pieces: list, arrays: list, points_type: str = "Float32") -> None:
    s = ['<?xml version="1.0"?>\n',
         '<VTKFile type="PUnstructuredGrid" version="0.1" byte_order="LittleEndian" '
         'compressor="vtkZLibDataCompressor">\n',
         '  <PUnstructuredGrid GhostLevel="0">\n',
         '    <PPointData Scalars="iam" Vectors="v" Normals="norm1">\n']
    for name, a, t in arrays:
        a = np.asarray(a)
        nc = f' NumberOfComponents="{a.shape[1]}"' if a.ndim == 2 else ""
        s.append(f'      <PDataArray type="{t}" Name="{name}"{nc}/>\n')
    s.append("    </PPointData>\n    <PPoints>\n")
    s.append(f'      <PDataArray type="{points_type}" NumberOfComponents="3"/>\n')
    s.append("    </PPoints>\n")
    for p in pieces:
        s.append(f'    <Piece Source="{os.path.basename(p)}"/>\n')
    s.append("  </PUnstructuredGrid>\n</VTKFile>\n")
    with open(path, "w") as fh:
        fh.write("".join(s))


# --------------------------------------------------------------------------
# particles <-> restart arrays

def restart_arrays(ps: dict, ndim: int, exact: bool = False) -> list:
    """Particle fields (tag order, the keys of capi.ParticleBuffers) -> the
    reference's restart arrays in its order."""
    n = ps["iam"].shape[0]

    def vec(k):
        a = np.zeros((n, 3))
        if k in ps and ps[k] is not None:
            a[:, :ndim] = np.asarray(ps[k])[:, :ndim]
        return a

    def sca(k, dflt=0.0):
        return np.asarray(ps[k], dtype=np.float64) if k in ps and ps[k] is not None else np.full(n, dflt)

    tag = np.asarray(ps["tag"]) if "tag" in ps and ps["tag"] is not None else np.arange(1, n + 1)
    arrays = [("dens", sca("dens"), "Float64"), ("h", sca("h"), "Float64"),
              ("eBForce", np.zeros(n), "Float64"), ("eViscF", sca("e_visc"), "Float64"),
              ("eViscB", np.zeros(n), "Float64"), ("eFF", np.zeros(n), "Float64"),
              ("u", sca("u"), "Float64"), ("mass", sca("mass"), "Float64"),
              ("colour", np.zeros(n), "Float64"), ("iam", np.asarray(ps["iam"], np.int32), "Int32"),
              ("tag", np.asarray(tag, np.int32), "Int32"), ("v", vec("v"), "Float64"),
              ("vhat", vec("vhat"), "Float64"), ("vort", np.zeros((n, 3)), "Float64"),
              ("norm1", vec("norm1"), "Float64"), ("norm2", vec("norm2"), "Float64")]
    if ndim == 3:
        arrays.append(("norm3", vec("norm3"), "Float64"))
    if exact:
        arrays += [("f", vec("f"), "Float64"), ("dddt", sca("dddt"), "Float64"),
                   ("fdrag", vec("fdrag"), "Float64"), ("radius", sca("radius"), "Float64"),
                   ("dudt", sca("dudt"), "Float64"), ("deViscFdt", sca("de_visc_dt"), "Float64")]
    return arrays


def particles_from_restart(d: dict, ndim: int) -> dict:
    """Restart arrays -> particle fields for sphdem_create / set_fields, in the
    file's order (sorted by tag if the pieces are not)."""
    a = d["arrays"]
    order = np.argsort(a["tag"], kind="stable") if "tag" in a else np.arange(d["n"])
    n = d["n"]

    def vec(k):
        out = np.zeros((n, 3))
        if k in a:
            v = a[k].reshape(n, -1)
            out[:, :min(ndim, v.shape[1])] = v[order, :min(ndim, v.shape[1])]
        return out

    def sca(k):
        return np.asarray(a[k], dtype=np.float64)[order] if k in a else np.zeros(n)

    r = np.zeros((n, 3))
    r[:, :ndim] = d["points"][order, :ndim]
    ps = {"iam": np.asarray(a["iam"], np.int32)[order], "tag": np.asarray(a["tag"], np.int32)[order],
          "r": r, "v": vec("v"), "vhat": vec("vhat") if "vhat" in a else vec("v"),
          "mass": sca("mass"), "dens": sca("dens"), "h": sca("h"),
          "norm1": vec("norm1"), "norm2": vec("norm2"), "norm3": vec("norm3"),
          "u": sca("u"), "e_visc": sca("eViscF")}
    for k_file, k in (("f", "f"), ("fdrag", "fdrag")):
        if k_file in a:
            ps[k] = vec(k_file)
    for k_file, k in (("dddt", "dddt"), ("radius", "radius"), ("dudt", "dudt"), ("deViscFdt", "de_visc_dt")):
        if k_file in a:
            ps[k] = sca(k_file)
    return ps


def write_restart(base: str, step: int, ps: dict, ndim: int, rank: int = 0, exact: bool = False) -> str:
    """<base>Restart%07d_<rank>.vtu + <base>Restart%07d.pvtu; returns the .pvtu path."""
    stem = f"{base}Restart{step:07d}"
    piece = f"{stem}_{rank}.vtu"
    arrays = restart_arrays(ps, ndim, exact)
    ptype = "Float64" if exact else "Float32"
    write_vtu(piece, np.asarray(ps["r"], dtype=np.float64), arrays, ptype)
    write_pvtu(stem + ".pvtu", [piece], arrays, ptype)
    return stem + ".pvtu"


# --------------------------------------------------------------------------
# Globals / Domain

GLOBALS_COLUMNS = ["OutStep", "SPHStep", "Time", "linMomX", "linMomY", "angMom", "KE", "eBForce", "eElast",
                   "eElastExact", "eViscF", "eViscB", "eFF", "eTotal", "wtTotalStep", "wtTotalForceCalc",
                   "wtTotalDddtCalc", "wtTotalReset", "wtTotalUpdateDomain", "wtTotalMPI", "maxV", "aveDens",
                   "varDens", "aveDensFromMass", "n", "nSph", "maxF", "maxFF", "rmsFF", "edElastdt",
                   "edViscFdt", "edFFdt"]


def globals_line(out_step: int, sph_step: int, time: float, ov: dict, custom=()) -> str:
    """One CioGlobals::myWriteLine row from sphdem_output_vars' dict."""
    vals = [out_step, sph_step, time, ov["lin_mom"][0], ov["lin_mom"][1], ov["ang_mom"], ov["e_ke"],
            ov["e_b_force"], ov["e_elast"], ov["e_elast_exact"], ov["e_visc_f"], ov["e_visc_b"], ov["e_ff"],
            ov["e_total"], 0, 0, 0, 0, 0, 0, ov["max_v"], ov["ave_dens"], ov["var_dens"],
            ov["ave_dens_from_mass"], ov["n"], ov["n_sph"], ov["max_f"], ov["max_ff"], ov["rms_ff"],
            ov["ed_elast_dt"], ov["ed_visc_f_dt"], ov["ed_ff_dt"]] + list(custom)
    return " ".join(repr(v) if isinstance(v, float) else str(v) for v in vals) + "\n"


def append_globals(path: str, out_step: int, sph_step: int, time: float, ov: dict, dt: float | None = None):
    """Append one row (creating the file with the reference's header line);
    dt, when given, goes in the first custom column."""
    if not os.path.exists(path):
        with open(path, "w") as fh:
            fh.write("# " + " ".join(GLOBALS_COLUMNS) + "\n")
    with open(path, "a") as fh:
        fh.write(globals_line(out_step, sph_step, time, ov, () if dt is None else (dt,)))


def read_globals(path: str) -> list:
    """Rows of a Globals file as dicts of the named columns (+ "custom": the rest)."""
    rows = []
    with open(path) as fh:
        for line in fh:
            if line.startswith("#") or not line.strip():
                continue
            t = line.split()
            row = {k: float(v) for k, v in zip(GLOBALS_COLUMNS, t)}
            row["custom"] = [float(v) for v in t[len(GLOBALS_COLUMNS):]]
            rows.append(row)
    return rows


def write_domain(path: str, ndim: int, proc_domain, rank: int = 0, neighbours=None) -> None:
    """CioDomain::writeDomain: rank, procDomain[2*NDIM], procNeighbrs[3^NDIM]
    (one process: every neighbour is the process itself)."""
    if neighbours is None:
        neighbours = [rank] * 3 ** ndim
        neighbours[(3 ** ndim) // 2] = -1  # the centre is -1, as readDomain sets it (ioDomain.cpp:14-15)
    vals = [rank] + [repr(float(x)) for x in proc_domain[:2 * ndim]] + list(neighbours)
    with open(path, "w") as fh:
        fh.write(" ".join(str(v) for v in vals) + " \n")


def read_domain(path: str, ndim: int) -> dict:
    t = open(path).read().split()
    return {"rank": int(t[0]), "proc_domain": [float(x) for x in t[1:1 + 2 * ndim]],
            "neighbours": [int(x) for x in t[1 + 2 * ndim:1 + 2 * ndim + 3 ** ndim]]}


def array_ranges(path: str) -> dict:
    """The RangeMin / RangeMax attributes VTK wrote for each point array of a
    piece (a check of decoded arrays against the writer's own numbers)."""
    out = {}
    txt = open(path).read()
    for m in re.finditer(r'<DataArray type="(\w+)" Name="([^"]+)"[^>]*RangeMin="([^"]+)" RangeMax="([^"]+)"', txt):
        out[m.group(2)] = (float(m.group(3)), float(m.group(4)))
    return out


# --------------------------------------------------------------------------
# a Simulation to and from the reference's files

def save_simulation(sim, base: str, out_step: int, exact: bool = False) -> str:
    """What the reference writes at an output step (run.cpp:124-140 with
    setup.cpp:105-118): the restart pair, one Globals row (calcOutputVars of
    the current state; dt in the first custom column) and the Domain file."""
    from . import capi
    buf = sim.get(capi.FIELD_ALL)
    ps = {k: buf[k] for k in buf.arrays}
    ndim = int(sim.cfg_struct.ndim)
    path = write_restart(base, out_step, ps, ndim, exact=exact)
    g = sim.globals()
    append_globals(f"{base}Globals0.dat", out_step, int(g.sph_step), float(g.time), sim.output_vars(),
                   dt=float(g.dt))
    dom = [x for d in range(ndim) for x in (sim.cfg_struct.domain_min[d], sim.cfg_struct.domain_max[d])]
    write_domain(f"{base}Domain.dat", ndim, dom)
    return path


def load_simulation(lib, cfg: dict, path: str, precision: int = 0, globals_path: str | None = None,
                    out_step: int | None = None):
    """A Simulation from a restart file (.pvtu or .vtu).  Arrays the exact
    form carries (f, dddt, fdrag, the energy rates) are set after creation;
    with a Globals file the step's time, dt and step count are restored."""
    from . import capi
    d = read_restart(path)
    ndim = int(cfg["ndim"])
    ps = particles_from_restart(d, ndim)
    init = {k: v for k, v in ps.items() if k in ("iam", "r", "v", "vhat", "mass", "dens", "h", "radius",
                                                   "norm1", "norm2", "norm3")}
    sim = capi.Simulation(lib, cfg, init, precision=precision)
    buf = sim.get(capi.FIELD_ALL)
    mask = capi.FIELD_ENERGY
    for k in ("u", "e_visc", "dudt", "de_visc_dt"):
        if k in ps:
            buf[k][...] = ps[k]
    if "f" in ps:
        buf["f"][...] = ps["f"]
        for k in ("fp", "fv", "fb"):
            buf[k][...] = 0.0
        mask |= capi.FIELD_F
    if "dddt" in ps:
        buf["dddt"][...] = ps["dddt"]
        mask |= capi.FIELD_DDDT
    if "fdrag" in ps:
        buf["fdrag"][...] = ps["fdrag"]
        mask |= capi.FIELD_COUPLING
    sim.set(buf, mask)
    if globals_path is not None:
        rows = read_globals(globals_path)
        row = rows[-1] if out_step is None else next(r for r in rows if int(r["OutStep"]) == out_step)
        g = sim.globals()
        g.time = row["Time"]
        g.sph_step = int(row["SPHStep"])
        if row["custom"]:
            g.dt = row["custom"][0]
        sim.set_globals(g)
    return sim
