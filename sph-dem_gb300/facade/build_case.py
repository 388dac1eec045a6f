"""Build a case directory (customConstants.h, customSim.{h,cpp},
customOutput.{h,cpp}) into a device-driven executable: the façade headers in
include/ stand in for the framework headers the case includes, and the
executable links libsphdem.so.

    python build_case.py <case_dir> <output_executable>
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.dirname(HERE)


def zlib_flags() -> list:
    """-lz where zlib's header is installed (the restart reader then also
    reads zlib-compressed pieces, and the writer compresses)."""
    probe = subprocess.run(["g++", "-E", "-x", "c++", "-", "-o", os.devnull], input="#include <zlib.h>\n",
                           capture_output=True, text=True)
    return ["-lz"] if probe.returncode == 0 else []


def build_case(case_dir: str, out: str, extra=(), libdir: str = LIBDIR) -> str:
    """libdir: the directory of the libsphdem.so to link (the device library
    by default)."""
    case_dir = os.path.abspath(case_dir)
    srcs = [os.path.join(HERE, "run_facade.cpp"), os.path.join(HERE, "io_data_vtk.cpp")]
    for f in ("customSim.cpp", "customOutput.cpp"):
        p = os.path.join(case_dir, f)
        if os.path.exists(p):
            srcs.append(p)
    cmd = ["g++", "-std=gnu++17", "-O2", "-w", f"-I{case_dir}", f"-I{os.path.join(HERE, 'include')}",
           *srcs, f"-L{libdir}", "-lsphdem", f"-Wl,-rpath,{libdir}", "-o", out, *zlib_flags(), *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("case build failed:\n" + res.stderr[-6000:])
    return out


if __name__ == "__main__":
    if len(sys.argv) != 3:
        sys.exit(__doc__)
    print(build_case(sys.argv[1], sys.argv[2]))
