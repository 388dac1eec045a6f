"""The C-ABI library loads and exports every entry point include/*.h declares
(no GPU needed: the library is only dlopen'ed, nothing is called on a device)."""
import ctypes
import glob
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(sphdem_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("sphdem_create", "sphdem_destroy", "sphdem_phase", "sphdem_step",
                     "sphdem_get_fields", "sphdem_set_fields", "sphdem_pairs", "sphdem_last_error"):
        assert required in names


def test_library_exports_all_declared_symbols():
    import __graft_entry__  # noqa: F401  (build() compiles the library)
    from sphdem import capi
    if not os.path.exists(capi.LIB_PATH):
        __graft_entry__.build()
    lib = ctypes.CDLL(capi.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    lib.sphdem_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.sphdem_version()


def test_config_struct_layout_matches_header():
    """ctypes mirror of SphDemConfig has every member of the C struct."""
    from sphdem import capi
    src = open(os.path.join(REPO, "include", "sphdem.h")).read()
    body = src[src.index("typedef struct SphDemConfig"):src.index("} SphDemConfig;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    members = re.findall(r"\b([a-z_0-9]+)\s*(?:\[[^\]]*\])?\s*[;,]", body)
    ours = [f for f, _ in capi.SphDemConfig._fields_]
    for m in members:
        assert m in ours, m


def test_integration_binding_compiles(tmp_path):
    """The reference-side binding of the integration notes (their first C++
    block) compiles against include/sphdem.h, with a case's constants and the
    façade's framework headers standing in for the reference's."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    block = re.search(r"```cpp\n(.*?)```", text, flags=re.S).group(1)
    src = tmp_path / "run_gpu.cpp"
    src.write_text("#include <cstdlib>\n#include <iostream>\n#include <vector>\n" + block)
    facade = os.path.join(REPO, "sph-dem_gb300", "facade")
    res = subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-I" + os.path.join(REPO, "include"),
                          "-I" + os.path.join(facade, "example_sediment"), "-I" + os.path.join(facade, "include"),
                          str(src)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]


def test_every_entry_point_cites_the_reference():
    """Each declaration of include/sphdem.h sits in a block (back to the
    previous blank line) that cites the reference interface it replaces
    (file:line) or states that it has no counterpart there."""
    lines = open(os.path.join(REPO, "include", "sphdem.h")).read().splitlines()
    decl = re.compile(r"^(int|const char \*)\s+(sphdem_\w+)\(")
    missing = []
    for i, line in enumerate(lines):
        m = decl.match(line)
        if not m:
            continue
        j = i - 1
        block = []
        while j >= 0 and lines[j].strip():
            block.append(lines[j])
            j -= 1
        text = " ".join(block)
        if not (re.search(r"\w+\.(h|cpp):\d+", text) or "counterpart" in text):
            missing.append(m.group(2))
    assert not missing, missing
