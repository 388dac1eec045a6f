"""The CPU oracle port against golden outputs of the reference itself.

tests/golden/*.npz were produced by tests/golden/make_golden.py, which builds
the unmodified reference sources (oracle/ref/build_ref.py) and runs them from
the same seeded initial state.  This pins the port: every neighbour relation
and every bucket index must match exactly; every field must match to 1e-11
of the field's own scale (the only freedom left is the order in which the
reference visits periodic ghosts and scatters Shepard sums).
"""
import os

import numpy as np
import pytest

from sphdem import cases
from sphdem.capi import PAIR_KIND_NAMES
from sphdem.state import pair_set
from oracle.port_api import OracleSim

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
WORKLOADS = ["dambreak2d_small", "dambreak2d_monaghan_small", "dem_small", "sediment3d_small",
             "dambreak2d_own_small", "dambreak2d_cg_varh_small", "sediment3d_reinit_small",
             "sediment3d_block_small", "dambreak2d_flow_small", "sediment3d_flow_small"]
FIELD_MAP = {"r": "r", "v": "v", "vhat": "vhat", "v0": "v0", "vhat0": "vhat0", "f": "f",
             "fp": "fp", "fv": "fv", "fb": "fb", "dens": "dens", "dddt": "dddt", "h": "h",
             "press": "press", "pdr2": "pdr2", "porosity": "porosity",
             "dporositydt": "dporositydt", "gradPorosity": "grad_porosity",
             "shepSum": "shep_sum", "fdrag": "fdrag", "fvel": "fvel", "omega": "omega",
             "mass": "mass", "u": "u", "dudt": "dudt", "eViscF": "e_visc", "deViscFdt": "de_visc_dt"}
# calcOutputVars globals in the order the fixtures store them
OUTPUT_VARS = ["lin_mom_x", "lin_mom_y", "lin_mom_z", "ang_mom", "e_ke", "e_elast", "e_elast_exact",
               "ed_elast_dt", "e_visc_f", "ed_visc_f_dt", "e_ff", "ed_ff_dt", "e_visc_b", "e_b_force",
               "e_total", "max_v", "max_f", "max_ff", "rms_ff", "ave_dens", "var_dens",
               "ave_dens_from_mass", "n", "n_sph"]
RTOL = 1e-11


def _load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.fixture(scope="module", params=WORKLOADS)
def ran(request):
    name = request.param
    g = _load(name)
    case = cases.workload(name)
    assert case.n == int(g["meta_n"])
    o = OracleSim(case.cfg, case.particles)
    cases.advance(o, case, int(g["meta_nsteps"]))
    ov = o.output_vars()   # on the lists of the last reset, before any rebuild below
    return name, g, o, o.get(), o.globals(), ov


def test_fields_match_reference(ran):
    name, g, o, got, glob, ov = ran
    assert glob.time == pytest.approx(float(g["time"]), rel=1e-15)
    assert glob.dt == float(g["dt"])
    # deleted particles: dead slots here, absent (alive = 0) in the reference
    alive = g["field_alive"] > 0 if "field_alive" in g else np.ones(got.n, bool)
    assert got.n == alive.size
    assert np.array_equal(got["iam"] >= 0, alive), name
    for k, ours in FIELD_MAP.items():
        key = "field_" + k
        if key not in g:
            continue
        ref = g[key][alive]
        a = got[ours][alive]
        if a.ndim == 2 and ref.ndim == 1:
            ref = ref.reshape(a.shape)
        scale = np.abs(ref).max()
        err = np.abs(a - ref).max()
        assert err <= RTOL * max(scale, 1e-300), f"{name}:{k} err {err:.3e} scale {scale:.3e}"


def test_pairs_and_cells_match_reference(ran):
    name, g, o, got, glob, ov = ran
    o.rebuild()
    for kind, kname in PAIR_KIND_NAMES.items():
        key = "pairs_" + kname + "_offs"
        if key not in g:
            continue
        po, pi = o.pairs(kind)
        ref = pair_set(g[key], g["pairs_" + kname + "_idx"])
        ours = pair_set(po, pi)
        assert np.array_equal(ours, ref), f"{name}:{kname} {ours.size} vs {ref.size}"
    alive = g["field_alive"] > 0 if "field_alive" in g else np.ones(g["cells"].shape[0], bool)
    assert np.array_equal(o.cells()[alive], g["cells"][alive])


def output_vars_vector(ov: dict) -> np.ndarray:
    """A SphDemOutputVars dict in the fixtures' order."""
    out = list(ov["lin_mom"])
    out += [ov[k] for k in OUTPUT_VARS[3:]]
    return np.array(out, dtype=np.float64)


def test_output_vars_match_reference(ran):
    name, g, o, got, glob, ov = ran
    ref = g["output_vars"]
    ours = output_vars_vector(ov)
    assert ours.shape == ref.shape
    for k, (a, b) in enumerate(zip(ours, ref)):
        assert abs(a - b) <= 1e-9 * abs(b) + 1e-12, f"{name}:{OUTPUT_VARS[k]} ours {a!r} reference {b!r}"


def test_golden_cases_are_not_trivial():
    # every relation the fixtures pin must be exercised by at least one case
    seen = {k: 0 for k in PAIR_KIND_NAMES.values()}
    for name in WORKLOADS:
        g = _load(name)
        for k in seen:
            key = "pairs_" + k + "_idx"
            if key in g:
                seen[k] += g[key].size
    assert all(v > 0 for v in seen.values()), seen
