"""Output-step diagnostics on the device (sphdem_output_vars, and the
calcEnergies integrals u, dudt, e_visc, de_visc_dt) against the reference's
own values in the golden fixtures (-m gpu).

FP64: the globals to 1e-8 relative, the per-particle integrals to 1e-9 of
their scale.  Mixed: 1e-3 relative (the FP32 pair sums feed dddt and the
viscous force, whose products are integrated), with an absolute floor of
1e-6 of each quantity's natural scale for the sums that cancel (momenta).
"""
import os

import numpy as np
import pytest

from sphdem import capi, cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
WORKLOADS = ["dambreak2d_small", "dambreak2d_monaghan_small", "dem_small", "sediment3d_small"]
ORDER = ["ang_mom", "e_ke", "e_elast", "e_elast_exact", "ed_elast_dt", "e_visc_f", "ed_visc_f_dt", "e_ff",
         "ed_ff_dt", "e_visc_b", "e_b_force", "e_total", "max_v", "max_f", "max_ff", "rms_ff", "ave_dens",
         "var_dens", "ave_dens_from_mass", "n", "n_sph"]
FIELDS = {"u": "u", "dudt": "dudt", "eViscF": "e_visc", "deViscFdt": "de_visc_dt"}


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def as_vector(ov):
    return np.array(list(ov["lin_mom"]) + [ov[k] for k in ORDER], dtype=np.float64)


@pytest.mark.parametrize("precision", [cases.PREC_FP64, cases.PREC_MIXED])
@pytest.mark.parametrize("name", WORKLOADS)
def test_output_vars_match_reference(lib, name, precision):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    case = cases.workload(name)
    sim = capi.Simulation(lib, case.cfg, case.particles, precision=precision)
    try:
        sim.step(int(g["meta_nsteps"]))
        ov = sim.output_vars()
        a = sim.get()
    finally:
        sim.close()
    ref = g["output_vars"]
    ours = as_vector(ov)
    names = ["lin_mom_x", "lin_mom_y", "lin_mom_z"] + ORDER
    mass = np.asarray(case.particles["mass"], dtype=np.float64)
    mom_scale = mass.sum() * max(1e-3, float(ref[names.index("max_v")]))
    rtol = 1e-8 if precision == cases.PREC_FP64 else 1e-3
    for k, nm in enumerate(names):
        floor = 1e-6 * mom_scale if nm.startswith("lin_mom") or nm == "ang_mom" else 1e-12
        assert abs(ours[k] - ref[k]) <= rtol * abs(ref[k]) + floor, f"{name}:{nm} ours {ours[k]!r} ref {ref[k]!r}"
    ftol = 1e-9 if precision == cases.PREC_FP64 else 1e-3
    for key, ours_name in FIELDS.items():
        refv = g["field_" + key]
        scale = np.abs(refv).max()
        err = np.abs(a[ours_name] - refv).max()
        assert err <= ftol * max(scale, 1e-300), f"{name}:{key} err {err:.3e} scale {scale:.3e}"
