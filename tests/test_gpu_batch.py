"""Batched ensembles (sphdem_batch_*) through the C ABI (-m gpu).

A batch replays one graph whose branches are the members' own step
sequences, so every member must end bit-identical to the same simulation
stepped alone; the autotuner only changes launch shapes, never the
per-particle arithmetic.
"""
import numpy as np
import pytest

from sphdem import capi, cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    return capi.Library()


def small_ensemble():
    # three uneven dam breaks (a few hundred to ~2k particles)
    return cases.dambreak_ensemble(3, seed=11, n_min=300, n_max=2000)


@pytest.mark.parametrize("precision", [cases.PREC_MIXED, cases.PREC_FP64])
def test_batch_matches_members_stepped_alone(lib, precision):
    ens = small_ensemble()
    alone = [capi.Simulation(lib, c.cfg, c.particles, precision=precision) for c in ens]
    members = [capi.Simulation(lib, c.cfg, c.particles, precision=precision) for c in ens]
    batch = capi.Batch(lib, members)
    try:
        batch.step(6)
        for s in alone:
            s.step(6)
        for k, (m, s) in enumerate(zip(members, alone)):
            a, b = m.get(), s.get()
            for f in ("r", "v", "dens", "f"):
                np.testing.assert_array_equal(a[f], b[f], err_msg=f"member {k} field {f}")
            assert m.globals().time == s.globals().time
    finally:
        batch.close()
        for s in alone + members:
            s.close()


def test_batch_tune_then_step(lib):
    ens = small_ensemble()
    alone = [capi.Simulation(lib, c.cfg, c.particles, precision=cases.PREC_MIXED) for c in ens]
    members = [capi.Simulation(lib, c.cfg, c.particles, precision=cases.PREC_MIXED) for c in ens]
    batch = capi.Batch(lib, members)
    try:
        chosen = batch.tune(steps_per_trial=2)
        assert len(chosen) == len(ens)
        assert all(blk in (64, 128) and div in (1, 4) and tile in (0, 1) for blk, div, tile in chosen)
        # tuning advanced each timed member by (2 + 1) steps per candidate; a
        # member of a class tuned before is not timed
        done = [int(m.globals().sph_step) for m in members]
        batch.step(3)
        for s, k in zip(alone, done):
            s.step(k + 3)
        for k, (m, s) in enumerate(zip(members, alone)):
            a, b = m.get(), s.get()
            for f in ("r", "dens"):
                np.testing.assert_array_equal(a[f], b[f], err_msg=f"member {k} field {f}")
        ms = batch.time_steps(2)
        assert ms > 0.0
    finally:
        batch.close()
        for s in alone + members:
            s.close()
