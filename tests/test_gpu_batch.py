"""Batches of independent replicas (uneven grids, temperatures, strain rates
and seeds) advanced together: each replica's trajectory must be exactly the
one it follows alone, and the stress error bar of the mixed form holds."""
import numpy as np
import pytest

from metallic_glasses_gb300 import api, configs

pytestmark = pytest.mark.gpu


def _replicas():
    ps = configs.replicas(count=4, sizes=(16, 24, 32))
    for p in ps:
        p.resolve_period = 100
    return ps


def test_batch_matches_replicas_run_alone(engine_lib):
    ps = _replicas()
    batch = api.Batch(ps)
    batch.run(60)
    for i, p in enumerate(ps):
        alone = api.Batch([p])
        alone.run(60)
        a = batch.replicas[i].events()
        b = alone.replicas[0].events()
        assert len(a) == len(b) > 0
        for k in ("step", "kind", "site", "mode"):
            assert np.array_equal(a[k], b[k]), (i, k)
        assert np.array_equal(a["time"], b["time"])
        sa, sb = batch.replicas[i].scalars(), alone.replicas[0].scalars()
        assert sa["kstep"] == sb["kstep"]
        assert sa["eps_avg"] == sb["eps_avg"]
        alone.close()
    batch.close()


def test_batch_replicas_advance_and_stay_accurate(engine_lib):
    ps = _replicas()
    batch = api.Batch(ps)
    batch.run(250)
    for r in batch.replicas:
        sc = r.scalars()
        assert sc["status"] == 0
        assert sc["kstep"] == 250 or sc["stopped"]
        if sc["n_resolves"]:
            assert sc["stress_err_rms_worst"] < 1e-5
    batch.close()


def test_athermal_trigger_forms_agree(engine_lib):
    """The single-grid main pass decides the athermal trigger per line from
    its 20 FP32 mode sums (an exact re-test of the lines whose sums reach half
    of the trigger's rate); the batched pass tests every site's largest
    argument. On a 32^3 grid under 4 GPa of shear stress, where avalanches
    start within the first 60 steps, both take the same steps."""
    p = configs.stress32(n=32)
    p.applied_stress[api.XY] = 4.0
    p.precision = api.PREC_MIXED
    p.solver = api.SOLVER_KERNEL
    p.resolve_period = 1000
    eng = api.Engine(p)
    eng.run(max_events=57)
    batch = api.Batch([p])
    batch.run(57)
    a, b = eng.events(), batch.replicas[0].events()
    sa, sb = eng.scalars(), batch.replicas[0].scalars()
    assert sa["astep"] > 0
    assert (sa["kstep"], sa["astep"]) == (sb["kstep"], sb["astep"])
    assert len(a) == len(b) > 0
    for k in ("step", "kind", "site", "mode"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["time"], b["time"])
    eng.close()
    batch.close()


def test_256_site_lines_match_general_pass(engine_lib):
    """The single-grid main pass for 256-site lines (staged and computed in two
    pieces of 128, the rate sums parked in shared memory between them) against
    the general pass that the batched form runs for such lines: the same
    events at the same times and the same stored field on a 16 x 16 x 256
    grid."""
    p = configs.mixed128(n=256, resolve_period=100)
    p.n[0], p.n[1], p.n[2] = 16, 16, 256
    eng = api.Engine(p)
    eng.run(max_events=250)
    batch = api.Batch([p])
    batch.run(250)
    r = batch.replicas[0]
    a, b = eng.events(), r.events()
    assert len(a) == len(b) == 250
    for k in ("step", "kind", "site", "mode"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["time"], b["time"])
    for c in range(5):
        assert np.array_equal(eng.field(api.FIELD_SDEV, c), r.field(api.FIELD_SDEV, c)), c
    eng.close()
    batch.close()
