"""The mixed-precision form (FP32 field, contraction and rates; selection exact
in distribution over its FP32 rates) against the FP64 oracle on the same seed.

FP32 rates move the cumulative-rate boundaries of the FP64 method by about
1e-8 of the total rate; at 128^3 one (site, mode) holds about 2.4e-8 of it, so
two free-running trajectories part after a few events (at 32^3 after about
ten), always by a neighbouring site. The comparison therefore replays the
engine's trajectory in the oracle (its forced path): at every thermal event
the oracle computes its own FP64 rates, total rate, dice (the same generator
words, including any the engine rejected), clock, full FP64 re-solve and
loading, takes the engine's (site, mode), and records what it would have
chosen with the same dice. Bars:
- the dice lies within 2^-18 of the total rate of the engine's chosen
  element's FP64 cumulative interval, at every event;
- every event whose engine margin is at least that tolerance is the oracle's
  own choice;
- total rate within 1e-5 and clock within 1e-6 relative: the FP32 field
  carries the roundings of up to 1000 incremental updates per site (about
  1e-6 of its size between re-solves), and a rate moves by about 8 times the
  stress change in GPa at 455 K;
- the engine's FP32 deviatoric stress within 1e-5 (max norm over the field's
  largest value, and relative L2) of the oracle's FP64 stress after the same
  events (the oracle re-solves the whole field at every event), and the mean
  stress within 1e-5 of its largest component.
"""
import numpy as np
import pytest

from metallic_glasses_gb300 import api, configs

pytestmark = pytest.mark.gpu

CUM_TOL = 2.0 ** -18     # cumulative-position tolerance (fraction of R)
RATE_RTOL = 1e-5
CLOCK_RTOL = 1e-6
FIELD_TOL = 1e-5


def dev5(sig):
    """Deviatoric coordinates of Voigt stresses (tensor shear) in the engine's
    orthonormal basis."""
    xx, yy, zz, yz, xz, xy = sig
    r2, r6, q2 = np.sqrt(0.5), 1 / np.sqrt(6.0), np.sqrt(2.0)
    return np.stack([(xx - yy) * r2, (2 * zz - xx - yy) * r6, q2 * yz, q2 * xz, q2 * xy])


def replay(oracle_lib, eng, p_oracle, events, bounded=0, run=True):
    """Run the engine (unless run is False: a batch replica that has run),
    replay its thermal events in the oracle; returns (engine events, oracle
    events, oracle checks, oracle model). bounded > 0: the oracle's own
    choices follow the line-bound rule of that slack."""
    if run:
        eng.run(max_events=events)
    ev = eng.events()
    assert (ev["kind"] != api.EV_ATHERMAL).all()
    th = ev[ev["kind"] == api.EV_THERMAL]
    assert len(th) == events
    ora = oracle_lib.Model(p_oracle)
    if bounded:
        ora.set_bounded_selection(bounded)
    ora.force_path(th["site"], th["mode"], th["draws"])
    ora.run(max_events=events)
    oe = ora.events()
    assert len(oe) == len(ev)
    assert np.array_equal(oe["kind"], ev["kind"])
    ck = ora.checks()
    assert len(ck) == events
    return ev, oe, ck, ora


def replay_stats(eng, ev, oe, ck, ora):
    e = ev[ev["kind"] == api.EV_THERMAL]
    own_same = (ck[:, 0].astype(np.int64) == e["site"]) & (ck[:, 1].astype(np.int64) == e["mode"])
    dice, lo, hi = ck[:, 2], ck[:, 3], ck[:, 4]
    dist = np.maximum(np.maximum(lo - dice, dice - hi), 0.0)
    flagged = e["margin"] < CUM_TOL
    sig = np.stack([ora.field(api.FIELD_SIGMA, c) for c in range(6)])
    want = dev5(sig)
    got = np.stack([eng.field(api.FIELD_SDEV, k) for k in range(5)])
    sa, so = eng.scalars(), ora.scalars()
    scale = max(np.abs(so["stress"]).max(), 1e-300)
    stats = dict(events=len(e), same=int(own_same.sum()), flagged=int(flagged.sum()),
                 unflagged_differ=int((~own_same & ~flagged).sum()),
                 dist_max=float(dist.max()), dist_p99=float(np.quantile(dist, 0.99)),
                 rejections=int(sa["rejections"]),
                 rate_rel_max=float(np.abs(e["total_rate"] / ck[:, 5] - 1).max()),
                 time_rel_max=float(np.abs(ev["time"] / oe["time"] - 1).max()),
                 field_max=float(np.abs(got - want).max() / np.abs(want).max()),
                 field_l2=float(np.linalg.norm(got - want) / np.linalg.norm(want)),
                 mean_stress_rel=float(np.abs(np.array(sa["stress"]) - np.array(so["stress"])).max() / scale))
    return stats, own_same, flagged, dist


def check_state(stats):
    """Rates, clock, field and mean stress follow the oracle on the same path."""
    assert stats["rate_rel_max"] <= RATE_RTOL and stats["time_rel_max"] <= CLOCK_RTOL, stats
    assert stats["field_max"] <= FIELD_TOL and stats["field_l2"] <= FIELD_TOL, stats
    assert stats["mean_stress_rel"] <= FIELD_TOL, stats


@pytest.mark.parametrize("n,events", [(32, 1500), (128, 24)])
def test_mixed_selections_follow_the_oracle(engine_lib, oracle_lib, n, events):
    """128^3 is the bench workload (the 128-site specialised pass); the oracle
    takes about 0.2 s per event there."""
    p = configs.mixed128(n=n, resolve_period=1000)
    p.resolve_fp64 = 1
    eng = api.Engine(p)
    ev, oe, ck, ora = replay(oracle_lib, eng, configs.plain128(n=n), events)
    stats, own_same, flagged, dist = replay_stats(eng, ev, oe, ck, ora)
    print("replay %d^3: %s" % (n, stats))
    assert dist.max() <= CUM_TOL, stats
    assert (own_same | flagged).all(), np.nonzero(~(own_same | flagged))[0][:5]
    assert stats["same"] >= 0.5 * events
    check_state(stats)
    eng.close()
    ora.close()


def test_mixed_rejected_draws_follow_the_oracle(engine_lib, oracle_lib):
    """The rejection path: with the line bounds inflated by a quarter
    (sel_slack_shift = 2) about one draw in five lands in a line's slack and
    is redrawn. The oracle follows the same line-bound rule in FP64
    (or_set_bounded_selection) on the engine's path: it takes as many
    generator words and the same (site, mode) at every event, but where a
    boundary lies within the FP32 tolerance of a draw; and rates, clock,
    field and mean stress stay on the oracle's (an undone commit of a
    rejected draw would move them)."""
    n, events, slack = 16, 400, 2
    p = configs.mixed128(n=n, resolve_period=100)
    p.resolve_fp64 = 1
    p.sel_slack_shift = slack
    eng = api.Engine(p)
    ev, oe, ck, ora = replay(oracle_lib, eng, configs.plain128(n=n), events, bounded=slack)
    th = ev[ev["kind"] == api.EV_THERMAL]
    stats, own_same, flagged, dist = replay_stats(eng, ev, oe, ck, ora)
    same_draws = ck[:, 6].astype(np.int64) == th["draws"]
    stats["draws_differ"] = int((~same_draws).sum())
    print("replay %d^3, slack 2^-%d: %s" % (n, slack, stats))
    assert stats["rejections"] == int((th["draws"] - 1).sum()) > 40
    assert (th["draws"] > 1).sum() > 30
    assert stats["draws_differ"] <= 2, stats
    ok = own_same | flagged | ~same_draws
    assert ok.all(), np.nonzero(~ok)[0][:5]
    assert stats["same"] >= 0.9 * events
    check_state(stats)
    eng.close()
    ora.close()


def test_batch_replicas_follow_the_oracle(engine_lib, oracle_lib):
    """Replicas of one batch (uneven grids, temperatures and strain rates,
    the shared seed-0 mode set, one launch per line-length class) replayed
    in the oracle: the same bars as a single grid."""
    ps = configs.replicas(count=4, sizes=(16, 24, 32))
    for p in ps:
        p.resolve_period = 100
        p.resolve_fp64 = 1
    events = 300
    batch = api.Batch(ps)
    batch.run(events)
    checked = 0
    for i, p in enumerate(ps):
        r = batch.replicas[i]
        if r.scalars()["kstep"] != events or (r.events()["kind"] == api.EV_ATHERMAL).any():
            continue  # stopped early or avalanched: not a pure thermal path to replay
        ev, oe, ck, ora = replay(oracle_lib, r, p, events, run=False)
        stats, own_same, flagged, dist = replay_stats(r, ev, oe, ck, ora)
        print("batch replica %d (%d^3, %.0f K): %s" % (i, p.n[0], p.temperature, stats))
        assert dist.max() <= CUM_TOL, stats
        assert (own_same | flagged).all(), np.nonzero(~(own_same | flagged))[0][:5]
        check_state(stats)
        checked += 1
        ora.close()
    assert checked >= 2
    batch.close()


def test_default_slack_rejects_rarely(engine_lib):
    """With the default bounds (slack 2^-18 of each line sum plus 3 quanta)
    rejections are a few per million draws."""
    p = configs.mixed128(n=32, resolve_period=1000)
    eng = api.Engine(p)
    eng.run(max_events=20000)
    sc = eng.scalars()
    th = eng.events()
    th = th[th["kind"] == api.EV_THERMAL]
    assert sc["kstep"] == 20000 and sc["status"] == 0
    assert sc["rejections"] == int((th["draws"] - 1).sum())
    assert sc["rejections"] <= 5
    eng.close()


def test_128_site_lines_match_general_pass(engine_lib):
    """The per-event pass specialised to 128-site lines (each lane's four
    sites in one pass; the bench workload) against the general pass on an
    8 x 8 x 128 grid: the same events at the same times and the same stored
    FP32 field, bit for bit."""
    out = []
    for general in (0, 1):
        p = configs.mixed128(n=128, resolve_period=100)
        p.n[0], p.n[1], p.n[2] = 8, 8, 128
        p.main_pass_general = general
        e = api.Engine(p)
        e.run(max_events=300)
        out.append((e.events(), np.stack([e.field(api.FIELD_SDEV, k) for k in range(5)]), e.scalars()))
        e.close()
    (a, fa, sa), (b, fb, sb) = out
    assert len(a) == len(b) and sa["kstep"] == sb["kstep"] == 300
    for k in ("step", "kind", "site", "mode", "draws"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("time", "total_rate", "margin"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(fa, fb)
