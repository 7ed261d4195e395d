"""GPU parity: the CUDA engine (through its C ABI) against the reference's own
fixtures and against the CPU oracle.

Bars: (site, mode) event sequences identical; clocks and fields within 1e-10
relative (the plain FP64 form); the mixed form's stress error against an FP64
re-solve of its own eigenstrain <= 1e-5.
"""
import numpy as np
import pytest

from conftest import golden
from metallic_glasses_gb300 import api, configs
from ref2d_cases import MATERIAL_CASES, MRO_CASES, MRO_SWITCH_CASES, SF_CASES, SWITCH_CASES, check_mro_state, params_for

pytestmark = pytest.mark.gpu

FIELD_RTOL = 1e-10


def rel_err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


# ----------------------------------------------------------------- solver
@pytest.mark.parametrize("model,shape", [
    (api.MODEL_GLOBAL3D, (8, 8, 8)), (api.MODEL_GLOBAL3D, (12, 6, 16)), (api.MODEL_GLOBAL3D, (16, 24, 32)),
    (api.MODEL_GLOBAL3D, (48, 48, 48)), (api.MODEL_REF2D, (1, 64, 64)), (api.MODEL_REF2D, (1, 48, 96)),
    (api.MODEL_REF2D, (1, 512, 512)),
])
def test_fft_green_solve_matches_oracle(engine_lib, oracle_lib, model, shape):
    """The hand-written R2C/C2R solve with the fused Green's pass against the
    oracle's complex-FFT solve that keeps the real part, as the reference does."""
    if model == api.MODEL_REF2D:
        p = configs.ref2d(shape[1], shape[2])
    else:
        p = configs.shear64(seed=2)
        p.n[0], p.n[1], p.n[2] = shape
    eng = api.Engine(p)
    ora = oracle_lib.Model(p)
    rng = np.random.default_rng(11)
    nc = eng.nc
    N = eng.N
    for c in range(nc):
        v = rng.standard_normal(N) * 0.02
        eng.set_field(api.FIELD_EPS0, c, v)
        ora.set_field(api.FIELD_EPS0, c, v)
    eng.solve()
    ora.solve()
    for c in range(nc):
        assert rel_err(eng.field(api.FIELD_SIGMA, c), ora.field(api.FIELD_SIGMA, c)) < 1e-11
    eng.close()


# ----------------------------------------------------- reference fixtures
def _shear_prefix_ok(eng, g):
    """SHEAR mode: after an avalanche the reference's mean-strain correction
    (evolution.c:92-97, first component masked in every mode) zeroes the mean
    shear stress, and its divergence test |Stress[2]| < 1e-17 (bmg.c:402)
    then compares rounding noise of the field average. Where the engine's
    noise falls below the bound first, it stops there with status 2; the
    events up to that step must still be the reference's."""
    sc = eng.scalars()
    if sc["stopped"] != 2:
        return False
    ev = eng.events()
    X = g["X"]
    tr = ev[ev["kind"] != api.EV_ELASTIC]
    k = len(tr)
    assert k <= len(X)
    assert np.array_equal(np.stack([tr["step"], tr["kind"], tr["site"], tr["mode"]], 1), X[:k])
    last = int(sc["step"])
    assert (X[:, 0] == last).any() and (X[X[:, 0] == last, 1] == 1).all(), "stop must follow an avalanche"
    return True


@pytest.mark.parametrize("case", ["ref2d_64_tension_s123", "ref2d_32_shear_s7", "ref2d_32_tension_nosoft_s5"] + MRO_CASES +
                         SF_CASES + SWITCH_CASES + MRO_SWITCH_CASES + MATERIAL_CASES)
def test_ref2d_event_sequence_matches_reference(engine_lib, case):
    g = golden(case)
    p = params_for(g)
    eng = api.Engine(p)
    hdr = g["hdr"]
    eng.run(max_steps=int(hdr[1]))
    if "shear" in case and _shear_prefix_ok(eng, g):
        return
    ev = eng.events()
    tr = ev[ev["kind"] != api.EV_ELASTIC]
    X = g["X"]
    assert len(tr) == len(X)
    for col, k in ((0, "step"), (1, "kind"), (2, "site"), (3, "mode")):
        assert np.array_equal(tr[k], X[:, col]), "first mismatch in %s at %s" % (
            k, np.nonzero(tr[k] != X[:, col])[0][:3])
    sc = eng.scalars()
    assert [sc["step"], sc["kstep"], sc["astep"], sc["estep"]] == [int(v) for v in hdr[1:]]
    S = g["S"]
    last_time = {}
    for e in ev:
        last_time[int(e["step"])] = e["time"]
    t = np.array([last_time[int(s)] for s in S[:, 0] if int(s) in last_time])
    assert len(t) == len(S)
    assert np.abs(t - S[:, 2]).max() <= FIELD_RTOL * np.abs(S[:, 2]).max()
    for c in range(3):
        assert rel_err(eng.field(api.FIELD_SIGMA, c), g["sigma"][c]) < FIELD_RTOL
        assert rel_err(eng.field(api.FIELD_EPS0, c), g["eps0"][c]) < FIELD_RTOL
    assert rel_err(eng.field(api.FIELD_TLAST), g["tlast"]) < FIELD_RTOL
    assert rel_err(eng.field(api.FIELD_PERM_SOFT), g["perm_soft"]) < FIELD_RTOL
    assert rel_err(eng.field(api.FIELD_TEMP_SOFT), g["temp_soft"]) < FIELD_RTOL
    assert np.allclose(sc["eps_avg"][:3], g["sc"][1:4], rtol=FIELD_RTOL, atol=1e-14)
    assert np.allclose(sc["stress"][:3], g["sc"][4:7], rtol=1e-9, atol=1e-12)
    if case in MRO_CASES + MRO_SWITCH_CASES:
        # the map bit for bit; the modes through the host's cos/sin (glibc of
        # the machine that runs the engine, not the one that made the fixture)
        # and the device-drawn barriers to an ulp
        check_mro_state(eng, g, exact=False)
    eng.close()


@pytest.mark.parametrize("no_sf", [1, 0])
def test_mro_map_matches_oracle(engine_lib, oracle_lib, no_sf):
    """Crystal-like sites drawn at 15 % (seed 11, 32^2, softening on) with the
    NO_SF_XTAL_MRO switch as shipped and switched off: the engine takes the
    oracle's transformations for 1500 thermal events, fields within 1e-10. The
    oracle is pinned bit for bit to the reference built either way on the same
    input (fixtures ref2d_32_mro_s11 and ref2d_32_mro_xsfoff_s11)."""
    from oracle import pyoracle
    kw = dict(end="0.5", seed="11", xfrac="0.15", xq0="1.8")
    p = configs.ref2d(32, 32, **kw)
    p.no_sf_xtal_mro = no_sf
    q = configs.ref2d(32, 32, defaults=pyoracle.default_params, from_input=pyoracle.params_from_input, **kw)
    q.no_sf_xtal_mro = no_sf
    eng = api.Engine(p)
    ora = oracle_lib.Model(q)
    eng.run(max_events=1500)
    ora.run(max_events=1500)
    a, b = eng.events(), ora.events()
    a, b = a[a["kind"] != api.EV_ELASTIC], b[b["kind"] != api.EV_ELASTIC]
    assert len(a) == len(b)
    for k in ("step", "kind", "site", "mode"):
        bad = np.nonzero(a[k] != b[k])[0]
        assert bad.size == 0, "first mismatch in %s at %d" % (k, bad[0])
    mro = eng.field(api.FIELD_MRO, 0)
    assert (mro == 1).sum() > 100 and np.isin(a["site"], np.nonzero(mro)[0]).any()
    for c in range(3):
        assert rel_err(eng.field(api.FIELD_SIGMA, c), ora.field(api.FIELD_SIGMA, c)) < FIELD_RTOL
    eng.close()


def test_ref2d_deterministic(engine_lib):
    p = configs.ref2d(32, 32)
    a, b = api.Engine(p), api.Engine(p)
    a.run(max_events=200)
    b.run(max_events=200)
    assert np.array_equal(a.events(), b.events())


# ------------------------------------------------------------- 3D vs oracle
@pytest.mark.parametrize("solver", [api.SOLVER_FFT, api.SOLVER_KERNEL])
@pytest.mark.parametrize("cfg,events", [("stress32", 400), ("shear16", 400)])
def test_global3d_plain_matches_oracle(engine_lib, oracle_lib, cfg, events, solver):
    """The FP64 forms against the oracle's full re-solve per event: the FFT
    re-solve (the reference's method) and the incremental update."""
    p = configs.stress32() if cfg == "stress32" else configs.shear64(seed=5, n=16)
    p.solver = solver
    eng = api.Engine(p)
    ora = oracle_lib.Model(p)
    eng.run(max_events=events)
    ora.run(max_events=events)
    a, b = eng.events(), ora.events()
    assert len(a) == len(b)
    for k in ("step", "kind", "site", "mode"):
        assert np.array_equal(a[k], b[k])
    assert np.abs(a["time"] - b["time"]).max() <= FIELD_RTOL * np.abs(b["time"]).max()
    for c in range(6):
        assert rel_err(eng.field(api.FIELD_SIGMA, c), ora.field(api.FIELD_SIGMA, c)) < FIELD_RTOL
        assert rel_err(eng.field(api.FIELD_EPS0, c), ora.field(api.FIELD_EPS0, c)) < FIELD_RTOL
    assert rel_err(eng.field(api.FIELD_DF), ora.field(api.FIELD_DF)) < 1e-15


@pytest.mark.parametrize("solver", [api.SOLVER_FFT, api.SOLVER_KERNEL])
def test_first_10k_events_match_oracle_32(engine_lib, oracle_lib, solver):
    """The 32^3 stress-controlled configuration (1 GPa of shear, seed 0): the
    plain FP64 form takes the oracle's (step, kind, site, mode) sequence for the
    first 10^4 events, at its times, and ends with its stress and eigenstrain
    fields within 1e-10 of their size; with the FFT re-solve after every event
    (the reference's method) and with the incremental update."""
    p = configs.stress32()
    p.solver = solver
    eng = api.Engine(p)
    ora = oracle_lib.Model(p)
    eng.run(max_events=10000)
    ora.run(max_events=10000)
    a, b = eng.events(), ora.events()
    assert len(a) == len(b) and (a["kind"] == api.EV_THERMAL).sum() == 10000
    for k in ("step", "kind", "site", "mode"):
        bad = np.nonzero(a[k] != b[k])[0]
        assert bad.size == 0, "first mismatch in %s at %d" % (k, bad[0])
    assert np.abs(a["time"] - b["time"]).max() <= FIELD_RTOL * np.abs(b["time"]).max()
    for c in range(6):
        assert rel_err(eng.field(api.FIELD_SIGMA, c), ora.field(api.FIELD_SIGMA, c)) < FIELD_RTOL
        assert rel_err(eng.field(api.FIELD_EPS0, c), ora.field(api.FIELD_EPS0, c)) < FIELD_RTOL
    eng.close()
    ora.close()


@pytest.mark.parametrize("model", ["shear32", "ref2d64"])
def test_fp64_incremental_form_matches_resolve_form(engine_lib, model):
    """The FP64 incremental form against the FFT re-solve after every event
    (the reference's method) over 2000 events: shear loading at 32^3, and the
    reference's 2D model at 64^2 on its shipped input (per-site modes re-drawn
    at each transformation, softening, prints and their re-solves). The same
    events at the same times, stress fields within 1e-12 of their size (FP64
    rounding of 2000 updates of the linear solve) and the same mean stress
    (C:(ebar - <eps*>) of the solve against the solved field's mean)."""
    out = []
    for solver in (api.SOLVER_FFT, api.SOLVER_KERNEL):
        p = configs.shear64(seed=3, n=32) if model == "shear32" else configs.ref2d(64, 64)
        p.solver = solver
        eng = api.Engine(p)
        eng.run(max_events=2000)
        nc = 6 if model == "shear32" else 3
        out.append((eng.events(), np.stack([eng.field(api.FIELD_SIGMA, c) for c in range(nc)]), eng.scalars()))
        eng.close()
    (a, fa, sa), (b, fb, sb) = out
    assert sa["status"] == sb["status"] == 0 and sa["kstep"] == sb["kstep"] == 2000
    for k in ("step", "kind", "site", "mode"):
        assert np.array_equal(a[k], b[k]), k
    assert np.abs(a["time"] - b["time"]).max() <= 1e-12 * np.abs(a["time"]).max()
    assert np.abs(fa - fb).max() <= 1e-12 * np.abs(fa).max()
    assert np.allclose(sa["stress"], sb["stress"], rtol=0, atol=1e-12 * np.abs(fa).max())


def test_ensemble_stress_strain_curves_agree():
    """Ensemble-mean stress-strain curves of the mixed form and the FP64 plain
    form (shear loading at 250 K to 3 % shear strain through the elastic rise,
    thermal yield and softening; 16^3, seeds 0..15, the same seeds in both
    forms) within 1 % of the plain curve's peak. The two forms' trajectories
    part after some events, so the difference of the means is mostly the
    sampling noise of 16 realisations per form."""
    from metallic_glasses_gb300 import timing
    out = timing.ensemble(16, 16)
    print("ensemble 16^3: %s" % {k: out[k] for k in ("rel_diff_max", "rel_diff_mean", "forms")})
    assert out["strain_xy_max"] > 0.029
    assert out["forms"]["plain"]["thermal_events"] > 1000
    assert out["rel_diff_max"] < 0.01, out["rel_diff_max"]


def test_ref2d_512_matches_oracle(engine_lib, oracle_lib):
    """The reference's 2D model at its own 512 x 512 grid on its shipped input
    (softening on): the engine takes the oracle's transformations (the oracle
    is pinned to the reference's code at this grid) for 30 thermal events,
    with the clock and fields within 1e-10."""
    p = configs.ref2d(512, 512)
    eng = api.Engine(p)
    ora = oracle_lib.Model(configs.ref2d(512, 512))
    eng.run(max_events=30)
    ora.run(max_events=30)
    a, b = eng.events(), ora.events()
    assert len(a) == len(b) and (a["kind"] == api.EV_THERMAL).sum() == 30
    for k in ("step", "kind", "site", "mode"):
        assert np.array_equal(a[k], b[k]), k
    assert np.abs(a["time"] - b["time"]).max() <= FIELD_RTOL * np.abs(b["time"]).max()
    for c in range(3):
        assert rel_err(eng.field(api.FIELD_SIGMA, c), ora.field(api.FIELD_SIGMA, c)) < FIELD_RTOL
        assert rel_err(eng.field(api.FIELD_EPS0, c), ora.field(api.FIELD_EPS0, c)) < FIELD_RTOL
    eng.close()
    ora.close()


def test_correlated_barrier_field_matches_oracle(engine_lib, oracle_lib):
    p = configs.grf256(n=16)
    p.precision = api.PREC_FP64
    p.solver = api.SOLVER_FFT
    eng = api.Engine(p)
    ora = oracle_lib.Model(p)
    a, b = eng.field(api.FIELD_DF), ora.field(api.FIELD_DF)
    assert np.abs(a - b).max() < 1e-10
    assert abs(a.mean() - 1.2) < 0.05


# ------------------------------------------------------------- mixed form
def test_mixed_rates_select_like_plain_for_a_while(engine_lib):
    """FP32 rates against the FP64 plain form on the same seed: the same
    events until a near-tie of the FP32 rates flips one."""
    pm = configs.mixed128(n=16)
    pp = configs.plain128(n=16)
    m, q = api.Engine(pm), api.Engine(pp)
    m.run(max_events=20)
    q.run(max_events=20)
    a, b = m.events(), q.events()
    same = 0
    for x, y in zip(a, b):
        if x["site"] != y["site"] or x["mode"] != y["mode"]:
            break
        same += 1
    assert same >= 5
    assert np.allclose(a["time"][:same], b["time"][:same], rtol=1e-5)


def test_mixed_stress_error_within_bound(engine_lib):
    """Stress error of the FP32 incremental field against FP64 re-solves of
    the same eigenstrain every 1000 events: relative L2 and max norms of the
    deviatoric stress <= 1e-5."""
    p = configs.mixed128(n=32, resolve_period=1000)
    m = api.Engine(p)
    m.run(max_events=3000)
    sc = m.scalars()
    assert sc["kstep"] == 3000 and sc["n_resolves"] == 3
    assert 0 < sc["stress_err_rms_worst"] < 1e-5
    assert sc["stress_err_max_worst"] < 1e-5


def test_mixed_first_resolve_error_small(engine_lib):
    """One event after the start: the incremental update of one voxel's
    response against the FP64 re-solve of the same state."""
    p = configs.mixed128(n=24, resolve_period=1)
    m = api.Engine(p)
    m.run(max_events=3)
    sc = m.scalars()
    assert sc["kstep"] == 3 and sc["n_resolves"] == 3
    assert 0 < sc["stress_err_rms_worst"] < 1e-6
    assert sc["stress_err_max_worst"] < 1e-6


@pytest.mark.parametrize("n", [32, 24])
def test_mixed_pair_resolve_matches_fp64(engine_lib, n):
    """The mixed form's field solves in FP32 pairs (the default) against the
    same solves in FP64 (resolve_fp64 = 1): after the start solve and three
    periodic re-solves of an n^3 run the stored FP32 field agrees to within one
    FP32 rounding, the events are the same, and the measured stress errors of
    the incremental field agree to 1e-4 of their size (the pair transform
    carries about 48 bits; its error norms are summed in FP32 per warp). At
    24^3 the wave numbers' 1/n is not a binary fraction and the transforms
    take radix-3 passes."""
    out = {}
    for fp64 in (0, 1):
        p = configs.mixed128(n=n, resolve_period=100)
        p.resolve_fp64 = fp64
        e = api.Engine(p)
        e.run(max_events=300)
        sc = e.scalars()
        assert sc["kstep"] == 300 and sc["n_resolves"] == 3
        out[fp64] = (e.events(), sc, np.stack([e.field(api.FIELD_SDEV, k) for k in range(5)]))
        e.close()
    (ea, sa, fa), (eb, sb, fb) = out[0], out[1]
    for k in ("site", "mode"):
        assert np.array_equal(ea[k], eb[k]), k
    scale = np.abs(fb).max()
    assert np.abs(fa - fb).max() <= 2 ** -23 * scale
    for k in ("stress_err_rms_worst", "stress_err_max_worst"):
        assert abs(sa[k] - sb[k]) <= 1e-4 * sb[k] + 1e-13, k


def test_displacement_gradient_is_the_solved_strain_3d(engine_lib):
    """3D displacement field (no reference code exists in 3D): its spectral
    symmetric gradient equals the fluctuation of the total strain of the stress
    solve, C^-1:sigma + eps*, on every wave vector off the Nyquist planes (where
    the operator is the average of the sign choices)."""
    p = configs.plain128(n=16)
    e = api.Engine(p)
    e.run(max_events=40)
    u = e.displacement()
    sig = np.stack([e.field(api.FIELD_SIGMA, c) for c in range(6)])
    eps0 = np.stack([e.field(api.FIELD_EPS0, c) for c in range(6)])
    e.close()
    lam, mu, n = p.lambda_, p.mu, 16
    assert np.abs(u.mean(axis=1)).max() <= 1e-12 * np.abs(u).max()
    tr = sig[0] + sig[1] + sig[2]
    eps = np.empty_like(sig)
    eps[:3] = (sig[:3] - lam / (3 * lam + 2 * mu) * tr) / (2 * mu)
    eps[3:] = sig[3:] / (2 * mu)  # tensor shear components
    eps += eps0
    f = np.fft.fftfreq(n)
    f0, f1, f2 = np.meshgrid(f, f, f, indexing="ij")
    k = [2 * np.pi * f2, 2 * np.pi * f1, 2 * np.pi * f0]  # x = axis 2, y = axis 1, z = axis 0
    mask = (np.abs(f0) < 0.5) & (np.abs(f1) < 0.5) & (np.abs(f2) < 0.5)
    mask[0, 0, 0] = False  # the mean strain is not a gradient
    U = [np.fft.fftn(u[a].reshape(n, n, n)) for a in range(3)]
    pairs = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]  # xx yy zz yz xz xy
    scale = np.abs(eps - eps.mean(axis=1, keepdims=True)).max()
    for c, (a, b) in enumerate(pairs):
        grad = np.real(np.fft.ifftn(0.5j * (k[a] * U[b] + k[b] * U[a]) * mask))
        want = np.real(np.fft.ifftn(np.fft.fftn(eps[c].reshape(n, n, n)) * mask))
        assert np.abs(grad - want).max() <= 1e-9 * scale, c


# -------------------------------------------- spatially varying moduli
def test_inhomogeneous_solve_matches_reference(engine_lib):
    """The polarisation fixed point of a medium whose Lame moduli vary between
    0.7 and 1.3 of the uniform ones, against the reference's own
    InhomogeneousStressSolver on the same eigenstrain, moduli and mean strain
    (tests/golden/inhom_32.npz, generated from the reference's sources): the
    stress field and its mean to 1e-9 of the field's size."""
    g = golden("inhom_32")
    p = configs.ref2d(int(g["nx"]), int(g["ny"]), end="0.5", seed="5", soft="0")
    assert np.allclose([p.lambda_, p.mu], g["lame"], rtol=1e-15)
    e = api.Engine(p)
    for c in range(3):
        e.set_field(api.FIELD_EPS0, c, g["eps0"][c])
    e.set_field(api.FIELD_LAMBDA, 0, g["lam"])
    e.set_field(api.FIELD_MU, 0, g["mu"])
    e.set_mean_strain(list(g["epsavg"]))
    e.solve()
    sig = np.stack([e.field(api.FIELD_SIGMA, c) for c in range(3)])
    stress = np.array(e.scalars()["stress"][:3])
    e.close()
    scale = np.abs(g["sigma"]).max()
    assert np.abs(sig - g["sigma"]).max() <= 1e-9 * scale
    assert np.abs(stress - g["stress"]).max() <= 1e-9 * scale


def test_inhomogeneous_medium_steps(engine_lib):
    """The plain form steps with spatially varying moduli (every solve the
    fixed point); uniform moduli set explicitly leave the event sequence of the
    uniform medium unchanged."""
    def run(moduli):
        p = configs.ref2d(32, 32, end="0.5", seed="5", soft="0")
        e = api.Engine(p)
        if moduli is not None:
            lam, mu = moduli(p)
            e.set_field(api.FIELD_LAMBDA, 0, lam)
            e.set_field(api.FIELD_MU, 0, mu)
        e.run(max_events=30)
        ev, sc = e.events(), e.scalars()
        e.close()
        return ev, sc
    n = 32 * 32
    ev0, sc0 = run(None)
    ev1, sc1 = run(lambda p: (np.full(n, p.lambda_), np.full(n, p.mu)))
    for k in ("step", "kind", "site", "mode"):
        assert np.array_equal(ev0[k], ev1[k]), k
    rng = np.random.default_rng(3)
    ev2, sc2 = run(lambda p: (p.lambda_ * rng.uniform(0.8, 1.2, n), p.mu * rng.uniform(0.8, 1.2, n)))
    assert sc2["status"] == 0 and sc2["kstep"] == 30
    assert np.all(np.isfinite(sc2["stress"]))
    assert not np.array_equal(ev0["site"], ev2["site"])
