"""Invariants of the oracle's Green's-function solve (3D generalisation of
elastic.c:779-828), and the 3D model on small grids. CPU only."""
import numpy as np

from metallic_glasses_gb300 import api, configs


def voigt_to_tensor(v):
    xx, yy, zz, yz, xz, xy = v
    return np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]])


def test_equilibrium_and_mean(oracle_lib, engine_lib):
    p = configs.shear64(seed=3, n=12)
    m = oracle_lib.Model(p)
    rng = np.random.default_rng(0)
    N = 12 ** 3
    eps = rng.standard_normal((6, N)) * 0.01
    for c in range(6):
        m.set_field(api.FIELD_EPS0, c, eps[c])
    m.solve()
    sig = np.stack([m.field(api.FIELD_SIGMA, c) for c in range(6)]).reshape(6, 12, 12, 12)
    # mean stress = C:(eps_avg - <eps*>) with eps_avg = 0
    lam, mu = p.lambda_, p.mu
    e = -eps.mean(axis=1)
    tr = e[:3].sum()
    want = np.array([lam * tr + 2 * mu * e[0], lam * tr + 2 * mu * e[1], lam * tr + 2 * mu * e[2],
                     2 * mu * e[3], 2 * mu * e[4], 2 * mu * e[5]])
    assert np.allclose(sig.reshape(6, -1).mean(axis=1), want, atol=1e-12)
    # k-space equilibrium sigma_hat . k = 0 away from the Nyquist planes
    S = np.fft.fftn(sig, axes=(1, 2, 3))
    f = np.fft.fftfreq(12)
    K0, K1, K2 = np.meshgrid(f, f, f, indexing="ij")
    k = np.stack([K2, K1, K0])  # x <- axis 2, y <- axis 1, z <- axis 0
    T = np.array([[S[0], S[5], S[4]], [S[5], S[1], S[3]], [S[4], S[3], S[2]]])
    div = np.einsum("ij...,j...->i...", T, k)
    nyq = (np.abs(K0) == 0.5) | (np.abs(K1) == 0.5) | (np.abs(K2) == 0.5)
    assert np.abs(div[:, ~nyq]).max() < 1e-9 * np.abs(S).max()


def test_uniform_eigenstrain_gives_uniform_stress(oracle_lib, engine_lib):
    p = configs.shear64(seed=3, n=8)
    m = oracle_lib.Model(p)
    N = 8 ** 3
    v = [0.01, -0.004, 0.002, 0.003, -0.001, 0.005]
    for c in range(6):
        m.set_field(api.FIELD_EPS0, c, np.full(N, v[c]))
    m.solve()
    for c in range(6):
        s = m.field(api.FIELD_SIGMA, c)
        assert np.ptp(s) < 1e-12


def test_3d_model_runs_and_is_deterministic(oracle_lib, engine_lib):
    p = configs.shear64(seed=1, n=12)
    a = oracle_lib.Model(p)
    b = oracle_lib.Model(p)
    a.run(max_events=50)
    b.run(max_events=50)
    ea, eb = a.events(), b.events()
    assert np.array_equal(ea, eb)
    assert (ea["kind"] == api.EV_THERMAL).sum() == 50


def test_stress_control_holds_applied_stress(oracle_lib, engine_lib):
    p = configs.stress32(n=8)
    m = oracle_lib.Model(p)
    m.run(max_events=30)
    sc = m.scalars()
    assert abs(sc["stress"][api.XY] - 1.0) < 1e-12
    assert all(abs(sc["stress"][c]) < 1e-12 for c in range(5))
    sig = np.stack([m.field(api.FIELD_SIGMA, c) for c in range(6)])
    assert abs(sig[api.XY].mean() - 1.0) < 1e-10


def test_ensemble_curve_machinery(oracle_lib, monkeypatch):
    """The stress-strain ensemble comparison (timing.ensemble) on CPU, with the
    FP64 oracle standing in for both forms: identical runs give identical
    curves, and the curves start at the origin with the elastic slope
    sigma_xy = 2 mu eps_xy (tensor shear strain) before the first events."""
    from metallic_glasses_gb300 import timing

    class Oracle(oracle_lib.Model):
        def __init__(self, p):
            p.precision = api.PREC_FP64
            p.solver = api.SOLVER_FFT
            super().__init__(p)

    monkeypatch.setattr(api, "Engine", Oracle)
    out = timing.ensemble(8, 2, max_steps=400, eng_end=0.02)
    assert out["rel_diff_max"] == 0.0
    for k in ("steps", "thermal_events", "athermal_steps"):
        assert out["forms"]["mixed"][k] == out["forms"]["plain"][k]
    assert out["forms"]["plain"]["steps"] > 0
    eps, sig = np.array(out["curve"]["eps_xy"]), np.array(out["curve"]["plain"])
    assert eps[0] == 0.0 and sig[0] == 0.0 and out["strain_xy_max"] > 0.005
    mu = timing._ensemble_params(8, 0, 0, 250.0, 1e-4, 0.02).mu
    assert abs(sig[1] / eps[1] - 2 * mu) < 1e-6 * 2 * mu
    inc = timing._ensemble_params(8, 0, 0, 250.0, 1e-4, 0.02, fp64_incremental=True)
    assert inc.precision == api.PREC_FP64 and inc.solver == api.SOLVER_KERNEL
    assert timing._ensemble_params(8, 0, 0, 250.0, 1e-4, 0.02).solver == api.SOLVER_FFT
