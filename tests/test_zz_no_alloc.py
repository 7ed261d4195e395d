"""stz_solve_noalloc, the stress solve that allocates no device memory.

It exists for callers that cannot call cudaMalloc: code that runs inside
another framework's memory pool or budget, or in a process whose allocator
someone else owns. The caller passes its own device buffers; the solver's scratch sits
in one fixed device array. Its result must equal that of the context solve
(stz_solve) on the same eigenstrain, within the solver tolerance of the other
tests, on two calls in a row (the second call reuses the array the first one
left behind).
"""
import ctypes as C

import numpy as np
import pytest

from metallic_glasses_gb300 import api, configs

pytestmark = pytest.mark.gpu


def _rel_err(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("case", ["3d_stress", "2d_ref"])
def test_noalloc_solve_matches_context_solve_twice(engine_lib, case):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    if case == "3d_stress":
        p = configs.stress32(n=16)
        p.n[0], p.n[1], p.n[2] = 16, 12, 24
        dim = 3
    else:
        p = configs.ref2d(48, 64)
        dim = 2
    eng = api.Engine(p)
    lib = api.load_library()
    nc, N = eng.nc, eng.N
    ebar = eng.scalars()["eps_avg"][:nc]
    rng = np.random.default_rng(5)
    for _ in range(2):
        eps = rng.standard_normal((nc, N)) * 0.02
        for c in range(nc):
            eng.set_field(api.FIELD_EPS0, c, eps[c])
        eng.solve()
        ref = np.stack([eng.field(api.FIELD_SIGMA, c) for c in range(nc)])
        d_eps = torch.tensor(eps, dtype=torch.float64, device="cuda")
        d_sig = torch.full((nc, N), float("nan"), dtype=torch.float64, device="cuda")
        eb = (C.c_double * nc)(*ebar)
        torch.cuda.synchronize()
        st = lib.stz_solve_noalloc(dim, p.n[0], p.n[1], p.n[2], p.lambda_, p.mu, d_eps.data_ptr(), eb,
                                   d_sig.data_ptr(), None)
        assert st == api.OK, lib.stz_last_error().decode()
        out = d_sig.cpu().numpy()
        assert np.isfinite(out).all()
        assert _rel_err(out, ref) < 1e-11
    eng.close()


def test_noalloc_rejects_grids_beyond_its_scratch(engine_lib):
    lib = api.load_library()
    eb = (C.c_double * 6)(*([0.0] * 6))
    st = lib.stz_solve_noalloc(3, 128, 128, 128, 81.7, 35.0, C.c_void_p(16), eb, C.c_void_p(16), None)
    assert st == api.ERR_INVALID
    assert b"fixed scratch" in lib.stz_last_error()
