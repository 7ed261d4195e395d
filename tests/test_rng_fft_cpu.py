"""Known answers for the oracle's generator and FFT (CPU)."""
import numpy as np
import pytest

from conftest import golden


def test_mt19937_known_answers(oracle_lib):
    k = golden("mt19937_kat")
    r = oracle_lib.Rng(5489)
    v = 0
    for _ in range(10000):
        v = r.get()
    assert v == int(k["v10000"]) == 4123659995
    r = oracle_lib.Rng(123)
    assert [r.get() for _ in range(8)] == [int(x) for x in k["s123"]]
    r0 = oracle_lib.Rng(0)  # GSL maps seed 0 to 4357
    assert [r0.get() for _ in range(8)] == [int(x) for x in k["s4357"]]
    r = oracle_lib.Rng(123)
    for _ in range(700):
        r.get()
    assert [r.get() for _ in range(4)] == [int(x) for x in k["s123_after700"]]


def test_uniform_and_gaussian_conventions(oracle_lib):
    r1, r2 = oracle_lib.Rng(42), oracle_lib.Rng(42)
    for _ in range(100):
        assert r1.uniform() == r2.get() / 4294967296.0
    g = np.array([oracle_lib.Rng(7 + i).gaussian(1.0) for i in range(2000)])
    assert abs(g.mean()) < 0.1 and abs(g.std() - 1) < 0.1


@pytest.mark.parametrize("shape", [(1, 8, 16), (1, 6, 12), (4, 8, 16), (3, 6, 12), (1, 32, 48), (2, 9, 24)])
def test_oracle_fft_matches_numpy(oracle_lib, shape):
    rng = np.random.default_rng(1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    f = oracle_lib.fft3(a, -1)
    assert np.allclose(f, np.fft.fftn(a), rtol=0, atol=1e-10 * np.abs(a).sum())
    b = oracle_lib.fft3(f, +1)
    assert np.allclose(b / a.size, a, atol=1e-12)


def test_exp_table_matches_its_generator():
    """The FP64 exponential's table (exp_table.h) is what exp_table.py
    generates: 2^(j/256) as hi + lo and the split of ln2/256."""
    import os
    import subprocess
    import sys
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "metallic_glasses_gb300", "csrc")
    out = subprocess.run([sys.executable, os.path.join(here, "exp_table.py")], capture_output=True, text=True,
                         check=True).stdout
    with open(os.path.join(here, "exp_table.h")) as f:
        assert f.read() == out
