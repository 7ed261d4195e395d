"""FFT schedules chosen per grid shape by timing (fft_autotune): every
candidate tile shape and radix order gives the default schedule's result
(none is rejected), the chosen one is a valid schedule of the shape, and the
contexts solve with it (the solver parity tests run on tuned plans)."""
import numpy as np
import pytest

from metallic_glasses_gb300 import api, configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(16, 16, 16), (24, 32, 48), (1, 64, 64)])
def test_tuned_schedule_valid(engine_lib, shape):
    if shape[0] == 1:
        p = configs.ref2d(shape[1], shape[2])
    else:
        p = configs.stress32(n=shape[2])
        p.n[0], p.n[1], p.n[2] = shape
    eng = api.Engine(p)
    sch = eng.fft_schedule()
    assert all(t >= 1 for t in sch["tiles"])
    assert sch["rejected"] == 0
    lengths = (shape[2] // 2, shape[1], shape[0])
    for order, n in zip(sch["radices"], lengths):
        assert int(np.prod(order)) == n and set(order) <= {2, 3, 4, 8}
    eng.close()
