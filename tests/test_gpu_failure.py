"""Failure detection without a GPU fault.

The only spin-waits of the kernels are the bounded waits of the per-event
pass on its staged lines (an mbarrier completed by bulk copies). The
self-test arms such a barrier for bytes that no copy delivers: the wait must
run out, report STZ_ERR_TIMEOUT through the status the host reads, take a
bounded time at the kernels' full limit, and leave the device usable."""
import pytest

from metallic_glasses_gb300 import api, configs

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_device_stays_usable(engine_lib):
    st, ms_short, kmax = api.selftest_wait(1 << 10)
    assert st == api.ERR_TIMEOUT
    st, ms, kmax = api.selftest_wait(1 << 16)
    assert st == api.ERR_TIMEOUT
    assert kmax >= 1 << 16
    # the per-event kernels give up after kmax attempts: a bounded time
    full_s = ms * kmax / (1 << 16) / 1e3
    print("bounded wait: %.3f ms for 2^16 attempts, about %.2f s at the kernels' limit of %d" % (ms, full_s, kmax))
    assert full_s < 5.0
    # the context is still usable afterwards
    e = api.Engine(configs.mixed128(n=16, resolve_period=100))
    e.run(max_events=20)
    sc = e.scalars()
    assert sc["kstep"] == 20 and sc["status"] == 0
    e.close()


@pytest.mark.parametrize("mixed", [0, 1])
def test_nan_in_a_host_staged_field_is_reported(engine_lib, mixed):
    """A NaN written into one site's barrier through the C ABI (a fault made on
    the host): the next step stops with STZ_ERR_NAN in the returned status and
    in the scalars, in the FP64 plain form and in the mixed form."""
    import numpy as np
    p = configs.mixed128(n=16, resolve_period=100) if mixed else configs.shear64(seed=1, n=16)
    e = api.Engine(p)
    e.run(max_events=5)
    dF = e.field(api.FIELD_DF)
    dF[123] = np.nan
    e.set_field(api.FIELD_DF, 0, dF)
    with pytest.raises(api.StzError) as ei:
        e.run(max_events=5)
    assert ei.value.code == api.ERR_NAN
    assert e.scalars()["status"] == api.ERR_NAN
    e.close()
