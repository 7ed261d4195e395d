"""CPU: the oracle's own parameter derivation and its forced-path replay.

The CPU timing arms run the oracle without the engine library, so the oracle
derives a run's parameters itself (defaults and the reference's labelled
input file through Init(), io.c:4-101, init.c:6-75). Both derivations must
give the same stz_params field by field. The forced path (the replay the GPU
parity tests use) must reproduce a free run when fed that run's own events,
and so must the line-bound selection rule the mixed form's rejection test
replays.
"""
import os

import numpy as np
import pytest

from metallic_glasses_gb300 import api, configs


def _fields(p):
    import ctypes as C
    out = {}
    for name, ctype in api.Params._fields_:
        v = getattr(p, name)
        if isinstance(v, C._Pointer):
            out[name] = C.cast(v, C.c_void_p).value  # the address (None: no map)
        else:
            out[name] = list(v) if hasattr(v, "__len__") else v
    return out


@pytest.mark.parametrize("model", [api.MODEL_REF2D, api.MODEL_GLOBAL3D])
def test_oracle_defaults_match_engine(engine_lib, oracle_lib, model):
    a = _fields(api.default_params(model))
    b = _fields(oracle_lib.default_params(model))
    assert a == b


@pytest.mark.parametrize("overrides", [{}, dict(E="80.5", nu="0.3", seed="9", soft="0", rate="2e-4", pp="7")])
def test_oracle_input_parse_matches_engine(engine_lib, oracle_lib, tmp_path, overrides):
    path = configs.write_input(os.path.join(tmp_path, "input"), **overrides)
    a = _fields(api.params_from_input(path, api.default_params(api.MODEL_REF2D)))
    b = _fields(oracle_lib.params_from_input(path, oracle_lib.default_params(api.MODEL_REF2D)))
    assert a == b


def test_configs_with_oracle_defaults(engine_lib, oracle_lib):
    for make in (configs.plain128, configs.mixed128, configs.stress32, configs.grf256):
        assert _fields(make(n=16)) == _fields(make(n=16, defaults=oracle_lib.default_params))
    assert _fields(configs.ref2d(32, 32)) == _fields(
        configs.ref2d(32, 32, defaults=oracle_lib.default_params, from_input=oracle_lib.params_from_input))


@pytest.mark.parametrize("slack", [0, 2])
def test_forced_path_reproduces_a_free_run(oracle_lib, slack):
    p = configs.plain128(n=8, defaults=oracle_lib.default_params)
    free = oracle_lib.Model(p)
    if slack:
        free.set_bounded_selection(slack)
    free.run(max_events=300)
    ev = free.events()
    th = ev[ev["kind"] == api.EV_THERMAL]
    if slack:
        assert (th["draws"] > 1).sum() > 10
    rep = oracle_lib.Model(p)
    if slack:
        rep.set_bounded_selection(slack)
    rep.force_path(th["site"], th["mode"], th["draws"])
    rep.run(max_events=300)
    ck = rep.checks()
    assert len(ck) == 300
    assert np.array_equal(ck[:, 0].astype(np.int64), th["site"])
    assert np.array_equal(ck[:, 1].astype(np.int64), th["mode"])
    assert np.array_equal(ck[:, 6].astype(np.int64), th["draws"])
    if not slack:
        assert ((ck[:, 3] < ck[:, 2]) & (ck[:, 2] <= ck[:, 4])).all()
    ev2 = rep.events()
    for k in ("step", "kind", "site", "mode", "time"):
        assert np.array_equal(ev[k], ev2[k]), k
    for c in range(6):
        assert np.array_equal(free.field(api.FIELD_SIGMA, c), rep.field(api.FIELD_SIGMA, c))
