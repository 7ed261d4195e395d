"""The oracle against the reference: fixtures produced by the reference's own
sources (tests/golden/make_golden.py). CPU only."""
import numpy as np
import pytest

from conftest import golden
from metallic_glasses_gb300 import api
from ref2d_cases import (CASES, MATERIAL_CASES, MRO_CASES, MRO_SWITCH_CASES, SF_CASES, SWITCH_CASES, check_mro_state,
                         params_for)


@pytest.mark.parametrize("case", CASES + MRO_CASES + SF_CASES + SWITCH_CASES + MRO_SWITCH_CASES + MATERIAL_CASES)
def test_oracle_matches_reference_bitwise(oracle_lib, engine_lib, case):
    g = golden(case)
    p = params_for(g)
    m = oracle_lib.Model(p)
    hdr = g["hdr"]
    m.run(max_steps=int(hdr[1]))
    ev = m.events()
    tr = ev[ev["kind"] != api.EV_ELASTIC]
    X = g["X"]
    # same (step, kind, site, mode) for every transformation
    assert len(tr) == len(X)
    assert np.array_equal(tr["step"], X[:, 0])
    assert np.array_equal(tr["kind"], X[:, 1])
    assert np.array_equal(tr["site"], X[:, 2])
    assert np.array_equal(tr["mode"], X[:, 3])
    sc = m.scalars()
    assert [sc["step"], sc["kstep"], sc["astep"], sc["estep"]] == [int(v) for v in hdr[1:]]
    # every step's clock
    S = g["S"]
    steps = np.unique(ev["step"])
    assert len(steps) == len(S)
    last_time = {}
    for e in ev:
        last_time[int(e["step"])] = e["time"]
    t_or = np.array([last_time.get(int(s), np.nan) for s in S[:, 0]])
    thermal_or_elastic = S[:, 1] != 1
    assert np.array_equal(t_or[thermal_or_elastic], S[thermal_or_elastic, 2])
    # final fields, bit for bit
    for c in range(3):
        assert np.array_equal(m.field(api.FIELD_SIGMA, c), g["sigma"][c])
        assert np.array_equal(m.field(api.FIELD_EPS0, c), g["eps0"][c])
    assert np.array_equal(m.field(api.FIELD_TLAST), g["tlast"])
    assert np.array_equal(m.field(api.FIELD_PERM_SOFT), g["perm_soft"])
    assert np.array_equal(m.field(api.FIELD_TEMP_SOFT), g["temp_soft"])
    deps = np.stack([m.field(api.FIELD_DEPS, k) for k in range(60)]).reshape(20, 3, -1)
    assert np.allclose(deps.sum(axis=(0, 2)), g["deps_sum"], rtol=0, atol=1e-12)
    assert sc["eps_avg"][:3] == list(g["sc"][1:4])
    assert sc["stress"][:3] == list(g["sc"][4:7])
    if case in MRO_CASES + MRO_SWITCH_CASES:
        check_mro_state(m, g)


def test_mro_fixtures_take_crystal_like_transformations():
    """The MRO fixtures exercise what they are for: crystal-like sites of
    every type the map holds transform (the reference's actQ.out records the
    chosen site's type), and their barriers were re-drawn."""
    for case, types in (("ref2d_32_mro_s11", {1}), ("ref2d_32_mrofile_s13", {1, 2, 3})):
        g = golden(case)
        assert set(np.unique(g["mro"])) == types | {0}
        chosen = set(np.unique(g["actq"][:, 0].astype(int)))
        assert types <= chosen
        X = g["X"]
        thermal = X[X[:, 1] == 0]
        assert np.array_equal(g["actq"][:, 0].astype(np.int8), g["mro"][thermal[:, 2]])
        assert (g["mro_iout"] == g["mro"]).all()


def _shipped(g):
    if "material" in g.files:
        return params_for(g, material="LOW_T")
    p = params_for(g)
    if "sf" in g.files:
        assert p.sf_scheme == int(g["sf"]) != api.SF_SQUARE_FWD
        p.sf_scheme = api.SF_SQUARE_FWD
    if "nse" in g.files:
        assert p.no_subtract_error == 1
        p.no_subtract_error = 0
    if "xsf" in g.files:
        assert p.no_sf_xtal_mro == 0
        p.no_sf_xtal_mro = 1
    return p


@pytest.mark.parametrize("case", SF_CASES + SWITCH_CASES + MRO_SWITCH_CASES + MATERIAL_CASES)
def test_switch_fixtures_depend_on_their_switch(oracle_lib, engine_lib, case):
    """Each scheme, NO_SUBTRACT_ERROR, NO_SF_XTAL_MRO or material-branch
    fixture is a run of its own switch: the oracle with the switch as shipped leaves the fixture's
    transformation sequence within the first quarter of it (within ten
    transformations for the schemes; 23 for NO_SUBTRACT_ERROR under SHEAR,
    which acts through the small normal stresses and after avalanches; 219 of
    3095 for NO_SF_XTAL_MRO, which acts only at crystal-like sites)."""
    g = golden(case)
    p = _shipped(g)
    m = oracle_lib.Model(p)
    m.run(max_steps=int(g["hdr"][1]))
    ev = m.events()
    tr = ev[ev["kind"] != api.EV_ELASTIC]
    X = g["X"]
    k = min(len(tr), len(X))
    got = np.stack([tr["step"], tr["kind"], tr["site"], tr["mode"]], 1)[:k]
    first = np.nonzero((got != X[:k]).any(axis=1))[0]
    assert len(first) and first[0] < len(X) // 4


def test_mro_structure_file_is_checked():
    """A structure line whose indices do not match its position is refused,
    as the reference aborts (init.c:412-416); so is a file with fewer lines than
    sites. Blank lines are skipped and sites are read in row-major order."""
    from metallic_glasses_gb300 import configs
    t, th = configs.read_mro_structure("1 1 0 0.5\n1 2 3 -0.25\n", 1, 2)
    assert t.tolist() == [0, 3] and th.tolist() == [0.5, -0.25]
    with pytest.raises(ValueError):
        configs.read_mro_structure("1 1 0 0.5\n1 3 3 -0.25\n", 1, 2)
    with pytest.raises(ValueError):
        configs.read_mro_structure("1 1 0 0.5\n", 1, 2)
    t, _ = configs.read_mro_structure("1 1 2 0\n\n1 2 1 0\n2 1 0 0\n2 2 3 0\n", 2, 2)
    assert t.tolist() == [2, 1, 0, 3]


def test_shear_instability_stop(oracle_lib, engine_lib):
    """In SHEAR mode the reference's athermal correction zeroes the mean shear
    stress and its divergence test (bmg.c:402) ends the run; the oracle does too."""
    g = golden("ref2d_32_shear_stop_s7")
    m = oracle_lib.Model(params_for(g))
    m.run(max_steps=100000)
    sc = m.scalars()
    assert sc["stopped"] == 2
    assert sc["step"] == int(g["hdr"][1])


@pytest.mark.parametrize("loading", ["TENSION", "SHEAR"])
def test_oracle_matches_reference_at_512(oracle_lib, engine_lib, loading):
    """At the reference's own 512 x 512 grid on its shipped input, live, under
    both loading switches: the reference's sources built against the
    single-rank stand-ins and the oracle take the same transformations and end
    with the same fields, bit for bit, over 8 thermal events (only where the
    reference tree is present)."""
    import os
    import subprocess
    import tempfile

    from metallic_glasses_gb300 import configs
    from oracle.build_oracle import build_ref2d, ref_available
    if not ref_available():
        pytest.skip("reference tree not present")
    exe = build_ref2d(512, 512, loading)
    d = tempfile.mkdtemp(prefix="stz_ref512_")
    configs.write_input(os.path.join(d, "input"))
    env = dict(os.environ, STZ_REF_LOG=os.path.join(d, "log.txt"), STZ_REF_MAX_EVENTS="8",
               STZ_REF_DUMP=os.path.join(d, "dump.bin"))
    subprocess.run([exe], cwd=d, env=env, stdout=subprocess.DEVNULL, check=True, timeout=300)
    X = np.array([[int(v) for v in line.split()[1:5]] for line in open(os.path.join(d, "log.txt"))
                  if line.startswith("X")], np.int64)
    raw = open(os.path.join(d, "dump.bin"), "rb").read()
    hdr = np.frombuffer(raw[:40], np.int64)
    N = int(hdr[0])
    arr = np.frombuffer(raw[96:], np.float64)
    sigma, eps0 = arr[:3 * N].reshape(3, N), arr[3 * N:6 * N].reshape(3, N)
    lc = api.LOAD_TENSION if loading == "TENSION" else api.LOAD_SHEAR
    m = oracle_lib.Model(configs.ref2d(512, 512, input_path=os.path.join(d, "input"), loading=lc))
    m.run(max_steps=int(hdr[1]))
    ev = m.events()
    tr = ev[ev["kind"] != api.EV_ELASTIC]
    assert N == 512 * 512 and len(X) >= 8
    assert np.array_equal(np.stack([tr["step"], tr["kind"], tr["site"], tr["mode"]], 1), X)
    sc = m.scalars()
    assert [sc["step"], sc["kstep"], sc["astep"], sc["estep"]] == [int(v) for v in hdr[1:]]
    for c in range(3):
        assert np.array_equal(m.field(api.FIELD_SIGMA, c), sigma[c])
        assert np.array_equal(m.field(api.FIELD_EPS0, c), eps0[c])
