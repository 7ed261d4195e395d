"""The reference's own entry points on the GB300 engine (refapi.c).

CPU: the reference's main (bmg.c), compiled unchanged from the reference
tree against the single-rank stand-ins of oracle/shim, links against the
drop-in layer and the engine library (only where the reference tree is
present), and so does the test driver.
GPU: the test driver, which follows the reference main's call sequence
(ReadInput ... Alloc, Energy_Init, DStrain, solve, then per step ActEnergy,
the Q < 0 scan, athermal_plasticity or KMC, ElasticEnergy, the print-time
RecordPrep / Q0 reset / uflag-2 solve), reproduces the reference's own
(step, kind, site, mode) sequence of the 32x32 tension fixture, its clock,
the positions XR (supercell position plus displacement field) its prints write
and the .iout records of Eps0 and Sigma (WriteScalarMPI, FULL_TENSOR_RECORD).
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, golden
from metallic_glasses_gb300 import build, configs
from oracle.build_oracle import REF_DIR  # the reference tree, where present

REFAPI = os.path.join(ROOT, "metallic_glasses_gb300", "refapi", "refapi.c")
TESTHDR = os.path.join(ROOT, "tests", "refapi")
SHIM = os.path.join(ROOT, "oracle", "shim")
CFLAGS = ["-O2", "-std=gnu11", "-w"]


def _lib_args():
    lib = build.build()
    d = os.path.dirname(lib)
    return ["-L", d, "-lstz_gb300", "-Wl,-rpath," + d, "-lm"]


def _support():
    # MPI stand-in (shim.c) and the generator it forwards to
    return [os.path.join(SHIM, "shim.c"), os.path.join(ROOT, "oracle", "stz_oracle.c")]


def build_driver(out, nx=32, ny=32):
    cmd = (["gcc", *CFLAGS, "-DREFAPI_NX=%d" % nx, "-DREFAPI_NY=%d" % ny, "-I", TESTHDR, "-I", SHIM,
            "-I", os.path.join(ROOT, "include"), os.path.join(TESTHDR, "driver.c"), REFAPI] + _support() +
           ["-o", out] + _lib_args())
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def test_driver_links(engine_lib):
    with tempfile.TemporaryDirectory() as d:
        build_driver(os.path.join(d, "driver"))


@pytest.mark.skipif(not os.path.isdir(REF_DIR), reason="reference tree not present")
@pytest.mark.parametrize("defs", [[], ["-DFULL_TENSOR_RECORD"]])
def test_reference_main_links_unchanged(engine_lib, defs):
    """bmg.c as shipped, and with the FULL_TENSOR_RECORD switch of its print
    block on (its .iout records through WriteScalarMPI)."""
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "bmg_gb300")
        cmd = (["gcc", *CFLAGS, *defs, "-DSTZ_SHIM_NX=32", "-DSTZ_SHIM_NY=32", "-I", SHIM, "-I", REF_DIR,
                "-I", os.path.join(ROOT, "include"), os.path.join(REF_DIR, "bmg.c"), REFAPI] + _support() +
               ["-o", out] + _lib_args())
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        assert os.path.getsize(out) > 0


@pytest.mark.gpu
def test_driver_reproduces_reference_events(engine_lib):
    g = golden("ref2d_32_tension_nosoft_s5")
    hdr = g["hdr"]
    with tempfile.TemporaryDirectory() as d:
        exe = build_driver(os.path.join(d, "driver"))
        configs.write_input(os.path.join(d, "input"), end="0.5", seed="5", soft="0")
        env = dict(os.environ, REFAPI_MAX_EVENTS=str(int(hdr[2])),
                   REFAPI_XR_PRINTS=",".join(str(int(k)) for k in g["xr_k"]))
        r = subprocess.run([exe], cwd=d, env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
        ev = np.loadtxt(os.path.join(d, "events.txt"), dtype=np.int64, ndmin=2)
        steps = np.loadtxt(os.path.join(d, "steps.txt"), ndmin=2)
        actq = np.loadtxt(os.path.join(d, "actQ.out"), ndmin=2)
        xr = np.array([[np.loadtxt(os.path.join(d, "X%dR%03d_P00.out" % (a, int(k)))).reshape(-1) for a in (1, 2)]
                       for k in g["xr_k"]])
        iout = np.array([[[np.fromfile(os.path.join(d, "%s_%02d_S%03d.iout" % (w, c + 1, int(k))), np.float64)
                           for c in range(3)] for w in ("Strain", "Stress")] for k in g["xr_k"]])
    X = g["X"]
    assert ev.shape == X.shape
    for col, name in enumerate(("step", "kind", "site", "mode")):
        bad = np.nonzero(ev[:, col] != X[:, col])[0]
        assert bad.size == 0, "first mismatch in %s at row %d" % (name, bad[0])
    assert len(steps) == int(hdr[1])
    # the reference's per-step record: (step, kind, time)
    S = g["S"]
    assert np.array_equal(steps[:, 0], S[:, 0]) and np.array_equal(steps[:, 1], S[:, 1])
    assert np.abs(steps[:, 2] - S[:, 2]).max() <= 1e-10 * np.abs(S[:, 2]).max()
    # EpsAvg and Stress every 10 steps
    S10 = g["S10"]
    rows = {int(s): k for k, s in enumerate(steps[:, 0])}
    for r10 in S10:
        got = steps[rows[int(r10[0])]]
        assert np.allclose(got[3:9], r10[3:9], rtol=1e-9, atol=1e-12)
    # actQ.out: one record per thermal event, the chosen site's MRO type (all
    # glass here) and its Q
    thermal = X[X[:, 1] == 0]
    assert len(actq) == len(thermal)
    assert (actq[:, 0] == 0).all()
    # the print files' positions: supercell position plus the displacement
    # field (up to ~1 nm here), both written with 6 decimals
    ref_xr = g["xr"]
    assert xr.shape == ref_xr.shape
    assert np.abs(xr - ref_xr).max() <= 2e-6
    # the same prints' .iout records (raw FP64 Eps0 and Sigma, FULL_TENSOR_RECORD
    # in the reference's main): the eigenstrain is the same sum of the same
    # draws; the stress is a different FFT of it
    ref_io = g["iout"]
    assert iout.shape == ref_io.shape
    assert np.abs(iout[:, 0] - ref_io[:, 0]).max() <= 1e-12 * np.abs(ref_io[:, 0]).max()
    assert np.abs(iout[:, 1] - ref_io[:, 1]).max() <= 1e-9 * np.abs(ref_io[:, 1]).max()


@pytest.mark.gpu
def test_driver_reproduces_reference_with_mro_structure(engine_lib):
    """InitMRO 1: the drop-in's Alloc reads the reference's MROstructure.ms
    (six-, two- and ten-fold sites), the run takes the reference's
    transformations, writes its Initial_MROstructure record (ten-fold sites
    turned two-fold by the same draws) and its actQ.out (the chosen site's MRO
    type and Q)."""
    import ast
    g = golden("ref2d_32_mrofile_s13")
    hdr = g["hdr"]
    ov = ast.literal_eval(str(g["overrides"]))
    with tempfile.TemporaryDirectory() as d:
        exe = build_driver(os.path.join(d, "driver"))
        configs.write_input(os.path.join(d, "input"), **ov)
        with open(os.path.join(d, "MROstructure.ms"), "w") as f:
            f.write(str(g["structure"]))
        env = dict(os.environ, REFAPI_MAX_EVENTS=str(int(hdr[2])), REFAPI_XR_PRINTS="1")
        r = subprocess.run([exe], cwd=d, env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-2000:])
        ev = np.loadtxt(os.path.join(d, "events.txt"), dtype=np.int64, ndmin=2)
        actq = np.loadtxt(os.path.join(d, "actQ.out"), ndmin=2)
        mro = np.fromfile(os.path.join(d, "Initial_MROstructure_S000.iout"), np.int32)
    X = g["X"]
    assert ev.shape == X.shape
    for col, name in enumerate(("step", "kind", "site", "mode")):
        bad = np.nonzero(ev[:, col] != X[:, col])[0]
        assert bad.size == 0, "first mismatch in %s at row %d" % (name, bad[0])
    assert np.array_equal(mro, g["mro_iout"])
    ref = g["actq"]
    assert actq.shape == ref.shape
    assert np.array_equal(actq[:, 0], ref[:, 0])
    # Q printed with 7 significant digits
    assert np.abs(actq[:, 1] - ref[:, 1]).max() <= 1e-6 * np.abs(ref[:, 1]).max()


def test_iout_records_are_the_raw_fields(engine_lib):
    """WriteScalarMPI / WriteScalarMPI_INT write "<name>_S<step>.iout" with the
    raw native values of the whole field in site order (one rank holds the
    grid): the bytes a single-rank reference run writes (CPU, no device)."""
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "iout_check")
        cmd = (["gcc", *CFLAGS, "-DREFAPI_NX=8", "-DREFAPI_NY=6", "-I", TESTHDR, "-I", SHIM,
                "-I", os.path.join(ROOT, "include"), os.path.join(TESTHDR, "iout_check.c"), REFAPI] + _support() +
               ["-o", exe] + _lib_args())
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr[-2000:]
        s = np.arange(48)
        f = np.fromfile(os.path.join(d, "Stress_02_S012.iout"), dtype=np.float64)
        assert np.array_equal(f, 0.25 * s - 3.0)
        g = np.fromfile(os.path.join(d, "Map_S003.iout"), dtype=np.int32)
        assert np.array_equal(g, 7 * s - 11)


@pytest.mark.parametrize("material", ["LOW_T", "HIGH_T_Vit1", "HIGH_T_PdNiP"])
def test_drop_in_init_material_branches(engine_lib, material):
    """Init() of the drop-in under each material branch (CPU, no device): the
    moduli and barrier amplitude the oracle reproduces the reference's own
    runs with (configs.high_t_material for the high-temperature branches,
    pinned by the ref2d_32_vit1/pdnip fixtures; the input derivation for
    LOW_T), to the last bit."""
    defs = [] if material == "LOW_T" else ["-DREFAPI_TEST_HIGH_T", "-D" + material]
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "init_check")
        cmd = (["gcc", *CFLAGS, *defs, "-DREFAPI_NX=8", "-DREFAPI_NY=6", "-I", TESTHDR, "-I", SHIM,
                "-I", os.path.join(ROOT, "include"), os.path.join(TESTHDR, "init_check.c"), REFAPI] + _support() +
               ["-o", exe] + _lib_args())
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr[-2000:]
        got = [float(v) for v in r.stdout.split()]
    p = configs.ref2d(8, 6, E="69.46", nu="0.365", q0amp="2.0")
    if material != "LOW_T":
        configs.high_t_material(p, material)
    assert got == [p.young, p.poisson, p.mu, p.lambda_, p.q0_mean]


@pytest.mark.parametrize("case,defs,overrides", [
    ("print_tension", [], {}),
    ("print_shear_nosoft", ["-DREFAPI_TEST_SHEAR"], {"soft": "0", "end": "0.1"}),
    ("print_vit1", ["-DREFAPI_TEST_HIGH_T", "-DHIGH_T_Vit1"], {"rate": "5e-5"}),
])
def test_drop_in_startup_printout_matches_reference(engine_lib, case, defs, overrides):
    """The flag block and the parameter block the drop-in prints at start-up
    (CPU, no device) are the reference's own, byte for byte
    (tests/golden/print_*.txt, written by the reference's build)."""
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "print_check")
        cmd = (["gcc", *CFLAGS, *defs, "-DREFAPI_NX=32", "-DREFAPI_NY=32", "-I", TESTHDR, "-I", SHIM,
                "-I", os.path.join(ROOT, "include"), os.path.join(TESTHDR, "print_check.c"), REFAPI] + _support() +
               ["-o", exe] + _lib_args())
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        configs.write_input(os.path.join(d, "input"), **overrides)
        r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, r.stderr[-2000:]
    want = open(os.path.join(ROOT, "tests", "golden", case + ".txt")).read()
    assert r.stdout == want


REFUSED_SWITCHES = [
    (["-DSTRAIN_RATE_SENSITIVITY"], "STRAIN_RATE_SENSITIVITY"),
    (["-DSTRAIN_RATE_SENSITIVITY", "-DLOCAL_RATE_V2"], "LOCAL_RATE_V2"),
    (["-DRELX_BIMOLE_FLAG"], "RELX_BIMOLE_FLAG"),
    (["-DRELX_FVT_FLAG"], "RELX_FVT_FLAG"),
    (["-DAVG_PERMSOFTENING"], "AVG_PERMSOFTENING"),
    (["-DHEAT_CONDUCT"], "HEAT_CONDUCT"),
    (["-DRESIDUAL_STRESS_CONST"], "RESIDUAL_STRESS_CONST"),
    (["-DRESIDUAL_STRESS_RELX"], "RESIDUAL_STRESS_RELX"),
    (["-DXTAL_VARIANTS"], "XTAL_VARIANTS"),
    (["-DSTRESS_FREE_BOUNDARY"], "STRESS_FREE_BOUNDARY"),
    (["-DREFAPI_TEST_NO_MICRO_MEMORY"], "MICRO_MEMORY"),
    (["-DREFAPI_TEST_NO_MICRO_MEMORY", "-DSF_EVEN", "-DSF_LINEAR_BWD"], "MICRO_MEMORY"),
    (["-DREFAPI_TEST_NO_SF"], "no softening-direction scheme"),
    (["-DREFAPI_TEST_NO_SF", "-DSF_Cubic_FWD"], "SF_Cubic_FWD"),
    (["-DREFAPI_TEST_HIGH_T"], "no material branch"),
]


def _syntax_check(defs):
    cmd = (["gcc", "-fsyntax-only", "-std=gnu11", *defs, "-DREFAPI_NX=8", "-DREFAPI_NY=8", "-I", TESTHDR,
            "-I", SHIM, "-I", os.path.join(ROOT, "include"), REFAPI])
    return subprocess.run(cmd, capture_output=True, text=True)


def test_drop_in_compiles_with_the_implemented_switches():
    for defs in ([], ["-DREFAPI_TEST_SHEAR"], ["-DNO_SUBTRACT_ERROR"], ["-DFULL_TENSOR_RECORD"],
                 ["-DPRE_RELAXATION", "-DUNIFORM_DEFECTS", "-DSTZ_DILATATION"],
                 ["-DREFAPI_TEST_NO_SF", "-DSF_CUBIC_FWD"], ["-DREFAPI_TEST_NO_SF", "-DSF_GAUSS_FWD"],
                 ["-DREFAPI_TEST_NO_MICRO_MEMORY", "-DREFAPI_TEST_NO_SF", "-DSF_EVEN"]):
        r = _syntax_check(defs)
        assert r.returncode == 0, (defs, r.stderr[-2000:])


@pytest.mark.parametrize("defs,scheme", [
    ([], "SQUARE_FWD"),
    (["-DSF_CUBIC_FWD"], "SQUARE_FWD"),
    (["-DSF_LINEAR_BWD"], "LINEAR_BWD"),
    (["-DSF_EVEN"], "EVEN"),
    (["-DREFAPI_TEST_NO_SF", "-DSF_GAUSS_FWD"], "GAUSS_FWD"),
    (["-DREFAPI_TEST_NO_SF", "-DSF_CUBIC_FWD", "-DSF_GAUSS_FWD"], "CUBIC_FWD"),
    (["-DREFAPI_TEST_NO_MICRO_MEMORY", "-DREFAPI_TEST_NO_SF", "-DSF_EVEN"], "EVEN"),
])
def test_drop_in_takes_the_scheme_actenergy_takes(defs, scheme):
    """With several SF_* switches defined, the first in ActEnergy's order
    (init.c:590-642) is the one the reference runs; the drop-in passes the
    same scheme to the engine."""
    cmd = (["gcc", "-E", "-P", "-std=gnu11", *defs, "-DREFAPI_NX=8", "-DREFAPI_NY=8", "-I", TESTHDR,
            "-I", SHIM, "-I", os.path.join(ROOT, "include"), REFAPI])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    got = [ln.split("=")[1].strip(" ;") for ln in r.stdout.splitlines() if "g_p.sf_scheme =" in ln]
    assert got == ["STZ_SF_" + scheme]


@pytest.mark.parametrize("defs,name", REFUSED_SWITCHES, ids=[n for _, n in REFUSED_SWITCHES])
def test_drop_in_refuses_unimplemented_switches(defs, name):
    """A bmgFlags.h switch whose physics the engine does not implement stops
    the drop-in build with an error that names it (instead of running the
    default physics)."""
    r = _syntax_check(defs)
    assert r.returncode != 0
    assert "#error" in r.stderr and name in r.stderr, r.stderr[-2000:]
