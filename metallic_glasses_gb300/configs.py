"""Workload configurations.

ref2d(...)      the reference's own 2D model, built from a reference-format
                input file (labels of io.c:4-101) at a chosen grid, with the
                text of an MROstructure.ms file when its input reads one
stress32()      32^3, FP64, constant applied pure shear stress 1 GPa, seed 0
plain128()      128^3 (or n^3), FP64, shear strain rate, the re-solve after every event
incr128()       the same with the FP64 incremental update
shear64(seed)   64^3, FP64, shear strain rate, seeds 0-3
mixed128()      128^3, mixed form, periodic full re-solve every 1000 events
grf256()        256^3, mixed form, correlated barrier field
replicas(...)   uneven 3D replicas (grids 32/48/64/96, T in [325, 585] K,
                log-uniform strain rates), seeds 0-255

Every function takes `defaults`, the function that fills a model's default
parameters (api.default_params, the engine library's, unless given), and
ref2d also `from_input`, the input-file parser (api.params_from_input unless
given): a caller that must not load the engine library (the CPU oracle's
timing) passes the oracle's own.

Common 3D physics: mu = 35 GPa, nu = 0.35, nu0 = 1e13 /s, Omega0 = 1 nm^3,
T = 455 K, dF ~ N(1.2, 0.1) eV truncated at 3 sd, 20 traceless modes of
magnitude 0.1 with orientations uniform on SO(3). The shear loading applies
the reference's SHEAR branch to the xy tensor component; an engineering shear
strain (rate) gamma corresponds to a tensor strain (rate) gamma/2.
"""
import math
import os

import numpy as np

from . import api

INPUT_LABELS = [
    ("Moduli(E, nu):", "{E} {nu}"),
    ("Stress-free energy barrier:", "{q0amp}"),
    ("Applied strain rate:", "{rate}"),
    ("Strain increment:", "{inc}"),
    ("Random seed:", "{seed}"),
    ("Random ratio of fluctuation in energy barrier:", "{rr}"),
    ("Print period:", "{pp}"),
    ("End Strain:", "{end}"),
    ("Softening Flag:", "{soft}"),
    ("Relaxation Time:", "{relx}"),
    ("Characteristic Xtal shear:", "{xs}"),
    ("Barrier for Xtal shear:", "{xq}"),
    ("Ratio for generating residual stress:", "{resi}"),
    ("Residual stress data file:", "{resfile}"),
    ("Volume fraction of crystal-like MRO:", "{xfrac}"),
    ("Initialization condition for MRO:", "{initmro}"),
    ("Stress-free energy barrier for crystal-like MRO:", "{xq0}"),
]

# values of the input file shipped with the reference
SHIPPED_INPUT = dict(E="69.46", nu="0.365", q0amp="2.0", rate="1e-4", inc="1e-4", seed="123", rr="0.2",
                     pp="5", end="0.06", soft="1", relx="0.", xs="0.04", xq="1.25", resi="0.06",
                     resfile="NullSpaceBasis_128x128_Nullity254.out", xfrac="0.0", initmro="0", xq0="2.0")


def write_input(path, **overrides):
    """Write a reference-format 'input' file (the labelled layout of io.c)."""
    v = dict(SHIPPED_INPUT)
    v.update({k: str(x) for k, x in overrides.items()})
    with open(path, "w") as f:
        for label, fmt in INPUT_LABELS:
            f.write(label + "\n" + fmt.format(**v) + "\n\n")
    return path


def read_mro_structure(text, nx, ny):
    """The crystal-like MRO map of a structure file in the reference's
    MROstructure.ms layout (init.c:398-420): one line per site in site order,
    "i j type angle" with 1-based i (slow axis) and j. Returns (types, angles);
    a line whose indices do not match its position raises ValueError, as the
    reference aborts."""
    rows = [ln.split() for ln in text.splitlines() if ln.strip()]
    if len(rows) < nx * ny:
        raise ValueError("structure file has %d lines for %d sites" % (len(rows), nx * ny))
    types = np.zeros(nx * ny, np.int32)
    theta = np.zeros(nx * ny, np.float64)
    for m in range(nx * ny):
        ii, jj, t, th = rows[m][:4]
        if (int(ii) - 1) * ny + int(jj) - 1 != m:
            raise ValueError("structure file line %d: inconsistent index" % (m + 1))
        types[m] = int(t)
        theta[m] = float(th)
    return types, theta


def high_t_material(p, branch):
    """The moduli and barrier amplitude of the reference's high-temperature
    material branches of Init() (bmgFlags.h HIGH_T_Vit1 / HIGH_T_PdNiP,
    init.c:28-42, with bmg.h:36-48's constants), in place of what the input
    file's LOW_T derivation gave (init.c:18-27): Vit1 follows the glass /
    supercooled-liquid interpolation in tanh((T - Tg)/DeltaE), PdNiP fixed
    values; lambda as in init.c:44. Returns p."""
    T = p.temperature
    if branch == "HIGH_T_Vit1":
        Tg = 623.
        E = (80.7 + 30.0) / 2. - (80.7 - 30.0) * math.tanh((T - Tg) / 24.0) / 2. - 39.0E-3 * (T - Tg)
        nu = (0.360 + 0.447) / 2. - (0.360 - 0.447) * math.tanh((T - Tg) / 24.0) / 2.
        q0 = 2.2
    elif branch == "HIGH_T_PdNiP":
        E, nu, q0 = 96., 0.36, 3.0
    else:
        raise ValueError("material branch %r" % branch)
    p.young, p.poisson = E, nu
    p.mu = E / (2 + 2 * nu)
    p.lambda_ = E * nu / (1 - nu * nu)
    p.q0_mean = q0
    return p


def ref2d(nx=64, ny=64, input_path=None, loading=api.LOAD_TENSION, defaults=None, from_input=None,
          mro_structure=None, solver=None, **overrides):
    p = (defaults or api.default_params)(api.MODEL_REF2D)
    if input_path is None:
        import tempfile
        d = tempfile.mkdtemp(prefix="stz_in_")
        input_path = write_input(os.path.join(d, "input"), **overrides)
    (from_input or api.params_from_input)(input_path, p)
    p.n[0], p.n[1], p.n[2] = 1, nx, ny
    p.loading = loading
    if mro_structure is not None:
        api.set_mro_map(p, *read_mro_structure(mro_structure, nx, ny))
    if solver is not None:
        p.solver = solver
    return p


def _g3(n, seed=0, defaults=None):
    p = (defaults or api.default_params)(api.MODEL_GLOBAL3D)
    p.n[0] = p.n[1] = p.n[2] = n
    p.seed = seed
    return p


def stress32(seed=0, n=32, defaults=None):
    p = _g3(n, seed, defaults)
    p.loading = api.LOAD_STRESS
    p.applied_stress[api.XY] = 1.0
    p.strain_rate = 0.0
    return p


def shear64(seed=0, n=64, eng_rate=1e-4, eng_end=0.05, defaults=None):
    p = _g3(n, seed, defaults)
    p.loading = api.LOAD_SHEAR
    p.strain_rate = eng_rate / 2
    p.end_strain = eng_end / 2
    p.strain_increment = 1e-4
    return p


def mixed128(seed=0, n=128, resolve_period=1000, defaults=None):
    p = shear64(seed, n, defaults=defaults)
    p.precision = api.PREC_MIXED
    p.solver = api.SOLVER_KERNEL
    p.resolve_period = resolve_period
    return p


def plain128(seed=0, n=128, defaults=None):
    return shear64(seed, n, defaults=defaults)


def incr128(seed=0, n=128, defaults=None):
    """The FP64 form with the incremental update (the mixed form's method in
    FP64) in place of the re-solve after every event."""
    p = shear64(seed, n, defaults=defaults)
    p.solver = api.SOLVER_KERNEL
    return p


def grf256(seed=0, n=256, defaults=None):
    p = shear64(seed, n, eng_rate=1e-3, eng_end=0.08, defaults=defaults)
    p.df_kind = api.DF_CORRELATED
    p.q0_sd = 0.15
    p.q0_corr_len = 4.0
    p.precision = api.PREC_MIXED
    p.solver = api.SOLVER_KERNEL
    return p


def replicas(count=256, seed_base=0, mixed=True, sizes=(32, 48, 64, 96)):
    """Uneven replicas: grid uniform over `sizes`, T uniform in [325, 585] K,
    engineering strain rate log-uniform in [1e-5, 1e-2] /s, barrier seeds
    0..count-1, and the 20 modes of the seed-0 configuration for every
    replica. The size, T and rate draws come from numpy's PCG64 seeded with
    2024 + seed_base."""
    rng = np.random.default_rng(2024 + seed_base)
    out = []
    for i in range(count):
        n = int(sizes[rng.integers(len(sizes))])
        T = float(rng.uniform(325.0, 585.0))
        rate = float(10 ** rng.uniform(-5, -2))
        p = shear64(seed_base + i, n, eng_rate=rate)
        p.mode_seed_set, p.mode_seed = 1, 0
        p.temperature = T
        p.t_temp = 1 / (p.trial_frequency * math.exp(-0.37 / (T * 1.380658e-23 / 1.60217733e-19)))
        if mixed:
            p.precision = api.PREC_MIXED
            p.solver = api.SOLVER_KERNEL
        out.append(p)
    return out
