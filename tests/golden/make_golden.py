"""Generate the parity fixtures in tests/golden/ from the reference itself.

Runs the reference's own STZ sources (compiled unmodified against the
single-rank stand-ins of oracle/shim by oracle/build_oracle.py) in a scratch
directory and stores, per case:
  <case>.npz   X     int64 [K, 4]  one row per VoxelShearTransform call:
                                   (step, kind 0 thermal / 1 athermal, site, mode)
               S     float64 [M, 9] one row per driver step:
                                   (step, kind 0/1/2, time, EpsAvg[3], Stress[3])
               hdr   int64 [5]     (N, steps done, kstep, astep, estep)
               sc    float64 [7]   (time, EpsAvg[3], Stress[3]) at the end
               sigma, eps0  float64 [3, N]  final stress and eigenstrain
               tlast, perm_soft, temp_soft  float64 [N]
               deps_sum   float64 [3] sum over modes and sites of DEps0[m][c]
               xr         float64 [P, 2, N] the positions the reference's main
                                   wrote at P = 4 of its prints spread over the
                                   run (X1R/X2R files, "%lf" text: 6 decimals)
               xr_k       int64 [P]  their print numbers (the files' %03d)
               iout       float64 [P, 2, 3, N] (cases in IOUT_CASES) Eps0 and
                                   Sigma of the same prints as the reference's
                                   main writes them with FULL_TENSOR_RECORD
                                   (Strain_0c/Stress_0c_S%03d.iout, raw FP64)
             cases with crystal-like MRO sites (MRO_CASES) also:
               mro        int8 [N]   the MRO map (0 glass, 1 six-, 2 two-, 3 ten-fold)
               theta      float64 [N] its angles MROthe0
               mro_iout   int32 [N]  the reference's Initial_MROstructure_S000.iout
               deps_mro   float64 [20, 3, M] the mode eigenstrains of the M
                                   crystal-like sites (kept through transformations)
               q0_mro     float64 [20, M] their barriers at the end
               actq       float64 [K, 2] the reference's actQ.out (MRO type of
                                   the chosen site, its Q), one row per thermal event
               structure  (InitMRO 1 cases) the MROstructure.ms the run read
             cases of another softening-direction scheme (SF_CASES) also:
               sf         int64      the scheme (STZ_SF_*) the reference was built with
             cases built with NO_SUBTRACT_ERROR (SWITCH_CASES) also:
               nse        int64      1
             MRO cases built without NO_SF_XTAL_MRO (MRO_SWITCH_CASES) also:
               xsf        int64      0
             cases of a high-temperature material branch (MATERIAL_CASES) also:
               material   str        HIGH_T_Vit1 or HIGH_T_PdNiP
the reference's start-up printout under a few switch and input combinations
(print_*.txt: its PrintFlags and ParameterPrint blocks), and
the MT19937 known answers of the GSL conventions (mt19937_kat.npz), and
the reference's InhomogeneousStressSolver on a spatially varying medium
(inhom_32.npz, from inhom_ref.c: eps0, lam, mu, epsavg, sigma, stress).

Only this script reads the reference tree; tests read the .npz files.
Usage: python tests/golden/make_golden.py [case ...]   (all fixtures when no case is named)
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from metallic_glasses_gb300 import configs  # noqa: E402
from oracle.build_oracle import build_ref2d, build_oracle_lib  # noqa: E402

CASES = {
    # name: (nx, ny, loading, input overrides, thermal events)
    "ref2d_64_tension_s123": (64, 64, "TENSION", {"end": "0.5"}, 10000),
    "ref2d_32_shear_s7": (32, 32, "SHEAR", {"end": "0.5", "seed": "7"}, 150),
    # runs into the reference's SHEAR instability stop after its first avalanche
    "ref2d_32_shear_stop_s7": (32, 32, "SHEAR", {"end": "0.5", "seed": "7"}, 100000),
    "ref2d_32_tension_nosoft_s5": (32, 32, "TENSION", {"end": "0.5", "seed": "5", "soft": "0"}, 3000),
    # a non-square grid: site index i*NY + j and the FFT over unequal axes
    "ref2d_32x48_tension_s51": (32, 48, "TENSION", {"end": "0.5", "seed": "51"}, 1500),
}


# cases whose reference build also writes the .iout records of its prints
IOUT_CASES = {"ref2d_32_tension_nosoft_s5"}

# cases with crystal-like MRO sites: (nx, ny, loading, input overrides, thermal
# events); initmro 1 cases read a structure file drawn by mro_structure()
MRO_CASES = {
    "ref2d_32_mro_s11": (32, 32, "TENSION", {"end": "0.5", "seed": "11", "xfrac": "0.15", "xq0": "1.8"}, 3000),
    "ref2d_32_mrofile_s13": (32, 32, "TENSION", {"end": "0.5", "seed": "13", "initmro": "1", "xq0": "2.2"}, 3000),
}


# cases of the other softening-direction schemes of ActEnergy (init.c:590-642;
# bmgFlags.h ships SF_SQUARE_FWD): (nx, ny, loading, input overrides, thermal
# events, STZ_SF_* number)
SF_CASES = {
    "ref2d_32_sf_linear_fwd_s21": (32, 32, "TENSION", {"end": "0.5", "seed": "21"}, 1500, 0),
    "ref2d_32_sf_linear_bwd_s22": (32, 32, "TENSION", {"end": "0.5", "seed": "22"}, 1500, 1),
    "ref2d_32_sf_even_s23": (32, 32, "TENSION", {"end": "0.5", "seed": "23"}, 1500, 2),
    "ref2d_32_sf_cubic_fwd_s24": (32, 32, "TENSION", {"end": "0.5", "seed": "24"}, 1500, 4),
    "ref2d_32_sf_gauss_fwd_s25": (32, 32, "TENSION", {"end": "0.5", "seed": "25"}, 1500, 5),
}


# the athermal and loading error correction switched off (NO_SUBTRACT_ERROR,
# evolution.c:91-95, 262-310): (nx, ny, loading, input overrides, thermal
# events, NO_SUBTRACT_ERROR). The reference's main does not compile under
# COMPRESSION (its print test, bmg.c:181-187, opens a block under TENSION and
# SHEAR only), so that switch has no fixture.
SWITCH_CASES = {
    "ref2d_32_tension_nse_s32": (32, 32, "TENSION", {"end": "0.5", "seed": "32"}, 1500, True),
    "ref2d_32_shear_nse_s33": (32, 32, "SHEAR", {"end": "0.5", "seed": "33"}, 1500, True),
}


# crystal-like sites with bmgFlags.h's NO_SF_XTAL_MRO taken out (ActEnergy
# then leaves their direction modifier and softening unscaled, init.c:645-668)
MRO_SWITCH_CASES = {
    "ref2d_32_mro_xsfoff_s11": (32, 32, "TENSION", {"end": "0.5", "seed": "11", "xfrac": "0.15", "xq0": "1.8"},
                                3000),
}


# the high-temperature material branches of Init() in place of LOW_T
# (init.c:28-42): (nx, ny, loading, input overrides, thermal events, branch)
MATERIAL_CASES = {
    "ref2d_32_vit1_s41": (32, 32, "TENSION", {"end": "0.5", "seed": "41"}, 1500, "HIGH_T_Vit1"),
    "ref2d_32_pdnip_s42": (32, 32, "TENSION", {"end": "0.5", "seed": "42"}, 1500, "HIGH_T_PdNiP"),
}


# the reference's start-up printout (PrintFlags, ParameterPrint; io.c:103-135, 374-434)
# under a few switch and input combinations: (loading, material, input overrides)
PRINT_CASES = {
    "print_tension": ("TENSION", None, {}),
    "print_shear_nosoft": ("SHEAR", None, {"soft": "0", "end": "0.1"}),
    "print_vit1": ("TENSION", "HIGH_T_Vit1", {"rate": "5e-5"}),
}


def print_case(name, loading, material, overrides):
    """Runs the reference for one thermal event and keeps its flag block and
    parameter block as <name>.txt."""
    exe = build_ref2d(32, 32, loading, material=material)
    d = tempfile.mkdtemp(prefix="stz_ref_print_")
    configs.write_input(os.path.join(d, "input"), **overrides)
    env = dict(os.environ, STZ_REF_LOG=os.path.join(d, "log.txt"), STZ_REF_MAX_EVENTS="1",
               STZ_REF_DUMP=os.path.join(d, "dump.bin"))
    out = subprocess.run([exe], cwd=d, env=env, capture_output=True, text=True, check=True).stdout
    lines = out.split("\n")
    i = lines.index("Active flags in bmgFlags.h:")
    j = i + 1
    while lines[j].startswith("#define"):
        j += 1
    k = lines.index("Simulation Geometry:") - 1
    m = next(n for n in range(k, len(lines)) if lines[n].startswith("Ratio for generating residual stress:"))
    text = "\n".join(lines[i:j] + lines[k:m + 1]) + "\n"
    with open(os.path.join(HERE, name + ".txt"), "w") as f:
        f.write(text)
    print(name, "->", name + ".txt")


def mro_structure(nx, ny, seed=2024):
    """A structure file in the reference's MROstructure.ms layout (one line
    per site in site order: 1-based i, 1-based j, type, angle): types 0/1/2/3
    with probabilities 0.6/0.15/0.1/0.15, angles uniform on [-pi/2, pi/2)."""
    rs = np.random.default_rng(seed)
    t = rs.choice(4, size=nx * ny, p=[0.6, 0.15, 0.1, 0.15])
    th = rs.uniform(-np.pi / 2, np.pi / 2, size=nx * ny)
    lines = ["%d %d %d %.17g" % (i + 1, j + 1, t[i * ny + j], th[i * ny + j]) for i in range(nx) for j in range(ny)]
    return "\n".join(lines) + "\n"


def run_case(name, nx, ny, loading, overrides, events, mro=False, sf=None, nse=False, xsf=True, material=None):
    ftr = name in IOUT_CASES
    exe = build_ref2d(nx, ny, loading, full_tensor=ftr, sf=sf, no_subtract_error=nse, no_sf_xtal_mro=xsf,
                      material=material)
    d = tempfile.mkdtemp(prefix="stz_ref_")
    configs.write_input(os.path.join(d, "input"), **overrides)
    structure = None
    if overrides.get("initmro") == "1":
        structure = mro_structure(nx, ny)
        with open(os.path.join(d, "MROstructure.ms"), "w") as f:
            f.write(structure)
    env = dict(os.environ, STZ_REF_LOG=os.path.join(d, "log.txt"), STZ_REF_MAX_EVENTS=str(events),
               STZ_REF_DUMP=os.path.join(d, "dump.bin"))
    subprocess.run([exe], cwd=d, env=env, stdout=subprocess.DEVNULL, check=True)
    X, S = [], []
    for line in open(os.path.join(d, "log.txt")):
        t = line.split()
        if t[0] == "X":
            X.append([int(v) for v in t[1:5]])
        else:
            S.append([float(v) for v in t[1:]])
    raw = open(os.path.join(d, "dump.bin"), "rb").read()
    hdr = np.frombuffer(raw[:40], np.int64).copy()
    sc = np.frombuffer(raw[40:96], np.float64).copy()
    N = int(hdr[0])
    arr = np.frombuffer(raw[96:], np.float64)
    off = 0

    def take(k):
        nonlocal off
        v = arr[off:off + k].copy()
        off += k
        return v

    sigma = take(3 * N).reshape(3, N)
    eps0 = take(3 * N).reshape(3, N)
    deps = take(60 * N).reshape(20, 3, N)
    q0 = take(20 * N).reshape(20, N)
    tlast = take(N)
    perm = take(N)
    temp = take(N)
    take(3 * N)  # PreDEps0 of the last transformations
    mro_map = take(N).astype(np.int8)
    theta = take(N)
    # the reference main's print files X1R%03d_P00.out / X2R%03d_P00.out:
    # four prints spread over the run
    n_prints = 0
    while os.path.exists(os.path.join(d, "X1R%03d_P00.out" % (n_prints + 1))):
        n_prints += 1
    xr_k = sorted({max(1, n_prints // 8), max(1, n_prints // 3), max(1, 2 * n_prints // 3), n_prints})
    xr = [[np.loadtxt(os.path.join(d, "X%dR%03d_P00.out" % (a, k))).reshape(-1) for a in (1, 2)] for k in xr_k]
    xr = np.array(xr, np.float64).reshape(len(xr_k), 2, N)
    extra = {}
    if ftr:
        extra["iout"] = np.array([[[np.fromfile(os.path.join(d, "%s_%02d_S%03d.iout" % (w, c + 1, k)), np.float64)
                                    for c in range(3)] for w in ("Strain", "Stress")] for k in xr_k])
    if mro:
        sel = np.nonzero(mro_map)[0]
        extra.update(mro=mro_map, theta=theta, deps_mro=deps[:, :, sel], q0_mro=q0[:, sel],
                     mro_iout=np.fromfile(os.path.join(d, "Initial_MROstructure_S000.iout"), np.int32),
                     actq=np.loadtxt(os.path.join(d, "actQ.out"), ndmin=2))
        if structure is not None:
            extra["structure"] = structure
    if sf is not None:
        extra["sf"] = np.int64(sf)
    if nse:
        extra["nse"] = np.int64(1)
    if not xsf:
        extra["xsf"] = np.int64(0)
    if material is not None:
        extra["material"] = material
    out = os.path.join(HERE, name + ".npz")
    S = np.array(S, np.float64)
    # per-step time for every step; mean strain and stress for every 10th
    np.savez_compressed(out, X=np.array(X, np.int64), S=S[:, :3], S10=S[::10], hdr=hdr, sc=sc, sigma=sigma,
                        eps0=eps0, tlast=tlast, perm_soft=perm, temp_soft=temp, deps_sum=deps.sum(axis=(0, 2)),
                        nx=nx, ny=ny, loading=loading, overrides=repr(overrides), events=events, xr=xr,
                        xr_k=np.array(xr_k, np.int64), **extra)
    print(name, "transforms", len(X), "steps", len(S), "hdr", hdr, "->", out)


def mt_kat():
    """MT19937 known answers: C++ std::mt19937 (the same generator and seeding
    recurrence) for seed 5489 gives 4123659995 as its 10000th output; the
    first outputs for seeds 123 and 4357 come from g++'s std::mt19937."""
    src = r'''
#include <random>
#include <cstdio>
int main(){ std::mt19937 a(5489u); unsigned v=0; for(int i=0;i<10000;i++) v=a(); printf("%u\n", v);
 for (unsigned s : {123u, 4357u}) { std::mt19937 g(s); for(int i=0;i<8;i++) printf("%u ", (unsigned)g()); printf("\n"); }
 std::mt19937 g(123u); for(int i=0;i<700;i++) g(); for(int i=0;i<4;i++) printf("%u ", (unsigned)g()); printf("\n"); }
'''
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "k.cpp"), "w") as f:
        f.write(src)
    subprocess.run(["g++", "-O1", "-o", os.path.join(d, "k"), os.path.join(d, "k.cpp")], check=True)
    outp = subprocess.run([os.path.join(d, "k")], capture_output=True, text=True, check=True).stdout.split("\n")
    v10000 = int(outp[0])
    s123 = [int(x) for x in outp[1].split()]
    s4357 = [int(x) for x in outp[2].split()]
    s123_700 = [int(x) for x in outp[3].split()]
    np.savez(os.path.join(HERE, "mt19937_kat.npz"), v10000=v10000, s123=np.array(s123, np.uint32),
             s4357=np.array(s4357, np.uint32), s123_after700=np.array(s123_700, np.uint32))
    print("mt19937 kat", v10000, s123[:2])


def inhom_case(nx=32, ny=32):
    """The reference's polarisation solver on a medium whose Lame moduli vary
    between 0.7 and 1.3 of the uniform ones (inhom_ref.c is the main; the
    reference's io.c, init.c, elastic.c, evolution.c compile unmodified against
    the stand-ins of oracle/shim)."""
    from oracle.build_oracle import HERE as OR, REF_DIR, CFLAGS
    d = tempfile.mkdtemp(prefix="stz_inhom_")
    exe = os.path.join(d, "inhom_ref")
    srcs = [os.path.join(REF_DIR, f) for f in ("io.c", "init.c", "elastic.c", "evolution.c")]
    cmd = (["gcc", *CFLAGS, "-w", "-DSTZ_SHIM_NX=%d" % nx, "-DSTZ_SHIM_NY=%d" % ny, "-I", os.path.join(OR, "shim"),
            "-I", REF_DIR] + srcs + [os.path.join(HERE, "inhom_ref.c"), os.path.join(OR, "shim", "shim.c"),
                                     os.path.join(OR, "stz_oracle.c"), "-o", exe, "-lm"])
    subprocess.run(cmd, check=True)
    configs.write_input(os.path.join(d, "input"), end="0.5", seed="5", soft="0")
    subprocess.run([exe], cwd=d, stdout=subprocess.DEVNULL, check=True)
    raw = open(os.path.join(d, "inhom.bin"), "rb").read()
    NX, NY = np.frombuffer(raw[:16], np.int64)
    N = int(NX * NY)
    sc = np.frombuffer(raw[16:80], np.float64)
    arr = np.frombuffer(raw[80:], np.float64)
    eps0, lam, mu, sigma = arr[:3 * N].reshape(3, N), arr[3 * N:4 * N], arr[4 * N:5 * N], arr[5 * N:8 * N].reshape(3, N)
    out = os.path.join(HERE, "inhom_%d.npz" % nx)
    np.savez_compressed(out, nx=nx, ny=ny, lame=sc[:2], epsavg=sc[2:5], stress=sc[5:8], eps0=eps0, lam=lam, mu=mu,
                        sigma=sigma)
    print("inhom", nx, ny, "stress", sc[5:8], "->", out)


if __name__ == "__main__":
    build_oracle_lib()
    only = sys.argv[1:]
    if not only:
        inhom_case()
        mt_kat()
    for name, (nx, ny, loading, ov, ev) in CASES.items():
        if not only or name in only:
            run_case(name, nx, ny, loading, ov, ev)
    for name, (nx, ny, loading, ov, ev) in MRO_CASES.items():
        if not only or name in only:
            run_case(name, nx, ny, loading, ov, ev, mro=True)
    for name, (nx, ny, loading, ov, ev, sf) in SF_CASES.items():
        if not only or name in only:
            run_case(name, nx, ny, loading, ov, ev, sf=sf)
    for name, (nx, ny, loading, ov, ev, nse) in SWITCH_CASES.items():
        if not only or name in only:
            run_case(name, nx, ny, loading, ov, ev, nse=nse)
    for name, (nx, ny, loading, ov, ev) in MRO_SWITCH_CASES.items():
        if not only or name in only:
            run_case(name, nx, ny, loading, ov, ev, mro=True, xsf=False)
    for name, (nx, ny, loading, ov, ev, mat) in MATERIAL_CASES.items():
        if not only or name in only:
            run_case(name, nx, ny, loading, ov, ev, material=mat)
    for name, (loading, mat, ov) in PRINT_CASES.items():
        if not only or name in only:
            print_case(name, loading, mat, ov)
