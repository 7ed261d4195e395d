"""TEST INFRASTRUCTURE ONLY: build recipe for the oracle.

Builds
  oracle/_build/liboracle.so      the C restatement (stz_oracle.c), OpenMP
  oracle/_ref/ref2d_<NX>x<NY>_<L>  the reference's own STZ sources, compiled
                                   unmodified by path against the single-rank
                                   stand-ins in oracle/shim, with the event
                                   logger oracle/ref_wrap.c (only where the
                                   reference tree is present)

Usage: python oracle/build_oracle.py [--ref] [--ref-dir DIR] [--nx 64 --ny 64 --loading TENSION]

The reference's STZ source directory is taken from --ref-dir, else from the
environment variable STZ_REFERENCE_DIR, else from the default checkout
location below.
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF_DIR = "/root/reference/Mesoscale simulation STZ model"
REF_DIR = os.environ.get("STZ_REFERENCE_DIR", DEFAULT_REF_DIR)
REF_SOURCES = ["bmg.c", "io.c", "init.c", "elastic.c", "evolution.c"]
CFLAGS = ["-O2", "-std=gnu11", "-ffp-contract=off", "-fno-strict-aliasing"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle_lib(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle.so")
    srcs = [os.path.join(HERE, "stz_oracle.c"), os.path.join(HERE, "stz_oracle.h"),
            os.path.join(HERE, "..", "include", "stz_api.h")]
    if force or not _newer(out, srcs):
        _run(["gcc", "-shared", "-fPIC", "-fopenmp", *CFLAGS, "-Wall",
              os.path.join(HERE, "stz_oracle.c"), "-o", out, "-lm"])
    return out


def ref_available():
    return os.path.isdir(REF_DIR)


def build_ref2d(nx=64, ny=64, loading="TENSION", force=False, full_tensor=False, sf=None,
                no_subtract_error=False, no_sf_xtal_mro=True, material=None):
    """Compile the reference at an NX x NY grid; returns the binary path.
    full_tensor: also define FULL_TENSOR_RECORD, so that the reference's main
    writes Eps0 and Sigma of every print as .iout records (bmg.c:269-277).
    sf: the softening-direction scheme (an STZ_SF_* number) in place of
    bmgFlags.h's, through the stand-ins' STZ_SHIM_SF. loading: TENSION,
    SHEAR (the reference's main does not compile under COMPRESSION: its print
    test, bmg.c:181-187, opens a block under TENSION and SHEAR only).
    no_subtract_error: also define NO_SUBTRACT_ERROR
    (commented out in bmgFlags.h). no_sf_xtal_mro False: take bmgFlags.h's
    NO_SF_XTAL_MRO out (STZ_SHIM_XTAL_SF_OFF). material: HIGH_T_Vit1 or
    HIGH_T_PdNiP in place of bmgFlags.h's LOW_T (STZ_SHIM_NO_LOW_T)."""
    if not ref_available():
        raise FileNotFoundError("reference tree not present")
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "ref2d_%dx%d_%s%s%s" % (nx, ny, loading, "_ftr" if full_tensor else "",
                                                        "" if sf is None else "_sf%d" % sf) +
                       ("_nse" if no_subtract_error else "") + ("" if no_sf_xtal_mro else "_xsfoff") +
                       ("" if material is None else "_" + material))
    mine = [os.path.join(HERE, f) for f in ("ref_wrap.c", "stz_oracle.c", "stz_oracle.h",
                                            "shim/shim.c", "shim/mpi.h", "shim/fftw_mpi.h",
                                            "shim/gsl/gsl_rng.h", "shim/gsl/gsl_randist.h")]
    refs = [os.path.join(REF_DIR, f) for f in REF_SOURCES]
    if not force and _newer(out, mine + refs):
        return out
    defs = ["-DSTZ_SHIM_NX=%d" % nx, "-DSTZ_SHIM_NY=%d" % ny]
    if loading == "SHEAR":
        defs.append("-DSTZ_SHIM_LOAD_SHEAR")
    elif loading != "TENSION":
        raise ValueError("loading %r" % loading)
    if full_tensor:
        defs.append("-DFULL_TENSOR_RECORD")
    if sf is not None:
        defs.append("-DSTZ_SHIM_SF=%d" % sf)
    if no_subtract_error:
        defs.append("-DNO_SUBTRACT_ERROR")
    if not no_sf_xtal_mro:
        defs.append("-DSTZ_SHIM_XTAL_SF_OFF")
    if material is not None:
        if material not in ("HIGH_T_Vit1", "HIGH_T_PdNiP"):
            raise ValueError("material %r" % material)
        defs += ["-D" + material, "-DSTZ_SHIM_NO_LOW_T"]
    inc = ["-I", os.path.join(HERE, "shim"), "-I", REF_DIR]
    wraps = ["-Wl,--wrap=VoxelShearTransform", "-Wl,--wrap=KMC",
             "-Wl,--wrap=athermal_plasticity", "-Wl,--wrap=ActEnergy", "-Wl,--wrap=Free"]
    cmd = (["gcc", *CFLAGS, "-w", *defs, *inc] + refs +
           [os.path.join(HERE, "ref_wrap.c"), os.path.join(HERE, "shim", "shim.c"),
            os.path.join(HERE, "stz_oracle.c")] + wraps + ["-o", out, "-lm"])
    _run(cmd)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", action="store_true")
    ap.add_argument("--ref-dir", default=None, help="the reference's STZ source directory")
    ap.add_argument("--nx", type=int, default=64)
    ap.add_argument("--ny", type=int, default=64)
    ap.add_argument("--loading", default="TENSION")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    if a.ref_dir:
        global REF_DIR
        REF_DIR = a.ref_dir
    print(build_oracle_lib(a.force))
    if a.ref:
        print(build_ref2d(a.nx, a.ny, a.loading, a.force))


if __name__ == "__main__":
    sys.exit(main())
