"""The C-ABI library loads without a GPU, exports every entry point declared
in include/*.h, and its structs match the Python mirror (CPU only, no
compute calls)."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(inc, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*([a-zA-Z_][A-Za-z0-9_]*)\s*\(", src, re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "switch", "return", "sizeof"):
                names.add(name)
    return sorted(names)


def test_library_exports_every_declared_symbol(engine_lib):
    names = declared_functions()
    assert "stz_create" in names and "stz_run" in names
    missing = [n for n in names if not hasattr(engine_lib, n)]
    assert not missing, "declared but not exported: %s" % missing


@pytest.mark.parametrize("compiler", [["gcc", "-x", "c", "-std=c99"], ["gcc", "-x", "c", "-std=c11"],
                                      ["g++", "-x", "c++", "-std=c++11"]])
def test_headers_compile_standalone(compiler, tmp_path):
    """Each public header is self-contained plain C (and C++) with no warnings
    under -Wall -Wextra -pedantic: what a C, cgo or FFI binding includes."""
    import subprocess
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            src = tmp_path / ("use_" + f + ".src")
            src.write_text('#include "%s"\nint main(void) { return 0; }\n' % f)
            r = subprocess.run(compiler + ["-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", "-I", inc,
                                           str(src)], capture_output=True, text=True)
            assert r.returncode == 0, (f, r.stderr[-2000:])


def test_struct_sizes_match(engine_lib):
    from metallic_glasses_gb300 import api
    assert engine_lib.stz_sizeof(0) == C.sizeof(api.Params)
    assert engine_lib.stz_sizeof(1) == C.sizeof(api.Event)
    assert engine_lib.stz_sizeof(2) == C.sizeof(api.Scalars)


def test_input_file_parse_matches_reference_init(engine_lib, tmp_path):
    from metallic_glasses_gb300 import api, configs
    path = configs.write_input(str(tmp_path / "input"))
    p = api.params_from_input(path)
    E, nu = 69.46, 0.365 * 2          # LOW_T doubles nu (init.c:26)
    assert p.young == E and p.poisson == nu
    assert p.mu == E / (2 + 2 * nu)
    assert p.lambda_ == E * nu / (1 - nu * nu)
    assert p.q0_mean == 2.0 and p.seed == 123 and p.softening == 1 and p.print_period == 5
    assert p.strain_rate == 1e-4 and p.strain_increment == 1e-4 and p.end_strain == 0.06


def test_bad_input_reports_io_error(engine_lib, tmp_path):
    from metallic_glasses_gb300 import api
    bad = tmp_path / "input"
    bad.write_text("nothing useful\n")
    with pytest.raises(api.StzError) as ei:
        api.params_from_input(str(bad))
    assert ei.value.code == api.ERR_IO
    with pytest.raises(api.StzError):
        api.params_from_input(str(tmp_path / "missing"))


def test_missing_engine_library_fails_loudly(tmp_path):
    """Without its CUDA library the package raises instead of running any
    other implementation."""
    from metallic_glasses_gb300 import api
    with pytest.raises(RuntimeError, match="not built"):
        api.load_library(str(tmp_path / "libstz_gb300.so"))


def test_no_device_reports_an_error_status(engine_lib):
    """Creating a context where no GPU answers (this CPU host) returns an error
    status from the C ABI, not a host fallback."""
    from metallic_glasses_gb300 import api, configs
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(api.StzError):
        api.Engine(configs.ref2d(16, 16))


@pytest.mark.parametrize("cmd", ["kernel", "solve", "batch", "run", "ensemble"])
def test_timing_commands_parse(cmd):
    """Every documented timing subcommand parses its options."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, "-m", "metallic_glasses_gb300.timing", cmd, "--help"], cwd=ROOT,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "usage" in r.stdout, r.stderr[-1000:]


def _refused(p):
    from metallic_glasses_gb300 import api
    with pytest.raises(api.StzError) as ei:
        api.Engine(p)
    return ei.value.code, str(ei.value)


def test_create_refuses_bad_parameters_before_any_device_call(engine_lib):
    """stz_create checks the parameters before it touches a device, so on this
    host (no GPU) each unsupported or invalid combination is reported with its
    own status and message, never as a CUDA failure."""
    from metallic_glasses_gb300 import api, configs
    p = configs.shear64(0, 16)
    p.xmro_frac = 0.1
    code, msg = _refused(p)
    assert code == api.ERR_UNSUPPORTED and "MRO" in msg
    p = configs.shear64(0, 16)
    p.softening = 1
    assert _refused(p)[0] == api.ERR_UNSUPPORTED
    p = configs.ref2d(16, 16)
    p.precision = api.PREC_MIXED
    code, msg = _refused(p)
    assert code == api.ERR_UNSUPPORTED and "3D" in msg
    p = configs.shear64(0, 16)
    p.precision, p.solver = api.PREC_MIXED, api.SOLVER_FFT
    assert _refused(p)[0] == api.ERR_UNSUPPORTED
    p = configs.shear64(0, 16)
    p.precision, p.solver = api.PREC_MIXED, api.SOLVER_KERNEL
    p.n[2] = 18
    code, msg = _refused(p)
    assert code == api.ERR_UNSUPPORTED and "multiple of 4" in msg
    p = configs.shear64(0, 16)
    p.n[2] = 15
    code, msg = _refused(p)
    assert code == api.ERR_INVALID and "not supported" in msg
    p = configs.shear64(0, 16)
    p.mu = 0.0
    assert _refused(p)[0] == api.ERR_INVALID
