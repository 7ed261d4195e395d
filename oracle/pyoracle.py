"""TEST INFRASTRUCTURE ONLY: ctypes binding of the C oracle (liboracle.so).

Imported by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, never by the product.
"""
import ctypes as C
import os

import numpy as np

from metallic_glasses_gb300.api import EVENT_DTYPE, Scalars, Params, scalars_dict

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from oracle.build_oracle import build_oracle_lib
            build_oracle_lib()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.or_create.argtypes = [C.POINTER(Params), C.POINTER(C.c_int)]
        L.or_create.restype = vp
        L.or_destroy.argtypes = [vp]
        L.or_destroy.restype = None
        L.or_run.argtypes = [vp, C.c_int64, C.c_int64]
        L.or_solve.argtypes = [vp]
        L.or_get_scalars.argtypes = [vp, C.POINTER(Scalars)]
        L.or_num_events.argtypes = [vp]
        L.or_num_events.restype = C.c_int64
        L.or_get_events.argtypes = [vp, C.c_int64, vp, C.c_int64, C.POINTER(C.c_int64)]
        L.or_get_field.argtypes = [vp, C.c_int, C.c_int, vp, C.c_int64]
        L.or_set_field.argtypes = [vp, C.c_int, C.c_int, vp, C.c_int64]
        L.or_elastic_energy.argtypes = [vp, C.POINTER(C.c_double)]
        L.or_fft3.argtypes = [C.c_int, C.c_int, C.c_int, vp, C.c_int]
        L.or_rng_seed.argtypes = [vp, C.c_ulong]
        L.or_rng_seed.restype = None
        L.or_rng_get.argtypes = [vp]
        L.or_rng_get.restype = C.c_uint32
        L.or_rng_uniform.argtypes = [vp]
        L.or_rng_uniform.restype = C.c_double
        L.or_ran_gaussian.argtypes = [vp, C.c_double]
        L.or_ran_gaussian.restype = C.c_double
        L.or_set_mean_strain.argtypes = [vp, C.POINTER(C.c_double)]
        L.or_force_path.argtypes = [vp, vp, vp, vp, C.c_int64]
        L.or_get_checks.argtypes = [vp, vp, C.c_int64]
        L.or_get_checks.restype = C.c_int64
        L.or_set_bounded_selection.argtypes = [vp, C.c_int]
        L.or_params_default.argtypes = [C.POINTER(Params), C.c_int]
        L.or_params_from_input_file.argtypes = [C.POINTER(Params), C.c_char_p]
        L.or_threads.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        L.or_set_threads.restype = None
        _lib = L
    return _lib


class Rng:
    """The oracle's GSL-convention MT19937."""

    def __init__(self, seed):
        self.buf = C.create_string_buffer(624 * 4 + 8)
        lib().or_rng_seed(self.buf, seed)

    def get(self):
        return lib().or_rng_get(self.buf)

    def uniform(self):
        return lib().or_rng_uniform(self.buf)

    def gaussian(self, sigma=1.0):
        return lib().or_ran_gaussian(self.buf, sigma)


def default_params(model):
    """Parameters of a model from the oracle's own defaults (no engine library)."""
    p = Params()
    st = lib().or_params_default(C.byref(p), model)
    if st != 0:
        raise ValueError("oracle: no defaults for model %d" % model)
    return p


def params_from_input(path, base=None):
    """A reference-format input file through the oracle's parser (no engine library)."""
    p = base if base is not None else default_params(0)
    st = lib().or_params_from_input_file(C.byref(p), path.encode())
    if st != 0:
        raise ValueError("oracle: cannot read input file %s (status %d)" % (path, st))
    return p


def fft3(a, sign):
    """Unnormalised complex DFT of a 3D complex array (sign -1 forward)."""
    b = np.ascontiguousarray(a, dtype=np.complex128).copy()
    n0, n1, n2 = b.shape
    st = lib().or_fft3(n0, n1, n2, b.ctypes.data, sign)
    if st != 0:
        raise ValueError("oracle fft: unsupported extents %s" % (b.shape,))
    return b


class Model:
    def __init__(self, params):
        st = C.c_int()
        self.h = lib().or_create(C.byref(params), C.byref(st))
        if not self.h:
            raise RuntimeError("oracle create failed with status %d" % st.value)
        self.N = params.n[0] * params.n[1] * params.n[2]
        self.nc = 3 if params.model == 0 else 6

    def close(self):
        if self.h:
            lib().or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, max_steps=0, max_events=0):
        st = lib().or_run(self.h, max_steps, max_events)
        if st != 0:
            raise RuntimeError("oracle run failed with status %d" % st)

    def solve(self):
        lib().or_solve(self.h)

    def scalars(self):
        s = Scalars()
        lib().or_get_scalars(self.h, C.byref(s))
        return scalars_dict(s)

    def events(self):
        n = lib().or_num_events(self.h)
        out = np.zeros(n, dtype=EVENT_DTYPE)
        got = C.c_int64()
        lib().or_get_events(self.h, 0, out.ctypes.data, n, C.byref(got))
        return out

    def field(self, which, comp=0):
        out = np.empty(self.N)
        if lib().or_get_field(self.h, which, comp, out.ctypes.data, self.N) != 0:
            raise ValueError("bad field %d/%d" % (which, comp))
        return out

    def set_field(self, which, comp, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        if lib().or_set_field(self.h, which, comp, v.ctypes.data, self.N) != 0:
            raise ValueError("bad field %d/%d" % (which, comp))

    def set_mean_strain(self, eps_avg):
        v = (C.c_double * 6)(*([float(x) for x in eps_avg] + [0.0] * (6 - len(eps_avg))))
        lib().or_set_mean_strain(self.h, v)

    def force_path(self, sites, modes, draws=None):
        """The next len(sites) thermal events take these (site, mode) pairs,
        each after discarding draws[k] - 1 generator words."""
        s = np.ascontiguousarray(sites, dtype=np.int64)
        mo = np.ascontiguousarray(modes, dtype=np.int32)
        d = np.ones(len(s), np.int32) if draws is None else np.ascontiguousarray(draws, dtype=np.int32)
        self._force = (s, mo, d)
        st = lib().or_force_path(self.h, s.ctypes.data, mo.ctypes.data, d.ctypes.data, len(s))
        if st != 0:
            raise ValueError("oracle: bad forced path (status %d)" % st)

    def checks(self):
        """Per forced event: own site, own mode, dice, the forced element's
        cumulative interval [lo, hi] (fractions of R), R and the words the
        own choice took."""
        n = len(self._force[0]) if getattr(self, "_force", None) else 0
        out = np.zeros((max(n, 1), 7))
        k = lib().or_get_checks(self.h, out.ctypes.data, n)
        return out[:k]

    def set_bounded_selection(self, slack):
        """Own choices by line bounds of slack 2^-slack with rejection."""
        if lib().or_set_bounded_selection(self.h, int(slack)) != 0:
            raise ValueError("oracle: bad slack %r" % slack)

    def elastic_energy(self):
        e = C.c_double()
        lib().or_elastic_energy(self.h, C.byref(e))
        return e.value


def threads():
    return lib().or_threads()


def set_threads(n):
    """Threads of the oracle's parallel loops from now on."""
    lib().or_set_threads(int(n))
