"""ctypes mirror of include/stz_api.h and a thin Python driver over it.

The product path is the CUDA library libstz_gb300.so built in-tree under
metallic_glasses_gb300/_lib/. Loading fails loudly when it is missing: there is
no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libstz_gb300.so")

MODES = 20
# status codes
OK, ERR_INVALID, ERR_CUDA, ERR_NAN, ERR_NO_EVENT, ERR_UNSUPPORTED, ERR_TIMEOUT, ERR_IO, ERR_NOMEM = range(9)
MODEL_REF2D, MODEL_GLOBAL3D = 0, 1
LOAD_TENSION, LOAD_SHEAR, LOAD_COMPRESSION, LOAD_STRESS = 0, 1, 2, 3
SF_LINEAR_FWD, SF_LINEAR_BWD, SF_EVEN, SF_SQUARE_FWD, SF_CUBIC_FWD, SF_GAUSS_FWD = range(6)
PREC_FP64, PREC_MIXED = 0, 1
SOLVER_FFT, SOLVER_KERNEL, SOLVER_AUTO = 0, 1, 2
DF_TRUNC_NORMAL, DF_CORRELATED = 0, 1
XX, YY, ZZ, YZ, XZ, XY = range(6)
EV_THERMAL, EV_ATHERMAL, EV_ELASTIC = 0, 1, 2
FIELD_SIGMA, FIELD_EPS0, FIELD_DF, FIELD_DEPS, FIELD_TLAST, FIELD_PERM_SOFT, FIELD_TEMP_SOFT, \
    FIELD_PREV_DEPS, FIELD_Q, FIELD_SDEV, FIELD_LAMBDA, FIELD_MU, FIELD_MRO = range(13)


class Params(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("n", C.c_int32 * 3),
        ("lambda_", C.c_double), ("mu", C.c_double), ("young", C.c_double), ("poisson", C.c_double),
        ("temperature", C.c_double), ("trial_frequency", C.c_double), ("voxel_volume", C.c_double),
        ("df_kind", C.c_int32),
        ("q0_mean", C.c_double), ("q0_sd", C.c_double), ("q0_trunc", C.c_double), ("q0_corr_len", C.c_double),
        ("gamma0", C.c_double),
        ("loading", C.c_int32), ("strain_rate", C.c_double), ("strain_increment", C.c_double),
        ("end_strain", C.c_double), ("applied_stress", C.c_double * 6),
        ("no_subtract_error", C.c_int32), ("shear_elastic_quirk", C.c_int32),
        ("softening", C.c_int32), ("sf_scheme", C.c_int32),
        ("perm_soft", C.c_double), ("temp_soft", C.c_double), ("perm_soft_cap", C.c_double), ("t_temp", C.c_double),
        ("xmro_frac", C.c_double), ("xq0amp", C.c_double), ("random_ratio", C.c_double),
        ("init_mro", C.c_int32), ("no_sf_xtal_mro", C.c_int32), ("perm_soft_mro", C.c_double), ("temp_soft_mro", C.c_double),
        ("mro_type", C.POINTER(C.c_int32)), ("mro_theta", C.POINTER(C.c_double)),
        ("print_period", C.c_int32), ("seed", C.c_uint64),
        ("precision", C.c_int32), ("solver", C.c_int32), ("resolve_period", C.c_int32), ("device", C.c_int32),
        ("log_capacity", C.c_int32), ("mode_seed_set", C.c_int32), ("mode_seed", C.c_int32),
        ("resolve_fp64", C.c_int32), ("sel_slack_shift", C.c_int32),
        ("main_pass_general", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


def set_mro_map(p, types, theta):
    """Give a REF2D Params the crystal-like MRO map of the reference's
    MROstructure.ms (init_mro 1): a type (0 glass, 1 six-fold, 2 two-fold,
    3 ten-fold) and an angle per site in site order. The arrays stay referenced
    by the Params object; the context reads them when it is created."""
    t = np.ascontiguousarray(types, dtype=np.int32)
    th = np.ascontiguousarray(theta, dtype=np.float64)
    if t.shape != th.shape or t.ndim != 1:
        raise ValueError("types and angles must be 1-D arrays of one length")
    p._mro_keep = (t, th)
    p.init_mro = 1
    p.mro_type = t.ctypes.data_as(C.POINTER(C.c_int32))
    p.mro_theta = th.ctypes.data_as(C.POINTER(C.c_double))
    return p


class Event(C.Structure):
    _fields_ = [("step", C.c_int64), ("site", C.c_int64), ("kind", C.c_int32), ("mode", C.c_int32),
                ("time", C.c_double), ("dt", C.c_double), ("q", C.c_double), ("total_rate", C.c_double),
                ("margin", C.c_double), ("draws", C.c_int32), ("reserved_ev", C.c_int32)]


class Scalars(C.Structure):
    _fields_ = [("time", C.c_double), ("eps_avg", C.c_double * 6), ("stress", C.c_double * 6),
                ("eps0_avg", C.c_double * 6), ("step", C.c_int64), ("kstep", C.c_int64), ("astep", C.c_int64),
                ("estep", C.c_int64), ("n_print", C.c_int64), ("n_events_logged", C.c_int64),
                ("stopped", C.c_int32), ("status", C.c_int32), ("stress_err_max", C.c_double),
                ("stress_err_rms", C.c_double), ("near_ties", C.c_int64), ("log_dropped", C.c_int64),
                ("n_resolves", C.c_int64), ("stress_err_rms_worst", C.c_double),
                ("stress_err_max_worst", C.c_double), ("rejections", C.c_int64), ("reserved", C.c_int64 * 1)]


EVENT_DTYPE = np.dtype([("step", np.int64), ("site", np.int64), ("kind", np.int32), ("mode", np.int32),
                        ("time", np.float64), ("dt", np.float64), ("q", np.float64), ("total_rate", np.float64),
                        ("margin", np.float64), ("draws", np.int32), ("reserved_ev", np.int32)])

_lib = None


def load_library(path=None):
    """Load libstz_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("the CUDA engine library %s is not built; run __graft_entry__.build()" % p)
    lib = C.CDLL(p)
    vp = C.c_void_p
    lib.stz_params_default.argtypes = [C.POINTER(Params), C.c_int32]
    lib.stz_params_from_input_file.argtypes = [C.POINTER(Params), C.c_char_p]
    lib.stz_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    lib.stz_destroy.argtypes = [vp]
    lib.stz_destroy.restype = None
    lib.stz_last_error.restype = C.c_char_p
    lib.stz_run.argtypes = [vp, C.c_int64, C.c_int64]
    lib.stz_solve.argtypes = [vp]
    lib.stz_get_scalars.argtypes = [vp, C.POINTER(Scalars)]
    lib.stz_get_events.argtypes = [vp, C.c_int64, vp, C.c_int64, C.POINTER(C.c_int64)]
    lib.stz_get_field.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int64]
    lib.stz_set_field.argtypes = [vp, C.c_int32, C.c_int32, vp, C.c_int64]
    lib.stz_set_mean_strain.argtypes = [vp, C.POINTER(C.c_double)]
    lib.stz_fft_schedule.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.stz_get_displacement.argtypes = [vp, C.c_void_p, C.c_int64]
    lib.stz_elastic_energy.argtypes = [vp, C.POINTER(C.c_double)]
    lib.stz_sync.argtypes = [vp]
    lib.stz_timer_start.argtypes = [vp]
    lib.stz_selftest_wait.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                      C.POINTER(C.c_int32)]
    lib.stz_timer_stop.argtypes = [vp, C.POINTER(C.c_float)]
    lib.stz_flush_l2.argtypes = [vp]
    lib.stz_kernel_launches.argtypes = [vp]
    lib.stz_kernel_launches.restype = C.c_int64
    lib.stz_kernel_time.argtypes = [vp, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.stz_transfer_bytes.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.stz_phase_times.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    lib.stz_solve_noalloc.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double,
                                      vp, C.POINTER(C.c_double), vp, vp]
    lib.stz_batch_create.argtypes = [C.POINTER(Params), C.c_int32, C.POINTER(vp)]
    lib.stz_batch_destroy.argtypes = [vp]
    lib.stz_batch_destroy.restype = None
    lib.stz_batch_run.argtypes = [vp, C.c_int64]
    lib.stz_batch_size.argtypes = [vp]
    lib.stz_batch_replica.argtypes = [vp, C.c_int32]
    lib.stz_batch_replica.restype = vp
    lib.stz_sizeof.argtypes = [C.c_int32]
    lib.stz_sizeof.restype = C.c_int64
    for name, s in ((0, Params), (1, Event), (2, Scalars)):
        if lib.stz_sizeof(name) != C.sizeof(s):
            raise RuntimeError("ABI mismatch for struct %d: C %d, Python %d" % (name, lib.stz_sizeof(name), C.sizeof(s)))
    if path is None:
        _lib = lib
    return lib


class StzError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("stz error %d: %s" % (code, msg))
        self.code = code


def _check(code):
    if code != OK:
        raise StzError(code, load_library().stz_last_error().decode(errors="replace"))


def default_params(model):
    p = Params()
    _check(load_library().stz_params_default(C.byref(p), model))
    return p


def params_from_input(path, base=None):
    p = base if base is not None else default_params(MODEL_REF2D)
    _check(load_library().stz_params_from_input_file(C.byref(p), path.encode()))
    return p


def scalars_dict(s):
    return {"time": s.time, "eps_avg": list(s.eps_avg), "stress": list(s.stress), "eps0_avg": list(s.eps0_avg),
            "step": s.step, "kstep": s.kstep, "astep": s.astep, "estep": s.estep, "n_print": s.n_print,
            "n_events_logged": s.n_events_logged, "stopped": s.stopped, "status": s.status,
            "stress_err_max": s.stress_err_max, "stress_err_rms": s.stress_err_rms, "near_ties": s.near_ties,
            "log_dropped": s.log_dropped, "n_resolves": s.n_resolves,
            "stress_err_rms_worst": s.stress_err_rms_worst, "stress_err_max_worst": s.stress_err_max_worst,
            "rejections": s.rejections}


class Engine:
    """One simulation context on one GPU (the device owns all state)."""

    def __init__(self, params):
        self.lib = load_library()
        self.params = params
        h = C.c_void_p()
        _check(self.lib.stz_create(C.byref(params), C.byref(h)))
        self.h = h
        self.N = params.n[0] * params.n[1] * params.n[2]
        self.nc = 3 if params.model == MODEL_REF2D else 6

    def close(self):
        if self.h and not getattr(self, "_borrowed", False):
            self.lib.stz_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, max_steps=0, max_events=0):
        _check(self.lib.stz_run(self.h, max_steps, max_events))

    def solve(self):
        _check(self.lib.stz_solve(self.h))

    def scalars(self):
        s = Scalars()
        _check(self.lib.stz_get_scalars(self.h, C.byref(s)))
        return scalars_dict(s)

    def events(self, first=0, count=None):
        total = self.scalars()["n_events_logged"]
        if count is None:
            count = max(0, total - first)
        out = np.zeros(count, dtype=EVENT_DTYPE)
        n = C.c_int64()
        _check(self.lib.stz_get_events(self.h, first, out.ctypes.data, count, C.byref(n)))
        return out[:n.value]

    def displacement(self):
        """The displacement field of the current eigenstrain, [dim][N] (dim = 2
        in 2D, axis order (j, i); 3 in 3D, axis order (2, 1, 0)), zero mean."""
        dim = 3 if self.params.n[0] > 1 else 2
        out = np.empty((dim, self.N), dtype=np.float64)
        _check(self.lib.stz_get_displacement(self.h, out.ctypes.data, dim * self.N))
        return out

    def field(self, which, comp=0):
        out = np.empty(self.N, dtype=np.float64)
        _check(self.lib.stz_get_field(self.h, which, comp, out.ctypes.data, self.N))
        return out

    def set_field(self, which, comp, values):
        v = np.ascontiguousarray(values, dtype=np.float64)
        _check(self.lib.stz_set_field(self.h, which, comp, v.ctypes.data, self.N))


    def fft_schedule(self):
        """(tiles, rejected, radix orders) of the tuned FFT plan."""
        t = (C.c_int32 * 4)()
        r = (C.c_int32 * 36)()
        _check(self.lib.stz_fft_schedule(self.h, t, r))
        orders = [[v for v in list(r)[12 * a:12 * a + 12] if v] for a in range(3)]
        return {"tiles": list(t)[:3], "rejected": t[3], "radices": orders}

    def set_mean_strain(self, eps_avg):
        """EpsAvg (Voigt, tensor shear) applied by the next solve."""
        v = (C.c_double * 6)(*(list(eps_avg) + [0.0] * (6 - len(eps_avg))))
        _check(self.lib.stz_set_mean_strain(self.h, v))
    def elastic_energy(self):
        e = C.c_double()
        _check(self.lib.stz_elastic_energy(self.h, C.byref(e)))
        return e.value

    def sync(self):
        _check(self.lib.stz_sync(self.h))

    def timer_start(self):
        _check(self.lib.stz_timer_start(self.h))

    def timer_stop(self):
        ms = C.c_float()
        _check(self.lib.stz_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def flush_l2(self):
        _check(self.lib.stz_flush_l2(self.h))

    def launches(self):
        return self.lib.stz_kernel_launches(self.h)

    def phase_times(self):
        a, b, n = C.c_double(), C.c_double(), C.c_int64()
        _check(self.lib.stz_phase_times(self.h, C.byref(a), C.byref(b), C.byref(n)))
        return a.value, b.value, n.value

    def transfer_bytes(self):
        a, b = C.c_int64(), C.c_int64()
        _check(self.lib.stz_transfer_bytes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    @classmethod
    def _borrow(cls, lib, handle, params):
        e = cls.__new__(cls)
        e.lib = lib
        e.params = params
        e.h = C.c_void_p(handle)
        e.N = params.n[0] * params.n[1] * params.n[2]
        e.nc = 3 if params.model == MODEL_REF2D else 6
        e._borrowed = True
        return e

    def kernel_time(self, steps=64, which=0):
        ms = C.c_double()
        n = C.c_int64(steps)
        _check(self.lib.stz_kernel_time(self.h, which, C.byref(ms), C.byref(n)))
        return ms.value, n.value


def selftest_wait(tries, device=0):
    """Run the bounded-wait self-test (stz_selftest_wait): returns (status,
    ms, kernel_tries); status is STZ_ERR_TIMEOUT when the wait ran out."""
    lib = load_library()
    st, ms, km = C.c_int32(), C.c_double(), C.c_int32()
    _check(lib.stz_selftest_wait(device, tries, C.byref(st), C.byref(ms), C.byref(km)))
    return st.value, ms.value, km.value


class Batch:
    """Independent replicas advanced together (mixed form, 3D)."""

    def __init__(self, params_list):
        self.lib = load_library()
        n = len(params_list)
        arr = (Params * n)(*params_list)
        self.params = list(params_list)
        h = C.c_void_p()
        _check(self.lib.stz_batch_create(arr, n, C.byref(h)))
        self.h = h
        self.replicas = [Engine._borrow(self.lib, self.lib.stz_batch_replica(h, i), params_list[i])
                         for i in range(n)]

    def run(self, events):
        _check(self.lib.stz_batch_run(self.h, events))

    def close(self):
        if self.h:
            for r in self.replicas:
                r.h = None
            self.lib.stz_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
