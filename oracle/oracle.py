"""Python binding of the CPU oracle (test infrastructure only).

Loads oracle/_build/libks_oracle.so (built by oracle/Makefile) and exposes the
same method names as kynema_sgf_gb300.Incflo so that parity tests can drive
both with identical calls.  Only the test-suite, the package smoke check and
the CPU-baseline leg of bench.py use this module; the product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def library_path():
    return os.path.join(_HERE, "_build", "libks_oracle.so")


def build(quiet=True):
    """Compile the oracle with its Makefile (g++ -O3 -fopenmp)."""
    r = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return library_path()


def load():
    global _LIB
    if _LIB is None:
        p = library_path()
        if not os.path.exists(p):
            build()
        lib = ctypes.CDLL(p)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.kso_create.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
        lib.kso_destroy.argtypes = [vp]
        lib.kso_destroy.restype = None
        lib.kso_last_error.argtypes = [vp]
        lib.kso_last_error.restype = ctypes.c_char_p
        for n in ["kso_init_data", "kso_step", "kso_pre_advance", "kso_prepare_time_step", "kso_update_mueff", "kso_compute_sources",
                  "kso_apply_corrector"]:
            getattr(lib, n).argtypes = [vp]
        lib.kso_evolve.argtypes = [vp, ip]
        lib.kso_compute_dt.argtypes = [vp, ctypes.POINTER(dp)]
        lib.kso_apply_predictor.argtypes = [vp, ip, ip]
        lib.kso_apply_projection.argtypes = [vp, dp, dp, ip]
        lib.kso_compute_divtau.argtypes = [vp, ip]
        lib.kso_predictor_rhs.argtypes = [vp, dp]
        lib.kso_improve_explicit_diffusion.argtypes = [vp]
        lib.kso_field_shape.argtypes = [vp, ctypes.c_char_p] + [ctypes.POINTER(ip)] * 4
        lib.kso_get_field.argtypes = [vp, ctypes.c_char_p, vp]
        lib.kso_set_field.argtypes = [vp, ctypes.c_char_p, vp]
        lib.kso_get_scalar.argtypes = [vp, ctypes.c_char_p]
        lib.kso_get_scalar.restype = dp
        lib.kso_set_scalar.argtypes = [vp, ctypes.c_char_p, dp]
        _LIB = lib
    return _LIB


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("oracle status %d: %s" % (code, msg))
        self.code = code


class Oracle:
    """CPU restatement driven with the Incflo method names."""

    def __init__(self, deck_text):
        self._lib = load()
        self._h = ctypes.c_void_p()
        rc = self._lib.kso_create(deck_text.encode(), ctypes.byref(self._h))
        if rc:
            msg = self._lib.kso_last_error(self._h).decode()
            self._lib.kso_destroy(self._h)
            self._h = None
            raise OracleError(rc, msg)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.kso_destroy(self._h)
            self._h = None

    def _check(self, rc, allow_done=False):
        if rc == 0 or (allow_done and rc == 7):
            return rc
        raise OracleError(rc, self._lib.kso_last_error(self._h).decode())

    def InitData(self):
        self._check(self._lib.kso_init_data(self._h))

    def compute_dt(self):
        dt = ctypes.c_double()
        self._check(self._lib.kso_compute_dt(self._h, ctypes.byref(dt)))
        return dt.value

    def pre_advance(self):
        self._check(self._lib.kso_pre_advance(self._h))

    def prepare_time_step(self):
        self._check(self._lib.kso_prepare_time_step(self._h))

    def ApplyPredictor(self, incremental_projection=False, fixed_point_iteration=0):
        self._check(self._lib.kso_apply_predictor(self._h, int(bool(incremental_projection)), int(fixed_point_iteration)))

    def ApplyCorrector(self):
        self._check(self._lib.kso_apply_corrector(self._h))

    def ApplyProjection(self, time, scaling_factor, incremental=False):
        self._check(self._lib.kso_apply_projection(self._h, float(time), float(scaling_factor), int(bool(incremental))))

    def step(self):
        return self._check(self._lib.kso_step(self._h), allow_done=True) == 0

    def Evolve(self, nsteps=1 << 30):
        self._check(self._lib.kso_evolve(self._h, int(nsteps)))

    def update_mueff(self):
        self._check(self._lib.kso_update_mueff(self._h))

    def compute_sources(self):
        self._check(self._lib.kso_compute_sources(self._h))

    def compute_divtau(self, use_new_state=False):
        self._check(self._lib.kso_compute_divtau(self._h, int(bool(use_new_state))))

    def predictor_rhs(self, fac=1.0):
        self._check(self._lib.kso_predictor_rhs(self._h, float(fac)))

    def improve_explicit_diffusion(self):
        self._check(self._lib.kso_improve_explicit_diffusion(self._h))

    def layout(self, name):
        v = [ctypes.c_int() for _ in range(4)]
        self._check(self._lib.kso_field_shape(self._h, name.encode(), *[ctypes.byref(x) for x in v]))
        return (v[0].value, v[3].value, v[2].value, v[1].value)

    def get_field(self, name):
        a = np.empty(self.layout(name), dtype=np.float64)
        self._check(self._lib.kso_get_field(self._h, name.encode(), a.ctypes.data_as(ctypes.c_void_p)))
        return a

    def set_field(self, name, value):
        a = np.ascontiguousarray(value, dtype=np.float64).reshape(self.layout(name))
        self._check(self._lib.kso_set_field(self._h, name.encode(), a.ctypes.data_as(ctypes.c_void_p)))

    def scalar(self, name):
        return self._lib.kso_get_scalar(self._h, name.encode())

    def set_scalar(self, name, value):
        self._check(self._lib.kso_set_scalar(self._h, name.encode(), float(value)))
