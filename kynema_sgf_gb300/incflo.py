"""ctypes binding of include/ks.h with the reference's incflo method names.

``Incflo`` mirrors ``class incflo`` (src/incflo.H:51-233 in Kynema-SGF):
``InitData``, ``Evolve``, ``advance``, ``ApplyPredictor``, ``ApplyCorrector``,
``ApplyProjection`` and ``compute_dt`` keep their names, argument meaning and
their failure behaviour (an invalid deck raises, ``ApplyCorrector`` on the
Godunov path raises as unsupported).  Field access by repository name
(``velocity``, ``p``, ``gp``, ...) replaces ``FieldRepo::get_field``.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

STATUS = {
    0: "KS_OK", 1: "KS_ERR_DECK", 2: "KS_ERR_UNSUPPORTED", 3: "KS_ERR_NOT_CONVERGED", 4: "KS_ERR_NONFINITE",
    5: "KS_ERR_OOM", 6: "KS_ERR_ARG", 7: "KS_DONE", 8: "KS_ERR_CUDA",
}
KS_DONE = 7
KS_HOST, KS_DEVICE = 0, 1

FIELDS = ["velocity", "velocity_old", "gp", "p", "src_term", "forces", "diff_term", "conv_term", "conv_term_old", "velocity_mueff",
          "u_mac", "v_mac", "w_mac", "actuator_src_term", "velocity_adjoint", "gp_adjoint", "temperature", "temperature_old",
          "temperature_mueff", "temperature_conv_term", "temperature_diff_term", "wall_grad"]

# every symbol declared in include/ks.h
SYMBOLS = ["ks_create", "ks_destroy", "ks_last_error", "ks_init_data", "ks_compute_dt", "ks_pre_advance",
           "ks_prepare_time_step", "ks_advance", "ks_apply_predictor", "ks_apply_corrector", "ks_apply_projection",
           "ks_evolve", "ks_step", "ks_field_layout", "ks_get_field", "ks_set_field", "ks_get_scalar",
           "ks_last_solver_stats", "ks_set_precision", "ks_synchronize", "ks_kernel_launches", "ks_get_stream",
           "ks_profile_kernels", "ks_profile_report", "ks_divtau_noalloc", "ks_fma_peak", "ks_set_objective_box",
           "ks_objective", "ks_adjoint_step", "ks_adjoint_run", "ks_get_ct_gradient", "ks_adjoint_reset",
           "ks_set_disk_ct", "ks_checkpoint_cost", "ks_write_plotfile", "ks_write_checkpoint", "ks_read_checkpoint",
           "ks_write_outputs", "ks_plotfile_write_host"]


class KsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class _Layout(ctypes.Structure):
    _fields_ = [("ncomp", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int)]


class _Stats(ctypes.Structure):
    _fields_ = [("mac_iterations", ctypes.c_int), ("mac_initial_residual", ctypes.c_double),
                ("mac_final_residual", ctypes.c_double), ("nodal_iterations", ctypes.c_int),
                ("nodal_initial_residual", ctypes.c_double), ("nodal_final_residual", ctypes.c_double)]


def library_path():
    return os.path.join(_HERE, "_build", "libks.so")


def build_library(verbose=False):
    from . import build as _b
    return _b.build(verbose=verbose)


def load_library(path=None):
    """Load libks.so (raises if it was not built)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or library_path()
    if not os.path.exists(p):
        raise KsError(8, "CUDA extension %s is missing: run kynema_sgf_gb300.build_library()" % p)
    lib = ctypes.CDLL(p)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.ks_create.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp)]
    lib.ks_destroy.argtypes = [vp]
    lib.ks_destroy.restype = None
    lib.ks_last_error.argtypes = [vp]
    lib.ks_last_error.restype = ctypes.c_char_p
    for name in ["ks_init_data", "ks_pre_advance", "ks_prepare_time_step", "ks_apply_corrector", "ks_synchronize", "ks_step"]:
        getattr(lib, name).argtypes = [vp]
    lib.ks_compute_dt.argtypes = [vp, ctypes.POINTER(dp)]
    lib.ks_advance.argtypes = [vp, ip]
    lib.ks_apply_predictor.argtypes = [vp, ip, ip]
    lib.ks_apply_projection.argtypes = [vp, dp, dp, ip]
    lib.ks_evolve.argtypes = [vp, ip]
    lib.ks_field_layout.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(_Layout)]
    lib.ks_get_field.argtypes = [vp, ctypes.c_char_p, vp, ip]
    lib.ks_set_field.argtypes = [vp, ctypes.c_char_p, vp, ip]
    lib.ks_get_scalar.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(dp)]
    lib.ks_last_solver_stats.argtypes = [vp, ctypes.POINTER(_Stats)]
    lib.ks_set_precision.argtypes = [vp, ip]
    lib.ks_kernel_launches.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
    lib.ks_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    lib.ks_profile_kernels.argtypes = [vp, ctypes.c_char_p]
    lib.ks_profile_report.argtypes = [vp, ctypes.c_char_p, ctypes.c_longlong]
    lib.ks_profile_report.restype = ctypes.c_longlong
    lib.ks_divtau_noalloc.argtypes = [vp, vp, vp, vp, ip, ip, ip, dp, dp, dp, ip, ip, vp]
    lib.ks_fma_peak.argtypes = [ip, ctypes.POINTER(dp)]
    d3 = ctypes.POINTER(dp)
    lib.ks_set_objective_box.argtypes = [vp, d3, d3]
    lib.ks_objective.argtypes = [vp, ip, d3]
    lib.ks_adjoint_step.argtypes = [vp]
    lib.ks_adjoint_run.argtypes = [vp, ip, ip, d3]
    lib.ks_get_ct_gradient.argtypes = [vp, d3, ip]
    lib.ks_adjoint_reset.argtypes = [vp]
    lib.ks_set_disk_ct.argtypes = [vp, d3, ip]
    lib.ks_checkpoint_cost.argtypes = [ip, ip, ctypes.POINTER(ctypes.c_longlong)]
    for name in ("ks_write_plotfile", "ks_write_checkpoint", "ks_read_checkpoint"):
        getattr(lib, name).argtypes = [vp, ctypes.c_char_p]
    lib.ks_write_outputs.argtypes = [vp, ip]
    i3 = ctypes.POINTER(ctypes.c_int)
    lib.ks_plotfile_write_host.argtypes = [ctypes.c_char_p, ip, ctypes.POINTER(ctypes.c_char_p), i3, d3, d3, dp, ip, vp]
    if path is None:
        _LIB = lib
    return lib


def fma_peak(fp64=True):
    """Measured FMA throughput of the current device, GFLOP/s."""
    lib = load_library()
    v = ctypes.c_double()
    rc = lib.ks_fma_peak(int(bool(fp64)), ctypes.byref(v))
    if rc != 0:
        raise KsError(rc, "ks_fma_peak failed")
    return v.value


def checkpoint_cost(nsteps, snapshots):
    """Forward steps a binomial schedule adds to reverse ``nsteps`` steps with
    ``snapshots`` checkpoint slots (host-only computation)."""
    lib = load_library()
    v = ctypes.c_longlong()
    rc = lib.ks_checkpoint_cost(int(nsteps), int(snapshots), ctypes.byref(v))
    if rc != 0:
        raise KsError(rc, "ks_checkpoint_cost failed")
    return v.value


def write_plotfile_host(path, names, data, prob_lo, prob_hi, time=0.0, step=0):
    """AMReX plot file from host data (no device): ``data`` is (nvars, nz, ny, nx)."""
    lib = load_library()
    a = np.ascontiguousarray(data, dtype=np.float64)
    nv, nz, ny, nx = a.shape
    if nv != len(names):
        raise ValueError("one name per variable")
    nm = (ctypes.c_char_p * nv)(*[n.encode() for n in names])
    n3 = (ctypes.c_int * 3)(nx, ny, nz)
    lo = (ctypes.c_double * 3)(*[float(x) for x in prob_lo])
    hi = (ctypes.c_double * 3)(*[float(x) for x in prob_hi])
    rc = lib.ks_plotfile_write_host(str(path).encode(), nv, nm, n3, lo, hi, float(time), int(step), a.ctypes.data)
    if rc != 0:
        raise KsError(rc, "ks_plotfile_write_host failed")


class Incflo:
    """One simulation on cuda:0 driven through the C ABI."""

    def __init__(self, deck_text, lib=None):
        self._lib = lib or load_library()
        self._h = ctypes.c_void_p()
        rc = self._lib.ks_create(deck_text.encode(), ctypes.byref(self._h))
        if rc != 0:
            msg = self._lib.ks_last_error(self._h).decode() if self._h else "ks_create failed"
            self._lib.ks_destroy(self._h)
            self._h = None
            raise KsError(rc, msg)

    def _check(self, rc, allow_done=False):
        if rc == 0 or (allow_done and rc == KS_DONE):
            return rc
        raise KsError(rc, self._lib.ks_last_error(self._h).decode())

    def close(self):
        if self._h:
            self._lib.ks_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- reference operator surface
    def InitData(self):
        self._check(self._lib.ks_init_data(self._h))

    def compute_dt(self):
        dt = ctypes.c_double()
        self._check(self._lib.ks_compute_dt(self._h, ctypes.byref(dt)))
        return dt.value

    def pre_advance(self):
        self._check(self._lib.ks_pre_advance(self._h))

    def prepare_time_step(self):
        self._check(self._lib.ks_prepare_time_step(self._h))

    def advance(self, fixed_point_iteration=0):
        self._check(self._lib.ks_advance(self._h, int(fixed_point_iteration)))

    def ApplyPredictor(self, incremental_projection=False, fixed_point_iteration=0):
        self._check(self._lib.ks_apply_predictor(self._h, int(bool(incremental_projection)), int(fixed_point_iteration)))

    def ApplyCorrector(self):
        self._check(self._lib.ks_apply_corrector(self._h))

    def ApplyProjection(self, time, scaling_factor, incremental=False):
        self._check(self._lib.ks_apply_projection(self._h, float(time), float(scaling_factor), int(bool(incremental))))

    def step(self):
        """One iteration of the Evolve loop; returns False once the run is finished."""
        return self._check(self._lib.ks_step(self._h), allow_done=True) == 0

    def Evolve(self, nsteps=1 << 30):
        self._check(self._lib.ks_evolve(self._h, int(nsteps)))

    # --- fields and scalars
    def layout(self, name):
        L = _Layout()
        self._check(self._lib.ks_field_layout(self._h, name.encode(), ctypes.byref(L)))
        return (L.ncomp, L.nz, L.ny, L.nx)

    def get_field(self, name, out=None):
        """Copy a field into a numpy array shaped (ncomp, nz, ny, nx), or into a
        torch CUDA tensor of that size when ``out`` is one."""
        shape = self.layout(name)
        if out is not None and hasattr(out, "data_ptr"):
            assert out.numel() == int(np.prod(shape)) and out.is_contiguous() and out.element_size() == 8
            where = KS_DEVICE if out.is_cuda else KS_HOST
            self._check(self._lib.ks_get_field(self._h, name.encode(), ctypes.c_void_p(out.data_ptr()), where))
            return out
        a = np.empty(shape, dtype=np.float64) if out is None else out
        self._check(self._lib.ks_get_field(self._h, name.encode(), a.ctypes.data_as(ctypes.c_void_p), KS_HOST))
        return a

    def set_field(self, name, value):
        shape = self.layout(name)
        if hasattr(value, "data_ptr"):
            assert value.numel() == int(np.prod(shape)) and value.is_contiguous() and value.element_size() == 8
            where = KS_DEVICE if value.is_cuda else KS_HOST
            self._check(self._lib.ks_set_field(self._h, name.encode(), ctypes.c_void_p(value.data_ptr()), where))
            return
        a = np.ascontiguousarray(value, dtype=np.float64).reshape(shape)
        self._check(self._lib.ks_set_field(self._h, name.encode(), a.ctypes.data_as(ctypes.c_void_p), KS_HOST))

    def scalar(self, name):
        v = ctypes.c_double()
        self._check(self._lib.ks_get_scalar(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    def solver_stats(self):
        s = _Stats()
        self._check(self._lib.ks_last_solver_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in _Stats._fields_}

    def set_precision(self, precision):
        self._check(self._lib.ks_set_precision(self._h, int(precision)))

    def synchronize(self):
        self._check(self._lib.ks_synchronize(self._h))

    def stream(self):
        """The cudaStream_t (as an int) all kernels of this handle run on."""
        p = ctypes.c_void_p()
        self._check(self._lib.ks_get_stream(self._h, ctypes.byref(p)))
        return p.value or 0

    def profile_kernels(self, kernel="*"):
        self._check(self._lib.ks_profile_kernels(self._h, kernel.encode() if kernel else None))

    def profile_report(self):
        """{kernel name: (launches, total ms, algorithmic bytes)} since the last report; clears it."""
        need = self._lib.ks_profile_report(self._h, None, 0)
        if need < 0:
            raise KsError(-need, self._lib.ks_last_error(self._h).decode())
        buf = ctypes.create_string_buffer(int(need))
        self._lib.ks_profile_report(self._h, buf, need)
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms, nbytes = line.split()
            out[name] = (int(n), float(ms), float(nbytes))
        return out

    def kernel_launches(self):
        c = ctypes.c_longlong()
        self._check(self._lib.ks_kernel_launches(self._h, ctypes.byref(c)))
        return c.value

    # --- reverse mode
    def set_objective_box(self, lo, hi):
        """J = mean of 0.5 |u|^2 over the cells whose centres lie in [lo, hi]."""
        a = (ctypes.c_double * 3)(*[float(x) for x in lo])
        b = (ctypes.c_double * 3)(*[float(x) for x in hi])
        self._check(self._lib.ks_set_objective_box(self._h, a, b))

    def objective(self, seed=False):
        J = ctypes.c_double()
        self._check(self._lib.ks_objective(self._h, int(bool(seed)), ctypes.byref(J)))
        return J.value

    def adjoint_step(self):
        self._check(self._lib.ks_adjoint_step(self._h))

    def adjoint_run(self, nsteps, snapshots):
        """Forward ``nsteps`` steps, J at the end, reverse sweep with binomial
        checkpointing in ``snapshots`` device slots; returns J."""
        J = ctypes.c_double()
        self._check(self._lib.ks_adjoint_run(self._h, int(nsteps), int(snapshots), ctypes.byref(J)))
        return J.value

    def ndisks(self):
        return int(self.scalar("ndisks"))

    def ct_gradient(self):
        n = self.ndisks()
        g = (ctypes.c_double * max(n, 1))()
        self._check(self._lib.ks_get_ct_gradient(self._h, g, n))
        return np.array(g[:n])

    def adjoint_reset(self):
        self._check(self._lib.ks_adjoint_reset(self._h))

    # ---- IOManager counterparts
    def write_plot_file(self, path):
        self._check(self._lib.ks_write_plotfile(self._h, str(path).encode()))

    def write_checkpoint_file(self, path):
        self._check(self._lib.ks_write_checkpoint(self._h, str(path).encode()))

    def read_checkpoint_file(self, path):
        self._check(self._lib.ks_read_checkpoint(self._h, str(path).encode()))

    def write_outputs(self, last=False):
        self._check(self._lib.ks_write_outputs(self._h, int(bool(last))))

    def set_disk_ct(self, ct):
        ct = [float(x) for x in ct]
        a = (ctypes.c_double * max(len(ct), 1))(*ct)
        self._check(self._lib.ks_set_disk_ct(self._h, a, len(ct)))
