"""Python binding of the GB300 block-DDA C ABI (``include/bdda.h``).

Thin ctypes layer over ``block-dda_gb300/_lib/libbdda.so`` used by the tests,
the benchmark and ``__graft_entry__``.  There is no CPU fallback: if the
library is missing, :func:`lib` raises.  Host matrices are numpy complex128
arrays in column-major (Fortran) order, exactly the reference's Eigen layout
(column l = right-hand side, row f*m + c = component c of dipole m; f = 3
electric dipoles, f = 6 electric then magnetic).
"""
from __future__ import annotations

import ctypes as ct
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_LIB = None

OK, ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_BREAKDOWN, ERR_NOT_CONVERGED = 0, 1, 2, 3, 4, 5
PREC_FP64, PREC_FP32, PREC_DF64 = 1, 2, 4
SOLVER_COCG_RQ, SOLVER_BICGSTAB, SOLVER_BICGGR = 0, 1, 2
SOLVE_FP64, SOLVE_MIXED = 0, 1
SOLVERS = {"cocg_rq": SOLVER_COCG_RQ, "bicgstab": SOLVER_BICGSTAB, "bicggr": SOLVER_BICGGR}
KERNEL_NAMES = ["passA_c64", "passB_c64", "passC_c64", "passD_c64", "passE_c64",
                "passA_c128", "passB_c128", "passC_c128", "passD_c128", "passE_c128",
                "gram", "update", "small", "other"]

# every symbol include/bdda.h declares
EXPORTS = [
    "bdda_op_create", "bdda_op_destroy", "bdda_op_set_dipoles", "bdda_op_info", "bdda_mbt_fft_mvp",
    "bdda_op_mvp_device", "bdda_solve_opts_default", "bdda_solve_device", "bdda_solve", "bdda_qr_reduced",
    "bdda_mie_a1b1", "bdda_aggregate", "bdda_incident_fields", "bdda_cross_sections", "bdda_op_set_timing",
    "bdda_op_set_graphs", "bdda_op_kernel_stats", "bdda_last_error", "bdda_op_mvp_bytes", "bdda_host_fft_line",
    "bdda_op_mvp_device_noalloc", "bdda_request_footprint", "bdda_server_create", "bdda_server_submit",
    "bdda_server_wait", "bdda_server_stats", "bdda_server_destroy", "bdda_batch_solve",
    "bdda_incident_fields_eh", "bdda_cross_sections_eh", "bdda_read_target_file", "bdda_shape_target",
    "bdda_material_load", "bdda_material_constant", "bdda_material_eval", "bdda_material_destroy",
    "bdda_polarizabilities", "bdda_diag_a", "bdda_op_set_wavenumber", "bdda_sweep", "bdda_mie_q",
    "bdda_format_result", "bdda_request_footprint_f", "bdda_server_set_spectrum_cache", "bdda_server_cache_stats",
    "bdda_op_set_autotune", "bdda_op_get_tuning", "bdda_op_check_status", "bdda_op_set_z_kernel",
    "bdda_op_test_z_stall",
]

SHAPES = {"sphere": 0, "cube": 1, "ellipsoid": 2, "cuboid": 3, "cylinder": 4, "rounded_cylinder": 5}


class BddaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"bdda error {code}: {msg}")
        self.code = code


class SolveOpts(ct.Structure):
    _fields_ = [("solver", ct.c_int), ("jacobi", ct.c_int), ("precision", ct.c_int), ("tol", ct.c_double),
                ("itermax", ct.c_int), ("true_tol", ct.c_double), ("inner_tol", ct.c_double),
                ("max_refine", ct.c_int), ("check_every", ct.c_int), ("warm_start", ct.c_int)]


class SweepTarget(ct.Structure):
    _fields_ = [("n", ct.c_int * 3), ("lf", ct.c_double), ("nocc", ct.c_int), ("address", ct.POINTER(ct.c_int)),
                ("vol", ct.POINTER(ct.c_double)), ("material", ct.POINTER(ct.c_int))]


class SweepSpec(ct.Structure):
    _fields_ = [("f", ct.c_int), ("n_wl", ct.c_int), ("wl0", ct.POINTER(ct.c_double)), ("n_targets", ct.c_int),
                ("targets", ct.POINTER(SweepTarget)), ("nmat", ct.c_int), ("materials", ct.POINTER(ct.c_void_p)),
                ("L", ct.c_int), ("uinc", ct.POINTER(ct.c_double)), ("einc", ct.POINTER(ct.c_double)),
                ("hinc", ct.POINTER(ct.c_double)), ("opts", SolveOpts), ("warm_start", ct.c_int), ("prec", ct.c_int)]


class SweepResult(ct.Structure):
    _fields_ = [("status", ct.c_int), ("iterations", ct.c_int), ("refinements", ct.c_int),
                ("mie_evaluations", ct.c_int), ("true_res_max", ct.c_double), ("final_err", ct.c_double),
                ("ms_solve", ct.c_double), ("alpha_e0", ct.c_double * 2), ("alpha_h0", ct.c_double * 2)]

    def as_dict(self):
        return {"status": self.status, "iterations": self.iterations, "refinements": self.refinements,
                "mie_evaluations": self.mie_evaluations, "true_res_max": self.true_res_max,
                "final_err": self.final_err, "ms_solve": self.ms_solve,
                "alpha_e0": complex(self.alpha_e0[0], self.alpha_e0[1]),
                "alpha_h0": complex(self.alpha_h0[0], self.alpha_h0[1])}


class ResultRecord(ct.Structure):
    _fields_ = [("wl0_index", ct.c_int), ("target_index", ct.c_int), ("wl0", ct.c_double), ("N_inc", ct.c_int),
                ("eper_medium", ct.c_double * 2), ("mper_medium", ct.c_double * 2), ("target_fname", ct.c_char_p),
                ("is_homogeneous", ct.c_int), ("eper_core", ct.c_double * 2), ("mper_core", ct.c_double * 2),
                ("volume_core", ct.c_double), ("density_core", ct.c_double), ("eper_coat", ct.c_double * 2),
                ("mper_coat", ct.c_double * 2), ("volume_coat", ct.c_double), ("L", ct.c_int),
                ("cext", ct.POINTER(ct.c_double)), ("cabs", ct.POINTER(ct.c_double)), ("f", ct.c_int),
                ("nx", ct.c_int), ("ny", ct.c_int), ("nz", ct.c_int), ("num_element_occupy", ct.c_int),
                ("solver_time", ct.c_double), ("append_mac_mie", ct.c_int)]


class Request(ct.Structure):
    _fields_ = [("n", ct.c_int * 3), ("lf", ct.c_double), ("k_re", ct.c_double), ("k_im", ct.c_double),
                ("address", ct.POINTER(ct.c_int)), ("nocc", ct.c_int), ("diag", ct.POINTER(ct.c_double)),
                ("B", ct.POINTER(ct.c_double)), ("L", ct.c_int), ("X", ct.POINTER(ct.c_double)), ("f", ct.c_int)]


class RequestResult(ct.Structure):
    _fields_ = [("status", ct.c_int), ("iterations", ct.c_int), ("refinements", ct.c_int),
                ("true_res_max", ct.c_double), ("t_submit", ct.c_double), ("t_start", ct.c_double),
                ("t_done", ct.c_double), ("footprint_bytes", ct.c_double), ("retried_fp64", ct.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SolveStats(ct.Structure):
    _fields_ = [("status", ct.c_int), ("iterations", ct.c_int), ("refinements", ct.c_int), ("mvps", ct.c_int),
                ("final_err", ct.c_double), ("true_res_max", ct.c_double), ("ms_solve", ct.c_double),
                ("fp64_inner_steps", ct.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = False):
    """Load libbdda.so (raises if it was not built)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"CUDA library not built: {path} (run __graft_entry__.build())")
        _build.build()
    L = ct.CDLL(path)
    vp, ip, dp = ct.c_void_p, ct.POINTER(ct.c_int), ct.POINTER(ct.c_double)
    L.bdda_op_create.argtypes = [ct.POINTER(vp), ip, ct.c_int, ct.c_double, ct.c_double, ct.c_double, ct.c_int]
    L.bdda_op_destroy.argtypes = [vp]
    L.bdda_op_set_wavenumber.argtypes = [vp, ct.c_double, ct.c_double]
    L.bdda_op_set_dipoles.argtypes = [vp, ip, ct.c_int]
    L.bdda_op_info.argtypes = [vp, ip, ip, ip]
    L.bdda_mbt_fft_mvp.argtypes = [vp, dp, dp]
    L.bdda_op_mvp_device.argtypes = [vp, ct.c_int, vp, ct.c_int, vp, ct.c_int, ct.c_int, vp, vp, vp]
    L.bdda_op_mvp_device_noalloc.argtypes = [vp, ct.c_int, vp, ct.c_int, vp, ct.c_int, ct.c_int, vp, vp, vp]
    L.bdda_solve_opts_default.argtypes = [ct.POINTER(SolveOpts)]
    L.bdda_solve_opts_default.restype = None
    L.bdda_solve_device.argtypes = [vp, ct.POINTER(SolveOpts), vp, vp, ct.c_int, vp, ct.c_int, ct.c_int,
                                    ct.POINTER(SolveStats), vp]
    L.bdda_solve.argtypes = [vp, ct.POINTER(SolveOpts), dp, dp, ct.c_int, dp, ct.c_int, ct.c_int,
                             ct.POINTER(SolveStats)]
    L.bdda_qr_reduced.argtypes = [dp, ct.c_int, ct.c_int, ct.c_int, dp, ct.c_int, dp]
    L.bdda_mie_a1b1.argtypes = [ct.c_double, ct.c_double, dp, dp, dp, dp, dp, dp]
    L.bdda_aggregate.argtypes = [ct.c_int, ct.c_double, ct.c_double, ct.c_ulonglong, ip, ip]
    L.bdda_incident_fields.argtypes = [ip, ct.c_double, ip, ct.c_int, ct.c_double, ct.c_int, dp, dp, dp, ct.c_int]
    L.bdda_cross_sections.argtypes = [ct.c_double, dp, dp, ct.c_int, dp, ct.c_int, ct.c_int, ct.c_int, dp]
    L.bdda_incident_fields_eh.argtypes = [ip, ct.c_double, ip, ct.c_int, ct.c_double, ct.c_int, dp, dp, dp, dp,
                                          ct.c_int]
    L.bdda_cross_sections_eh.argtypes = [ct.c_double, dp, dp, dp, ct.c_int, dp, ct.c_int, ct.c_int, ct.c_int, dp]
    L.bdda_read_target_file.argtypes = [ct.c_char_p, ct.c_double, ip, dp, ip, ct.c_int, ip, dp, ip]
    L.bdda_shape_target.argtypes = [ct.c_int, ct.c_int, dp, ip, dp, ip, ct.c_int, ip]
    L.bdda_material_load.argtypes = [ct.c_char_p, ct.c_double, ct.POINTER(vp)]
    L.bdda_material_constant.argtypes = [dp, dp, ct.c_double, ct.POINTER(vp)]
    L.bdda_material_eval.argtypes = [vp, ct.c_double, dp, dp, dp]
    L.bdda_material_destroy.argtypes = [vp]
    L.bdda_polarizabilities.argtypes = [ct.c_double, ct.c_int, dp, ip, ct.POINTER(vp), ct.c_int, dp, dp, ip]
    L.bdda_diag_a.argtypes = [ct.c_int, ct.c_int, dp, dp, dp]
    L.bdda_sweep.argtypes = [ct.POINTER(SweepSpec), dp, ct.POINTER(SweepResult)]
    L.bdda_mie_q.argtypes = [ct.c_double, ct.c_double, dp, dp, dp, dp, dp]
    L.bdda_format_result.argtypes = [ct.POINTER(ResultRecord), ct.c_char_p, ct.c_int, ip]
    L.bdda_op_mvp_bytes.argtypes = [vp, ct.c_int, ct.c_int, ct.c_int, ct.c_int, dp]
    L.bdda_op_set_timing.argtypes = [vp, ct.c_int]
    L.bdda_op_set_graphs.argtypes = [vp, ct.c_int]
    L.bdda_op_set_autotune.argtypes = [vp, ct.c_int]
    L.bdda_op_get_tuning.argtypes = [vp, ct.c_int, ip, ct.POINTER(ct.c_float)]
    L.bdda_op_check_status.argtypes = [vp]
    L.bdda_op_set_z_kernel.argtypes = [vp, ct.c_int]
    L.bdda_op_test_z_stall.argtypes = [vp, ct.c_int]
    L.bdda_op_kernel_stats.argtypes = [vp, dp, ct.POINTER(ct.c_longlong), ct.c_int, ct.c_int]
    L.bdda_last_error.restype = ct.c_char_p
    L.bdda_request_footprint.argtypes = [ip, ct.c_int, ct.c_int, ct.c_int]
    L.bdda_request_footprint.restype = ct.c_double
    L.bdda_request_footprint_f.argtypes = [ip, ct.c_int, ct.c_int, ct.c_int, ct.c_int]
    L.bdda_request_footprint_f.restype = ct.c_double
    L.bdda_server_create.argtypes = [ct.POINTER(vp), ct.c_int, ct.c_double, ct.POINTER(SolveOpts), ct.c_int]
    L.bdda_server_submit.argtypes = [vp, ct.POINTER(Request), ct.POINTER(ct.c_longlong)]
    L.bdda_server_wait.argtypes = [vp, ct.c_longlong, ct.POINTER(RequestResult)]
    L.bdda_server_stats.argtypes = [vp, dp, ip, ct.POINTER(ct.c_longlong)]
    L.bdda_server_destroy.argtypes = [vp]
    L.bdda_server_set_spectrum_cache.argtypes = [vp, ct.c_double]
    L.bdda_server_cache_stats.argtypes = [vp, ct.POINTER(ct.c_longlong), ct.POINTER(ct.c_longlong),
                                          ct.POINTER(ct.c_double)]
    L.bdda_batch_solve.argtypes = [ct.POINTER(Request), ct.c_int, ct.c_int, ct.c_double, ct.POINTER(SolveOpts),
                                   ct.POINTER(RequestResult)]
    L.bdda_host_fft_line.argtypes = [ct.c_int, ct.c_int, ct.c_int, ct.c_int, dp, ip]
    _LIB = L
    return L


def _check(rc, allow=()):
    if rc != OK and rc not in allow:
        raise BddaError(rc, lib().bdda_last_error().decode())
    return rc


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ct.POINTER(ct.c_double))


def _iptr(a: np.ndarray):
    return a.ctypes.data_as(ct.POINTER(ct.c_int))


def _cmat(a, rows=None):
    """complex128 column-major copy (or view) of a matrix / vector."""
    a = np.asarray(a, dtype=np.complex128)
    if a.ndim == 1:
        a = a[:, None]
    return np.asfortranarray(a)


# ---------------------------------------------------------------------------
# operator
# ---------------------------------------------------------------------------

class Operator:
    """Green-tensor operator of one lattice box (``bdda_op``)."""

    def __init__(self, n, lf, k, prec=PREC_FP64 | PREC_FP32 | PREC_DF64, f=3):
        self._h = ct.c_void_p()
        n3 = np.ascontiguousarray(n, dtype=np.int32)
        k = complex(k)
        _check(lib().bdda_op_create(ct.byref(self._h), _iptr(n3), f, float(lf), k.real, k.imag, prec))
        self.n = tuple(int(v) for v in n3)
        self.lf = float(lf)
        self.k = k
        self.f = int(f)    # 3: electric dipoles; 6: electric + magnetic (rows f*m + c)
        self.nocc = 0

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().bdda_op_destroy(self._h)
            self._h = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_wavenumber(self, k):
        """New wavenumber (next wavelength): rebuilds the Green spectra only."""
        k = complex(k)
        _check(lib().bdda_op_set_wavenumber(self._h, k.real, k.imag))
        self.k = k

    def set_dipoles(self, address):
        a = np.ascontiguousarray(address, dtype=np.int32)
        _check(lib().bdda_op_set_dipoles(self._h, _iptr(a), int(a.size)))
        self.nocc = int(a.size)

    def info(self):
        P = np.zeros(3, np.int32)
        nocc, nl = ct.c_int(), ct.c_int()  # nl: occupied (y, z-tile) tiles
        _check(lib().bdda_op_info(self._h, _iptr(P), ct.byref(nocc), ct.byref(nl)))
        return tuple(int(v) for v in P), nocc.value, nl.value

    def plans(self):
        """Radix sequences of the complex FP32 FFT plans per axis (x, y: the
        tile passes' tables; z: the fused z pass's table)."""
        P, _, _ = self.info()
        return {ax: host_fft_line(np.zeros(P[i]), prec=PREC_FP32, max_radix=16 if i == 2 else 8)[1]
                for i, ax in enumerate("xyz")}

    def mbt_fft_mvp(self, p_hat):
        """Reference ``MBT_fft_mvp`` on a full cuboid vector (host, complex128)."""
        x = np.ascontiguousarray(p_hat, dtype=np.complex128)
        y = np.empty_like(x)
        _check(lib().bdda_mbt_fft_mvp(self._h, _dptr(x), _dptr(y)))
        return y

    def mvp_device(self, x, y, L, ldx, ldy, prec=PREC_FP64, diag=None, jpre=None, stream=None):
        """Block MVP on device pointers (ints, e.g. ``torch.Tensor.data_ptr()``)."""
        _check(lib().bdda_op_mvp_device(self._h, prec, ct.c_void_p(x), ldx, ct.c_void_p(y), ldy, L,
                                        ct.c_void_p(diag) if diag else None, ct.c_void_p(jpre) if jpre else None,
                                        ct.c_void_p(stream) if stream else None))

    def mvp_bytes(self, L, prec=PREC_FP32, with_diag=True, with_jpre=True):
        """Algorithmic HBM bytes of one block MVP, per pass (A..E)."""
        b = np.zeros(5)
        _check(lib().bdda_op_mvp_bytes(self._h, prec, int(L), int(with_diag), int(with_jpre), _dptr(b)))
        return b

    def mvp_device_noalloc(self, x, y, L, ldx, ldy, prec=PREC_FP64, diag=None, jpre=None, stream=None):
        """Same as mvp_device, with the workspace in the library's fixed device
        array instead of memory allocated by the call (bdda_op_mvp_device_noalloc)."""
        _check(lib().bdda_op_mvp_device_noalloc(self._h, prec, ct.c_void_p(x), ldx, ct.c_void_p(y), ldy, L,
                                                ct.c_void_p(diag) if diag else None,
                                                ct.c_void_p(jpre) if jpre else None,
                                                ct.c_void_p(stream) if stream else None))

    def set_timing(self, on=True):
        """True / 1: time every kernel class; 2: the fused z pass only; False / 0: off."""
        _check(lib().bdda_op_set_timing(self._h, int(on) if not isinstance(on, bool) else (1 if on else 0)))

    def set_graphs(self, on=True):
        """Captured CUDA graphs for the solvers' poll cycles (default on); off: launch by launch."""
        _check(lib().bdda_op_set_graphs(self._h, 1 if on else 0))

    def set_autotune(self, on=True):
        """Measured FFT launch schedule for the complex FP32 MVP (default on)."""
        _check(lib().bdda_op_set_autotune(self._h, 1 if on else 0))

    def tuning(self, L):
        """(schedule dict, candidate ms dict, measured?) for nrhs L (bdda_op_get_tuning)."""
        sch = np.zeros(6, np.int32)
        ms = (ct.c_float * 22)()
        rc = lib().bdda_op_get_tuning(self._h, int(L), _iptr(sch), ms)
        _check(rc, (ERR_NOT_CONVERGED,))
        cand = {"y": {f"buf{1 + i // 4}_waves{(2, 4, 8, 16)[i % 4]}": ms[i] for i in range(8)},
                "y_inverse": {f"buf{1 + i // 4}_waves{(2, 4, 8, 16)[i % 4]}": ms[14 + i] for i in range(8)},
                "z_pass": {"scalar": ms[8], "packed": ms[9], "pipelined": ms[13]},
                "x_cta_per_sm": {str(v): ms[10 + i] for i, v in enumerate((5, 10, 20))}}
        return ({"y_waves": int(sch[0]), "y_buffers": int(sch[1]),
                 "z_pass": {-1: "default", 0: "scalar", 1: "packed", 2: "pipelined"}[int(sch[2])],
                 "x_cta_per_sm": int(sch[3]), "y_inverse_waves": int(sch[4]), "y_inverse_buffers": int(sch[5])},
                cand, rc == OK)

    def set_z_kernel(self, kind="default"):
        """Force the complex FP32 pass C kernel: "default", "scalar", "packed" or "pipelined"."""
        _check(lib().bdda_op_set_z_kernel(self._h, {"default": -1, "scalar": 0, "packed": 1, "pipelined": 2}[kind]))

    def test_z_stall(self, on=True):
        """Test hook: the pipelined z pass gives up one bounded wait (bdda_op_test_z_stall)."""
        _check(lib().bdda_op_test_z_stall(self._h, 1 if on else 0))

    def check_status(self):
        """Raise if a kernel of this operator reported a failed bounded wait (bdda_op_check_status)."""
        _check(lib().bdda_op_check_status(self._h))

    def kernel_stats(self, reset=False):
        n = len(KERNEL_NAMES)
        ms = (ct.c_double * n)()
        la = (ct.c_longlong * n)()
        m = lib().bdda_op_kernel_stats(self._h, ms, la, n, 1 if reset else 0)
        return {KERNEL_NAMES[i]: {"ms": ms[i], "launches": la[i]} for i in range(m)}


def solve_opts(solver="cocg_rq", jacobi=True, precision=SOLVE_FP64, tol=1e-2, itermax=300, true_tol=0.0,
               inner_tol=0.0, max_refine=8, check_every=4, warm_start=False) -> SolveOpts:
    o = SolveOpts()
    lib().bdda_solve_opts_default(ct.byref(o))
    o.solver = SOLVERS[solver] if isinstance(solver, str) else int(solver)
    o.jacobi = 1 if jacobi else 0
    o.precision = int(precision)
    o.tol = float(tol)
    o.itermax = int(itermax)
    o.true_tol = float(true_tol)
    o.inner_tol = float(inner_tol)
    o.max_refine = int(max_refine)
    o.check_every = int(check_every)
    o.warm_start = 1 if warm_start else 0
    return o


def solve(op: Operator, diag, B, opts: SolveOpts, allow_not_converged=True, X0=None):
    """Host-buffer solve (``bdda_solve``).  Returns (X, stats dict).  X0: initial
    guess for a warm-started refinement (``opts.warm_start``)."""
    d = np.ascontiguousarray(diag, dtype=np.complex128)
    Bm = _cmat(B)
    n, L = Bm.shape
    X = np.zeros((n, L), dtype=np.complex128, order="F") if X0 is None else np.array(X0, dtype=np.complex128,
                                                                                      order="F")
    st = SolveStats()
    allow = (ERR_NOT_CONVERGED,) if allow_not_converged else ()
    _check(lib().bdda_solve(op.handle, ct.byref(opts), _dptr(d), _dptr(Bm), n,
                            _dptr(X), n, L, ct.byref(st)), allow)
    return X, st.as_dict()


def solve_device(op: Operator, diag_ptr, B_ptr, ldb, X_ptr, ldx, L, opts: SolveOpts, stream=None,
                 allow_not_converged=True):
    st = SolveStats()
    allow = (ERR_NOT_CONVERGED,) if allow_not_converged else ()
    _check(lib().bdda_solve_device(op.handle, ct.byref(opts), ct.c_void_p(diag_ptr), ct.c_void_p(B_ptr), ldb,
                                   ct.c_void_p(X_ptr), ldx, L, ct.byref(st), ct.c_void_p(stream) if stream else None),
           allow)
    return st.as_dict()


def qr_reduced(A):
    a = _cmat(A)
    m, n = a.shape
    Q = np.zeros((m, n), dtype=np.complex128, order="F")
    R = np.zeros((n, n), dtype=np.complex128, order="F")
    _check(lib().bdda_qr_reduced(_dptr(a), m, n, m, _dptr(Q), m,
                                 _dptr(R)))
    return Q, R


# ---------------------------------------------------------------------------
# host physics (C++)
# ---------------------------------------------------------------------------

def mie_a1b1(wl0, r_p, eps_p, mu_p=1 + 0j, eps_m=1 + 0j, mu_m=1 + 0j):
    vals = [np.array([complex(v).real, complex(v).imag]) for v in (eps_p, mu_p, eps_m, mu_m)]
    a1 = np.zeros(2)
    b1 = np.zeros(2)
    _check(lib().bdda_mie_a1b1(float(wl0), float(r_p), *[_dptr(v) for v in vals], _dptr(a1), _dptr(b1)))
    return complex(a1[0], a1[1]), complex(b1[0], b1[1])


def polarizability(wl0, r_p, eps_p, k, mu_p=1 + 0j):
    """alpha = 3 i a1 / (2 k^3) (Target_manager.cpp:232)."""
    a1, _ = mie_a1b1(wl0, r_p, eps_p, mu_p)
    return 3j * a1 / (2.0 * k ** 3)


def polarizabilities(wl0, r_p, eps_p, k, mu_p=1 + 0j):
    """(alpha_E, alpha_H) = 3 i (a1, b1) / (2 k^3) (Target_manager.cpp:246-247)."""
    a1, b1 = mie_a1b1(wl0, r_p, eps_p, mu_p)
    return 3j * a1 / (2.0 * k ** 3), 3j * b1 / (2.0 * k ** 3)


def diag_a(alpha_e, alpha_h=None):
    """DIAG_A per row (``bdda_diag_a``): 1/alpha_E over rows 3m..3m+2 (f=3,
    Solver.cpp:33-36), or 1/alpha_E then 1/alpha_H over rows 6m..6m+5 (f=6,
    Solver.cpp:40-45)."""
    ae = np.ascontiguousarray(np.asarray(alpha_e, dtype=np.complex128).reshape(-1))
    f = 3 if alpha_h is None else 6
    ah = None if alpha_h is None else np.ascontiguousarray(np.asarray(alpha_h, dtype=np.complex128).reshape(-1))
    d = np.zeros(f * ae.size, dtype=np.complex128)
    _check(lib().bdda_diag_a(f, int(ae.size), _dptr(ae), _dptr(ah) if ah is not None else None, _dptr(d)))
    return d


def read_target_file(path, scale_factor=1.0):
    """Target file ``DDA_target_*.out`` -> (n, lf, address, vol, material) (``bdda_read_target_file``)."""
    n = np.zeros(3, np.int32)
    lf, nocc = ct.c_double(), ct.c_int()
    bp = os.fsencode(path)
    _check(lib().bdda_read_target_file(bp, float(scale_factor), _iptr(n), ct.byref(lf), ct.byref(nocc), 0,
                                       None, None, None))
    m = nocc.value
    addr, vol, mat = np.zeros(m, np.int32), np.zeros(m), np.zeros(m, np.int32)
    _check(lib().bdda_read_target_file(bp, float(scale_factor), _iptr(n), ct.byref(lf), ct.byref(nocc), m,
                                       _iptr(addr), _dptr(vol), _iptr(mat)))
    return tuple(int(v) for v in n), lf.value, addr, vol, mat


def shape_target(shape, nmax, side_lengths):
    """Lattice sites of a shape (``bdda_shape_target``) -> (n, lf, address); element volume lf^3."""
    code = SHAPES[shape] if isinstance(shape, str) else int(shape)
    s3 = np.ascontiguousarray(side_lengths, dtype=np.float64)
    n = np.zeros(3, np.int32)
    lf, nocc = ct.c_double(), ct.c_int()
    _check(lib().bdda_shape_target(code, int(nmax), _dptr(s3), _iptr(n), ct.byref(lf), ct.byref(nocc), 0, None))
    addr = np.zeros(nocc.value, np.int32)
    _check(lib().bdda_shape_target(code, int(nmax), _dptr(s3), _iptr(n), ct.byref(lf), ct.byref(nocc), nocc.value,
                                   _iptr(addr)))
    return tuple(int(v) for v in n), lf.value, addr


class Material:
    """Material table or constant (``bdda_material``)."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def load(cls, path, density):
        h = ct.c_void_p()
        _check(lib().bdda_material_load(os.fsencode(path), float(density), ct.byref(h)))
        return cls(h)

    @classmethod
    def constant(cls, eper, mper=1 + 0j, density=0.0):
        h = ct.c_void_p()
        e = np.array([complex(eper).real, complex(eper).imag])
        m = np.array([complex(mper).real, complex(mper).imag])
        _check(lib().bdda_material_constant(_dptr(e), _dptr(m), float(density), ct.byref(h)))
        return cls(h)

    @property
    def handle(self):
        return self._h

    def __call__(self, wl0):
        """(eper, mper) at the free-space wavelength wl0."""
        e, m, d = np.zeros(2), np.zeros(2), ct.c_double()
        _check(lib().bdda_material_eval(self._h, float(wl0), _dptr(e), _dptr(m), ct.byref(d)))
        return complex(e[0], e[1]), complex(m[0], m[1])

    @property
    def density(self):
        d = ct.c_double()
        _check(lib().bdda_material_eval(self._h, 0.0, None, None, ct.byref(d)))
        return d.value

    def close(self):
        if self._h:
            lib().bdda_material_destroy(self._h)
            self._h = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dipole_polarizabilities(wl0, vol, materials, material_index=None):
    """(alpha_E, alpha_H, Mie evaluations) of every dipole in vacuum (``bdda_polarizabilities``)."""
    v = np.ascontiguousarray(vol, dtype=np.float64)
    mi = None if material_index is None else np.ascontiguousarray(material_index, dtype=np.int32)
    hs = (ct.c_void_p * len(materials))(*[m.handle.value for m in materials])
    ae = np.zeros(v.size, np.complex128)
    ah = np.zeros(v.size, np.complex128)
    nev = ct.c_int()
    _check(lib().bdda_polarizabilities(float(wl0), int(v.size), _dptr(v), _iptr(mi) if mi is not None else None,
                                       ct.cast(hs, ct.POINTER(ct.c_void_p)), len(materials), _dptr(ae), _dptr(ah),
                                       ct.byref(nev)))
    return ae, ah, nev.value


def aggregate(nocc, kf=1.0, Df=2.8, seed=1):
    n = np.zeros(3, np.int32)
    addr = np.zeros(nocc, np.int32)
    _check(lib().bdda_aggregate(int(nocc), float(kf), float(Df), int(seed), _iptr(n), _iptr(addr)))
    return tuple(int(v) for v in n), addr


def incident_fields(n, lf, address, k, uinc, einc, hinc=None):
    """EHinc: f=3 rows e exp(i k u.r); with ``hinc`` the f=6 rows [e, h] exp(i k u.r)."""
    n3 = np.ascontiguousarray(n, dtype=np.int32)
    a = np.ascontiguousarray(address, dtype=np.int32)
    u = np.ascontiguousarray(uinc, dtype=np.float64).reshape(-1, 3)
    e = np.ascontiguousarray(einc, dtype=np.complex128).reshape(-1, 3)
    L = u.shape[0]
    if hinc is None:
        B = np.zeros((3 * a.size, L), dtype=np.complex128, order="F")
        _check(lib().bdda_incident_fields(_iptr(n3), float(lf), _iptr(a), int(a.size), float(k), L, _dptr(u),
                                          _dptr(e), _dptr(B), 3 * a.size))
        return B
    h = np.ascontiguousarray(hinc, dtype=np.complex128).reshape(-1, 3)
    B = np.zeros((6 * a.size, L), dtype=np.complex128, order="F")
    _check(lib().bdda_incident_fields_eh(_iptr(n3), float(lf), _iptr(a), int(a.size), float(k), L, _dptr(u),
                                         _dptr(e), _dptr(h), _dptr(B), 6 * a.size))
    return B


def cross_sections(k, alpha0, E, P, alpha_h0=None):
    """(Cext, Cabs, Csca) per column; with ``alpha_h0`` the f=6 form (rows 6m + c)."""
    Em = _cmat(E)
    Pm = _cmat(P)
    n, L = Em.shape
    out = np.zeros(3 * L)
    a0 = np.array([complex(alpha0).real, complex(alpha0).imag])
    if alpha_h0 is None:
        _check(lib().bdda_cross_sections(float(k), _dptr(a0), _dptr(Em), n, _dptr(Pm),
                                         n, n, L, _dptr(out)))
    else:
        h0 = np.array([complex(alpha_h0).real, complex(alpha_h0).imag])
        _check(lib().bdda_cross_sections_eh(float(k), _dptr(a0), _dptr(h0), _dptr(Em), n, _dptr(Pm), n, n // 6, L,
                                            _dptr(out)))
    out = out.reshape(L, 3)
    return out[:, 0].copy(), out[:, 1].copy(), out[:, 2].copy()


def host_fft_line(x, inverse=False, prec=1, nvalid=0, max_radix=8, c64_schedule=False):
    """Run the device FFT core on the CPU (unit tests).  Returns (y, radices).

    The schedule is the operator's for an axis of this length and the element
    width of prec: max_radix > 8 selects the z axis (three-line fused pass),
    otherwise the x / y axes; c64_schedule the complex FP32 schedule (first-
    stage radices up to 32) in any arithmetic."""
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    rad = np.zeros(16, np.int32)
    rad[0] = int(max_radix)
    rad[1] = 1 if c64_schedule else 0
    nst = lib().bdda_host_fft_line(int(a.size), 1 if inverse else 0, int(prec), int(nvalid), _dptr(a), _iptr(rad))
    if nst < 0:
        raise BddaError(ERR_INVALID, "unsupported FFT length")
    return a, [int(v) for v in rad[:nst]]


@dataclass
class Problem:
    """A DDA problem on a lattice aggregate (f=3, vacuum medium)."""
    n: tuple
    lf: float
    address: np.ndarray
    k: float
    alpha: np.ndarray   # per dipole
    diag: np.ndarray    # 3*nocc (1/alpha)
    B: np.ndarray       # 3*nocc x L, column-major

    @property
    def nocc(self):
        return int(self.address.size)


def directions(n_dirs, seed):
    """Seeded propagation directions, uniform on the sphere, with two
    orthonormal polarisations each: returns (uinc, einc) for L = 2*n_dirs."""
    rng = np.random.default_rng(seed)
    us, es = [], []
    for i in range(n_dirs):
        if i == 0:
            u = np.array([0.0, 0.0, 1.0])
        else:
            v = rng.standard_normal(3)
            u = v / np.linalg.norm(v)
        a = np.array([1.0, 0.0, 0.0]) if abs(u[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        e1 = a - np.dot(a, u) * u
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(u, e1)
        us += [u, u]
        es += [e1.astype(np.complex128), e2.astype(np.complex128)]
    return np.array(us), np.array(es)


def make_problem(nocc, m, wl0=0.55, kf=1.0, Df=2.8, seed=1, n_dirs=1, mkd=0.5):
    """Synthetic aggregate problem: |m| k d = mkd, dipole volume d^3,
    alpha from the Mie a1 of the volume-equivalent sphere."""
    n, addr = aggregate(nocc, kf, Df, seed)
    k = 2 * np.pi / wl0
    m = complex(m)
    d = mkd / (abs(m) * k)
    r_eq = d * (3.0 / (4.0 * np.pi)) ** (1.0 / 3.0)
    alpha0 = polarizability(wl0, r_eq, m * m, k)
    alpha = np.full(nocc, alpha0, dtype=np.complex128)
    diag = np.repeat(1.0 / alpha, 3)
    u, e = directions(n_dirs, seed + 1000)
    B = incident_fields(n, d, addr, k, u, e)
    return Problem(n=n, lf=d, address=addr, k=k, alpha=alpha, diag=diag, B=B)


def target_problem(n, lf, address, vol, m, wl0=0.55, seed=1, n_dirs=1, mkd=0.5):
    """Problem on a target read from a file (``read_target_file``): the file's
    lattice spacing ``lf`` and site volume ``vol`` (same length unit, e.g. the
    monomer radius r_pp of the reference's aggregates) are scaled so that
    |m| k d = mkd; every site is one dipole of the volume-equivalent radius of
    ``vol`` (``Target.cpp:13-19``) and one material."""
    k = 2 * np.pi / wl0
    m = complex(m)
    d = mkd / (abs(m) * k)
    scale = d / float(lf)
    r_eq = (3.0 * float(vol) / (4.0 * np.pi)) ** (1.0 / 3.0) * scale
    address = np.ascontiguousarray(address, dtype=np.int32)
    alpha0 = polarizability(wl0, r_eq, m * m, k)
    alpha = np.full(address.size, alpha0, dtype=np.complex128)
    u, e = directions(n_dirs, seed + 1000)
    B = incident_fields(n, d, address, k, u, e)
    return Problem(n=tuple(int(v) for v in n), lf=d, address=address, k=k, alpha=alpha,
                   diag=np.repeat(1.0 / alpha, 3), B=B)


# ---------------------------------------------------------------------------
# batched solves and the request server
# ---------------------------------------------------------------------------

def footprint(n, nocc, L, precision=SOLVE_MIXED, f=3):
    n3 = (ct.c_int * 3)(*[int(v) for v in n])
    return float(lib().bdda_request_footprint_f(n3, int(nocc), int(L), int(precision), int(f)))


class _Held:
    """Keeps the numpy buffers of a request alive while the server uses them."""

    def __init__(self, prob: Problem):
        self.address = np.ascontiguousarray(prob.address, dtype=np.int32)
        self.diag = np.ascontiguousarray(prob.diag, dtype=np.complex128)
        self.B = np.asfortranarray(prob.B, dtype=np.complex128)
        self.X = np.zeros_like(self.B, order="F")
        self.req = Request()
        for i in range(3):
            self.req.n[i] = int(prob.n[i])
        self.req.lf = float(prob.lf)
        self.req.k_re = float(np.real(prob.k))
        self.req.k_im = float(np.imag(prob.k))
        self.req.address = _iptr(self.address)
        self.req.nocc = int(self.address.size)
        self.req.diag = _dptr(self.diag)
        self.req.B = _dptr(self.B)
        self.req.L = int(self.B.shape[1])
        self.req.X = _dptr(self.X)
        self.req.f = int(self.B.shape[0] // max(1, self.address.size))  # 3 or 6 rows per dipole


class Server:
    """Request server (``bdda_server_*``): concurrent solves admitted by memory footprint."""

    def __init__(self, slots, mem_budget_bytes, opts: SolveOpts, dry_run=False):
        self._h = ct.c_void_p()
        self._opts = opts
        _check(lib().bdda_server_create(ct.byref(self._h), int(slots), float(mem_budget_bytes), ct.byref(opts),
                                        1 if dry_run else 0))
        self._held = {}

    def submit(self, prob: Problem):
        h = _Held(prob)
        t = ct.c_longlong()
        _check(lib().bdda_server_submit(self._h, ct.byref(h.req), ct.byref(t)))
        self._held[t.value] = h
        return t.value

    def wait(self, ticket, allow_fail=False):
        r = RequestResult()
        rc = lib().bdda_server_wait(self._h, ticket, ct.byref(r))
        h = self._held.pop(ticket)
        if not allow_fail:
            _check(rc)
        return h.X, r.as_dict()

    def stats(self):
        pb, pr, done = ct.c_double(), ct.c_int(), ct.c_longlong()
        _check(lib().bdda_server_stats(self._h, ct.byref(pb), ct.byref(pr), ct.byref(done)))
        ru, bu, cb = ct.c_longlong(), ct.c_longlong(), ct.c_double()
        _check(lib().bdda_server_cache_stats(self._h, ct.byref(ru), ct.byref(bu), ct.byref(cb)))
        return {"peak_inflight_bytes": pb.value, "peak_running": pr.value, "completed": done.value,
                "spectra_reused": ru.value, "spectra_built": bu.value, "cached_bytes": cb.value}

    def set_spectrum_cache(self, max_bytes):
        """Device bytes of idle operators (Green spectra) kept for later requests; 0 disables."""
        _check(lib().bdda_server_set_spectrum_cache(self._h, float(max_bytes)))

    def close(self):
        if self._h:
            lib().bdda_server_destroy(self._h)
            self._h = ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_solve(problems, slots, mem_budget_bytes, opts: SolveOpts):
    """Solve many problems concurrently (``bdda_batch_solve``).  Returns [(X, result dict)]."""
    held = [_Held(p) for p in problems]
    reqs = (Request * len(held))(*[h.req for h in held])
    res = (RequestResult * len(held))()
    rc = lib().bdda_batch_solve(reqs, len(held), int(slots), float(mem_budget_bytes), ct.byref(opts), res)
    out = [(h.X, res[i].as_dict()) for i, h in enumerate(held)]
    if rc != OK and rc != ERR_NOT_CONVERGED:
        _check(rc)
    return out


def random_problem(rng, n_range=(64, 8192), wl_range=(0.55, 0.55), L_choices=(2, 4, 8, 16), L_range=None,
                   seed=None):
    """One seeded aggregate problem with the batched/serving parameter ranges:
    N log-uniform, Df ~ U[1.8, 2.8], kf ~ U[1.0, 1.3], Re m ~ U[1.3, 2.4],
    Im m ~ U[0, 0.9], L from L_choices (or uniform in L_range)."""
    lo, hi = np.log(n_range[0]), np.log(n_range[1])
    nocc = int(round(np.exp(rng.uniform(lo, hi))))
    df = rng.uniform(1.8, 2.8)
    kf = rng.uniform(1.0, 1.3)
    m = complex(rng.uniform(1.3, 2.4), rng.uniform(0.0, 0.9))
    wl0 = rng.uniform(*wl_range)
    if L_range is not None:
        L = int(rng.integers(L_range[0], L_range[1] + 1))
    else:
        L = int(rng.choice(L_choices))
    s = int(rng.integers(1, 2 ** 31 - 1)) if seed is None else seed
    prob = make_problem(nocc, m, wl0=wl0, kf=kf, Df=df, seed=s, n_dirs=(L + 1) // 2)
    if prob.B.shape[1] != L:
        prob.B = np.asfortranarray(prob.B[:, :L])
    return prob


def sweep(wl0_list, targets, materials, uinc, einc, hinc=None, opts=None, warm_start=False, f=None, prec=0):
    """Wavelength x target sweep (``bdda_sweep``).

    targets: list of (n, lf, address, vol, material_index or None); materials:
    list of :class:`Material`.  f = 6 when ``hinc`` is given, else 3.  Returns
    (cross, results): cross[w, t, l] = (Cext, Cabs, Csca), results[w][t] dicts.
    """
    f = f or (6 if hinc is not None else 3)
    keep = []

    def arr(a, dt):
        v = np.ascontiguousarray(a, dtype=dt)
        keep.append(v)
        return v
    wl = arr(wl0_list, np.float64)
    tg = (SweepTarget * len(targets))()
    for i, (n, lf, address, vol, mat) in enumerate(targets):
        a = arr(address, np.int32)
        tg[i].n[:] = [int(v) for v in n]
        tg[i].lf = float(lf)
        tg[i].nocc = int(a.size)
        tg[i].address = _iptr(a)
        tg[i].vol = _dptr(arr(vol, np.float64))
        tg[i].material = _iptr(arr(mat, np.int32)) if mat is not None else None
    mh = (ct.c_void_p * len(materials))(*[m.handle.value for m in materials])
    u = arr(np.reshape(uinc, (-1, 3)), np.float64)
    e = arr(np.reshape(einc, (-1, 3)), np.complex128)
    spec = SweepSpec()
    spec.f, spec.n_wl, spec.wl0 = f, int(wl.size), _dptr(wl)
    spec.n_targets, spec.targets = len(targets), ct.cast(tg, ct.POINTER(SweepTarget))
    spec.nmat, spec.materials = len(materials), ct.cast(mh, ct.POINTER(ct.c_void_p))
    spec.L, spec.uinc, spec.einc = int(u.shape[0]), _dptr(u), _dptr(e)
    spec.hinc = _dptr(arr(np.reshape(hinc, (-1, 3)), np.complex128)) if hinc is not None else None
    spec.opts = opts if opts is not None else solve_opts()
    spec.warm_start = 1 if warm_start else 0
    spec.prec = int(prec)
    cross = np.zeros((wl.size, len(targets), spec.L, 3))
    res = (SweepResult * (wl.size * len(targets)))()
    rc = lib().bdda_sweep(ct.byref(spec), _dptr(cross), ct.cast(res, ct.POINTER(SweepResult)))
    _check(rc, (ERR_NOT_CONVERGED,))
    out = [[res[w * len(targets) + t].as_dict() for t in range(len(targets))] for w in range(wl.size)]
    return cross, out


def mie_q(wl0, r_p, eps_p, mu_p=1 + 0j, eps_m=1 + 0j, mu_m=1 + 0j):
    """(Qsca, Qabs, Qext) of a sphere (``bdda_mie_q``)."""
    vals = [np.array([complex(v).real, complex(v).imag]) for v in (eps_p, mu_p, eps_m, mu_m)]
    q = np.zeros(3)
    _check(lib().bdda_mie_q(float(wl0), float(r_p), *[_dptr(v) for v in vals], _dptr(q)))
    return tuple(float(v) for v in q)


def format_result(wl0, cext, cabs, eper, volume, density, n, nocc, f, target_fname="", N_inc=None, wl0_index=0,
                  target_index=0, mper=1 + 0j, eper_medium=1 + 0j, mper_medium=1 + 0j, coat=None, solver_time=0.0,
                  mac_mie=True):
    """One result section of the reference's DDA_result.dat (``bdda_format_result``).

    eper / mper / volume / density are the particle's (or the core's when
    ``coat`` = (eper, mper, volume) is given)."""
    ce = np.ascontiguousarray(cext, dtype=np.float64)
    ca = np.ascontiguousarray(cabs, dtype=np.float64)
    r = ResultRecord()
    r.wl0_index, r.target_index, r.wl0 = int(wl0_index), int(target_index), float(wl0)
    r.N_inc = int(N_inc if N_inc is not None else ce.size)
    r.eper_medium[:] = [complex(eper_medium).real, complex(eper_medium).imag]
    r.mper_medium[:] = [complex(mper_medium).real, complex(mper_medium).imag]
    r.target_fname = target_fname.encode()
    r.is_homogeneous = 1 if coat is None else 0
    r.eper_core[:] = [complex(eper).real, complex(eper).imag]
    r.mper_core[:] = [complex(mper).real, complex(mper).imag]
    r.volume_core, r.density_core = float(volume), float(density)
    if coat is not None:
        r.eper_coat[:] = [complex(coat[0]).real, complex(coat[0]).imag]
        r.mper_coat[:] = [complex(coat[1]).real, complex(coat[1]).imag]
        r.volume_coat = float(coat[2])
    r.L, r.cext, r.cabs = int(ce.size), _dptr(ce), _dptr(ca)
    r.f, (r.nx, r.ny, r.nz), r.num_element_occupy = int(f), [int(v) for v in n], int(nocc)
    r.solver_time, r.append_mac_mie = float(solver_time), 1 if mac_mie else 0
    ln = ct.c_int()
    _check(lib().bdda_format_result(ct.byref(r), None, 0, ct.byref(ln)))
    buf = ct.create_string_buffer(ln.value + 1)
    _check(lib().bdda_format_result(ct.byref(r), buf, ln.value + 1, ct.byref(ln)))
    return buf.value.decode()
