"""GB300 (sm_103a) SPD factor-and-solve -- Python mirror of linfa-linalg's
`cholesky` and `triangular` trait methods over the C ABI in
include/lla_gb300.h.

Every function mirrors one reference method (src/cholesky.rs,
src/triangular.rs) with the same name, argument meaning, mutation and error
behaviour; numpy arrays play the role of ndarray views (any strides, including
negative and transposed ones).  All computation happens in the CUDA library
liblla_gb300.so: importing this module fails when the library has not been
built, and every compute call raises `DeviceError` when no GPU is present --
there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblla_gb300.so")

OK, NOT_SQUARE, NOT_POSITIVE_DEFINITE, WRONG_ROWS = 0, 1, 2, 3
ERR_CUDA, ERR_NO_MEMORY, ERR_INVALID_ARG, ERR_TIMEOUT, ERR_NO_DEVICE = 16, 17, 18, 19, 20
ERR_NOT_CONVERGED, ERR_BUSY = 21, 22
UPPER, LOWER = 0, 1
ALGO_AUTO, ALGO_EXACT, ALGO_FAST = 0, 1, 2


class LinalgError(Exception):
    """Mirror of linfa_linalg::LinalgError (src/lib.rs:33-60)."""


class NotSquare(LinalgError):
    def __init__(self, rows, cols):
        super().__init__(f"Matrix of ({rows}, {cols}) is not square")
        self.rows, self.cols = rows, cols


class NotPositiveDefinite(LinalgError):
    def __init__(self, index=None):
        super().__init__("Matrix is not positive definite")
        self.index = index


class WrongRows(LinalgError):
    def __init__(self, expected, actual):
        super().__init__(f"Matrix must have {expected} rows, not {actual}")
        self.expected, self.actual = expected, actual


class DeviceError(RuntimeError):
    """A device-side condition the reference cannot have (CUDA error, no
    device, out of memory, bounded wait timed out, ...)."""

    def __init__(self, code, cuda_error=0, msg=""):
        super().__init__(f"lla status {code} (cuda error {cuda_error}) {msg}".strip())
        self.code, self.cuda_error = code, cuda_error


class Error(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("cuda_error", ctypes.c_int32),
                ("rows", ctypes.c_int64), ("cols", ctypes.c_int64),
                ("expected", ctypes.c_int64), ("actual", ctypes.c_int64),
                ("index", ctypes.c_int64)]


class RefineOpts(ctypes.Structure):
    _fields_ = [("update", ctypes.c_int32), ("max_iters", ctypes.c_int32), ("tol", ctypes.c_double),
                ("equilibrate", ctypes.c_int32), ("fallback", ctypes.c_int32), ("update_epilogue", ctypes.c_int32),
                ("residual", ctypes.c_int32), ("substitution", ctypes.c_int32),
                ("update_kchunk", ctypes.c_int32)]


class RefineReport(ctypes.Structure):
    _fields_ = [("update", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("fell_back", ctypes.c_int32),
                ("factor_failed", ctypes.c_int32), ("schedule", ctypes.c_int32),
                ("backward_error", ctypes.c_double), ("backward_error0", ctypes.c_double),
                ("ms_factor", ctypes.c_double), ("ms_refine", ctypes.c_double),
                ("ms_fallback", ctypes.c_double), ("ms_total", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


UPDATE_FP32, UPDATE_BF16, UPDATE_BF16X3, UPDATE_BF16X6, UPDATE_FP16, UPDATE_FP16X3 = 0, 1, 3, 6, 11, 13
UPDATE_NAMES = {"fp32": 0, "bf16": 1, "bf16x3": 3, "bf16x6": 6, "fp16": 11, "fp16x3": 13}
RESIDUAL_NAMES = {"fp64": 0, "slices": 1}

_V = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
_E = ctypes.POINTER(Error)

EXPORTS = {
    "lla_set_algorithm": ([ctypes.c_int], ctypes.c_int),
    "lla_get_algorithm": ([], ctypes.c_int),
    "lla_device_count": ([], ctypes.c_int),
    "lla_version": ([], ctypes.c_char_p),
    "lla_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "lla_kernel_launches": ([], ctypes.c_int64),
    "lla_profile_start": ([], None),
    "lla_profile_stop": ([], ctypes.c_int),
    "lla_profile_query": ([ctypes.c_char_p, ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double)],
                          ctypes.c_int),
    "lla_profile_kernel_name": ([ctypes.c_int], ctypes.c_char_p),
    "lla_measure_peak_tflops": ([ctypes.c_int], ctypes.c_double),
    "lla_refine_opts_default": ([ctypes.POINTER(RefineOpts)], None),
    "lla_dposv_refined_device": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                  ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                  ctypes.POINTER(RefineOpts), ctypes.POINTER(RefineReport),
                                  ctypes.c_void_p, _E], ctypes.c_int),
    "lla_dposv_refined": (_V + _V + [ctypes.POINTER(RefineOpts), ctypes.POINTER(RefineReport), _E],
                          ctypes.c_int),
    "lla_spotrf_mixed_device": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_void_p, _E], ctypes.c_int),
    "lla_refine_autotune": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                             ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(RefineOpts),
                             ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, _E], ctypes.c_int),
    "lla_dresidual_device": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                              ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                              ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, _E],
                             ctypes.c_int),
    "lla_batch_plan_create": ([ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                               ctypes.POINTER(ctypes.c_void_p), _E], ctypes.c_int),
    "lla_batch_plan_destroy": ([ctypes.c_void_p], None),
    "lla_batch_plan_info": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                             ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                             ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "lla_batch_set_shape": ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "lla_batch_set_refined": ([ctypes.c_void_p, ctypes.c_int, _E], ctypes.c_int),
    "lla_dbatch_posv_device": ([ctypes.c_void_p] * 5 + [_E], ctypes.c_int),
    "lla_sbatch_posv_device": ([ctypes.c_void_p] * 5 + [_E], ctypes.c_int),
    "lla_batch_posv_graph": ([ctypes.c_void_p] * 5 + [_E], ctypes.c_int),
    "lla_batch_autotune": ([ctypes.c_void_p] * 5 + [ctypes.POINTER(ctypes.c_double), _E],
                           ctypes.c_int),
    "lla_serve_opts_default": ([ctypes.c_void_p], None),
    "lla_server_create": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), _E], ctypes.c_int),
    "lla_server_submit": ([ctypes.c_void_p, ctypes.c_void_p, _E], ctypes.c_int),
    "lla_server_poll": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                         ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
    "lla_server_drain": ([ctypes.c_void_p, ctypes.c_double], ctypes.c_int),
    "lla_server_release_factor": ([ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "lla_server_get_stats": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "lla_server_destroy": ([ctypes.c_void_p], None),
    "lla_device_status": ([ctypes.c_void_p, _E], ctypes.c_int),
    "lla_dtrsm_device_noalloc_status": ([ctypes.c_void_p, _E], ctypes.c_int),
    "lla_debug_inject_lost_handoff": ([ctypes.c_int64], ctypes.c_int),
}
for _p in "ds":
    EXPORTS.update({
        f"lla_{_p}cholesky_inplace": (_V + [ctypes.c_int, _E], ctypes.c_int),
        f"lla_{_p}solvec_inplace": (_V + _V + [_E], ctypes.c_int),
        f"lla_{_p}invc_inplace": (_V + [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, _E],
                                  ctypes.c_int),
        f"lla_{_p}solve_triangular_inplace": (_V + _V + [ctypes.c_int, _E], ctypes.c_int),
        f"lla_{_p}solve_triangular_diag": (_V + [ctypes.c_void_p] + _V + [ctypes.c_int, _E],
                                           ctypes.c_int),
        f"lla_{_p}triangular_inplace": (_V + [ctypes.c_int, _E], ctypes.c_int),
        f"lla_{_p}is_triangular": (_V + [ctypes.c_int, ctypes.POINTER(ctypes.c_int), _E],
                                   ctypes.c_int),
        f"lla_{_p}orthonormalize": (_V + _V + _V + [_E], ctypes.c_int),
        f"lla_{_p}apply_constraints": (_V + _V + _V + [_E], ctypes.c_int),
        f"lla_{_p}potrf_device": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_void_p, _E], ctypes.c_int),
        f"lla_{_p}triangular_device": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_int, ctypes.c_void_p, _E], ctypes.c_int),
        f"lla_{_p}is_triangular_device": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, _E], ctypes.c_int),
        f"lla_{_p}trsm_device": ([ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                  ctypes.c_void_p, _E], ctypes.c_int),
    })


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() "
                          "(the CUDA library is required: there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


lib = _load()


def _raise(e):
    c = e.code
    if c == OK:
        return
    if c == NOT_SQUARE:
        raise NotSquare(e.rows, e.cols)
    if c == NOT_POSITIVE_DEFINITE:
        raise NotPositiveDefinite(e.index)
    if c == WRONG_ROWS:
        raise WrongRows(e.expected, e.actual)
    raise DeviceError(c, e.cuda_error, lib.lla_status_string(c).decode())


def _prefix(a):
    if a.dtype == np.float64:
        return "d"
    if a.dtype == np.float32:
        return "s"
    raise TypeError(f"unsupported dtype {a.dtype} (f32 and f64, like NdFloat)")


def _view(a):
    if not isinstance(a, np.ndarray) or a.ndim != 2:
        raise TypeError("expected a 2-D numpy array")
    isz = a.itemsize
    rs, cs = a.strides
    if rs % isz or cs % isz:
        raise ValueError("strides must be multiples of the element size")
    return [ctypes.c_void_p(a.__array_interface__["data"][0]), a.shape[0], a.shape[1],
            rs // isz, cs // isz]


def _writable(a):
    if not a.flags.writeable:
        raise ValueError("array is read-only")


def _uplo(uplo):
    if isinstance(uplo, str):
        u = uplo.lower()
        if u not in ("upper", "lower"):
            raise ValueError(uplo)
        return UPPER if u == "upper" else LOWER
    if uplo not in (UPPER, LOWER):
        raise ValueError(uplo)
    return uplo


def _same_dtype(a, b):
    if a.dtype != b.dtype:
        raise TypeError("both arrays must have the same element type")


# ---- algorithm selection -------------------------------------------------

def set_algorithm(algo):
    """ALGO_EXACT (the reference's operation order, bit-identical results),
    ALGO_FAST (blocked FMA; errors still decided in exact order) or ALGO_AUTO
    (exact up to n = 1024).  Returns the previous setting."""
    prev = lib.lla_set_algorithm(int(algo))
    if prev < 0:
        raise ValueError(algo)
    return prev


def get_algorithm():
    return lib.lla_get_algorithm()


def device_count():
    return lib.lla_device_count()


def kernel_launches():
    """Kernels launched by the library since it was loaded."""
    return lib.lla_kernel_launches()


def profile_start():
    lib.lla_profile_start()


def profile_stop():
    """Returns {kernel: (total_ms, launches, work)} for kernels launched while profiling."""
    rc = lib.lla_profile_stop()
    if rc:
        raise DeviceError(rc)
    out = {}
    i = 0
    while True:
        name = lib.lla_profile_kernel_name(i)
        if name is None:
            break
        ms, cnt, work = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
        lib.lla_profile_query(name, ctypes.byref(ms), ctypes.byref(cnt), ctypes.byref(work))
        if cnt.value:
            out[name.decode()] = (ms.value, cnt.value, work.value)
        i += 1
    return out


def measure_peak_tflops(which):
    """0: FP64 tensor pipe (mma .f64), 1: DFMA, 2: FFMA -- measured on this GPU."""
    return lib.lla_measure_peak_tflops(which)


# ---- CholeskyInplace / Cholesky (src/cholesky.rs:16-115) -------------------

def cholesky_inplace_dirty(a):
    """CholeskyInplace::cholesky_inplace_dirty: A = L L^T in place, upper triangle untouched."""
    _writable(a)
    e = Error()
    getattr(lib, f"lla_{_prefix(a)}cholesky_inplace")(*_view(a), 1, ctypes.byref(e))
    _raise(e)
    return a


def cholesky_inplace(a):
    """CholeskyInplace::cholesky_inplace: in place, upper triangle zeroed."""
    _writable(a)
    e = Error()
    getattr(lib, f"lla_{_prefix(a)}cholesky_inplace")(*_view(a), 0, ctypes.byref(e))
    _raise(e)
    return a


def cholesky_into_dirty(a):
    return cholesky_inplace_dirty(a)


def cholesky_into(a):
    return cholesky_inplace(a)


def cholesky_dirty(a):
    """Cholesky::cholesky_dirty: factor of a copy (to_owned)."""
    return cholesky_inplace_dirty(np.array(a))


def cholesky(a):
    """Cholesky::cholesky: factor of a copy (to_owned)."""
    return cholesky_inplace(np.array(a))


# ---- SolveCInplace / SolveC / InverseC (src/cholesky.rs:117-199) ------------

def solvec_inplace(a, b):
    """SolveCInplace::solvec_inplace: b <- A^{-1} b; `a` keeps the dirty factor."""
    _writable(a)
    _writable(b)
    _same_dtype(a, b)
    e = Error()
    getattr(lib, f"lla_{_prefix(a)}solvec_inplace")(*_view(a), *_view(b), ctypes.byref(e))
    _raise(e)
    return b


def solvec_into(a, b):
    return solvec_inplace(a, b)


def solvec(a, b):
    """SolveC::solvec: solves into a copy of b (a is still used as scratch)."""
    return solvec_inplace(a, np.array(b))


def invc_inplace(a):
    """InverseCInplace::invc_inplace: returns A^{-1}; `a` keeps the dirty factor."""
    _writable(a)
    n = a.shape[0]
    out = np.zeros((n, n), dtype=a.dtype)
    e = Error()
    getattr(lib, f"lla_{_prefix(a)}invc_inplace")(*_view(a), ctypes.c_void_p(out.ctypes.data),
                                                  n, 1, ctypes.byref(e))
    _raise(e)
    return out


def invc(a):
    """InverseC::invc: inverse of a copy."""
    return invc_inplace(np.array(a))


# ---- triangular.rs ----------------------------------------------------------

def solve_triangular_inplace(a, b, uplo, diag=None):
    """SolveTriangularInplace::solve_triangular_inplace (src/triangular.rs:147-169);
    with `diag`, the crate-internal solve_triangular_system's diag_fn (:133-144)."""
    _writable(b)
    _same_dtype(a, b)
    e = Error()
    p = _prefix(a)
    if diag is None:
        getattr(lib, f"lla_{p}solve_triangular_inplace")(*_view(a), *_view(b), _uplo(uplo),
                                                         ctypes.byref(e))
    else:
        d = np.ascontiguousarray(diag, dtype=a.dtype)
        if d.shape != (min(a.shape),):
            raise ValueError("diag must have one entry per row")
        getattr(lib, f"lla_{p}solve_triangular_diag")(*_view(a), ctypes.c_void_p(d.ctypes.data),
                                                      *_view(b), _uplo(uplo), ctypes.byref(e))
    _raise(e)
    return b


def solve_triangular_into(a, b, uplo):
    return solve_triangular_inplace(a, b, uplo)


def solve_triangular(a, b, uplo):
    """SolveTriangular::solve_triangular: solves into a copy of b."""
    return solve_triangular_inplace(a, np.array(b), uplo)


def orthonormalize(v):
    """LOBPCG's Cholesky-QR `orthonormalize` (src/lobpcg/algorithm.rs:81-96):
    returns (U, L) with L = cholesky_into(V^T V) and U = V L^-T."""
    if not isinstance(v, np.ndarray) or v.ndim != 2:
        raise TypeError("expected a 2-D numpy array")
    n, k = v.shape
    u = np.empty((n, k), dtype=v.dtype)
    l = np.empty((k, k), dtype=v.dtype)
    e = Error()
    getattr(lib, f"lla_{_prefix(v)}orthonormalize")(*_view(v), *_view(u), *_view(l), ctypes.byref(e))
    _raise(e)
    return u, l


def apply_constraints(v, cholesky_yy, y):
    """LOBPCG's `apply_constraints` (src/lobpcg/algorithm.rs:63-76): v -= y U with
    cholesky_yy U = y^T v; updates v in place and returns it."""
    _writable(v)
    _same_dtype(v, y)
    _same_dtype(v, cholesky_yy)
    e = Error()
    getattr(lib, f"lla_{_prefix(v)}apply_constraints")(*_view(v), *_view(y), *_view(cholesky_yy),
                                                        ctypes.byref(e))
    _raise(e)
    return v


def triangular_inplace(a, uplo):
    """IntoTriangular::triangular_inplace (src/triangular.rs:37-53)."""
    _writable(a)
    e = Error()
    getattr(lib, f"lla_{_prefix(a)}triangular_inplace")(*_view(a), _uplo(uplo), ctypes.byref(e))
    _raise(e)
    return a


def into_triangular(a, uplo):
    return triangular_inplace(a, uplo)


def is_triangular(a, uplo):
    """Triangular::is_triangular (src/triangular.rs:67-90)."""
    e = Error()
    r = ctypes.c_int(0)
    getattr(lib, f"lla_{_prefix(a)}is_triangular")(*_view(a), _uplo(uplo), ctypes.byref(r),
                                                   ctypes.byref(e))
    _raise(e)
    return bool(r.value)


# ---- device-resident helpers (torch tensors; column-major = transposed view) ----

def _stream_ptr(stream):
    return ctypes.c_void_p(stream.cuda_stream if stream is not None else 0)


def _ld(T):
    """Leading dimension of a column-major (stride(0) == 1) tensor; a single
    column's stride is arbitrary in torch, so its leading dimension is n."""
    return T.stride(1) if T.shape[1] > 1 else max(1, T.shape[0])


def potrf_device(A, algo=ALGO_FAST, info=None, stream=None):
    """Cholesky of a column-major CUDA tensor in place.  `A` is a torch tensor
    whose transpose is contiguous (A.T.is_contiguous(), i.e. Fortran order);
    returns the device int64 info tensor (-1 = success, else failing row)."""
    import torch
    n = A.shape[0]
    assert A.is_cuda and A.shape == (n, n) and A.stride(0) == 1
    if info is None:
        info = torch.empty(1, dtype=torch.int64, device=A.device)
    e = Error()
    p = "d" if A.dtype == torch.float64 else "s"
    getattr(lib, f"lla_{p}potrf_device")(ctypes.c_void_p(A.data_ptr()), n, _ld(A), algo,
                                         ctypes.c_void_p(info.data_ptr()), _stream_ptr(stream),
                                         ctypes.byref(e))
    _raise(e)
    return info


def trsm_device(L, B, trans, algo=ALGO_FAST, stream=None):
    """Solves L X = B (trans=0) or L^T X = B (trans=1) in place on the
    column-major CUDA tensor B, with the lower factor in column-major L."""
    import torch
    n = L.shape[0]
    assert L.stride(0) == 1 and B.stride(0) == 1 and B.shape[0] == n
    e = Error()
    p = "d" if L.dtype == torch.float64 else "s"
    getattr(lib, f"lla_{p}trsm_device")(ctypes.c_void_p(L.data_ptr()), n, _ld(L), trans,
                                        ctypes.c_void_p(B.data_ptr()), B.shape[1], _ld(B), algo,
                                        _stream_ptr(stream), ctypes.byref(e))
    _raise(e)
    return B


def triangular_device(A, uplo, stream=None):
    """IntoTriangular::triangular_inplace on a column-major CUDA tensor in place
    (src/triangular.rs:37-53); NotSquare for a non-square tensor."""
    import torch
    assert A.is_cuda and A.dim() == 2 and (A.stride(0) == 1 or A.numel() == 0)
    e = Error()
    p = "d" if A.dtype == torch.float64 else "s"
    getattr(lib, f"lla_{p}triangular_device")(ctypes.c_void_p(A.data_ptr()), A.shape[0], A.shape[1],
                                              max(1, _ld(A) if A.shape[1] > 0 else A.shape[0]), _uplo(uplo),
                                              _stream_ptr(stream), ctypes.byref(e))
    _raise(e)
    return A


def is_triangular_device(A, uplo, result=None, stream=None):
    """Triangular::is_triangular on a column-major CUDA tensor (src/triangular.rs:67-90):
    returns a device int32 tensor holding 1 or 0 (no host round trip)."""
    import torch
    assert A.is_cuda and A.dim() == 2 and (A.stride(0) == 1 or A.numel() == 0)
    if result is None:
        result = torch.empty(1, dtype=torch.int32, device=A.device)
    e = Error()
    p = "d" if A.dtype == torch.float64 else "s"
    getattr(lib, f"lla_{p}is_triangular_device")(ctypes.c_void_p(A.data_ptr()), A.shape[0], A.shape[1],
                                                 max(1, _ld(A) if A.shape[1] > 0 else A.shape[0]),
                                                 _uplo(uplo), ctypes.c_void_p(result.data_ptr()),
                                                 _stream_ptr(stream), ctypes.byref(e))
    _raise(e)
    return result


def device_status(stream=None):
    """Synchronises `stream` and raises DeviceError(LLA_ERR_TIMEOUT) when a
    bounded wait of an asynchronous device call of this thread gave up since
    the last query (that call's result is not valid); clears the record."""
    e = Error()
    lib.lla_device_status(_stream_ptr(stream), ctypes.byref(e))
    _raise(e)


def debug_inject_lost_handoff(spin_limit=1000):
    """Test-only: the next triangular-solve launch loses its first block and its
    waits give up after `spin_limit` polls (see include/lla_gb300.h)."""
    rc = lib.lla_debug_inject_lost_handoff(int(spin_limit))
    if rc != OK:
        raise ValueError(spin_limit)


# ---- mixed-precision refined solve (no counterpart in the reference) --------

def refine_opts(update="bf16x6", max_iters=30, tol=1e-13, equilibrate=True, fallback=True, update_epilogue=0,
                residual="fp64", substitution="auto", update_kchunk=0):
    o = RefineOpts()
    lib.lla_refine_opts_default(ctypes.byref(o))
    o.substitution = {"auto": 0, "chain": 1, "lookback": 2}[substitution] if isinstance(substitution, str) \
        else int(substitution)
    o.update_kchunk = update_kchunk
    o.update = UPDATE_NAMES[update] if isinstance(update, str) else int(update)
    o.residual = RESIDUAL_NAMES[residual] if isinstance(residual, str) else int(residual)
    o.max_iters, o.tol = max_iters, tol
    o.equilibrate, o.fallback = int(bool(equilibrate)), int(bool(fallback))
    o.update_epilogue = update_epilogue
    return o


def posv_refined(a, b, **kw):
    """Solves A X = B (host numpy views; `a` read only, `b` overwritten with X)
    by the low-precision factorisation plus FP64 refinement; returns the report."""
    _writable(b)
    if a.dtype != np.float64 or b.dtype != np.float64:
        raise TypeError("the refined solve is f64")
    o, r, e = refine_opts(**kw), RefineReport(), Error()
    lib.lla_dposv_refined(*_view(a), *_view(b), ctypes.byref(o), ctypes.byref(r), ctypes.byref(e))
    _raise(e)
    return r.as_dict()


def posv_refined_device(A, B, X, stream=None, **kw):
    """Device form on column-major CUDA tensors (stride(0) == 1): A (n x n),
    B (n x m) read, X (n x m) written.  Returns the report."""
    n, m = A.shape[0], B.shape[1]
    assert A.stride(0) == 1 and B.stride(0) == 1 and X.stride(0) == 1
    o, r, e = refine_opts(**kw), RefineReport(), Error()
    lib.lla_dposv_refined_device(ctypes.c_void_p(A.data_ptr()), n, _ld(A),
                                 ctypes.c_void_p(B.data_ptr()), m, _ld(B),
                                 ctypes.c_void_p(X.data_ptr()), _ld(X),
                                 ctypes.byref(o), ctypes.byref(r), _stream_ptr(stream),
                                 ctypes.byref(e))
    _raise(e)
    return r.as_dict()


def refine_autotune(A, B, X, stream=None, **kw):
    """Per-shape autotuner of the refined solve's schedule (lla_refine_autotune):
    times the candidates on this system (column-major CUDA tensors as in
    posv_refined_device), records the winner in the autotune cache and returns
    ({"update_kchunk", "update_epilogue", "substitution"}, best_ms)."""
    n, m = A.shape[0], B.shape[1]
    assert A.stride(0) == 1 and B.stride(0) == 1 and X.stride(0) == 1
    o, e, ms = refine_opts(**kw), Error(), ctypes.c_double(0.0)
    lib.lla_refine_autotune(ctypes.c_void_p(A.data_ptr()), n, _ld(A), ctypes.c_void_p(B.data_ptr()), m, _ld(B),
                            ctypes.c_void_p(X.data_ptr()), _ld(X), ctypes.byref(o), ctypes.byref(ms),
                            _stream_ptr(stream), ctypes.byref(e))
    _raise(e)
    return ({"update_kchunk": o.update_kchunk, "update_epilogue": o.update_epilogue,
             "substitution": o.substitution}, ms.value)


def spotrf_mixed_device(A, update="bf16x6", info=None, stream=None):
    """Low-precision Cholesky of a column-major FP32 CUDA tensor in place (FP32
    diagonal blocks and panels, tensor-core trailing updates); returns the
    device int64 info tensor."""
    import torch
    n = A.shape[0]
    assert A.is_cuda and A.dtype == torch.float32 and A.stride(0) == 1
    if info is None:
        info = torch.empty(1, dtype=torch.int64, device=A.device)
    u = UPDATE_NAMES[update] if isinstance(update, str) else int(update)
    e = Error()
    lib.lla_spotrf_mixed_device(ctypes.c_void_p(A.data_ptr()), n, _ld(A), u,
                                ctypes.c_void_p(info.data_ptr()), _stream_ptr(stream), ctypes.byref(e))
    _raise(e)
    return info


# ---- batched solves of many small systems (no counterpart in the reference) --

class BatchPlan:
    """Packs `count` SPD systems (orders n[i] <= 256, m[i] <= 8 right-hand
    sides) into two device pools and solves them all in one persistent launch.
    Use pack() to copy host matrices into pools, solve() / solve_graph() to run,
    unpack_x() to read the solutions."""

    def __init__(self, n, m, dtype="f64"):
        self.n = np.ascontiguousarray(n, dtype=np.int32)
        self.m = np.ascontiguousarray(m, dtype=np.int32)
        self.count = len(self.n)
        self.elem = 8 if dtype in ("f64", np.float64) else 4
        self.np_dtype = np.float64 if self.elem == 8 else np.float32
        h = ctypes.c_void_p()
        e = Error()
        lib.lla_batch_plan_create(self.count, ctypes.c_void_p(self.n.ctypes.data),
                                  ctypes.c_void_p(self.m.ctypes.data), self.elem, ctypes.byref(h),
                                  ctypes.byref(e))
        _raise(e)
        self.h = h
        ae, be = ctypes.c_int64(), ctypes.c_int64()
        self.a_off = np.zeros(self.count, dtype=np.int64)
        self.b_off = np.zeros(self.count, dtype=np.int64)
        lib.lla_batch_plan_info(h, ctypes.byref(ae), ctypes.byref(be),
                                ctypes.c_void_p(self.a_off.ctypes.data),
                                ctypes.c_void_p(self.b_off.ctypes.data), None, None, None)
        self.a_elems, self.b_elems = ae.value, be.value

    def shape(self):
        c, t, f = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        lib.lla_batch_plan_info(self.h, None, None, None, None, ctypes.byref(c), ctypes.byref(t),
                                ctypes.byref(f))
        return {"ctas_per_sm": c.value, "threads": t.value, "flops": f.value}

    def set_shape(self, ctas_per_sm, threads):
        if lib.lla_batch_set_shape(self.h, ctas_per_sm, threads):
            raise ValueError((ctas_per_sm, threads))

    def set_refined(self, refined=True):
        """f64 plans: solve through an FP32 factorisation with per-system FP64
        refinement (A read only, B receives X), or back to plain FP64."""
        e = Error()
        lib.lla_batch_set_refined(self.h, int(bool(refined)), ctypes.byref(e))
        _raise(e)

    def pack(self, As, Bs):
        """Host pools (numpy) holding the column-major A_i and B_i."""
        ap = np.zeros(self.a_elems, dtype=self.np_dtype)
        bp = np.zeros(self.b_elems, dtype=self.np_dtype)
        for i, (a, b) in enumerate(zip(As, Bs)):
            n, m = self.n[i], self.m[i]
            ap[self.a_off[i]:self.a_off[i] + n * n] = np.asarray(a, self.np_dtype).ravel(order="F")
            bp[self.b_off[i]:self.b_off[i] + n * m] = np.asarray(b, self.np_dtype).ravel(order="F")
        return ap, bp

    def unpack_x(self, bp):
        return [np.asarray(bp[self.b_off[i]:self.b_off[i] + self.n[i] * self.m[i]]).reshape(
            (self.n[i], self.m[i]), order="F") for i in range(self.count)]

    def _call(self, name, dA, dB, info, stream):
        e = Error()
        getattr(lib, name)(self.h, ctypes.c_void_p(dA.data_ptr()), ctypes.c_void_p(dB.data_ptr()),
                           ctypes.c_void_p(info.data_ptr()), _stream_ptr(stream), ctypes.byref(e))
        _raise(e)

    def solve(self, dA, dB, info, stream=None):
        """dA, dB: device tensors of the pools; info: int32 device tensor (count)."""
        self._call("lla_dbatch_posv_device" if self.elem == 8 else "lla_sbatch_posv_device",
                   dA, dB, info, stream)

    def solve_graph(self, dA, dB, info, stream=None):
        self._call("lla_batch_posv_graph", dA, dB, info, stream)

    def autotune(self, dA, dB, info, stream=None):
        e = Error()
        ms = ctypes.c_double()
        lib.lla_batch_autotune(self.h, ctypes.c_void_p(dA.data_ptr()), ctypes.c_void_p(dB.data_ptr()),
                               ctypes.c_void_p(info.data_ptr()), _stream_ptr(stream),
                               ctypes.byref(ms), ctypes.byref(e))
        _raise(e)
        return ms.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib.lla_batch_plan_destroy(self.h)
                self.h = None
        except Exception:
            pass


# ---- serving loop (no counterpart in the reference) --------------------------

REQ_SOLVE, REQ_RESOLVE, REQ_TRSM = 0, 1, 2
PATH_NAMES = {1: "batched", 2: "mixed", 3: "fp64", 4: "kept_factor", 5: "trsm"}


class ServeOpts(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_double), ("slots", ctypes.c_int32),
                ("small_n", ctypes.c_int32), ("batch_max", ctypes.c_int32),
                ("device_ctas", ctypes.c_int32), ("batch_window_us", ctypes.c_double)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("dtype", ctypes.c_int32), ("n", ctypes.c_int64),
                ("m", ctypes.c_int64), ("A", ctypes.c_void_p), ("lda", ctypes.c_int64),
                ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64), ("tol", ctypes.c_double),
                ("factor_handle", ctypes.c_int64), ("keep_factor", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("user_tag", ctypes.c_uint64)]


class Result(ctypes.Structure):
    _fields_ = [("user_tag", ctypes.c_uint64), ("status", ctypes.c_int32), ("path", ctypes.c_int32),
                ("factor_handle", ctypes.c_int64), ("backward_error", ctypes.c_double),
                ("iterations", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("t_submit_us", ctypes.c_double), ("t_admit_us", ctypes.c_double),
                ("t_start_us", ctypes.c_double), ("t_done_us", ctypes.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}
        d["path"] = PATH_NAMES.get(self.path, self.path)
        return d


class ServerStats(ctypes.Structure):
    _fields_ = [("bytes_in_use", ctypes.c_double), ("bytes_peak", ctypes.c_double),
                ("queued", ctypes.c_int64), ("running", ctypes.c_int64),
                ("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("kept_factors", ctypes.c_int64), ("device_loop_launches", ctypes.c_int64)]


class Server:
    """Continuous-batching solve server over device-resident (column-major)
    CUDA tensors: small systems are served by a device-resident loop of
    persistent CTAs, large ones by concurrent streams.  submit() returns
    immediately; poll()/drain() collect results."""

    def __init__(self, hbm_budget_bytes=40e9, slots=6, small_n=256, batch_max=1024,
                 batch_window_us=2000.0, device_ctas=0):
        o = ServeOpts()
        lib.lla_serve_opts_default(ctypes.byref(o))
        o.hbm_budget_bytes, o.slots, o.small_n = hbm_budget_bytes, slots, small_n
        o.batch_max, o.batch_window_us, o.device_ctas = batch_max, batch_window_us, device_ctas
        h, e = ctypes.c_void_p(), Error()
        lib.lla_server_create(ctypes.byref(o), ctypes.byref(h), ctypes.byref(e))
        _raise(e)
        self.h = h
        self._keep = {}

    def submit(self, kind, A, B, tol=0.0, keep_factor=False, handle=0, tag=0):
        import torch
        assert A.stride(0) == 1 and B.stride(0) == 1
        r = Request()
        r.kind, r.dtype = kind, 8 if A.dtype == torch.float64 else 4
        r.n, r.m = A.shape[0], B.shape[1]
        r.A, r.lda = A.data_ptr(), _ld(A)
        r.B, r.ldb = B.data_ptr(), _ld(B)
        r.tol, r.factor_handle, r.keep_factor, r.user_tag = tol, handle, int(keep_factor), tag
        self._keep[tag] = (A, B)  # keep the tensors alive until the result is polled
        e = Error()
        lib.lla_server_submit(self.h, ctypes.byref(r), ctypes.byref(e))
        _raise(e)

    def poll(self, max_results=4096):
        buf = (Result * max_results)()
        got = ctypes.c_int()
        lib.lla_server_poll(self.h, buf, max_results, ctypes.byref(got))
        out = [buf[i].as_dict() for i in range(got.value)]
        for r in out:
            self._keep.pop(r["user_tag"], None)
        return out

    def drain(self, timeout_s=600.0):
        rc = lib.lla_server_drain(self.h, timeout_s)
        if rc:
            raise DeviceError(rc)

    def release(self, handle):
        rc = lib.lla_server_release_factor(self.h, handle)
        if rc:
            raise DeviceError(rc)

    def stats(self):
        st = ServerStats()
        lib.lla_server_get_stats(self.h, ctypes.byref(st))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "h", None):
            lib.lla_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def residual_device(A, X, B, R, method="fp64", stream=None):
    """R = B - A_sym X on column-major CUDA tensors (A_sym from A's lower triangle)."""
    n, m = A.shape[0], X.shape[1]
    e = Error()
    lib.lla_dresidual_device(ctypes.c_void_p(A.data_ptr()), n, _ld(A), ctypes.c_void_p(X.data_ptr()),
                             _ld(X), ctypes.c_void_p(B.data_ptr()), _ld(B),
                             ctypes.c_void_p(R.data_ptr()), _ld(R), m,
                             RESIDUAL_NAMES[method] if isinstance(method, str) else int(method),
                             _stream_ptr(stream), ctypes.byref(e))
    _raise(e)
    return R
