"""ctypes front end of the CPU oracle (oracle/lla_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker.  The shipped library never imports
it.  Each function mirrors one reference trait method (citations in
lla_oracle.c) and mutates its numpy arguments in place, exactly as the Rust
`&mut` methods do; numpy views with any strides (negative, transposed) are
passed through unchanged as (ptr, rows, cols, row_stride, col_stride).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblla_oracle.so")

OK, NOT_SQUARE, NOT_POSITIVE_DEFINITE, WRONG_ROWS = 0, 1, 2, 3
UPPER, LOWER = 0, 1


class Error(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int32), ("cuda_error", ctypes.c_int32),
                ("rows", ctypes.c_int64), ("cols", ctypes.c_int64),
                ("expected", ctypes.c_int64), ("actual", ctypes.c_int64),
                ("index", ctypes.c_int64)]

    def as_dict(self):
        d = {"code": self.code}
        if self.code == NOT_SQUARE:
            d.update(rows=self.rows, cols=self.cols)
        elif self.code == WRONG_ROWS:
            d.update(expected=self.expected, actual=self.actual)
        elif self.code == NOT_POSITIVE_DEFINITE:
            d.update(index=self.index)
        return d


def build():
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_V = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
_E = ctypes.POINTER(Error)


def _declare(L):
    for p in "ds":
        getattr(L, f"ora_{p}cholesky_inplace_dirty").argtypes = _V + [_E]
        getattr(L, f"ora_{p}cholesky_inplace").argtypes = _V + [_E]
        getattr(L, f"ora_{p}triangular_inplace").argtypes = _V + [ctypes.c_int, _E]
        getattr(L, f"ora_{p}is_triangular").argtypes = _V + [ctypes.c_int]
        getattr(L, f"ora_{p}solve_triangular_system").argtypes = (
            _V + [ctypes.c_void_p] + _V + [ctypes.c_int, _E])
        getattr(L, f"ora_{p}solvec_inplace").argtypes = _V + _V + [_E]
        getattr(L, f"ora_{p}invc_inplace").argtypes = _V + [ctypes.c_void_p, ctypes.c_int64,
                                                            ctypes.c_int64, _E]
    L.ora_build_info.restype = ctypes.c_char_p


def view(a):
    """(ptr to element [0,0], rows, cols, row_stride, col_stride) of a 2-D numpy view."""
    assert a.ndim == 2 and a.dtype in (np.float64, np.float32)
    isz = a.itemsize
    rs, cs = a.strides
    assert rs % isz == 0 and cs % isz == 0
    return [ctypes.c_void_p(a.__array_interface__["data"][0]), a.shape[0], a.shape[1],
            rs // isz, cs // isz]


def _p(a):
    return "d" if a.dtype == np.float64 else "s"


def _uplo(u):
    if isinstance(u, str):
        return UPPER if u.lower() == "upper" else LOWER
    return u


def cholesky_inplace_dirty(a):
    e = Error()
    getattr(lib(), f"ora_{_p(a)}cholesky_inplace_dirty")(*view(a), ctypes.byref(e))
    return e.as_dict()


def cholesky_inplace(a):
    e = Error()
    getattr(lib(), f"ora_{_p(a)}cholesky_inplace")(*view(a), ctypes.byref(e))
    return e.as_dict()


def triangular_inplace(a, uplo):
    e = Error()
    getattr(lib(), f"ora_{_p(a)}triangular_inplace")(*view(a), _uplo(uplo), ctypes.byref(e))
    return e.as_dict()


def is_triangular(a, uplo):
    return bool(getattr(lib(), f"ora_{_p(a)}is_triangular")(*view(a), _uplo(uplo)))


def solve_triangular_inplace(a, b, uplo, diag=None):
    e = Error()
    dptr = None
    if diag is not None:
        diag = np.ascontiguousarray(diag, dtype=a.dtype)
        dptr = ctypes.c_void_p(diag.ctypes.data)
    getattr(lib(), f"ora_{_p(a)}solve_triangular_system")(*view(a), dptr, *view(b),
                                                           _uplo(uplo), ctypes.byref(e))
    return e.as_dict()


def solvec_inplace(a, b):
    e = Error()
    getattr(lib(), f"ora_{_p(a)}solvec_inplace")(*view(a), *view(b), ctypes.byref(e))
    return e.as_dict()


def invc_inplace(a):
    """Returns (status dict, inverse as a C-order array of shape (rows, rows))."""
    e = Error()
    out = np.zeros((a.shape[0], a.shape[0]), dtype=a.dtype)
    getattr(lib(), f"ora_{_p(a)}invc_inplace")(*view(a), ctypes.c_void_p(out.ctypes.data),
                                                out.shape[0], 1, ctypes.byref(e))
    return e.as_dict(), out


def build_info():
    return lib().ora_build_info().decode()


def orthonormalize(v):
    """LOBPCG's Cholesky-QR (src/lobpcg/algorithm.rs:81-96) composed from the
    restated path: G = V^T V (ndarray's `dot`, i.e. the matrixmultiply crate,
    is not part of this restatement: numpy's product stands in for it, so G
    matches the reference to rounding), L = cholesky_into(G)
    (src/cholesky.rs:24-43), U = solve_triangular_into(V^T, Lower)^T
    (src/triangular.rs:161-168).  Returns (status dict, U, L)."""
    g = np.array(v.T @ v, order="C")
    st = cholesky_inplace(g)
    if st["code"] != 0:
        return st, None, None
    vt = np.array(v.T, order="C")
    st = solve_triangular_inplace(g, vt, "lower")
    return st, np.array(vt.T), g
