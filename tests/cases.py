"""Seeded input generators that restate the reference's proptest strategies.

tests/common.rs:9-95 draws f64 entries uniformly from -100..=100
(FLOAT_RANGE, :9), dimensions from 1..=10 (DIM_RANGE, :10), and applies a
random Layout (:12-33): invert the row axis, invert the column axis and/or
transpose the backing array, so every property test also runs on negative
strides and column-major views.  tests/cholesky.rs:9-19 builds SPD inputs as
A^T A + I; tests/triangular.rs:9-20 masks a random square matrix to one
triangle and replaces diagonal entries with |d| < 1 by 1.  The reference
draws fresh proptest cases each run (no pinned seed), so these generators use
their own numpy seeds.
"""
import json
import os

import numpy as np

FLOAT_RANGE = (-100.0, 100.0)
DIM_RANGE = (1, 10)
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kats():
    with open(os.path.join(GOLDEN, "reference_kats.json")) as f:
        return json.load(f)["cases"]


def kat(name):
    for c in kats():
        if c["name"] == name:
            return c
    raise KeyError(name)


def apply_layout(arr, rng, allow_transpose=True):
    """Layout::apply (tests/common.rs:20-33): same logical values are NOT
    preserved -- like the reference, the layout changes which matrix is
    tested; it is applied before the matrix is used to build the system."""
    if rng.random() < 0.5:
        arr = arr[::-1, :]
    if rng.random() < 0.5:
        arr = arr[:, ::-1]
    if allow_transpose and arr.shape[0] == arr.shape[1] and rng.random() < 0.5:
        arr = arr.T
    return arr


def matrix(rng, rows, cols, dtype=np.float64):
    data = rng.uniform(FLOAT_RANGE[0], FLOAT_RANGE[1], size=(rows, cols)).astype(dtype)
    return apply_layout(data, rng, allow_transpose=(rows == cols))


def square(rng, dtype=np.float64):
    n = int(rng.integers(DIM_RANGE[0], DIM_RANGE[1] + 1))
    return matrix(rng, n, n, dtype)


def relayout(m, rng):
    """Same logical values, random memory layout: C or F order, each axis
    optionally stored reversed (negative stride)."""
    store = np.array(m, order="F" if rng.random() < 0.5 else "C")
    if rng.random() < 0.5:
        store = np.array(store[::-1, :], order="C")[::-1, :]
    if rng.random() < 0.5:
        store = np.array(store[:, ::-1], order="F")[:, ::-1]
    assert np.array_equal(store, m, equal_nan=True)
    return store


def hpd(rng, dtype=np.float64):
    """hpd_arr (tests/cholesky.rs:9-19): A^T A + I from a layout-randomised
    square_arr; the result is then stored in a random memory layout (the
    reference's own result is standard layout; the extra relayout exercises
    strided views on the factor path too)."""
    a = square(rng, np.float64)
    m = a.T @ a + np.eye(a.shape[0])
    return relayout(np.array(m, dtype=dtype), rng)


def system(rng, a, dtype=np.float64):
    """system_of_arr (tests/common.rs:83-95): x has a.ncols rows and 1..=10 columns."""
    cols = int(rng.integers(DIM_RANGE[0], DIM_RANGE[1] + 1))
    return matrix(rng, a.shape[1], cols, dtype)


def tri(rng, uplo, dtype=np.float64):
    """tri_system's matrix (tests/triangular.rs:9-20)."""
    a = square(rng, dtype)  # a strided view with a random layout, masked in place
    n = a.shape[0]
    if uplo == "upper":
        a[np.tril_indices(n, -1)] = 0
    else:
        a[np.triu_indices(n, 1)] = 0
    d = np.diag(a).copy()
    d[np.abs(d) < 1.0] = 1.0
    a[np.diag_indices(n)] = d
    return a


def spd_gram(rng, n, dtype=np.float64):
    """The single-matrix workload's construction: A = G G^T / n + I, G ~ N(0,1)."""
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + np.eye(n)
    return a.astype(dtype)


def same_layout_copy(src, like):
    """Copy of `src` (C order values) stored with the memory layout of `like`."""
    out = np.empty_like(like)
    out[...] = src
    return out
