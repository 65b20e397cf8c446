"""CPU-side checks of the C ABI: the library loads, exports every symbol that
include/lla_gb300.h declares, and answers the host-only questions (versions,
status strings, argument and shape errors that the reference raises before any
arithmetic) without a GPU.  Compute calls are not made here; on a machine
without a device they must fail loudly with LLA_ERR_NO_DEVICE rather than
fall back to the CPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "lla_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lla_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(lla):
    syms = header_symbols()
    assert len(syms) >= 23
    raw = ctypes.CDLL(lla.LIB_PATH)
    missing = [s for s in syms if not hasattr(raw, s)]
    assert not missing, missing


def test_python_bindings_cover_header(lla):
    declared = set(header_symbols())
    bound = set(lla.EXPORTS)
    assert bound <= declared, bound - declared


def test_version_and_status_strings(lla):
    assert b"sm_103a" in lla.lib.lla_version()
    assert lla.lib.lla_status_string(2) == b"matrix is not positive definite"
    assert lla.lib.lla_status_string(999) == b"unknown status"


def test_algorithm_option(lla):
    prev = lla.set_algorithm(lla.ALGO_FAST)
    assert lla.get_algorithm() == lla.ALGO_FAST
    lla.set_algorithm(prev)
    with pytest.raises(ValueError):
        lla.set_algorithm(7)


def test_shape_errors_precede_device_use(lla):
    """NotSquare / WrongRows (src/lib.rs:64-71, src/triangular.rs:102-108) are
    raised before any device work, as in the reference."""
    with pytest.raises(lla.NotSquare) as e:
        lla.cholesky(np.zeros((2, 3)))
    assert (e.value.rows, e.value.cols) == (2, 3)
    with pytest.raises(lla.NotSquare):
        lla.solvec(np.zeros((2, 3)), np.zeros((2, 3)))
    with pytest.raises(lla.NotSquare):
        lla.invc(np.zeros((3, 2)))
    with pytest.raises(lla.NotSquare):
        lla.solve_triangular(np.zeros((1, 2)), np.zeros((1, 2)), "lower")
    with pytest.raises(lla.WrongRows) as e:
        lla.solve_triangular(np.eye(2), np.zeros((1, 2)), "upper")
    assert (e.value.expected, e.value.actual) == (2, 1)
    assert not lla.is_triangular(np.zeros((2, 3)), "lower")
    with pytest.raises(lla.NotSquare):
        lla.triangular_inplace(np.zeros((3, 2)), "upper")


def test_empty_inputs_need_no_device(lla):
    e = np.zeros((0, 0))
    assert lla.cholesky(e).shape == (0, 0)
    assert lla.invc(e).shape == (0, 0)
    assert lla.solve_triangular(e, e, "upper").shape == (0, 0)
    assert lla.is_triangular(e, "lower") and lla.is_triangular(e, "upper")


def test_no_cpu_fallback_without_device(lla):
    if lla.device_count() > 0:
        pytest.skip("a device is present")
    with pytest.raises(lla.DeviceError) as e:
        lla.cholesky(np.eye(3))
    assert e.value.code == lla.ERR_NO_DEVICE
    with pytest.raises(lla.DeviceError):
        lla.solve_triangular(np.eye(3), np.ones((3, 1)), "lower")


def test_dtype_checks(lla):
    with pytest.raises(TypeError):
        lla.cholesky(np.eye(3, dtype=np.int64))
    with pytest.raises(TypeError):
        lla.solvec(np.eye(3), np.ones((3, 1), dtype=np.float32))
