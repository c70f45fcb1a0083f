"""Host-side validation of factors handed over through
gbchol_create_from_factor (no GPU: every check runs before any CUDA call).

The reference hands CHOLMOD's factor to kernels whose spin-waits are
unbounded (kernels/kernels.cu:20-21, 108-109, 176-177), so a malformed
factor there hangs the GPU. Here a factor whose structure could make a sweep
wait on a row that never comes is refused with GBCHOL_EINVAL first."""
import ctypes as C

import numpy as np
import pytest

from cholespy_gb300 import _ffi


def _create(gblib, n, perm, colptr, rowidx, store=_ffi.STORE_F64):
    perm = np.ascontiguousarray(perm, np.int32)
    colptr = np.ascontiguousarray(colptr, np.int32)
    rowidx = np.ascontiguousarray(rowidx, np.int32)
    vals = np.ones(max(len(rowidx), 1))
    h = C.c_void_p()
    st = gblib.gbchol_create_from_factor(n, perm.ctypes.data, colptr.ctypes.data, rowidx.ctypes.data,
                                         vals.ctypes.data, store, C.byref(h))
    return st, h


# A valid 3x3 pattern: L = [[x], [x, x], [x, x, x]] (CSC, diagonal first).
GOOD = dict(perm=[0, 1, 2], colptr=[0, 3, 5, 6], rowidx=[0, 1, 2, 1, 2, 2])

BAD = {
    "perm not a permutation": (dict(GOOD, perm=[0, 0, 2]), "permutation"),
    "perm out of range": (dict(GOOD, perm=[0, 1, 3]), "permutation"),
    "colptr[0] != 0": (dict(GOOD, colptr=[1, 3, 5, 6]), "colptr"),
    "empty column": (dict(GOOD, colptr=[0, 3, 3, 6], rowidx=[0, 1, 2, 1, 2, 2]), "diagonal"),
    "missing diagonal": (dict(GOOD, rowidx=[1, 1, 2, 1, 2, 2], colptr=[0, 1, 3, 4]), "diagonal"),
    "diagonal not first": (dict(GOOD, rowidx=[1, 0, 2, 1, 2, 2]), "diagonal"),
    "unsorted rows": (dict(GOOD, rowidx=[0, 2, 1, 1, 2, 2]), "sorted"),
    "duplicate row": (dict(GOOD, rowidx=[0, 1, 1, 1, 2, 2]), "sorted"),
    "row out of range": (dict(GOOD, rowidx=[0, 1, 3, 1, 2, 2]), "< n"),
}


@pytest.mark.parametrize("case", list(BAD))
def test_malformed_factor_refused(gblib, case):
    arrays, words = BAD[case]
    st, h = _create(gblib, 3, **arrays)
    assert st == _ffi.EINVAL, case
    assert not h.value
    assert words in _ffi.last_error(), (case, _ffi.last_error())


def test_bad_storage_flags_refused(gblib):
    st, _ = _create(gblib, 3, store=0, **GOOD)
    assert st == _ffi.EINVAL and "storage" in _ffi.last_error()
    st, _ = _create(gblib, 3, store=8 | _ffi.STORE_F32, **GOOD)
    assert st == _ffi.EINVAL


def test_null_arrays_refused(gblib):
    h = C.c_void_p()
    assert gblib.gbchol_create_from_factor(3, None, None, None, None, _ffi.STORE_F32, C.byref(h)) == _ffi.EINVAL
    assert gblib.gbchol_create_from_factor(-1, None, None, None, None, _ffi.STORE_F32, C.byref(h)) == _ffi.EINVAL
