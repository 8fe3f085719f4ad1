"""bem_dense_solve_noalloc: the dense solve for callers that cannot allocate
device memory (their application owns all device memory through its own pool
allocator, or cudaMalloc's implicit synchronization is not acceptable where
they call from).  Its result must match the allocating bem_dense_solve on the
same input, call after call, although every call shares one fixed scratch
array that keeps the previous call's contents.  Kept in a file of its own that
pytest collects last."""
import ctypes

import numpy as np
import pytest

from conftest import normwise

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def L():
    import bemuse_gb300
    bemuse_gb300.build.build()
    lib = bemuse_gb300.lib()
    lib.bem_dense_solve_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _dp]
    lib.bem_dense_solve_noalloc.restype = ctypes.c_int
    return lib


def _system(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    A = 0.5 * np.eye(n) + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    B = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    return np.ascontiguousarray(A), np.ascontiguousarray(B)


def _noalloc(L, A, B):
    X = np.array(B, dtype=np.complex128, order="C")
    st = L.bem_dense_solve_noalloc(0, A.shape[0], A.view(np.float64).ctypes.data_as(_dp), X.shape[1],
                                   X.view(np.float64).ctypes.data_as(_dp))
    return st, X


def test_noalloc_matches_allocating_solve_twice_in_a_row(L):
    import bemuse_gb300 as bg
    # a larger system first, then a smaller one that reuses the same scratch
    for n, nrhs, seed in ((300, 9, 1), (200, 5, 2)):
        A, B = _system(n, nrhs, seed)
        st, X = _noalloc(L, A, B)
        assert st == 0, L.bem_last_error(None)
        ref, _, _ = bg.dense_solve(A, B, bg.PLAIN_FP64)
        assert normwise(X, ref) < 1e-11
        assert normwise(X, np.linalg.solve(A, B)) < 1e-11


def _free_device_bytes():
    """cudaMemGetInfo's free bytes on the current device, through the CUDA runtime the
    library itself loaded (libcudart.so.13)."""
    rt = ctypes.CDLL("libcudart.so.13")
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_call_allocates_no_device_memory(L):
    # after one call (which, with lazy module loading, is when the scratch array
    # itself is reserved) a further call leaves the free device memory unchanged
    A, B = _system(400, 7, 4)
    st, _ = _noalloc(L, A, B)
    assert st == 0, L.bem_last_error(None)
    before = _free_device_bytes()
    st, X = _noalloc(L, A, B)
    after = _free_device_bytes()
    assert st == 0, L.bem_last_error(None)
    assert after == before, (before, after)
    assert normwise(X, np.linalg.solve(A, B)) < 1e-11


def test_noalloc_rejects_orders_beyond_its_scratch(L):
    A, B = _system(8, 1, 3)
    big = np.zeros((513, 513), np.complex128)
    st = L.bem_dense_solve_noalloc(0, 513, big.view(np.float64).ctypes.data_as(_dp), 1,
                                   B.view(np.float64).ctypes.data_as(_dp))
    assert st == 1  # BEM_ERR_ARG
    assert b"513" in L.bem_last_error(None)
