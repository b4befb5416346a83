"""afp_matrix_vmult_noalloc, the y = A x entry point that allocates no device
memory.  It serves callers that cannot let the library allocate on the device
when they call it (an application that reserved the device for its own
memory arena, a process under a hard device-memory cap, a time-step loop
whose allocator must not grow).  It stages x and y in a fixed static device
array instead of per-call buffers, so it must agree with afp_matrix_vmult
call after call, whatever an earlier call left in that array, and refuse
matrices larger than the array.

The file name makes pytest collect it after every other test file; it also
passes when run on its own.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIMIT = 1 << 21  # AFP_NOALLOC_MAX_ENTRIES


def _call(native, name, A, x, y):
    st = getattr(native, name)(A.handle, C.c_void_p(x.ctypes.data), C.c_void_p(y.ctypes.data))
    return st


def _vmult(native, name, A, x):
    y = np.full(A.m(), np.nan)
    st = _call(native, name, A, x, y)
    assert st == 0, native.afp_last_error()
    return y


def test_noalloc_vmult_matches_vmult_on_consecutive_calls(native, ctx):
    from afepack_gb300 import workloads as W
    from afepack_gb300.fem import Space, assemble
    wl = W.poisson3d_p1(12)
    K, M = assemble(Space(ctx, wl.space), wl.acc_stiff, wl.acc_mass)
    small = W.poisson2d_p1(8)
    Ks, _ = assemble(Space(ctx, small.space), small.acc_stiff, small.acc_mass)
    rng = np.random.default_rng(11)
    # two calls in a row on each matrix with different x, then a smaller
    # matrix after the larger ones (the array keeps the previous contents)
    for A in (K, K, M, M, Ks, Ks):
        x = rng.standard_normal(A.n())
        ref = _vmult(native, "afp_matrix_vmult", A, x)
        got = _vmult(native, "afp_matrix_vmult_noalloc", A, x)
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())


def test_noalloc_vmult_device_pointers(native, ctx):
    import torch
    from afepack_gb300.fem import SparseMatrix
    n = 1000
    d = np.linspace(1.0, 2.0, n)
    A = SparseMatrix.from_csr(ctx, np.arange(n + 1), np.arange(n), d)
    x = torch.arange(n, dtype=torch.float64, device="cuda")
    y = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    st = native.afp_matrix_vmult_noalloc(A.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()))
    assert st == 0, native.afp_last_error()
    assert np.allclose(y.cpu().numpy(), np.arange(n) * d, rtol=1e-15)


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        try:
            return C.CDLL(f"{d}/libcudart.so")
        except OSError:
            continue
    pytest.skip("no shared CUDA runtime to read the memory pool with")


USED_MEM_HIGH, USED_MEM_CURRENT = 8, 7  # cudaMemPoolAttrUsedMemHigh / UsedMemCurrent


def _pool_high_after(rt, pool, fn):
    """Peak bytes in use from the device's default stream-ordered pool while fn
    runs, above what was in use before (the pool serves cudaMallocAsync, the
    library's device allocator)."""
    import torch
    torch.cuda.synchronize()
    zero = C.c_uint64(0)
    assert rt.cudaMemPoolSetAttribute(pool, USED_MEM_HIGH, C.byref(zero)) == 0
    cur0, high = C.c_uint64(0), C.c_uint64(0)
    assert rt.cudaMemPoolGetAttribute(pool, USED_MEM_CURRENT, C.byref(cur0)) == 0
    fn()
    torch.cuda.synchronize()
    assert rt.cudaMemPoolGetAttribute(pool, USED_MEM_HIGH, C.byref(high)) == 0
    return high.value - cur0.value


def test_noalloc_vmult_allocates_nothing(native, ctx):
    """The promise itself: after the context exists, calls neither take bytes
    from the device's stream-ordered pool (which the ordinary vmult does, the
    control below) nor change the device's free memory."""
    import torch
    from afepack_gb300 import workloads as W
    from afepack_gb300.fem import Space, assemble
    wl = W.poisson2d_p1(64)
    K, _ = assemble(Space(ctx, wl.space), wl.acc_stiff, wl.acc_mass)
    x = np.random.default_rng(5).standard_normal(K.n())
    y = np.zeros(K.m())
    rt = _cudart()
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), 0) == 0
    assert _pool_high_after(rt, pool, lambda: _vmult(native, "afp_matrix_vmult", K, x)) > 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    grew = _pool_high_after(rt, pool, lambda: [_call(native, "afp_matrix_vmult_noalloc", K, x, y) for _ in range(3)])
    free1, _ = torch.cuda.mem_get_info()
    assert grew == 0
    assert free1 == free0


def test_noalloc_vmult_refuses_matrices_above_the_limit(native, ctx):
    from afepack_gb300.fem import SparseMatrix
    n = LIMIT + 1
    A = SparseMatrix.from_csr(ctx, np.arange(n + 1), np.arange(n), np.ones(n))
    x = np.ones(n)
    y = np.zeros(n)
    st = _call(native, "afp_matrix_vmult_noalloc", A, x, y)
    assert st == 9  # AFP_ERR_UNSUPPORTED, before anything is copied
    assert b"AFP_NOALLOC_MAX_ENTRIES" in native.afp_last_error()
    assert not y.any()
