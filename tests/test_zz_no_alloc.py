"""The allocation-free split GEMM (``tnr_gemm_split_noalloc``) against the allocating one.

Some callers cannot call cudaMalloc: code that runs inside another allocator's arena (a
CUDA.jl memory pool, a server that has reserved all free HBM) or on a latency-critical
path where cudaMalloc's implicit device synchronisation would stall other streams.  The
entry point keeps its BF16 plane scratch in a file-scope device array instead; the
caller still owns A, B and C.  Its name sorts after every other test file, so pytest
collects it last; it must pass alone in a fresh process as well as after the rest of the
suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tnr():
    import __graft_entry__ as ge
    ge.build()
    return ge.package()


@pytest.fixture(scope="module")
def rt(tnr):
    tnr.lib()                      # loads the CUDA runtime the library links
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            lib = C.CDLL(name)
            break
        except OSError:
            lib = None
    if lib is None:
        pytest.skip("CUDA runtime library not found")
    lib.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    lib.cudaFree.argtypes = [C.c_void_p]
    lib.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    lib.cudaDeviceSynchronize.argtypes = []
    return lib


def to_device(rt, a):
    """Caller-owned device copy of a numpy matrix in column-major order."""
    f = np.asfortranarray(a, dtype=np.float64)
    p = C.c_void_p()
    assert rt.cudaMalloc(C.byref(p), f.nbytes) == 0
    assert rt.cudaMemcpy(p, f.ctypes.data, f.nbytes, 1) == 0      # host -> device
    return p, f.shape


def from_device(rt, p, shape):
    out = np.empty(shape, dtype=np.float64, order="F")
    assert rt.cudaMemcpy(out.ctypes.data, p, out.nbytes, 2) == 0  # device -> host
    return out


def noalloc_gemm(tnr, rt, A, B, ta, tb, alpha=1.0, beta=0.0, C0=None):
    """C = alpha op(A) op(B) + beta C0 through the allocation-free entry point; with beta = 0
    C starts as NaN, which the kernel must overwrite without reading."""
    m = A.shape[1] if ta else A.shape[0]
    k = A.shape[0] if ta else A.shape[1]
    n = B.shape[0] if tb else B.shape[1]
    dA, _ = to_device(rt, A)
    dB, _ = to_device(rt, B)
    dC, _ = to_device(rt, np.full((m, n), np.nan) if C0 is None else C0)
    err = C.create_string_buffer(512)
    try:
        st = tnr.lib().tnr_gemm_split_noalloc(int(ta), int(tb), m, n, k, alpha, dA, A.shape[0], dB, B.shape[0], beta,
                                              dC, m, None, err, 512)
        assert st == 0, err.value.decode()
        return from_device(rt, dC, (m, n))
    finally:
        for p in (dA, dB, dC):
            rt.cudaFree(p)


def test_noalloc_matches_allocating_entry_point(tnr, rt):
    rng = np.random.default_rng(11)
    # two calls in a row with different shapes: the shared scratch keeps the first call's
    # planes, the second call must not see them
    for m, n, k, ta, tb in [(300, 200, 77, False, True), (256, 512, 384, True, False), (192, 96, 48, False, False)]:
        A = rng.standard_normal((k, m) if ta else (m, k))
        B = rng.standard_normal((n, k) if tb else (k, n))
        got = noalloc_gemm(tnr, rt, A, B, ta, tb)
        ref = tnr.debug_gemm(A, B, ta, tb, tnr.PREC_SPLIT)      # existing (allocating) entry point
        assert np.isfinite(got).all()
        if k <= 64:
            # one accumulation in both entry points: the same kernel, the same result
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
        else:
            # the allocating entry point accumulates K in chunks of 64 (the contraction path)
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 6e-8 * np.sqrt(k)
        exact = (A.T if ta else A) @ (B.T if tb else B)
        assert np.linalg.norm(got - exact) / np.linalg.norm(exact) < 6e-8 * np.sqrt(k)


def test_noalloc_rejects_oversized_operands(tnr):
    err = C.create_string_buffer(512)
    # 6 * (m + n) * ceil8(k) bytes of planes must fit in 16 MiB; 2048^3 needs 48 MiB
    st = tnr.lib().tnr_gemm_split_noalloc(0, 0, 2048, 2048, 2048, 1.0, C.c_void_p(16), 2048, C.c_void_p(16), 2048,
                                          0.0, C.c_void_p(16), 2048, None, err, 512)
    assert st == 1
    assert b"16777216" in err.value


def test_noalloc_alpha_beta_epilogue(tnr, rt):
    """alpha != 1 and beta != 0 on a pre-filled, finite C: the epilogue reads C0 and writes
    alpha op(A) op(B) + beta C0; the product part agrees with the allocating entry point."""
    rng = np.random.default_rng(12)
    for m, n, k in [(128, 64, 40), (200, 136, 200)]:
        A, B = rng.standard_normal((m, k)), rng.standard_normal((k, n))
        C0 = rng.standard_normal((m, n))
        alpha, beta = -0.75, 1.5
        got = noalloc_gemm(tnr, rt, A, B, False, False, alpha, beta, C0)
        ref = tnr.debug_gemm(A, B, False, False, tnr.PREC_SPLIT)
        want = alpha * ref + beta * C0
        scale = np.linalg.norm(alpha * (A @ B)) + np.linalg.norm(beta * C0)
        tol = 1e-12 if k <= 64 else 6e-8 * np.sqrt(k)
        assert np.linalg.norm(got - want) / scale < tol
        exact = alpha * (A @ B) + beta * C0
        assert np.linalg.norm(got - exact) / scale < 6e-8 * np.sqrt(k)
