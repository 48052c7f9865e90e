"""The batched GEMM engines (tcgen05 3xTF32 and SIMT FP32) against FP64 NumPy,
over transposes, partial tiles, unaligned strides and K splits."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _op(X, ld, rows, cols, t, b, s):
    """op(X)[b] as an FP64 [rows, cols] matrix from flat storage."""
    flat = X[b * s:]
    if t:
        return np.stack([flat[k * ld:k * ld + rows] for k in range(cols)], axis=1)
    return np.stack([flat[m * ld:m * ld + cols] for m in range(rows)], axis=0)


CASES = [
    # M, N, K, ta, tb, lda, ldb, batch, kchunk
    (300, 200, 257, False, False, 260, 200, 3, 0),       # forward layer shape, partial tiles
    (257, 130, 96, False, True, 96, 96, 2, 0),           # dH W^T
    (257, 256, 4096, True, False, 260, 256, 2, 1024),    # weight gradient, K split
    (33, 256, 1000, True, False, 36, 260, 2, 0),         # narrow M, no split
    (130, 70, 33, False, False, 33, 71, 2, 0),           # unaligned ld: scalar loads
    (64, 40, 20, True, True, 65, 21, 1, 0),              # both transposed, unaligned
]


@pytest.mark.parametrize("M,N,K,ta,tb,lda,ldb,batch,kchunk", CASES)
@pytest.mark.parametrize("engine", ["tc", "simt"])
def test_gemm_matches_fp64(cuda, M, N, K, ta, tb, lda, ldb, batch, kchunk, engine):
    from edward_gb300 import ops
    rng = np.random.default_rng(M * 7 + N)
    arows, bcols = (K, lda) if ta else (M, lda), (N, ldb) if tb else (K, ldb)
    sA = arows[0] * arows[1] + 3          # odd batch strides
    sB = bcols[0] * bcols[1] + 5
    A = rng.standard_normal(sA * batch).astype(np.float32)
    B = rng.standard_normal(sB * batch).astype(np.float32)
    C = ops.gemm(torch.as_tensor(A, device=cuda), torch.as_tensor(B, device=cuda), M, N, K, ta, tb,
                 lda, ldb, batch, sA, sB, engine, kchunk).cpu().numpy()
    for b in range(batch):
        a = _op(A.astype(np.float64), lda, M, K, ta, b, sA)
        bb = _op(B.astype(np.float64), ldb, K, N, tb, b, sB)
        ref = a @ bb
        err = np.abs(C[b] - ref).max() / np.abs(ref).max()
        print(f"gemm {engine} M{M} N{N} K{K} ta{int(ta)} tb{int(tb)} b{b}: max rel err {err:.2e}")
        assert err < 1e-5, (b, err)


def test_gemm_tc_aligned_large(cuda):
    """A forward-layer shape of the Bayesian NN step (float4 paths, many tiles)."""
    from edward_gb300 import ops
    M, N, K, batch = 4096, 256, 257, 4
    rng = np.random.default_rng(0)
    A = torch.as_tensor(rng.standard_normal((batch, M, 260)).astype(np.float32), device=cuda)
    B = torch.as_tensor(rng.standard_normal((batch, K, N)).astype(np.float32), device=cuda)
    C = ops.gemm(A, B, M, N, K, lda=260, ldb=N, batch=batch, sA=M * 260, sB=K * N)
    ref = torch.bmm(A[:, :, :K].double(), B.double())
    err = ((C.double() - ref).abs().max() / ref.abs().max()).item()
    print(f"gemm tc large: max rel err {err:.2e}")
    assert err < 1e-5, err


def test_gemm_status_clean_after_gemm(cuda):
    """edg_gemm reports bounded-wait timeouts through edg_gemm_status; a normal
    call leaves the status at EDG_OK."""
    import ctypes
    from edward_gb300 import _lib, ops
    A = torch.randn(300, 64, device=cuda)
    B = torch.randn(64, 200, device=cuda)
    C = ops.gemm(A, B, 300, 200, 64)
    st = ctypes.c_int32(99)
    _lib.call("edg_gemm_status", ctypes.byref(st), _lib.stream_ptr())
    assert st.value == 0
    np.testing.assert_allclose(C[0].cpu().numpy(), (A @ B).cpu().numpy(), rtol=1e-4, atol=1e-3)


def test_bounded_wait_gives_up_and_context_survives(cuda):
    """A wait on an mbarrier that nothing completes gives up after about one
    second with EDG_E_TIMEOUT (the bounded wait of every tensor-core kernel);
    the CUDA context stays usable afterwards."""
    import ctypes
    import time
    from edward_gb300 import _lib, ops
    st = ctypes.c_int32(0)
    t0 = time.perf_counter()
    _lib.call("edg_check_bounded_wait", ctypes.byref(st), _lib.stream_ptr())
    dt = time.perf_counter() - t0
    assert st.value == _lib.EDG_E_TIMEOUT
    assert dt < 30.0
    A = torch.randn(128, 32, device=cuda)
    B = torch.randn(32, 64, device=cuda)
    C = ops.gemm(A, B, 128, 64, 32)
    torch.cuda.synchronize()
    np.testing.assert_allclose(C[0].cpu().numpy(), (A @ B).cpu().numpy(), rtol=1e-4, atol=1e-3)
