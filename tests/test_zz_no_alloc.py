"""The allocation-free log-joint entry point, through the C ABI.

edg_glm_logjoint_grad_noalloc serves callers that cannot allocate device
memory when they call in (a host framework that owns all device memory in its
own pool, or an integration held to a fixed memory budget): its scratch is a
fixed array inside the library.  This file is named so that pytest collects
it last; it runs alone in a fresh process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def _model(cuda, N=3000, D=20, seed=0):
    from edward_gb300 import _lib
    rng = np.random.default_rng(seed)
    X = torch.as_tensor(rng.standard_normal((N, D)).astype(np.float32), device=cuda)
    y = torch.as_tensor((rng.random(N) < 0.4).astype(np.float32), device=cuda)
    loc = torch.full((D + 1,), 0.2, device=cuda)
    scale = torch.full((D + 1,), 1.5, device=cuda)
    g = _lib.EdgGLM()
    g.X, g.y, g.N, g.D, g.bias, g.lik, g.lik_scale = X.data_ptr(), y.data_ptr(), N, D, 1, 0, 1.0
    g.prior_loc, g.prior_scale = loc.data_ptr(), scale.data_ptr()
    return g, (X, y, loc, scale)


def _reference_call(lib, g, Z, B, P, cuda):
    from edward_gb300 import _lib
    ws_bytes = lib.edg_glm_logjoint_grad_workspace_bytes(ctypes.byref(g), B)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    lp = torch.empty(B, dtype=torch.float64, device=cuda)
    gr = torch.empty(B, P, device=cuda)
    _lib.call("edg_glm_logjoint_grad", ctypes.byref(g), _lib.ptr(Z), B, 1, 1.0, _lib.ptr(lp),
              _lib.ptr(gr), _lib.ptr(ws), ws_bytes, _lib.stream_ptr())
    return lp, gr


def test_no_alloc_matches_workspace_entry_point_twice(cuda):
    from edward_gb300 import _lib
    lib = _lib.load()
    g, keep = _model(cuda)
    P = 21
    for call, B in enumerate((70, 33)):     # two calls in a row, different shapes
        Z = torch.as_tensor(np.random.default_rng(10 + call).standard_normal((B, P))
                            .astype(np.float32) * 0.3, device=cuda)
        lp_ref, g_ref = _reference_call(lib, g, Z, B, P, cuda)
        lp = torch.full((B,), float("nan"), dtype=torch.float64, device=cuda)
        gr = torch.full((B, P), float("nan"), device=cuda)
        _lib.call("edg_glm_logjoint_grad_noalloc", ctypes.byref(g), _lib.ptr(Z), B, 1, 1.0,
                  _lib.ptr(lp), _lib.ptr(gr), _lib.stream_ptr())
        torch.cuda.synchronize()
        a, b = lp.cpu().numpy(), lp_ref.cpu().numpy()
        np.testing.assert_allclose(a, b, rtol=RTOL, atol=RTOL * np.abs(b).max())
        a, b = gr.cpu().numpy(), g_ref.cpu().numpy()
        np.testing.assert_allclose(a, b, rtol=RTOL, atol=RTOL * np.abs(b).max())


def test_no_alloc_rejects_oversized_call(cuda):
    from edward_gb300 import _lib
    lib = _lib.load()
    g, keep = _model(cuda, N=20000, D=60)
    B = 60000                                   # partial sums would need > 8 MiB
    Z = torch.zeros(B, 61, device=cuda)
    lp = torch.empty(B, dtype=torch.float64, device=cuda)
    rc = lib.edg_glm_logjoint_grad_noalloc(ctypes.byref(g), _lib.ptr(Z), B, 1, 1.0, _lib.ptr(lp),
                                           None, _lib.stream_ptr())
    assert rc == _lib.EDG_E_WORKSPACE
    assert b"fixed scratch" in lib.edg_last_error_string()
