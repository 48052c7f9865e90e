"""Bayesian-NN KLqp step (batched forward + hand-written adjoint) against the
FP64 oracle and FP64 central finite differences, through the C ABI."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import bnn
from oracle.klqp import TFAdam

pytestmark = pytest.mark.gpu


def _setup(cuda, D, H1, H2, M, S, noise=0.3, dscale=2.5, prior=1.0, seed=0):
    from edward_gb300 import _lib
    lib = _lib.load()
    cfg = _lib.EdgBNN()
    cfg.D, cfg.H1, cfg.H2, cfg.n_samples = D, H1, H2, S
    cfg.noise, cfg.prior_scale, cfg.data_scale, cfg.seed = noise, prior, dscale, 17
    P = lib.edg_bnn_num_params(D, H1, H2)
    assert P == bnn.n_params(D, H1, H2)
    rng = np.random.default_rng(seed)
    X, y = bnn.synthetic(M, D, H1, H2, noise=0.1, seed=seed)
    mu = (rng.standard_normal(P) * 0.2).astype(np.float32)
    rho = (rng.standard_normal(P) * 0.2 - 2.0).astype(np.float32)
    eps = rng.standard_normal((S, P)).astype(np.float32)
    ws_bytes = lib.edg_bnn_workspace_bytes(ctypes.byref(cfg), M)
    t = {k: torch.as_tensor(v, device=cuda) for k, v in
         dict(X=X, y=y, mu=mu, rho=rho, eps=eps).items()}
    t["ws"] = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    t["slots"] = torch.zeros(4 * P, device=cuda)
    t["grad"] = torch.zeros(2 * P, device=cuda)
    t["state"] = _lib.new_state(cuda)
    return cfg, P, (X, y, mu, rho, eps), t, ws_bytes


def _step(cfg, t, M, ws_bytes, apply, opt=None):
    from edward_gb300 import _lib, train
    o = (opt or train.AdamOptimizer(0.01)).to_c()
    _lib.call("edg_bnn_klqp_step", ctypes.byref(cfg), ctypes.byref(o), _lib.ptr(t["X"]),
              _lib.ptr(t["y"]), M, _lib.ptr(t["mu"]), _lib.ptr(t["rho"]), _lib.ptr(t["slots"]),
              _lib.ptr(t["state"]), _lib.ptr(t["eps"]), _lib.ptr(t["grad"]), 1 if apply else 0,
              _lib.ptr(t["ws"]), ws_bytes, _lib.stream_ptr())
    torch.cuda.synchronize()


def close(a, b, rtol):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=rtol * np.abs(b).max())


@pytest.mark.parametrize("D,H1,H2,M,S", [(5, 24, 20, 70, 3), (32, 256, 256, 300, 4)])
def test_bnn_loss_and_gradient_parity(cuda, D, H1, H2, M, S):
    from edward_gb300 import _lib
    cfg, P, (X, y, mu, rho, eps), t, ws = _setup(cuda, D, H1, H2, M, S)
    _step(cfg, t, M, ws, apply=False)
    st = _lib.read_state(t["state"])
    loss, gmu, grho = bnn.klqp_loss_and_grads(mu, rho, eps, X, y, cfg.noise, cfg.data_scale,
                                              D, H1, H2, cfg.prior_scale)
    assert abs(st.loss - loss) <= 1e-5 * abs(loss)
    g = t["grad"].cpu().numpy()
    close(g[:P], gmu, 2e-5)
    close(g[P:], grho, 2e-5)


def test_bnn_gradient_vs_fp64_finite_differences(cuda):
    """The hand-written adjoint against FP64 central differences of the loss."""
    D, H1, H2, M, S = 4, 9, 7, 33, 2
    cfg, P, (X, y, mu, rho, eps), t, ws = _setup(cuda, D, H1, H2, M, S, seed=3)
    _step(cfg, t, M, ws, apply=False)
    g = t["grad"].cpu().numpy().astype(np.float64)
    h = 1e-6
    args = (X, y, cfg.noise, cfg.data_scale, D, H1, H2, cfg.prior_scale)
    mu64, rho64 = mu.astype(np.float64), rho.astype(np.float64)
    for p in range(0, P, 3):
        a, b = mu64.copy(), mu64.copy()
        a[p] += h
        b[p] -= h
        fd = (bnn.klqp_loss_and_grads(a, rho64, eps, *args)[0] -
              bnn.klqp_loss_and_grads(b, rho64, eps, *args)[0]) / (2 * h)
        assert abs(fd - g[p]) <= 2e-5 * max(1.0, abs(fd)), (p, fd, g[p])
        a, b = rho64.copy(), rho64.copy()
        a[p] += h
        b[p] -= h
        fd = (bnn.klqp_loss_and_grads(mu64, a, eps, *args)[0] -
              bnn.klqp_loss_and_grads(mu64, b, eps, *args)[0]) / (2 * h)
        assert abs(fd - g[P + p]) <= 2e-5 * max(1.0, abs(fd)), (p, fd, g[P + p])


def test_bnn_adam_steps(cuda):
    """Three fused steps with Adam equal the oracle gradient + TF Adam."""
    from edward_gb300 import _lib
    D, H1, H2, M, S = 6, 16, 12, 64, 2
    cfg, P, (X, y, mu, rho, eps), t, ws = _setup(cuda, D, H1, H2, M, S, seed=5)
    opt = TFAdam(2 * P)
    th = np.concatenate([mu, rho]).astype(np.float64)
    for k in range(3):
        _step(cfg, t, M, ws, apply=True)
        _, gmu, grho = bnn.klqp_loss_and_grads(th[:P], th[P:], eps, X, y, cfg.noise,
                                               cfg.data_scale, D, H1, H2, cfg.prior_scale)
        th = opt.apply(th, np.concatenate([gmu, grho]), 0.01)
        got = torch.cat([t["mu"], t["rho"]]).cpu().numpy()
        close(got, th, 5e-5)
    assert _lib.read_state(t["state"]).t == 3
