"""Bayesian-NN KLqp step (batched forward + hand-written adjoint) against the
FP64 oracle and FP64 central finite differences, through the C ABI."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import bnn
from oracle.klqp import TFAdam

pytestmark = pytest.mark.gpu


def _setup(cuda, D, H1, H2, M, S, noise=0.3, dscale=2.5, prior=1.0, seed=0, engine=0):
    from edward_gb300 import _lib
    lib = _lib.load()
    cfg = _lib.EdgBNN()
    cfg.D, cfg.H1, cfg.H2, cfg.n_samples = D, H1, H2, S
    cfg.gemm_engine = engine
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


ENGINES = pytest.mark.parametrize("engine", [0, 1], ids=["tc", "simt"])


@pytest.mark.parametrize("D,H1,H2,M,S", [(5, 24, 20, 70, 3), (32, 256, 256, 300, 4),
                                         (32, 256, 256, 4096, 2)])
@ENGINES
def test_bnn_loss_and_gradient_parity(cuda, D, H1, H2, M, S, engine):
    from edward_gb300 import _lib
    cfg, P, (X, y, mu, rho, eps), t, ws = _setup(cuda, D, H1, H2, M, S, engine=engine)
    _step(cfg, t, M, ws, apply=False)
    st = _lib.read_state(t["state"])
    loss, gmu, grho = bnn.klqp_loss_and_grads(mu, rho, eps, X, y, cfg.noise, cfg.data_scale,
                                              D, H1, H2, cfg.prior_scale)
    assert abs(st.loss - loss) <= 1e-5 * abs(loss)
    g = t["grad"].cpu().numpy()
    close(g[:P], gmu, 1e-5)
    close(g[P:], grho, 1e-5)


@ENGINES
def test_bnn_gradient_vs_fp64_finite_differences(cuda, engine):
    """The hand-written adjoint against FP64 central differences of the loss."""
    D, H1, H2, M, S = 4, 9, 7, 33, 2
    cfg, P, (X, y, mu, rho, eps), t, ws = _setup(cuda, D, H1, H2, M, S, seed=3, engine=engine)
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


@ENGINES
def test_bnn_adam_steps(cuda, engine):
    """Three fused steps with Adam equal the oracle gradient + TF Adam."""
    from edward_gb300 import _lib
    D, H1, H2, M, S = 6, 16, 12, 64, 2
    cfg, P, (X, y, mu, rho, eps), t, ws = _setup(cuda, D, H1, H2, M, S, seed=5, engine=engine)
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


# ------------------------------------------------------------- public API

def _oracle_args(inf, X, y, scale):
    spec = inf._spec
    return (X, y, spec.noise, scale, spec.D, spec.H1, spec.H2, spec.prior_scale)


def test_bnn_klqp_api_full_batch_matches_oracle(cuda):
    """ed.KLqp on the network of examples/bayesian_nn.py: the loss and gradients
    for given draws, then two update() calls with in-kernel Philox draws, against
    the oracle with the same draws and TF's Adam."""
    import edward_gb300 as ed
    from bnn_model import example_model, example_q, flat_q
    from oracle import philox
    D, H1, H2, N, S = 3, 12, 9, 57, 3
    X, y = bnn.synthetic(N, D, H1, H2, seed=11)
    latents, _, yrv = example_model(D, H1, H2, X=X, noise=0.2)
    qs = example_q(latents, np.random.default_rng(1))
    inf = ed.KLqp(qs, data={yrv: y})
    inf.initialize(n_samples=S, optimizer=ed.train.AdamOptimizer(0.01))
    mu, rho = flat_q(qs, latents, "loc"), flat_q(qs, latents, "scale")
    P = mu.size
    args = _oracle_args(inf, X, y, 1.0)
    eps = np.random.default_rng(2).standard_normal((S, P)).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    l0, m0, r0 = bnn.klqp_loss_and_grads(mu, rho, eps, *args)
    assert abs(loss - l0) <= 1e-5 * abs(l0)
    close(gmu.cpu().numpy(), m0, 1e-5)
    close(grho.cpu().numpy(), r0, 1e-5)
    opt = TFAdam(2 * P)
    th = np.concatenate([mu, rho]).astype(np.float64)
    for t in range(2):
        e = philox.normals(inf.seed, philox.KIND_EPS, t, S, P)
        lo, gm, gr = bnn.klqp_loss_and_grads(th[:P], th[P:], e, *args)
        info = inf.update()
        assert info["t"] == t + 1
        assert abs(info["loss"] - lo) <= 1e-5 * abs(lo)
        th = opt.apply(th, np.concatenate([gm, gr]), 0.01)
        got = np.concatenate([flat_q(qs, latents, "loc"), flat_q(qs, latents, "scale")])
        close(got, th, 5e-5)


def test_bnn_klqp_api_feed_dict_minibatches(cuda):
    """Placeholders X [M, D] / y [M] fed per update, scale = N / M, as the
    reference's minibatch loops do."""
    import edward_gb300 as ed
    from bnn_model import example_model, example_q, flat_q
    from oracle import philox
    D, H1, H2, N, M, S = 4, 10, 6, 200, 32, 2
    X, y = bnn.synthetic(N, D, H1, H2, seed=4)
    Xp = ed.placeholder(shape=[M, D], name="X")
    yp = ed.placeholder(shape=[M], name="y")
    latents, _, yrv = example_model(D, H1, H2, X=Xp, noise=0.3)
    qs = example_q(latents, np.random.default_rng(3))
    inf = ed.KLqp(qs, data={yrv: yp})
    inf.initialize(n_samples=S, scale={yrv: N / M}, optimizer=ed.train.AdamOptimizer(0.01))
    with pytest.raises(ValueError):
        inf.update()                         # nothing fed yet
    th = np.concatenate([flat_q(qs, latents, "loc"), flat_q(qs, latents, "scale")])
    th = th.astype(np.float64)
    P = th.size // 2
    opt = TFAdam(2 * P)
    for t in range(3):
        sl = slice(t * M, (t + 1) * M)
        info = inf.update(feed_dict={Xp: X[sl], yp: y[sl]})
        e = philox.normals(inf.seed, philox.KIND_EPS, t, S, P)
        lo, gm, gr = bnn.klqp_loss_and_grads(th[:P], th[P:], e, X[sl], y[sl], 0.3, N / M,
                                             D, H1, H2, 1.0)
        assert abs(info["loss"] - lo) <= 1e-5 * abs(lo)
        th = opt.apply(th, np.concatenate([gm, gr]), 0.01)
    got = np.concatenate([flat_q(qs, latents, "loc"), flat_q(qs, latents, "scale")])
    close(got, th, 5e-5)


def test_bnn_klqp_api_device_minibatch(cuda):
    """n_minibatch=M gathers M rows on the device (Philox stream 4) with scale
    N / M; the rows and the step equal the oracle's."""
    import edward_gb300 as ed
    from bnn_model import example_model, example_q, flat_q
    from oracle import philox
    D, H1, H2, N, M, S = 5, 16, 8, 1000, 48, 2
    X, y = bnn.synthetic(N, D, H1, H2, seed=6)
    latents, _, yrv = example_model(D, H1, H2, X=X, noise=0.25)
    qs = example_q(latents, np.random.default_rng(5))
    inf = ed.KLqp(qs, data={yrv: y})
    inf.initialize(n_samples=S, n_minibatch=M, optimizer=ed.train.AdamOptimizer(0.01))
    th = np.concatenate([flat_q(qs, latents, "loc"), flat_q(qs, latents, "scale")])
    th = th.astype(np.float64)
    P = th.size // 2
    opt = TFAdam(2 * P)
    for t in range(2):
        info = inf.update()
        rows = bnn.minibatch_rows(inf._bnn.seed, t, M, N)
        np.testing.assert_array_equal(inf._bnn.Xb.cpu().numpy(), X[rows])
        e = philox.normals(inf.seed, philox.KIND_EPS, t, S, P)
        lo, gm, gr = bnn.klqp_loss_and_grads(th[:P], th[P:], e, X[rows], y[rows], 0.25, N / M,
                                             D, H1, H2, 1.0)
        assert abs(info["loss"] - lo) <= 1e-5 * abs(lo)
        th = opt.apply(th, np.concatenate([gm, gr]), 0.01)
    got = np.concatenate([flat_q(qs, latents, "loc"), flat_q(qs, latents, "scale")])
    close(got, th, 5e-5)


def test_bnn_reparameterization_klqp_monte_carlo_kl(cuda):
    """ReparameterizationKLqp (Monte Carlo KL, klqp.py:642-704) on the network."""
    import edward_gb300 as ed
    from bnn_model import example_model, example_q, flat_q
    D, H1, H2, N, S = 3, 8, 8, 40, 4
    X, y = bnn.synthetic(N, D, H1, H2, seed=8)
    latents, _, yrv = example_model(D, H1, H2, X=X, noise=0.2, prior_scale=1.5)
    qs = example_q(latents, np.random.default_rng(7))
    inf = ed.ReparameterizationKLqp(qs, data={yrv: y})
    inf.initialize(n_samples=S)
    mu, rho = flat_q(qs, latents, "loc"), flat_q(qs, latents, "scale")
    eps = np.random.default_rng(9).standard_normal((S, mu.size)).astype(np.float32)
    loss, gmu, grho = inf.loss_and_gradients(eps)
    l0, m0, r0 = bnn.klqp_loss_and_grads(mu, rho, eps, X, y, 0.2, 1.0, D, H1, H2, 1.5, method=1)
    assert abs(loss - l0) <= 1e-5 * abs(l0)
    close(gmu.cpu().numpy(), m0, 1e-5)
    close(grho.cpu().numpy(), r0, 1e-5)


@ENGINES
def test_bnn_log_lik_autograd_function(cuda, engine):
    """The torch.autograd.Function over the hand-written adjoint: backward of a
    weighted sum of per-sample log-likelihoods equals the oracle's gradient."""
    from edward_gb300 import ops
    D, H1, H2, M, S = 6, 20, 12, 90, 3
    X, y = bnn.synthetic(M, D, H1, H2, seed=12)
    P = bnn.n_params(D, H1, H2)
    theta = (np.random.default_rng(13).standard_normal((S, P)) * 0.3).astype(np.float32)
    cfg = ops.bnn_config(D, H1, H2, S, noise=0.4, data_scale=3.0, engine=engine)
    th = torch.tensor(theta, device=cuda, requires_grad=True)
    ll = ops.bnn_log_lik(cfg, torch.as_tensor(X, device=cuda), torch.as_tensor(y, device=cuda), th)
    w = torch.tensor([1.0, -0.5, 2.0], device=cuda)
    (ll * w).sum().backward()
    ll0, g0 = bnn.log_lik_and_grad(theta, X, y, 0.4, 3.0, D, H1, H2)
    close(ll.detach().cpu().numpy(), ll0, 1e-5)
    close(th.grad.cpu().numpy(), g0 * np.array([1.0, -0.5, 2.0])[:, None], 1e-5)
