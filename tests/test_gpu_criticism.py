"""Criticism on the device sample store: edg_glm_predict against NumPy, and
ed.evaluate / ed.ppc on GLM posteriors (edward/criticisms/evaluate.py, ppc.py)."""
import numpy as np
import pytest
import torch

from oracle import densities as dn
from oracle import glm as oglm

pytestmark = pytest.mark.gpu


def _model(ed, N=300, D=6, seed=0, lik="bernoulli"):
    from edward_gb300.models import Bernoulli, Normal
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((N, D)).astype(np.float32)
    w_true = rng.standard_normal(D).astype(np.float32)
    X_ph = ed.placeholder(shape=[N, D])
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = Normal(loc=0.0, scale=1.0)
    if lik == "bernoulli":
        y = Bernoulli(logits=ed.dot(X_ph, w) + b)
        y_obs = (rng.random(N) < dn.sigmoid(X @ w_true + 0.3)).astype(np.float32)
    else:
        y = Normal(loc=ed.dot(X_ph, w) + b, scale=0.5)
        y_obs = (X @ w_true + 0.3 + 0.5 * rng.standard_normal(N)).astype(np.float32)
    return X, X_ph, w, b, y, y_obs


@pytest.mark.parametrize("lik", ["bernoulli", "normal"])
def test_predict_kernel_matches_numpy(cuda, lik):
    import edward_gb300 as ed
    from edward_gb300 import _lib
    from edward_gb300.compile import compile_glm
    from edward_gb300.ops import GLMDevice
    X, X_ph, w, b, y, y_obs = _model(ed, lik=lik)
    glm = GLMDevice(compile_glm([w, b], {y: y_obs, X_ph: X}), cuda)
    S = 37
    Z = np.random.default_rng(1).standard_normal((S, 7)).astype(np.float32)
    Zt = torch.as_tensor(Z, device=cuda)
    eta = X.astype(np.float64) @ Z[:, :6].T.astype(np.float64) + Z[:, 6]
    mean = torch.empty(300, device=cuda)
    _lib.call("edg_glm_predict", glm.ref(), _lib.ptr(Zt), S, _lib.PREDICT_MEAN, 0, 0,
              _lib.ptr(mean), _lib.stream_ptr())
    ref = (dn.sigmoid(eta) if lik == "bernoulli" else eta).mean(axis=1)
    np.testing.assert_allclose(mean.cpu().numpy(), ref, rtol=1e-5, atol=1e-5)
    et = torch.empty(S, 300, device=cuda)
    _lib.call("edg_glm_predict", glm.ref(), _lib.ptr(Zt), S, _lib.PREDICT_ETA, 0, 0,
              _lib.ptr(et), _lib.stream_ptr())
    np.testing.assert_allclose(et.cpu().numpy(), eta.T, rtol=1e-5, atol=1e-4)
    # replicated data: the average over many replications approaches E[y | z]
    S2 = 4000
    Z2 = torch.as_tensor(np.repeat(Z[:1], S2, 0), device=cuda)
    rep = torch.empty(S2, 300, device=cuda)
    _lib.call("edg_glm_predict", glm.ref(), _lib.ptr(Z2), S2, _lib.PREDICT_SAMPLE, 7, 3,
              _lib.ptr(rep), _lib.stream_ptr())
    m1 = dn.sigmoid(eta[:, 0]) if lik == "bernoulli" else eta[:, 0]
    sd = np.sqrt(m1 * (1 - m1)) if lik == "bernoulli" else np.full(300, 0.5)
    assert np.all(np.abs(rep.mean(0).cpu().numpy() - m1) < 6 * sd / np.sqrt(S2) + 1e-6)


def test_evaluate_on_a_point_posterior(cuda):
    """An Empirical whose rows are all the same sample: every metric is then
    deterministic and equals the NumPy value."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical
    X, X_ph, w, b, y, y_obs = _model(ed)
    w_hat = np.random.default_rng(2).standard_normal(6).astype(np.float32) * 0.7
    qw = Empirical(ed.Variable(np.repeat(w_hat[None], 50, 0)))
    qb = Empirical(ed.Variable(np.full(50, 0.25, np.float32)))
    y_post = ed.copy(y, {w: qw, b: qb})
    acc, ll = ed.evaluate(["binary_accuracy", "log_likelihood"],
                          data={y_post: y_obs, X_ph: X}, n_samples=64, seed=3)
    eta = X.astype(np.float64) @ w_hat + 0.25
    pred = np.round(dn.sigmoid(eta))
    assert acc == pytest.approx(np.mean(pred == y_obs), abs=1e-6)
    model = oglm.GLM(X, y_obs, bias=True)
    ref_ll = model.log_lik(np.append(w_hat, 0.25)[None], scaled=False)[0] / len(y_obs)
    assert ll == pytest.approx(ref_ll, rel=1e-5)
    logloss = ed.evaluate("log_loss", data={y_post: y_obs, X_ph: X}, n_samples=8, seed=1)
    ref = np.mean(np.maximum(pred, 0) - pred * y_obs + np.log1p(np.exp(-np.abs(pred))))
    assert logloss == pytest.approx(ref, rel=1e-5)


def test_evaluate_and_ppc_after_hmc(cuda):
    """HMC on a logistic regression, then criticism on its device sample store."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical
    ed.set_seed(5)
    X, X_ph, w, b, y, y_obs = _model(ed, N=400)
    qw = Empirical(ed.Variable(np.zeros((300, 6), np.float32)))
    qb = Empirical(ed.Variable(np.zeros(300, np.float32)))
    inf = ed.HMC({w: qw, b: qb}, data={y: y_obs, X_ph: X})
    inf.run(step_size=0.02, n_steps=10, n_print=0)
    y_post = ed.copy(y, {w: qw, b: qb})
    acc = ed.evaluate("binary_accuracy", data={y_post: y_obs, X_ph: X}, n_samples=200, seed=0)
    assert acc > 0.8
    Trep, Tobs = ed.ppc(lambda xs, zs: xs[y_post].mean(), data={y_post: y_obs, X_ph: X},
                        n_samples=100)
    assert Trep.shape == (100,) and Tobs.shape == (100,)
    np.testing.assert_allclose(Tobs, y_obs.mean(), rtol=1e-6)
    assert abs(Trep.mean() - y_obs.mean()) < 0.05


def test_evaluate_regression_metrics(cuda):
    import edward_gb300 as ed
    from edward_gb300.models import Empirical
    X, X_ph, w, b, y, y_obs = _model(ed, lik="normal")
    w_hat = np.random.default_rng(4).standard_normal(6).astype(np.float32)
    qw = Empirical(ed.Variable(np.repeat(w_hat[None], 20, 0)))
    qb = Empirical(ed.Variable(np.full(20, 0.3, np.float32)))
    y_post = ed.copy(y, {w: qw, b: qb})
    mse, mae = ed.evaluate(["mse", "mae"], data={y_post: y_obs, X_ph: X}, n_samples=2000, seed=9)
    mean = X.astype(np.float64) @ w_hat + 0.3
    # the predictive average carries noise of scale 0.5 / sqrt(2000)
    assert mse == pytest.approx(np.mean((mean - y_obs) ** 2), rel=2e-2)
    assert mae == pytest.approx(np.mean(np.abs(mean - y_obs)), rel=2e-2)
