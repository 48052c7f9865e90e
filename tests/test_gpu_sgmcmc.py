"""SGLD / SGHMC (stochastic-gradient MCMC) for the GLM family: chains against
the FP64 oracle with the same draws, and the reference's Normal-Normal
posterior checks (tests/inferences/sgld_test.py, sghmc_test.py)."""
import numpy as np
import pytest
import torch

from oracle import glm as oglm
from oracle import sgmcmc

pytestmark = pytest.mark.gpu


def _logreg(ed, C, N=400, D=5, seed=0):
    from edward_gb300.models import Bernoulli, Empirical, Normal
    X, y, _, _ = oglm.synthetic_logreg(N, D, seed=seed)
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = Normal(loc=0.0, scale=1.0)
    yv = Bernoulli(logits=ed.dot(X, w) + b)
    rng = np.random.default_rng(seed)
    w0 = (rng.standard_normal((C, D)) * 0.1).astype(np.float32)
    qw = Empirical(ed.Variable(np.repeat(w0[None], 20, 0)), n_chains=C)
    qb = Empirical(ed.Variable(np.zeros((20, C), np.float32)), n_chains=C)
    model = oglm.GLM(X, y, bias=True)
    return {w: qw, b: qb}, {yv: y}, model, np.concatenate([w0, np.zeros((C, 1))], 1)


@pytest.mark.parametrize("method", ["sgld", "sghmc"])
@pytest.mark.parametrize("given_noise", [True, False])
def test_sgmcmc_chains_match_oracle(cuda, method, given_noise):
    import edward_gb300 as ed
    C, n = 6, 5
    lv, data, model, z0 = _logreg(ed, C)
    cls = ed.SGLD if method == "sgld" else ed.SGHMC
    inf = cls(lv, data=data, n_chains=C)
    kw = dict(step_size=1e-3) if method == "sgld" else dict(step_size=0.05, friction=0.2)
    inf.initialize(n_print=0, **kw)
    P = z0.shape[1]
    noise = np.random.default_rng(1).standard_normal((n, C, P)).astype(np.float32)
    inf.run_iterations(n, noise=noise if given_noise else None)
    got = inf._samples[:n].cpu().numpy()
    noise_fn = (lambda t: noise[t]) if given_noise else None
    ref, _, _ = sgmcmc.run(model, z0, n, kw["step_size"], method, kw.get("friction", 0.1),
                           seed=inf._cfg.seed, noise_fn=noise_fn)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    assert inf.t == n
    assert np.all(inf.n_accept.cpu().numpy() == n)


@pytest.mark.parametrize("cls_name,step", [("SGLD", 0.10), ("SGHMC", 0.025)])
def test_sgmcmc_normal_normal_posterior(cuda, cls_name, step):
    """The reference's check: x = 50 zeros, mu ~ N(0, 1), x ~ N(mu, 1), posterior
    N(0, 1/51); 2,000 iterations from mu = 1."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical, Normal
    ed.set_seed(42)
    x_data = np.zeros(50, np.float32)
    mu = Normal(loc=0.0, scale=1.0)
    x = Normal(loc=mu, scale=1.0, sample_shape=50)
    qmu = Empirical(params=ed.Variable(np.ones(2000, np.float32)))
    inference = getattr(ed, cls_name)({mu: qmu}, data={x: x_data})
    inference.run(step_size=step, n_print=0)
    assert abs(float(qmu.mean())) < 0.1
    assert abs(float(qmu.stddev()) - np.sqrt(1 / 51)) < 0.1
    assert inference.t == 2000
    assert inference.n_accept > 0.1
    inference.reset()
    assert inference.t == 0 and inference.n_accept == 0
