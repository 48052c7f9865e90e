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


@pytest.mark.parametrize("engine", ["simt", "tc"])
@pytest.mark.parametrize("walk", [True, False])
def test_mh_chains_match_oracle(cuda, walk, engine):
    """Per iteration: the FP64 ratio against the oracle's at the same state and
    draws, the accept decisions (away from log u = ratio) and the kept states,
    for the SIMT and the tensor-core engines."""
    import edward_gb300 as ed
    from edward_gb300.models import Normal
    from oracle import mh
    from oracle.philox import normals
    C, n = 8, 6
    lv, data, model, z0 = _logreg(ed, C)
    (w, qw), (b, qb) = lv.items()
    if walk:
        props = {w: Normal(loc=w, scale=0.05 * ed.ones(5)), b: Normal(loc=b, scale=0.05)}
        loc = None
    else:
        props = {w: Normal(loc=0.3 * ed.ones(5), scale=0.2 * ed.ones(5)),
                 b: Normal(loc=0.0, scale=0.2)}
        loc = np.array([0.3] * 5 + [0.0])
    scale = np.array([0.05] * 6) if walk else np.array([0.2] * 6)
    inf = ed.MetropolisHastings(lv, props, data=data, n_chains=C)
    inf.initialize(n_print=0, engine=engine)
    assert inf.engine == engine
    z = z0.copy()
    for t in range(n):
        ratio = torch.empty(C, dtype=torch.float64, device=cuda)
        inf.run_iterations(1, ratio_out=ratio)
        z_ref, acc, r_ref = mh.step(model, z, t, scale, loc, seed=inf._cfg.seed)
        r = ratio.cpu().numpy()
        np.testing.assert_allclose(r, r_ref, rtol=0, atol=1e-5 * max(1.0, np.abs(model.log_joint(z)).max()))
        got = inf._samples[t].cpu().numpy()
        from oracle.philox import uniforms64
        logu = np.log(uniforms64(inf._cfg.seed, mh.KIND_UNIFORM, t, C))
        clear = np.abs(logu - r_ref) > 1e-3
        np.testing.assert_allclose(got[clear], z_ref[clear], rtol=1e-5, atol=1e-5)
        z = got.astype(np.float64)      # continue from the device's state
    assert inf.t == n


@pytest.mark.parametrize("proposal", ["prior", "walk"])
def test_mh_normal_normal_posterior(cuda, proposal):
    """The reference's check (tests/inferences/metropolishastings_test.py:20-45):
    the prior as an independence proposal ({mu: mu}), or a random walk
    N(mu, 0.5); 2,000 iterations, posterior N(0, 1/51)."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical, Normal
    ed.set_seed(42)
    x_data = np.zeros(50, np.float32)
    mu = Normal(loc=0.0, scale=1.0)
    x = Normal(loc=mu, scale=1.0, sample_shape=50)
    qmu = Empirical(params=ed.Variable(np.ones(2000, np.float32)))
    g = mu if proposal == "prior" else Normal(loc=mu, scale=0.5)
    inference = ed.MetropolisHastings({mu: qmu}, {mu: g}, data={x: x_data})
    inference.run(n_print=0)
    assert abs(float(qmu.mean())) < 0.1
    assert abs(float(qmu.stddev()) - np.sqrt(1 / 51)) < 0.1
    assert inference.t == 2000 and inference.n_accept > 0.1
    inference.reset()
    assert inference.t == 0 and inference.n_accept == 0


def _logreg_scaled(ed, C, N, D, seed, dscale, lik="bernoulli"):
    from edward_gb300.models import Bernoulli, Empirical, Normal
    if lik == "bernoulli":
        X, y, _, _ = oglm.synthetic_logreg(N, D, seed=seed)
    else:
        rng = np.random.default_rng(seed)
        X = rng.standard_normal((N, D)).astype(np.float32)
        y = (X @ rng.standard_normal(D) + 0.3 * rng.standard_normal(N)).astype(np.float32)
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = Normal(loc=0.0, scale=1.0)
    eta = ed.dot(X, w) + b
    yv = Bernoulli(logits=eta) if lik == "bernoulli" else Normal(loc=eta, scale=0.7)
    rng = np.random.default_rng(seed + 1)
    w0 = (rng.standard_normal((C, D)) * 0.1).astype(np.float32)
    qw = Empirical(ed.Variable(np.repeat(w0[None], 20, 0)), n_chains=C)
    qb = Empirical(ed.Variable(np.zeros((20, C), np.float32)), n_chains=C)
    kw = {} if lik == "bernoulli" else dict(lik=oglm.NORMAL, lik_scale=0.7)
    model = oglm.GLM(X, y, bias=True, data_scale=dscale, **kw)
    return ({w: qw, b: qb}, {yv: y}, {yv: dscale}, model,
            np.concatenate([w0, np.zeros((C, 1))], 1))


@pytest.mark.parametrize("method", ["sgld", "sghmc"])
@pytest.mark.parametrize("given_noise", [True, False])
@pytest.mark.parametrize("shape", [(400, 5, 6, 1.0, "bernoulli"), (3000, 20, 200, 2.5, "bernoulli"),
                                   (1500, 63, 130, 0.5, "normal")])
def test_sgmcmc_tensor_core_matches_oracle(cuda, method, given_noise, shape):
    """The tensor-core engine (one 3xTF32 gradient evaluation per iteration,
    the update fused into the kernel) against the FP64 oracle with the same
    draws: several clusters of 128 chains (200 and 130 chains: a partial
    last cluster), P up to 64, the data scale, and the iterations split over
    two launches so the cached gradient carries over."""
    import edward_gb300 as ed
    N, D, C, dscale, lik = shape
    n1, n2 = 2, 3
    n = n1 + n2
    lv, data, scale, model, z0 = _logreg_scaled(ed, C, N, D, 3, dscale, lik)
    cls = ed.SGLD if method == "sgld" else ed.SGHMC
    inf = cls(lv, data=data, n_chains=C)
    kw = dict(step_size=1e-3) if method == "sgld" else dict(step_size=0.05, friction=0.2)
    inf.initialize(n_print=0, scale=scale, engine="tc", **kw)
    assert inf.engine == "tc"
    P = z0.shape[1]
    noise = np.random.default_rng(1).standard_normal((n, C, P)).astype(np.float32)
    inf.run_iterations(n1, noise=noise[:n1] if given_noise else None)
    inf.run_iterations(n2, noise=noise[n1:] if given_noise else None)
    got = inf._samples[:n].cpu().numpy()
    noise_fn = (lambda t: noise[t]) if given_noise else None
    ref, _, _ = sgmcmc.run(model, z0, n, kw["step_size"], method, kw.get("friction", 0.1),
                           seed=inf._cfg.seed, noise_fn=noise_fn)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    assert inf.t == n
    assert np.all(inf.n_accept.cpu().numpy() == n)


@pytest.mark.parametrize("method", ["sgld", "sghmc"])
def test_sgmcmc_engines_agree(cuda, method):
    """The tensor-core and SIMT engines draw the same Philox noise: the same
    chains to FP32 rounding over 20 iterations."""
    import edward_gb300 as ed
    C, n = 256, 20
    out = {}
    for engine in ("tc", "simt"):
        ed.set_seed(7)
        lv, data, scale, model, z0 = _logreg_scaled(ed, C, 2000, 12, 5, 1.0)
        cls = ed.SGLD if method == "sgld" else ed.SGHMC
        inf = cls(lv, data=data, n_chains=C)
        kw = dict(step_size=1e-3) if method == "sgld" else dict(step_size=0.05, friction=0.2)
        inf.initialize(n_print=0, engine=engine, **kw)
        assert inf.engine == engine
        inf.run_iterations(n)
        out[engine] = inf._samples[:n].cpu().numpy()
    np.testing.assert_allclose(out["tc"], out["simt"], rtol=1e-5,
                               atol=1e-5 * np.abs(out["simt"]).max())


def test_sgmcmc_tensor_core_reset_rebuilds_cache(cuda):
    """reset() restarts t at 0 from params[0] (the reference keeps the
    Empirical's values and re-initialises t and n_accept only): the cached
    gradient belongs to the last state, so it is rebuilt for params[0]."""
    import edward_gb300 as ed
    C, n = 64, 4
    lv, data, scale, model, z0 = _logreg_scaled(ed, C, 800, 8, 2, 1.0)
    inf = ed.SGLD(lv, data=data, n_chains=C)
    inf.initialize(n_print=0, step_size=1e-3, engine="tc")
    inf.run_iterations(n)
    start = inf._samples[0].cpu().numpy().astype(np.float64)
    inf.reset()
    inf.run_iterations(n)
    got = inf._samples[:n].cpu().numpy()
    ref, _, _ = sgmcmc.run(model, start, n, 1e-3, "sgld", seed=inf._cfg.seed)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
    assert inf.t == n


@pytest.mark.parametrize("method", ["sgld", "sghmc"])
def test_sgmcmc_tensor_core_single_chain_bias_only(cuda, method):
    """The tensor-core engine with one chain of a bias-only Normal model
    (P = 1: x ~ N(mu, 1), the reference tests' Normal-Normal shape) against the
    oracle, 6 iterations with Philox noise."""
    import edward_gb300 as ed
    from edward_gb300.models import Empirical, Normal
    x_data = np.random.default_rng(3).standard_normal(50).astype(np.float32) * 0.3
    mu = Normal(loc=0.0, scale=1.0)
    x = Normal(loc=mu, scale=1.0, sample_shape=50)
    qmu = Empirical(params=ed.Variable(np.full(10, 0.5, np.float32)))
    cls = ed.SGLD if method == "sgld" else ed.SGHMC
    inf = cls({mu: qmu}, data={x: x_data})
    kw = dict(step_size=0.01) if method == "sgld" else dict(step_size=0.05, friction=0.2)
    inf.initialize(n_print=0, engine="tc", **kw)
    assert inf.engine == "tc"
    n = 6
    inf.run_iterations(n)
    got = inf._samples[:n].cpu().numpy().reshape(n, 1, -1)
    model = oglm.GLM(np.zeros((50, 0)), x_data, bias=True, lik=oglm.NORMAL)
    ref, _, _ = sgmcmc.run(model, np.array([[0.5]]), n, kw["step_size"], method,
                           kw.get("friction", 0.1), seed=inf._cfg.seed)
    np.testing.assert_allclose(got.reshape(ref.shape), ref, rtol=1e-5,
                               atol=1e-5 * np.abs(ref).max())


@pytest.mark.parametrize("walk", [True, False])
def test_mh_engines_agree(cuda, walk):
    """The tensor-core and SIMT engines draw the same Philox proposals and
    uniforms: over 10 iterations of 300 chains (three clusters of 128, the last
    partial) the ratios agree to 1e-5 of the log joint and, where every
    decision matched, the chains agree to FP32 rounding."""
    import edward_gb300 as ed
    from edward_gb300.models import Normal
    C, n = 300, 10
    out = {}
    for engine in ("tc", "simt"):
        ed.set_seed(11)
        lv, data, scale, model, z0 = _logreg_scaled(ed, C, 1500, 10, 4, 1.0)
        (w, qw), (b, qb) = lv.items()
        if walk:
            props = {w: Normal(loc=w, scale=0.03 * ed.ones(10)), b: Normal(loc=b, scale=0.03)}
        else:
            props = {w: Normal(loc=0.1 * ed.ones(10), scale=0.2 * ed.ones(10)),
                     b: Normal(loc=0.0, scale=0.2)}
        inf = ed.MetropolisHastings(lv, props, data=data, n_chains=C)
        inf.initialize(n_print=0, engine=engine)
        assert inf.engine == engine
        ratio = torch.empty(n * C, dtype=torch.float64, device=cuda)
        inf.run_iterations(n, ratio_out=ratio)
        out[engine] = (inf._samples[:n].cpu().numpy(), ratio.cpu().numpy(),
                       inf.n_accept.cpu().numpy())
    (sa, ra, na), (sb, rb, nb) = out["simt"], out["tc"]
    lj_scale = 1500 * 0.7
    np.testing.assert_allclose(rb[:C], ra[:C], rtol=0, atol=1e-5 * lj_scale)
    if np.array_equal(na, nb):
        np.testing.assert_allclose(sb, sa, rtol=1e-5, atol=1e-5 * np.abs(sa).max())
        np.testing.assert_allclose(rb, ra, rtol=0, atol=1e-5 * lj_scale)
