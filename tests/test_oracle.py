"""Pins of the CPU oracle (no GPU): Philox known answers, FP64 finite
differences, the golden fixtures and the closed-form posteriors that the
reference's own tests assert."""
import os

import numpy as np
import pytest

from oracle import densities as dn
from oracle.glm import GLM, NORMAL, conjugate_linreg_posterior, synthetic_logreg
from oracle.hmc import glm_lj_grad, hmc_step, run_hmc
from oracle.klqp import REPARAM, REPARAM_KL, SCORE, TFAdam, klqp_glm_loss_and_grads, run_klqp_glm
from oracle.philox import philox4x32_10, raw_u32, normals, uniforms64

GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")


# Published Philox4x32-10 known-answer vectors (Salmon et al., SC 2011;
# the Random123 distribution's kat_vectors): (counter, key) -> output.
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_known_answers(ctr, key, expect):
    out = philox4x32_10(*ctr, *key)
    assert tuple(int(x) for x in out) == expect


def test_philox_normals_moments():
    z = normals(7, 0, 3, 4000, 64).ravel()
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01
    u = uniforms64(7, 2, 3, 100000)
    assert 0 < u.min() and u.max() < 1 and abs(u.mean() - 0.5) < 0.005


def _fd(f, x, h=1e-6):
    g = np.zeros_like(x)
    for i in range(x.size):
        xp, xm = x.copy(), x.copy()
        xp.flat[i] += h
        xm.flat[i] -= h
        g.flat[i] = (f(xp) - f(xm)) / (2 * h)
    return g


@pytest.mark.parametrize("lik", [0, 1])
def test_glm_gradient_finite_differences(lik):
    X, y, _, _ = synthetic_logreg(60, 4, seed=2)
    if lik == 1:
        y = X @ np.arange(4) * 0.3 + 0.1
    m = GLM(X, y, bias=True, lik=lik, lik_scale=0.7, prior_loc=0.3, prior_scale=2.0)
    Z = np.random.default_rng(0).standard_normal((3, 5))
    g = m.grad_log_joint(Z)
    for b in range(3):
        fd = _fd(lambda z: m.log_joint(z[None])[0], Z[b])
        np.testing.assert_allclose(g[b], fd, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("method", [REPARAM_KL, REPARAM])
def test_klqp_gradient_finite_differences(method):
    X, y, _, _ = synthetic_logreg(40, 3, seed=5)
    m = GLM(X, y, bias=True, prior_scale=1.3, data_scale=2.0)
    rng = np.random.default_rng(1)
    mu, rho, eps = rng.standard_normal(4), rng.standard_normal(4), rng.standard_normal((3, 4))
    _, gmu, grho, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, method, latent_scale=1.5)
    fmu = _fd(lambda v: klqp_glm_loss_and_grads(m, v, rho, eps, method, latent_scale=1.5)[0], mu)
    frho = _fd(lambda v: klqp_glm_loss_and_grads(m, mu, v, eps, method, latent_scale=1.5)[0], rho)
    np.testing.assert_allclose(gmu, fmu, rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(grho, frho, rtol=1e-6, atol=1e-6)


def test_score_gradient_is_unbiased():
    """E_eps[score gradient] = gradient of the exact negative ELBO (checked
    against the reparameterisation gradient averaged over many draws)."""
    m = GLM(np.ones((5, 1)), np.zeros(5), bias=False, lik=NORMAL, lik_scale=1.0)
    mu, rho = np.array([0.4]), np.array([-0.5])
    eps = np.random.default_rng(3).standard_normal((200000, 1))
    _, gs_mu, gs_rho, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, SCORE)
    _, gr_mu, gr_rho, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, REPARAM)
    np.testing.assert_allclose(gs_mu, gr_mu, rtol=0.05, atol=0.05)
    np.testing.assert_allclose(gs_rho, gr_rho, rtol=0.05, atol=0.05)


def test_golden_fixture_regression():
    """The oracle still produces the committed fixtures (make_golden.py)."""
    g = np.load(GOLD)
    seed = 0x0123456789ABCDEF
    np.testing.assert_array_equal(raw_u32(seed, 1, 7, 5, 10), g["philox_u32"])
    np.testing.assert_allclose(normals(seed, 1, 7, 5, 10), g["philox_normal"], rtol=0, atol=0)
    m = GLM(g["lr_X"], g["lr_y"], bias=True, prior_loc=0.25, prior_scale=1.5)
    np.testing.assert_allclose(m.log_joint(g["lr_Z"]), g["lr_lp"], rtol=1e-12)
    np.testing.assert_allclose(m.grad_log_joint(g["lr_Z"]), g["lr_grad"], rtol=1e-12)
    for name, meth in (("kl", REPARAM_KL), ("re", REPARAM), ("sc", SCORE)):
        loss, gmu, grho, _ = klqp_glm_loss_and_grads(m, g["kq_mu"], g["kq_rho"], g["kq_eps"], meth)
        np.testing.assert_allclose(loss, g[f"kq_{name}_loss"], rtol=1e-12)
        np.testing.assert_allclose(gmu, g[f"kq_{name}_gmu"], rtol=1e-12)
        np.testing.assert_allclose(grho, g[f"kq_{name}_grho"], rtol=1e-12)
    f = glm_lj_grad(m)
    lj0, g0 = f(g["hmc_z0"])
    res = hmc_step(f, g["hmc_z0"], g0, lj0, g["hmc_r0"], g["hmc_u"], 0.05, 3)
    np.testing.assert_allclose(res["z_prop"], g["hmc_zprop"], rtol=1e-12)
    np.testing.assert_array_equal(res["accept"].astype(np.int32), g["hmc_accept"])


def test_tf_adam_first_step():
    """TF's Adam: the first step moves each parameter by ~lr * sign(g)."""
    opt = TFAdam(3)
    p = opt.apply(np.zeros(3), np.array([2.0, -0.5, 1e-3]), 0.1)
    np.testing.assert_allclose(p, [-0.1, 0.1, -0.1], rtol=1e-3)


def test_kl_normal_normal_closed_form():
    kl = dn.kl_normal_normal(0.3, 0.7, -0.2, 1.4)
    x = np.linspace(-12, 12, 200001)
    q = np.exp(dn.normal_log_prob(x, 0.3, 0.7))
    num = np.trapezoid(q * (dn.normal_log_prob(x, 0.3, 0.7) - dn.normal_log_prob(x, -0.2, 1.4)), x)
    assert abs(kl - num) < 1e-8


# ------------------------------------------------ statistical pins (reference tests)

def test_oracle_klqp_normal_normal_posterior():
    """klqp_test.py:14-35: q -> N(0, sqrt(1/51)) for x = 0 (x50)."""
    m = GLM(np.ones((50, 1)), np.zeros(50), bias=False, lik=NORMAL, lik_scale=1.0)
    mu, rho, _ = run_klqp_glm(m, [0.5], [0.3], 1500, 1, seed=11)
    assert abs(mu[0]) < 0.05
    assert abs(dn.softplus(rho[0]) - np.sqrt(1 / 51)) < 0.02


def test_oracle_hmc_normal_normal_posterior():
    """hmc_test.py:14-45 (mean ~ 0, std ~ sqrt(1/51), acceptance > 0.1)."""
    m = GLM(np.ones((50, 1)), np.zeros(50), bias=False, lik=NORMAL, lik_scale=1.0)
    s, na = run_hmc(glm_lj_grad(m), np.ones((8, 1)), 1500, 0.25, 2, seed=5)
    post = s[300:].reshape(-1)
    assert abs(post.mean()) < 0.02
    assert abs(post.std() - np.sqrt(1 / 51)) < 0.01
    assert (na / 1500).min() > 0.1


def test_oracle_hmc_linear_regression_conjugate():
    """hmc_test.py:48-91 against the closed-form conjugate posterior."""
    rng = np.random.default_rng(0)
    N, D = 40, 10
    w_true = rng.standard_normal(D)
    X = rng.standard_normal((N, D))
    y = X @ w_true + rng.normal(0, 0.1, N)
    m = GLM(X, y, bias=True, lik=NORMAL, lik_scale=0.1)
    mean, cov = conjugate_linreg_posterior(X, y, 0.1)
    s, na = run_hmc(glm_lj_grad(m), np.tile(mean, (8, 1)), 400, 0.01, 10, seed=3)
    est = s[100:].reshape(-1, D + 1).mean(0)
    sd = np.sqrt(np.diag(cov))
    assert np.all(np.abs(est - mean) < 4 * sd / np.sqrt(8 * 300 / 20) + 1e-3)
    np.testing.assert_allclose(est[:D], w_true, atol=0.5, rtol=0.5)


# ------------------------------------------------------------- sigmoid belief network

def _tiny_sbn(seed=0, V=3, H0=2, H1=2, B=2):
    from oracle import sbn
    rng = np.random.default_rng(seed)
    theta = rng.standard_normal(sbn.n_params(V, H0, H1)) * 0.7
    X = (rng.random((B, V)) < 0.5).astype(np.float64)
    pl = rng.standard_normal(H1) * 0.3
    return rng, theta, X, pl


def test_sbn_score_gradient_matches_finite_differences():
    """p-part: d loss at fixed draws; q-part: d of the surrogate
    -mean_s sum_b A_sb log q(z_sb) at fixed draws and signal (klqp.py:900-904)."""
    from oracle import sbn
    V, H0, H1, S = 3, 2, 2, 3
    rng, th, X, pl = _tiny_sbn()
    z0, z1, _ = sbn.sample_z(th, X, rng.random((S, 2, H0)), rng.random((S, 2, H1)), V, H0, H1)
    for mode, stats in ((sbn.NONE, None), (sbn.MEAN, np.array([-4.0, 1, 1, .9, .999, 0, 0, 0]))):
        out = sbn.score_step(th, X, pl, z0, z1, V, H0, H1, mode=mode, stats=stats)
        A = out["A"]
        nq = (V + 1) * H0 + (H0 + 1) * H1

        def surrogate(t):
            Wq0, Wq1, _, _ = sbn.unpack(t, V, H0, H1)
            lq = sbn.bern_logp(z0, (sbn.aug(X) @ Wq0)[None]).sum(-1) + \
                sbn.bern_logp(z1, sbn.aug(z0) @ Wq1).sum(-1)
            return -(lq * A).sum() / S

        def loss(t):
            return sbn.score_step(t, X, pl, z0, z1, V, H0, H1)["loss"]

        for p in range(th.size):
            a, b = th.copy(), th.copy()
            a[p] += 1e-6
            b[p] -= 1e-6
            fn = surrogate if p < nq else loss
            fd = (fn(a) - fn(b)) / 2e-6
            assert abs(fd - out["grad"][p]) <= 1e-6 * max(1.0, abs(fd))


def test_sbn_rao_blackwell_gradient():
    """ScoreRB (klqp.py:1110-1139): q(z1 | z0)'s surrogate weights its log
    density by F_s - sum_b log p(x_b | z0) (its Markov blanket); q(z0 | x)'s and
    the model's gradients are those of the plain estimator."""
    from oracle import sbn
    V, H0, H1, S = 3, 2, 2, 3
    rng, th, X, pl = _tiny_sbn(4)
    z0, z1, _ = sbn.sample_z(th, X, rng.random((S, 2, H0)), rng.random((S, 2, H1)), V, H0, H1)
    plain = sbn.score_step(th, X, pl, z0, z1, V, H0, H1)
    rb = sbn.score_step(th, X, pl, z0, z1, V, H0, H1, rb=True)
    nq0 = (V + 1) * H0
    nq = nq0 + (H0 + 1) * H1
    np.testing.assert_allclose(rb["grad"][:nq0], plain["grad"][:nq0])
    np.testing.assert_allclose(rb["grad"][nq:], plain["grad"][nq:])
    Wq0, Wq1, Wp1, Wp0 = sbn.unpack(th, V, H0, H1)
    lx = sbn.bern_logp(X[None], sbn.aug(z0) @ Wp0).sum(-1).sum(-1)
    A1 = plain["F"] - lx

    def surrogate(t):
        W1 = sbn.unpack(t, V, H0, H1)[1]
        lq1 = sbn.bern_logp(z1, sbn.aug(z0) @ W1).sum(-1).sum(-1)
        return -(lq1 * A1).sum() / S

    for p in range(nq0, nq):
        a, b = th.copy(), th.copy()
        a[p] += 1e-6
        b[p] -= 1e-6
        fd = (surrogate(a) - surrogate(b)) / 2e-6
        assert abs(fd - rb["grad"][p]) <= 1e-6 * max(1.0, abs(fd))


def test_sbn_estimators_are_unbiased_against_exact_enumeration():
    """The reference estimator and both per-row baselines average to the
    exact ELBO gradient (enumeration over every z) within Monte Carlo error,
    and the baselines reduce the variance."""
    from oracle import sbn
    V, H0, H1, B, BH = 3, 2, 2, 2, 4
    rng, th, X, pl = _tiny_sbn(1)
    g_exact = sbn.exact_grad(th, X, pl, V, H0, H1)
    n, nb = 40000, 40
    z0, z1, _ = sbn.sample_z(th, X, rng.random((n, B, H0)), rng.random((n, B, H1)), V, H0, H1)
    bp = rng.standard_normal(sbn.n_baseline_params(V, BH)) * 0.3
    var = {}
    for mode, stats, rb in ((sbn.NONE, None, False),
                            (sbn.MEAN, np.array([-5.0, 1, 3, .9, .999, 0, 0, 0]), False),
                            (sbn.MLP, np.array([-5.0, 2.0, 3, .9, .999, 0, 0, 0]), False),
                            (sbn.NONE, None, True)):
        gs = np.array([sbn.score_step(th, X, pl, z0[k::nb], z1[k::nb], V, H0, H1, mode=mode,
                                      stats=stats, bparams=bp, BH=BH, rb=rb)["grad"]
                       for k in range(nb)])
        se = gs.std(axis=0) / np.sqrt(nb)
        assert np.all(np.abs(gs.mean(axis=0) - g_exact) < 5 * se + 1e-9)
        var[(mode, rb)] = gs.var(axis=0).sum()
    assert var[(sbn.MEAN, False)] < var[(sbn.NONE, False)]
    assert var[(sbn.NONE, True)] <= var[(sbn.NONE, False)]


def test_sbn_baseline_regression_gradient():
    """The MLP baseline's update uses the gradient of mean_b (o_b - t_b)^2."""
    from oracle import sbn
    V, BH, B = 5, 3, 7
    rng = np.random.default_rng(2)
    X = (rng.random((B, V)) < 0.5).astype(np.float64)
    bp = rng.standard_normal(sbn.n_baseline_params(V, BH)) * 0.4
    f = rng.standard_normal((4, B)) * 3 - 20
    stats = np.array([-19.0, 2.5, 5, 0.9, 0.999, 0, 0, 0])
    Hb, o = sbn.mlp_forward(bp, X, V, BH)
    t = (f.mean(0) - stats[0]) / stats[1]
    # one SGD-like probe: Adam's first step moves each parameter by -lr * sign(g)
    new_stats, new_bp, _ = sbn.baseline_update({"f": f, "mlp_out": o, "Hb": Hb}, X, stats, bp,
                                               np.zeros(2 * bp.size), V, BH, sbn.MLP, 0.9,
                                               lr=1e-4, beta1=0.9, beta2=0.999)

    def mse(p):
        return np.mean((sbn.mlp_forward(p, X, V, BH)[1] - t) ** 2)

    for p in range(bp.size):
        a, b = bp.copy(), bp.copy()
        a[p] += 1e-6
        b[p] -= 1e-6
        g = (mse(a) - mse(b)) / 2e-6
        if abs(g) > 1e-8:
            assert np.sign(bp[p] - new_bp[p]) == np.sign(g)
    assert new_stats[2] == 6 and new_stats[5] == pytest.approx(mse(bp))


def test_cpu_baseline_hmc_matches_oracle():
    """The timed CPU restatement (one chain, GEMV per gradient, FP32) follows
    the same chain as the FP64 oracle fed the same Philox draws."""
    from oracle.cpu_baseline import hmc_logreg_chain
    X, y, _, _ = synthetic_logreg(300, 6, seed=3)
    P = 7
    m = GLM(X, y, bias=True)
    f = glm_lj_grad(m)
    z0 = np.random.default_rng(1).standard_normal((4, P)) * 0.1
    samples, n_acc = run_hmc(f, z0, 3, 0.02, 4, seed=11)
    for c in range(4):
        z, acc = hmc_logreg_chain(X, y, z0[c].astype(np.float32), 3, 0.02, 4, 11, c,
                                  np.zeros(P, np.float32), np.ones(P, np.float32))
        assert acc == n_acc[c]
        np.testing.assert_allclose(z, samples[-1, c], rtol=1e-4, atol=1e-5)


def test_cpu_baseline_klqp_matches_oracle():
    """The timed CPU KLqp step (one model copy per sample, unfused TF Adam)
    follows the oracle's optimisation trajectory with the same draws."""
    from oracle.cpu_baseline import klqp_logreg_step
    from oracle.klqp import default_learning_rate
    X, y, _, _ = synthetic_logreg(400, 5, seed=2)
    P = 6
    m = GLM(X, y, bias=True)
    mu0 = np.zeros(P)
    rho0 = np.full(P, -1.0)
    e_mu, e_rho, e_losses = run_klqp_glm(m, mu0, rho0, 5, 3, seed=21)
    mu, rho = mu0.astype(np.float32), rho0.astype(np.float32)
    mm, vv = np.zeros(2 * P, np.float32), np.zeros(2 * P, np.float32)
    for t in range(5):
        loss = klqp_logreg_step(X, y, mu, rho, mm, vv, t, 3, 21, np.zeros(P, np.float32),
                                np.ones(P, np.float32), default_learning_rate(t))
        assert abs(loss - e_losses[t]) <= 1e-4 * abs(e_losses[t])
    np.testing.assert_allclose(mu, e_mu, rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(rho, e_rho, rtol=1e-3, atol=1e-4)


def test_cpu_baseline_bnn_step_matches_oracle():
    """The timed CPU Bayesian-NN step (one network copy per sample, FP32)
    gives the oracle's loss, and its first Adam step moves every parameter
    against the oracle's gradient."""
    from oracle import bnn
    from oracle.cpu_baseline import bnn_klqp_step
    from oracle.philox import KIND_EPS, normals
    D, H1, H2, M, S = 6, 12, 10, 80, 3
    rng = np.random.default_rng(0)
    X = rng.standard_normal((M, D)).astype(np.float32)
    y = rng.standard_normal(M).astype(np.float32)
    P = bnn.n_params(D, H1, H2)
    mu = (rng.standard_normal(P) * 0.3).astype(np.float32)
    rho = np.full(P, -2.0, np.float32)
    eps = normals(5, KIND_EPS, 0, S, P)
    loss64, gmu64, _ = bnn.klqp_loss_and_grads(mu, rho, eps, X, y, 0.3, 2.0, D, H1, H2)
    mu0 = mu.copy()
    m, v = np.zeros(2 * P, np.float32), np.zeros(2 * P, np.float32)
    loss = bnn_klqp_step(X, y, mu, rho, m, v, 0, S, 5, 0.3, 2.0, D, H1, H2, 1e-3)
    assert abs(loss - loss64) <= 1e-4 * abs(loss64)
    big = np.abs(gmu64) > 1e-3 * np.abs(gmu64).max()
    assert np.all(np.sign(mu0 - mu)[big] == np.sign(gmu64)[big])


@pytest.mark.parametrize("transform", [True, False])
@pytest.mark.parametrize("family", [0, 1, 2])
def test_expfam_gradients_finite_differences(family, transform):
    """The constrained-latent log joints' hand-written gradients, in the
    unconstrained space and on the support itself, against FP64 central
    differences; on the support, NaN outside it (the reference's densities give
    NaN for such draws: inference_auto_transform_test.py:46-63)."""
    from oracle import expfam as ef
    if family == ef.DIRICHLET and not transform:
        pytest.skip("the Dirichlet latent is worked in the unconstrained space only")
    rng = np.random.default_rng(family)
    if family == ef.BETA:
        prior, stats = (1.5, 2.0), ef.sufficient_stats(ef.BETA, rng.integers(0, 2, 12))
        U = rng.uniform(0.1, 0.9, (5, 1)) if not transform else rng.standard_normal((5, 1))
    elif family == ef.GAMMA:
        prior, stats = (2.0, 0.5), ef.sufficient_stats(ef.GAMMA, rng.poisson(3.0, 9))
        U = rng.uniform(0.5, 6.0, (5, 1)) if not transform else rng.standard_normal((5, 1))
    else:
        prior = np.array([1.0, 2.0, 0.5, 3.0])
        stats = ef.sufficient_stats(ef.DIRICHLET, rng.integers(0, 4, 20), 4)
        U = rng.standard_normal((5, 3))
    lj = ef.log_joint if transform else ef.log_joint_support
    glj = ef.grad_log_joint if transform else ef.grad_log_joint_support
    g = glj(family, prior, stats, U)
    h = 1e-6
    for j in range(U.shape[1]):
        e = np.zeros_like(U)
        e[:, j] = h
        fd = (lj(family, prior, stats, U + e) - lj(family, prior, stats, U - e)) / (2 * h)
        np.testing.assert_allclose(g[:, j], fd, rtol=1e-6, atol=1e-6)
    if not transform:
        out = np.array([[-0.5], [1.5]]) if family == ef.BETA else np.array([[-0.5], [0.0]])
        assert np.all(np.isnan(lj(family, prior, stats, out)))
        assert np.all(np.isnan(glj(family, prior, stats, out)))


def test_expfam_support_and_unconstrained_log_joints_agree():
    """log p(x, z) on the support equals the unconstrained log joint minus the
    bijector's log|dz/du| at z = bijector(u)."""
    from oracle import expfam as ef
    rng = np.random.default_rng(3)
    U = rng.standard_normal((7, 1))
    for family, prior, stats in ((ef.BETA, (1.5, 2.0), (4.0, 6.0)),
                                 (ef.GAMMA, (2.0, 0.5), (25.0, 9.0, 11.3))):
        Z = ef.constrain(family, U)
        ldj = (-dn.softplus(-U) - dn.softplus(U))[:, 0] if family == ef.BETA \
            else -dn.softplus(-U)[:, 0]
        np.testing.assert_allclose(ef.log_joint_support(family, prior, stats, Z),
                                   ef.log_joint(family, prior, stats, U) - ldj, rtol=1e-12)


def test_cpu_baseline_sgld_mh_hier_follow_the_oracle():
    """The timed CPU restatements of SGLD, Metropolis-Hastings and
    hierarchical HMC (FP32, one chain at a time, as the reference runs) track
    the FP64 oracle with the same Philox draws."""
    import numpy as np
    from oracle import cpu_baseline as cb, glm as oglm, hier, mh, sgmcmc
    from oracle.hmc import hmc_step
    from oracle.philox import normals, uniforms64
    X, y, _, _ = oglm.synthetic_logreg(300, 5, seed=1)
    m = oglm.GLM(X, y, bias=True)
    z0 = (np.random.default_rng(0).standard_normal(6) * 0.1).astype(np.float32)
    loc, sc = np.zeros(6, np.float32), np.ones(6, np.float32)
    zc = cb.sgld_logreg_chain(X, y, z0, 4, 1e-3, 9, 2, loc, sc)
    Z0 = np.zeros((3, 6))
    Z0[2] = z0
    _, zr, _ = sgmcmc.run(m, Z0, 4, 1e-3, "sgld", seed=9)
    np.testing.assert_allclose(zc, zr[2], rtol=1e-5, atol=1e-5 * np.abs(zr[2]).max())
    s = 0.02 * np.ones(6, np.float32)
    zc2, _ = cb.mh_logreg_chain(X, y, z0, 5, s, 9, 0, loc, sc)
    zz = z0[None].astype(np.float64)
    for t in range(5):
        zz, _, _ = mh.step(m, zz, t, s.astype(np.float64), None, seed=9)
    np.testing.assert_allclose(zc2, zz[0], rtol=1e-5, atol=1e-6)
    Xs, ys = hier.synthetic_instances(1, seed=3, n_range=(200, 200), d_range=(7, 7))
    f = hier.lj_grad_fn(Xs[0], ys[0])
    zh = (np.random.default_rng(1).standard_normal(9) * 0.2).astype(np.float32)
    zc3, _ = cb.hier_chain(Xs[0], ys[0], zh, 1, 0.02, 4, 5, 3)
    zi = zh[None].astype(np.float64)
    lj, g = f(zi)
    res = hmc_step(f, zi, g, lj, normals(5, 1, 0, 1, 9, row0=3), uniforms64(5, 2, 0, 1, row0=3),
                   0.02, 4)
    np.testing.assert_allclose(zc3, res["z"][0], rtol=1e-5, atol=1e-5)
