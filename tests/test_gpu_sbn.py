"""Sigmoid belief network under ScoreKLqp (score-function gradient, with no
baseline, a running-mean baseline or the learned MLP baseline) against the
FP64 oracle, through the public API and the C ABI."""
import numpy as np
import pytest
import torch

from oracle import sbn

pytestmark = pytest.mark.gpu


def close(a, b, rtol):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    np.testing.assert_allclose(a, b, rtol=rtol, atol=rtol * max(np.abs(b).max(), 1e-30))


def _setup(V, H0, H1, B, S, baseline=None, seed=0, data=None, jitter=0.3, **kw):
    import edward_gb300 as ed
    from sbn_model import example_sbn
    ed.set_seed(seed)
    lv, xr, x_ph, weights = example_sbn(V, H0, H1, B, prior_logit=0.2)
    rng = np.random.default_rng(seed)
    for w in weights:      # non-trivial parameters (dense() zero-initialises biases)
        w.assign(w.numpy() + rng.standard_normal(w.shape).astype(np.float32) * jitter)
    inf = ed.ScoreKLqp(lv, data={xr: data if data is not None else x_ph})
    inf.initialize(n_samples=S, baseline=baseline, baseline_hidden=16, n_print=0, **kw)
    X = (rng.random((B, V)) < 0.4).astype(np.float32)
    return inf, x_ph, weights, X, np.full(H1, 0.2)


def _draws(rng, S, B, H0, H1):
    return ((rng.random((S, B, H0)) < 0.5).astype(np.float32),
            (rng.random((S, B, H1)) < 0.5).astype(np.float32))


@pytest.mark.parametrize("V,H0,H1,B,S", [(20, 12, 8, 16, 3), (784, 200, 200, 64, 4),
                                          (50, 20, 10, 512, 4)])
@pytest.mark.parametrize("baseline", [None, "mean", "mlp"])
@pytest.mark.parametrize("engine", ["tc", "simt"])
def test_sbn_score_gradient_parity_given_draws(cuda, V, H0, H1, B, S, baseline, engine):
    from sbn_model import flat_theta
    inf, x_ph, weights, X, pl = _setup(V, H0, H1, B, S, baseline, gemm_engine=engine)
    inf._feed({x_ph: X})
    stats, bp = None, None
    if baseline is not None:        # a baseline that has seen earlier steps
        stats = np.array([-30.0 if V < 100 else -600.0, 4.0, 3, .9, .999, 0, 0, 0])
        inf._bstats.copy_(torch.as_tensor(stats, dtype=torch.float32))
        bp = np.random.default_rng(7).standard_normal(inf._bparams.numel()) * 0.05
        inf._bparams.copy_(torch.as_tensor(bp, dtype=torch.float32))
    z0, z1 = _draws(np.random.default_rng(3), S, B, H0, H1)
    loss, g, f, A = inf.score_gradients(z=(z0, z1), signal=True)
    mode = {None: sbn.NONE, "mean": sbn.MEAN, "mlp": sbn.MLP}[baseline]
    ref = sbn.score_step(flat_theta(weights), X, pl, z0.astype(np.float64), z1.astype(np.float64),
                         V, H0, H1, mode=mode, stats=stats, bparams=bp, BH=16)
    assert abs(loss - ref["loss"]) <= 1e-5 * abs(ref["loss"])
    close(f.cpu().numpy(), ref["f"], 1e-5)
    close(A.cpu().numpy(), ref["A"], 1e-5)
    close(g.cpu().numpy(), ref["grad"], 1e-5)


@pytest.mark.parametrize("V,H0,H1,B,S", [(20, 12, 8, 16, 3), (784, 200, 200, 64, 4),
                                          (50, 20, 10, 512, 4)])
@pytest.mark.parametrize("engine", ["tc", "simt"])
def test_sbn_rao_blackwell_parity_given_draws(cuda, V, H0, H1, B, S, engine):
    """ed.KLqp on the network dispatches to the Rao-Blackwellised score
    estimator (klqp.py:153-163, 1058-1152); gradients against the oracle."""
    import edward_gb300 as ed
    from sbn_model import example_sbn, flat_theta
    ed.set_seed(0)
    lv, xr, x_ph, weights = example_sbn(V, H0, H1, B, prior_logit=0.2)
    rng = np.random.default_rng(0)
    for w in weights:
        w.assign(w.numpy() + rng.standard_normal(w.shape).astype(np.float32) * 0.3)
    inf = ed.KLqp(lv, data={xr: x_ph})
    inf.initialize(n_samples=S, n_print=0, gemm_engine=engine)
    X = (rng.random((B, V)) < 0.4).astype(np.float32)
    inf._feed({x_ph: X})
    z0, z1 = _draws(np.random.default_rng(3), S, B, H0, H1)
    loss, g = inf.score_gradients(z=(z0, z1))
    ref = sbn.score_step(flat_theta(weights), X, np.full(H1, 0.2), z0.astype(np.float64),
                         z1.astype(np.float64), V, H0, H1, rb=True)
    assert abs(loss - ref["loss"]) <= 1e-5 * abs(ref["loss"])
    close(g.cpu().numpy(), ref["grad"], 1e-5)


def test_sbn_philox_draws_follow_the_bernoulli_rule(cuda):
    """Without overrides z = u < sigmoid(logit) with u from Philox stream 3;
    the oracle repeats the draw (no u within 1e-5 of its threshold here)."""
    from sbn_model import flat_theta
    V, H0, H1, B, S = 30, 10, 6, 12, 5
    inf, x_ph, weights, X, pl = _setup(V, H0, H1, B, S)
    inf._feed({x_ph: X})
    loss, g, f, _ = inf.score_gradients(signal=True)
    th = flat_theta(weights)
    u0, u1 = sbn.draw_uniforms(inf.seed, 0, S, B, H0, H1)
    z0, z1, (p0, p1) = sbn.sample_z(th, X, u0, u1, V, H0, H1)
    assert min(np.abs(u0 - p0[None]).min(), np.abs(u1 - p1).min()) > 1e-5
    ref = sbn.score_step(th, X, pl, z0, z1, V, H0, H1)
    assert abs(loss - ref["loss"]) <= 1e-5 * abs(ref["loss"])
    close(f.cpu().numpy(), ref["f"], 1e-5)
    close(g.cpu().numpy(), ref["grad"], 1e-5)


@pytest.mark.parametrize("V,H0,H1,B,S", [(24, 10, 8, 16, 4), (300, 12, 8, 1024, 2),
                                          (784, 200, 200, 32, 4)])
def test_sbn_training_steps_with_mlp_baseline_match_oracle(cuda, V, H0, H1, B, S):
    """Three training steps, each checked as a transition from the device's
    state before it: the model step (plain gradient descent, so the parameter
    change is lr times the gradient), the MLP baseline's own Adam step and the
    running statistics, against the oracle (the second size splits every
    gradient GEMM over the rows).  The draws are given: a Bernoulli draw
    u < sigmoid(l) flips when u is within the logits' rounding error of its
    threshold, which among ~10^5 draws happens; the Philox draw rule has its
    own test at a size where no draw is that close."""
    import edward_gb300 as ed
    from sbn_model import flat_theta
    BH = 16
    lr = 0.05
    inf, x_ph, weights, X, pl = _setup(V, H0, H1, B, S, "mlp",
                                       optimizer=ed.train.GradientDescentOptimizer(lr))
    inf._feed({x_ph: X})
    rng = np.random.default_rng(11)
    for t in range(3):
        th = flat_theta(weights)
        stats = inf._bstats.cpu().numpy().astype(np.float64)
        bp = inf._bparams.cpu().numpy().astype(np.float64)
        bsl = inf._bslots.cpu().numpy().astype(np.float64)
        z0, z1 = _draws(rng, S, B, H0, H1)
        ref = sbn.score_step(th, X, pl, z0.astype(np.float64), z1.astype(np.float64), V, H0, H1,
                             mode=sbn.MLP, stats=stats, bparams=bp, BH=BH)
        zo = torch.cat([torch.as_tensor(z0).reshape(-1), torch.as_tensor(z1).reshape(-1)]).to(cuda)
        inf._step(apply=True, eps=zo)
        loss = inf._read_state().loss
        assert abs(loss - ref["loss"]) <= 1e-5 * abs(ref["loss"])
        close(flat_theta(weights) - th, -lr * ref["grad"], 2e-5)
        stats1, bp1, _ = sbn.baseline_update(ref, X, stats, bp, bsl, V, BH, sbn.MLP, 0.9, 1e-2)
        np.testing.assert_allclose(inf._bparams.cpu().numpy(), bp1, rtol=1e-4, atol=2e-5)
        np.testing.assert_allclose(inf._bstats.cpu().numpy()[:6], stats1[:6], rtol=2e-5, atol=1e-6)
    assert inf.t == 3


def test_sbn_device_minibatch_from_uint8_data(cuda):
    """n_minibatch=B gathers rows of uint8 data on the device (Philox stream 4)."""
    from oracle import bnn
    V, H0, H1, N, B = 40, 8, 6, 500, 32
    data = sbn.synthetic(N, V, H0, H1, seed=3)
    inf, _, _, _, _ = _setup(V, H0, H1, B, 2, data=data, n_minibatch=B)
    for t in range(2):
        inf.update()
        rows = bnn.minibatch_rows(inf._sbn.seed, t, B, N)
        np.testing.assert_array_equal(inf._sbn.Xb.cpu().numpy(), data[rows].astype(np.float32))


def test_sbn_learned_baseline_reduces_gradient_variance(cuda):
    """After training with the MLP baseline, at fixed parameters the
    q-gradient variance over independent draws is ordered
    none > running mean > learned MLP (all three estimators share their mean)."""
    import edward_gb300 as ed
    V, H0, H1, N, B, S = 784, 200, 200, 4096, 64, 4
    data = sbn.synthetic(N, V, H0, H1, seed=1)
    inf, _, _, _, _ = _setup(V, H0, H1, B, S, "mlp", data=data, n_minibatch=B, jitter=0.0,
                             optimizer=ed.train.AdamOptimizer(1e-3))
    for _ in range(8):
        inf.steps(50)
    inf._sbn.gather = False          # freeze one minibatch
    P = inf._P
    nq = (V + 1) * H0 + (H0 + 1) * H1
    var = {}
    for mode in (0, 1, 2):
        inf._cfg.baseline = mode
        gs = []
        for k in range(48):
            inf.seed = 1000 + k
            gs.append(inf.score_gradients()[1][:nq].double())
        gs = torch.stack(gs)
        var[mode] = float(gs.var(dim=0).sum())
        assert P > nq
    assert var[2] < var[1] < var[0], var
