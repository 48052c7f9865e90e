"""Host-side logic of the drop-in surface (no GPU): model compilation,
optimizer resolution and the reference's error behaviour."""
import numpy as np
import pytest

import edward_gb300 as ed
from edward_gb300 import train
from edward_gb300.compile import UnsupportedModel, compile_glm
from edward_gb300.models import Bernoulli, Empirical, HalfNormal, Normal


def logreg(N=20, D=3, bias=True):
    X = np.random.default_rng(0).standard_normal((N, D)).astype(np.float32)
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    eta = ed.dot(X, w)
    lat = [w]
    if bias:
        b = Normal(loc=0.5, scale=2.0)
        eta = eta + b
        lat.append(b)
    y = Bernoulli(logits=eta)
    return X, lat, y


def test_compile_logistic_regression():
    X, lat, y = logreg()
    spec = compile_glm(lat, {y: np.zeros(20)})
    assert spec.P == 4 and spec.bias and spec.lik == 0
    np.testing.assert_array_equal(spec.prior_loc, [0, 0, 0, 0.5])
    np.testing.assert_array_equal(spec.prior_scale, [1, 1, 1, 2])
    assert [b.offset for b in spec.blocks] == [0, 3]


def test_compile_normal_normal():
    mu = Normal(loc=0.0, scale=1.0)
    x = Normal(loc=mu, scale=1.0, sample_shape=50)
    spec = compile_glm([mu], {x: np.zeros(50)})
    assert spec.X.shape == (50, 1) and not spec.bias and spec.lik == 1 and spec.P == 1


def test_compile_placeholder_linear_regression():
    N, D = 40, 10
    X = ed.placeholder(np.float32, [N, D])
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = Normal(loc=ed.zeros(1), scale=ed.ones(1))
    y = Normal(loc=ed.dot(X, w) + b, scale=0.1 * np.ones(N, np.float32))
    xv = np.ones((N, D), np.float32)
    spec = compile_glm([w, b], {X: xv, y: np.zeros(N)})
    assert spec.bias and abs(spec.lik_scale - 0.1) < 1e-7 and spec.P == 11


@pytest.mark.parametrize("bad", ["two_dots", "unused", "prior"])
def test_compile_unsupported(bad):
    X = np.ones((5, 2), np.float32)
    w = Normal(loc=ed.zeros(2), scale=ed.ones(2))
    v = Normal(loc=ed.zeros(2), scale=ed.ones(2))
    if bad == "two_dots":
        y = Bernoulli(logits=ed.dot(X, w) + ed.dot(X, v))
        lat = [w, v]
    elif bad == "unused":
        y = Bernoulli(logits=ed.dot(X, w))
        lat = [w, v]
    else:
        h = HalfNormal(scale=1.0)
        y = Bernoulli(logits=ed.dot(X, w) + h)
        lat = [w, h]
    with pytest.raises(NotImplementedError):
        compile_glm(lat, {y: np.zeros(5)})


def test_klqp_n_samples_check():
    """klqp_test.py:63-80."""
    X, lat, y = logreg()
    inf = ed.KLqp(lat, data={y: np.zeros(20)})
    with pytest.raises(ValueError, match="n_samples should be greater than zero: 0"):
        inf.initialize(n_samples=0)


def test_klqp_list_latents_build_normal_q():
    X, lat, y = logreg()
    inf = ed.KLqp(lat, data={y: np.zeros(20)})
    for z, q in inf.latent_vars.items():
        assert isinstance(q, Normal) and q.mean().shape == z.shape


def test_klqp_rejects_discrete_list_latent():
    z = Bernoulli(logits=0.0)
    with pytest.raises(AttributeError):
        ed.KLqp([z], data={})


def test_kl_scaling_requires_analytic_kl():
    X, lat, y = logreg()
    inf = ed.ReparameterizationKLqp(lat, data={y: np.zeros(20)})
    inf.latent_vars = {z: Bernoulli(logits=0.0) for z in lat}
    with pytest.raises(TypeError, match="kl_scaling must be None"):
        inf.initialize(n_samples=1, kl_scaling={lat[0]: 2.0})


def test_hmc_requires_empirical():
    X, lat, y = logreg()
    with pytest.raises(TypeError, match="Empirical"):
        ed.HMC({lat[0]: Normal(0.0, 1.0)}, data={y: np.zeros(20)})


def test_hmc_requires_auto_transform():
    X, lat, y = logreg()
    inf = ed.HMC(lat, data={y: np.zeros(20)})
    with pytest.raises(ValueError, match="unconstrained support"):
        inf.initialize(auto_transform=False)


def test_hmc_list_latents_default_store():
    """monte_carlo.py:78-83: list latents get Empirical(zeros([1e4, ...]))."""
    X, lat, y = logreg()
    inf = ed.HMC(lat, data={y: np.zeros(20)})
    assert all(isinstance(q, Empirical) and q.n == 10000 for q in inf.latent_vars.values())
    inf2 = ed.HMC(lat, data={y: np.zeros(20)}, n_chains=8)
    assert inf2.latent_vars[lat[0]].params.shape == (10000, 8, 3)


def test_optimizer_resolution():
    """variational_inference.py:83-116."""
    o = train.resolve(None, None)
    assert isinstance(o, train.AdamOptimizer)
    assert isinstance(o.learning_rate, train.ExponentialDecay)
    assert o.learning_rate.staircase and o.learning_rate.decay_steps == 100
    o = train.resolve("adam", None)
    assert o.learning_rate == 0.01
    assert isinstance(train.resolve("rmsprop", None), train.RMSPropOptimizer)
    with pytest.raises(ValueError):
        train.resolve("nope", None)
    with pytest.raises(TypeError):
        train.resolve(3, None)


def test_compute_fails_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    X, lat, y = logreg()
    inf = ed.KLqp(lat, data={y: np.zeros(20)})
    with pytest.raises(RuntimeError, match="CUDA"):
        inf.run(n_samples=2, n_iter=3)


def test_scale_must_be_dict():
    X, lat, y = logreg()
    inf = ed.KLqp(lat, data={y: np.zeros(20)})
    with pytest.raises(TypeError, match="scale must be a dict"):
        inf.initialize(scale=3.0)


def _hier_model(Dmax=7):
    X = ed.placeholder(np.float32, [None, None])
    mu = Normal(loc=0.0, scale=1.0)
    tau = HalfNormal(scale=1.0)
    tau.support = "nonnegative"
    w = Normal(loc=mu * ed.ones(Dmax), scale=tau * ed.ones(Dmax))
    y = Bernoulli(logits=ed.dot(X, w))
    return X, mu, tau, w, y


def test_compile_hierarchical_ragged_lists():
    from edward_gb300.compile import compile_hier
    X, mu, tau, w, y = _hier_model()
    Xs = [np.ones((5, 3), np.float32), np.ones((9, 7), np.float32)]
    ys = [np.zeros(5), np.ones(9)]
    with pytest.raises(NotImplementedError):
        compile_glm([w, mu, tau], {X: Xs, y: ys})
    spec = compile_hier([w, mu, tau], {X: Xs, y: ys})
    assert len(spec.Xs) == 2 and spec.Xs[1].shape == (9, 7) and spec.tau_scale == 1.0
    assert spec.w is w and spec.mu is mu and spec.tau is tau


def test_compile_hierarchical_requires_nonnegative_support():
    from edward_gb300.compile import compile_hier
    X, mu, tau, w, y = _hier_model()
    tau.support = None
    with pytest.raises(NotImplementedError, match="nonnegative"):
        compile_hier([w, mu, tau], {X: [np.ones((4, 7))], y: [np.zeros(4)]})


def test_hmc_validates_hierarchical_model_on_host():
    X, mu, tau, w, y = _hier_model()
    inf = ed.HMC([w, mu, tau], data={X: [np.ones((5, 7), np.float32)], y: [np.zeros(5)]},
                 n_chains=4)
    inf.auto_transform = True
    inf._validate()
    assert inf._family == "hier"


# ------------------------------------------------------------- Bayesian NN family

def test_compile_bayesian_nn_example_model():
    from bnn_model import example_model
    from edward_gb300.compile import compile_mlp
    X = np.zeros((40, 3), np.float32)
    y = np.zeros(40, np.float32)
    latents, _, yrv = example_model(3, 10, 7, X=ed.placeholder(shape=[40, 3]), noise=0.1,
                                    prior_scale=2.0)
    spec = compile_mlp(latents, {yrv: y})
    assert (spec.D, spec.H1, spec.H2) == (3, 10, 7)
    assert spec.noise == pytest.approx(0.1) and spec.prior_scale == 2.0
    assert spec.batch == 40 and spec.X is None
    assert [b.offset for b in spec.blocks] == [0, 30, 40, 110, 117, 124]
    assert spec.P == 125
    Xp = spec.X_node
    spec = compile_mlp(latents, {yrv: y, Xp: X})
    assert spec.X.shape == (40, 3) and spec.y.shape == (40,)


def test_compile_bayesian_nn_rejects_other_networks():
    from bnn_model import example_model
    from edward_gb300.compile import compile_mlp
    latents, Xn, yrv = example_model(2, 4, 4, X=np.zeros((5, 2), np.float32))
    with pytest.raises(UnsupportedModel):   # a latent missing from the dict
        compile_mlp(latents[:-1], {yrv: np.zeros(5)})
    W0 = latents[0]
    W0.loc = ed.ones([2, 4])                # non-zero prior mean
    with pytest.raises(UnsupportedModel):
        compile_mlp(latents, {yrv: np.zeros(5)})
    latents, Xn, _ = example_model(2, 4, 4, X=np.zeros((5, 2), np.float32))
    h = ed.sigmoid(ed.matmul(Xn, latents[0]) + latents[1])
    h = ed.tanh(ed.matmul(h, latents[2]) + latents[3])
    y2 = Normal(loc=ed.reshape(ed.matmul(h, latents[4]) + latents[5], [-1]), scale=0.1)
    with pytest.raises(UnsupportedModel):   # sigmoid hidden layer
        compile_mlp(latents, {y2: np.zeros(5)})


def test_klqp_dispatches_bayesian_nn_on_host():
    """KLqp recognises the network (GLM compile fails, MLP compile succeeds)
    before any device work; the checks that need no GPU run here."""
    from bnn_model import example_model, example_q
    latents, Xn, yrv = example_model(2, 4, 4, X=np.zeros((5, 2), np.float32))
    qs = example_q(latents, np.random.default_rng(0))
    inf = ed.KLqp(qs, data={yrv: np.zeros(5, np.float32)})
    with pytest.raises(NotImplementedError):
        inf.initialize(kl_scaling={latents[0]: 2.0})
    inf = ed.ScoreKLqp(qs, data={yrv: np.zeros(5, np.float32)})
    with pytest.raises(NotImplementedError):
        inf.initialize()
    inf = ed.KLqp(qs, data={yrv: np.zeros(5, np.float32)})
    with pytest.raises(RuntimeError):       # the model compiles; the step needs the GPU
        inf.initialize(n_samples=2)
    assert inf._family == "bnn"


def test_minibatch_rows_oracle_is_uniform():
    from oracle import bnn
    rows = bnn.minibatch_rows(5, 3, 20000, 7)
    assert rows.min() == 0 and rows.max() == 6
    counts = np.bincount(rows, minlength=7)
    assert np.all(np.abs(counts - 20000 / 7) < 5 * np.sqrt(20000 / 7))


# ------------------------------------------------------------- sigmoid belief network

def test_compile_sigmoid_belief_network():
    from sbn_model import example_sbn
    from edward_gb300.compile import compile_sbn
    lv, xr, x_ph, weights = example_sbn(12, 5, 4, 8, prior_logit=0.5)
    spec = compile_sbn(lv, {xr: x_ph})
    assert (spec.V, spec.H0, spec.H1, spec.batch) == (12, 5, 4, 8)
    assert spec.x_node is x_ph and spec.X is None
    np.testing.assert_array_equal(spec.prior_logits, np.full(4, 0.5, np.float32))
    assert [id(w) for w in spec.weights] == [id(w) for w in weights]
    data = (np.random.default_rng(0).random((30, 12)) < 0.5).astype(np.uint8)
    spec = compile_sbn(lv, {xr: data})
    assert spec.X.dtype == np.uint8 and spec.X.shape == (30, 12)


def test_compile_sbn_rejects_other_networks():
    from sbn_model import example_sbn
    from edward_gb300.compile import compile_sbn
    lv, xr, x_ph, _ = example_sbn(6, 3, 2, 4)
    (z0, qz0), (z1, qz1) = lv.items()
    with pytest.raises(UnsupportedModel):      # q(z1) not fed by q(z0)
        bad = Bernoulli(logits=ed.layers.dense(ed.cast(x_ph), 2))
        compile_sbn({z0: qz0, z1: bad}, {xr: x_ph})
    with pytest.raises(UnsupportedModel):      # non-constant top logits
        z1.logits = ed.layers.dense(ed.cast(x_ph), 2)
        compile_sbn(lv, {xr: x_ph})


def test_sbn_dispatch_on_host():
    """KLqp on discrete latents dispatches to the Rao-Blackwellised score
    estimator (klqp.py:153-163), ScoreKLqp to the plain one; both compile the
    network on the host and then need the GPU."""
    from sbn_model import example_sbn
    lv, xr, x_ph, _ = example_sbn(6, 3, 2, 4)
    for cls in (ed.KLqp, ed.ScoreRBKLqp):
        inf = cls(lv, data={xr: x_ph})
        with pytest.raises(RuntimeError):
            inf.initialize(n_samples=2)
        assert inf._family == "sbn" and inf._rao_blackwell
    inf = ed.ScoreKLqp(lv, data={xr: x_ph})
    with pytest.raises(ValueError):
        inf.initialize(baseline="median")
    inf = ed.ScoreKLqp(lv, data={xr: x_ph})
    with pytest.raises(RuntimeError):
        inf.initialize(n_samples=2, baseline="mlp")
    assert inf._family == "sbn"


def test_sgmcmc_validates_on_host():
    """SGLD / SGHMC compile the GLM on the host, then need the GPU."""
    from edward_gb300.models import Empirical
    X = np.zeros((10, 3), np.float32)
    w = Normal(loc=ed.zeros(3), scale=ed.ones(3))
    y = Bernoulli(logits=ed.dot(X, w))
    for cls in (ed.SGLD, ed.SGHMC):
        inf = cls({w: Empirical(ed.Variable(np.zeros((5, 3), np.float32)))},
                  data={y: np.zeros(10, np.float32)})
        with pytest.raises(RuntimeError):
            inf.initialize(step_size=0.1)
        assert inf._spec.P == 3


def test_criticism_argument_checks():
    X = np.zeros((4, 2), np.float32)
    w = Normal(loc=ed.zeros(2), scale=ed.ones(2))
    y = Bernoulli(logits=ed.dot(X, w))
    qw = Empirical(ed.Variable(np.zeros((3, 2), np.float32)))
    y_post = ed.copy(y, {w: qw})
    assert ed.copy(y, None) is y
    with pytest.raises(TypeError):
        ed.evaluate(3, data={y_post: np.zeros(4)})
    with pytest.raises(TypeError):
        ed.evaluate("binary_accuracy", data={y_post: np.zeros(4)}, n_samples=2.5)
    with pytest.raises(TypeError):
        ed.ppc("not callable", data={y_post: np.zeros(4)})
