"""Model compiler: recognises the model families the CUDA kernels implement.

Edward evaluates arbitrary models by cloning their TF subgraph per Monte
Carlo sample / leapfrog step (``copy``, ``edward/util/random_variables.py:
139-445``).  The GB300 build instead compiles the model once into a dense
description of a supported family and evaluates it with fused kernels:

* ``GLMSpec`` -- y ~ Bernoulli(logits = X.w [+ b]) or Normal(loc = X.w [+ b], s)
  with Normal priors on w and b.  Covers ``ed.dot`` regressions
  (``tests/inferences/hmc_test.py:48-91``) and the Normal-Normal model
  (``tests/inferences/klqp_test.py:14-44``: x ~ Normal(mu, 1), X = ones).
  w or b may also be trainable Variables of the model (model parameters, the
  reference's p_vars: ``klqp.py:902-904``, ``variational_inference.py:62-64``;
  ``klqp_test.py:46-56`` fits Bernoulli(probs=sigmoid(Variable))).

Models outside the supported families raise NotImplementedError.  This
module is host-only and runs without a GPU.
"""
from dataclasses import dataclass, field
from typing import List, Tuple

import numpy as np

from .expr import Const, Node, Op, Placeholder, Variable, const_value, flatten_add
from .models import Bernoulli, Empirical, Normal, RandomVariable

LIK_BERNOULLI, LIK_NORMAL = 0, 1


@dataclass
class LatentBlock:
    rv: RandomVariable      # prior random variable (a Variable for a model parameter)
    offset: int             # first coordinate in the flat parameter vector z
    size: int
    shape: Tuple[int, ...]
    point: bool = False     # a model parameter: no prior, no q, point value


@dataclass
class GLMSpec:
    X: np.ndarray           # [N, D] float32
    y: np.ndarray           # [N] float32
    bias: bool
    lik: int
    lik_scale: float
    prior_loc: np.ndarray   # [P]
    prior_scale: np.ndarray
    blocks: List[LatentBlock] = field(default_factory=list)
    observed: RandomVariable = None

    @property
    def N(self):
        return self.X.shape[0]

    @property
    def D(self):
        return self.X.shape[1]

    @property
    def P(self):
        return self.D + (1 if self.bias else 0)


class UnsupportedModel(NotImplementedError):
    pass


def _split_data(data):
    observed, bindings = {}, {}
    for k, v in data.items():
        if isinstance(k, RandomVariable):
            observed[k] = v
        elif isinstance(k, Placeholder):
            bindings[k] = v
        else:
            raise TypeError(f"data key {k!r} must be a RandomVariable or a placeholder")
    return observed, bindings


def _const_param(node, what, bindings):
    v = const_value(node, bindings)
    if v is None:
        raise UnsupportedModel(f"{what} must be a constant in the supported model families")
    return np.asarray(v, np.float64)


def _prior(rv, bindings):
    if not isinstance(rv, Normal):
        raise UnsupportedModel(
            f"latent {rv.name}: the GLM family needs Normal priors (got {type(rv).__name__})")
    loc = _const_param(rv.loc, f"prior loc of {rv.name}", bindings)
    scale = _const_param(rv.scale, f"prior scale of {rv.name}", bindings)
    shp = rv.shape
    return np.broadcast_to(loc, shp).reshape(-1), np.broadcast_to(scale, shp).reshape(-1), shp


def compile_glm(latents, data, params=False):
    """``latents``: list of prior RandomVariables; ``data``: Edward data dict.
    ``params``: trainable Variables in the linear predictor are model
    parameters (KLqp fits them; the samplers do not take them).  Returns a
    GLMSpec or raises UnsupportedModel."""
    observed, bindings = _split_data(data)
    if len(observed) != 1:
        raise UnsupportedModel("the GLM family has exactly one observed random variable")
    (yrv, yval), = observed.items()
    if isinstance(yval, RandomVariable):
        raise UnsupportedModel("observed values must be arrays, not random variables")
    if isinstance(yval, (list, tuple)) and yval and np.ndim(yval[0]) > 0:
        raise UnsupportedModel("a list of observed arrays (ragged instances) is not a GLM")
    if isinstance(yval, Node):
        yval = const_value(yval, bindings)
        if yval is None:
            raise UnsupportedModel("the GLM family needs the observed values bound to an array")
    y = np.asarray(yval, np.float32).reshape(-1)
    if isinstance(yrv, Bernoulli):
        if yrv.logits is not None:
            eta = yrv.logits
        elif isinstance(yrv.probs, Op) and yrv.probs.op == "sigmoid":
            eta = yrv.probs.args[0]        # Bernoulli(probs=sigmoid(e)) = Bernoulli(logits=e)
        else:
            raise UnsupportedModel("Bernoulli likelihood must be parameterised by logits "
                                   "or probs=sigmoid(...)")
        lik, lik_scale = LIK_BERNOULLI, 1.0
    elif isinstance(yrv, Normal):
        eta, lik = yrv.loc, LIK_NORMAL
        s = _const_param(yrv.scale, "likelihood scale", bindings)
        if s.size > 1 and not np.all(s == s.reshape(-1)[0]):
            raise UnsupportedModel("Normal likelihood scale must be one constant")
        lik_scale = float(s.reshape(-1)[0])
    else:
        raise UnsupportedModel(f"unsupported likelihood {type(yrv).__name__}")

    latent_set = set(id(z) for z in latents)

    def is_param(n):
        return params and isinstance(n, Variable) and n.trainable

    dot_terms, bias_terms = [], []
    for term in flatten_add(eta):
        if isinstance(term, Op) and term.op == "dot":
            Xn, w = term.args
            if not (isinstance(w, RandomVariable) and id(w) in latent_set) and not is_param(w):
                raise UnsupportedModel("ed.dot(X, w) needs w to be a latent random variable or a "
                                       "trainable Variable")
            if isinstance(Xn, Placeholder) and isinstance(bindings.get(Xn), (list, tuple)):
                raise UnsupportedModel("X bound to a list (ragged instances) is not a GLM")
            X = const_value(Xn, bindings)
            if X is None:
                raise UnsupportedModel("X in ed.dot(X, w) must be data (an array or a bound placeholder)")
            dot_terms.append((np.asarray(X, np.float32), w))
        elif (isinstance(term, RandomVariable) and id(term) in latent_set) or is_param(term):
            bias_terms.append(term)
        else:
            raise UnsupportedModel(f"term {term!r} of the linear predictor is not supported")
    if len(dot_terms) > 1 or len(bias_terms) > 1:
        raise UnsupportedModel("the GLM family supports one ed.dot term and one intercept")
    used = [w for _, w in dot_terms] + bias_terms
    used_rv = [z for z in used if isinstance(z, RandomVariable)]
    if set(id(z) for z in used_rv) != latent_set or len(used_rv) != len(latent_set):
        raise UnsupportedModel("every latent variable must appear once in the linear predictor")
    if not used:
        raise UnsupportedModel("the linear predictor has no latent variable or model parameter")

    def block(rv, offset, size):
        """(LatentBlock, prior loc, prior scale); a model parameter gets a
        placeholder N(0, 1) prior that no kernel reads."""
        if is_param(rv):
            if int(np.prod(rv.shape)) != size:
                raise ValueError(f"{rv.name} has {int(np.prod(rv.shape))} elements; {size} needed")
            return (LatentBlock(rv, offset, size, tuple(rv.shape), point=True),
                    np.zeros(size), np.ones(size))
        loc, scale, shp = _prior(rv, bindings)
        if int(np.prod(shp)) != size:
            raise ValueError(f"{rv.name} has {int(np.prod(shp))} elements; {size} needed")
        return LatentBlock(rv, offset, size, shp), loc, scale

    N = y.shape[0]
    blocks, locs, scales = [], [], []
    if dot_terms:
        X, w = dot_terms[0]
        if X.ndim != 2 or X.shape[0] != N:
            raise ValueError(f"X has shape {X.shape}; expected [{N}, D]")
        blk, loc, scale = block(w, 0, X.shape[1])
        blocks.append(blk)
        locs.append(loc)
        scales.append(scale)
        bias = bool(bias_terms)
        if bias:
            b = bias_terms[0]
            if int(np.prod(getattr(b, "shape", ()) or (1,))) != 1:
                raise UnsupportedModel("the intercept must be a scalar (or shape [1])")
            blk, loc, scale = block(b, X.shape[1], 1)
            blocks.append(blk)
            locs.append(loc)
            scales.append(scale)
    else:
        # x ~ Lik(mu): a scalar latent (Normal-Normal) or model parameter broadcast
        # over all rows
        mu = bias_terms[0]
        if int(np.prod(getattr(mu, "shape", ()) or (1,))) != 1:
            raise UnsupportedModel("a latent or parameter used without ed.dot must be a scalar")
        X = np.ones((N, 1), np.float32)
        blk, loc, scale = block(mu, 0, 1)
        blocks.append(blk)
        locs.append(loc)
        scales.append(scale)
        bias = False
    ps = np.concatenate(scales)
    if np.any(ps <= 0):
        raise ValueError("prior scales must be positive")
    return GLMSpec(X=np.ascontiguousarray(X, np.float32), y=y, bias=bias, lik=lik,
                   lik_scale=lik_scale, prior_loc=np.concatenate(locs).astype(np.float32),
                   prior_scale=ps.astype(np.float32), blocks=blocks, observed=yrv)


# ------------------------------------------------------------- variational families

@dataclass
class NormalQ:
    """q = Normal(loc=Variable, scale=softplus(Variable)) for one latent."""
    loc_var: Variable
    rho_var: Variable


def parse_normal_q(qz):
    """Returns NormalQ if ``qz`` is the mean-field Normal family with free loc
    and softplus-transformed scale (``klqp.py:76-80``), else raises."""
    if not isinstance(qz, Normal):
        raise UnsupportedModel(f"variational family {type(qz).__name__} is not supported here")
    if not isinstance(qz.loc, Variable):
        raise UnsupportedModel("q loc must be a Variable")
    sc = qz.scale
    if not (isinstance(sc, Op) and sc.op == "softplus" and isinstance(sc.args[0], Variable)):
        raise UnsupportedModel("q scale must be softplus(Variable)")
    return NormalQ(qz.loc, sc.args[0])


# ------------------------------------------------------------- hierarchical family

@dataclass
class HierSpec:
    """Ragged batch of hierarchical logistic regressions (one model instance
    per (X_i, y_i)): mu ~ N(mu_loc, mu_scale), tau ~ HalfNormal(tau_scale)
    with support 'nonnegative', w ~ N(mu, tau) elementwise, y ~ Bernoulli(X w)."""
    Xs: list
    ys: list
    mu_loc: float
    mu_scale: float
    tau_scale: float
    w: RandomVariable = None
    mu: RandomVariable = None
    tau: RandomVariable = None


def _strip_ones(node):
    """x, x * ones(..) or ones(..) * x  ->  x."""
    if isinstance(node, Op) and node.op == "mul":
        a, b = node.args
        for u, v in ((a, b), (b, a)):
            cv = const_value(v)
            if cv is not None and np.all(cv == 1.0):
                return u
    return node


def compile_hier(latents, data):
    """Recognises  mu ~ Normal, tau ~ HalfNormal (support 'nonnegative'),
    w ~ Normal(mu, tau), y ~ Bernoulli(logits = ed.dot(X, w)).  X and y may be
    bound to lists of arrays: each element is one independent instance."""
    from .models import HalfNormal
    observed, bindings = _split_data(data)
    if len(observed) != 1:
        raise UnsupportedModel("the hierarchical family has one observed variable")
    (yrv, yval), = observed.items()
    if not (isinstance(yrv, Bernoulli) and yrv.logits is not None):
        raise UnsupportedModel("hierarchical family: y must be Bernoulli(logits=ed.dot(X, w))")
    eta = yrv.logits
    if not (isinstance(eta, Op) and eta.op == "dot" and isinstance(eta.args[1], Normal)):
        raise UnsupportedModel("hierarchical family: logits must be ed.dot(X, w)")
    Xn, w = eta.args
    mu, tau = _strip_ones(w.loc), _strip_ones(w.scale)
    if not (isinstance(mu, Normal) and isinstance(tau, HalfNormal)):
        raise UnsupportedModel("hierarchical family: w ~ Normal(mu, tau), mu Normal, tau HalfNormal")
    if set(map(id, latents)) != {id(w), id(mu), id(tau)}:
        raise UnsupportedModel("hierarchical family: latent variables must be exactly w, mu, tau")
    if getattr(tau, "support", None) != "nonnegative":
        raise UnsupportedModel("set tau.support = 'nonnegative' so that auto_transform samples "
                               "u = softplus^{-1}(tau) on the real line")
    if isinstance(Xn, Placeholder):
        Xv = bindings.get(Xn)
    else:
        Xv = const_value(Xn)
    if Xv is None:
        raise UnsupportedModel("X must be data")
    Xs = list(Xv) if isinstance(Xv, (list, tuple)) else [np.asarray(Xv, np.float32)]
    ys = list(yval) if isinstance(yval, (list, tuple)) else [np.asarray(yval, np.float32)]
    if len(Xs) != len(ys):
        raise ValueError("X and y must hold the same number of instances")
    Xs = [np.ascontiguousarray(np.asarray(x, np.float32)) for x in Xs]
    ys = [np.asarray(v, np.float32).reshape(-1) for v in ys]
    mu_loc = float(_const_param(mu.loc, "mu loc", bindings).reshape(-1)[0])
    mu_scale = float(_const_param(mu.scale, "mu scale", bindings).reshape(-1)[0])
    tau_scale = float(_const_param(tau.scale, "tau scale", bindings).reshape(-1)[0])
    return HierSpec(Xs, ys, mu_loc, mu_scale, tau_scale, w=w, mu=mu, tau=tau)


# ------------------------------------------------------------- Bayesian NN family

@dataclass
class MLPSpec:
    """y ~ Normal(loc = reshape(tanh(tanh(X W0 + b0) W1 + b1) W2 + b2, [-1]), noise)
    with every weight ~ Normal(0, prior_scale): the regression network of
    ``examples/bayesian_nn.py:120-150``.  ``X`` / ``y`` are arrays when the data
    dict binds them, else None (placeholders fed per update)."""
    D: int
    H1: int
    H2: int
    noise: float
    prior_scale: float
    X: np.ndarray = None
    y: np.ndarray = None
    X_node: Node = None
    y_node: Node = None
    blocks: List[LatentBlock] = field(default_factory=list)
    observed: RandomVariable = None
    batch: int = None       # rows per step when X is a placeholder of static shape

    @property
    def P(self):
        return self.D * self.H1 + self.H1 + self.H1 * self.H2 + self.H2 + self.H2 + 1


def _strip_reshape(node):
    while isinstance(node, Op) and node.op == "reshape":
        node = node.args[0]
    return node


def _affine(node, latent_set):
    """matmul(a, W) + b  ->  (a, W, b) with W, b latent random variables."""
    terms = flatten_add(node)
    mm = [t for t in terms if isinstance(t, Op) and t.op == "matmul"]
    bs = [t for t in terms if isinstance(t, RandomVariable) and id(t) in latent_set]
    if len(mm) != 1 or len(bs) != 1 or len(terms) != 2:
        raise UnsupportedModel("each layer must be tf.matmul(h, W) + b with latent W and b")
    a, W = mm[0].args
    if not (isinstance(W, RandomVariable) and id(W) in latent_set):
        raise UnsupportedModel("layer weights must be latent random variables")
    return a, W, bs[0]


def compile_mlp(latents, data):
    """Recognises the two-hidden-layer tanh regression network.  Raises
    UnsupportedModel for anything else."""
    observed, bindings = _split_data(data)
    if len(observed) != 1:
        raise UnsupportedModel("the Bayesian NN family has exactly one observed variable")
    (yrv, yval), = observed.items()
    if not isinstance(yrv, Normal):
        raise UnsupportedModel("the Bayesian NN family needs a Normal likelihood")
    latent_set = set(map(id, latents))
    h, W2, b2 = _affine(_strip_reshape(yrv.loc), latent_set)
    if not (isinstance(h, Op) and h.op == "tanh"):
        raise UnsupportedModel("hidden layers must be tf.tanh(...)")
    h, W1, b1 = _affine(h.args[0], latent_set)
    if not (isinstance(h, Op) and h.op == "tanh"):
        raise UnsupportedModel("hidden layers must be tf.tanh(...)")
    Xn, W0, b0 = _affine(h.args[0], latent_set)
    order = [W0, b0, W1, b1, W2, b2]
    if len(set(map(id, order))) != 6 or set(map(id, order)) != latent_set:
        raise UnsupportedModel("latent variables must be exactly W_0, b_0, W_1, b_1, W_2, b_2")
    shp = [tuple(int(v) for v in z.shape) for z in order]
    if len(shp[0]) != 2 or len(shp[2]) != 2:
        raise UnsupportedModel("W_0 and W_1 must be matrices")
    D, H1 = shp[0]
    H2 = shp[2][1]
    want = [(D, H1), (H1,), (H1, H2), (H2,), (H2, 1), (1,)]
    for z, s, w in zip(order, shp, want):
        if int(np.prod(s)) != int(np.prod(w)) or (len(s) == 2 and s != w):
            raise UnsupportedModel(f"{z.name} has shape {s}; the network needs {w}")
    prior_scale = None
    for z in order:
        loc = _const_param(z.loc, f"prior loc of {z.name}", bindings)
        sc = _const_param(z.scale, f"prior scale of {z.name}", bindings)
        if np.any(loc != 0.0):
            raise UnsupportedModel("weight priors must have loc 0")
        if np.any(sc != sc.reshape(-1)[0]) or (prior_scale is not None and sc.reshape(-1)[0] != prior_scale):
            raise UnsupportedModel("every weight prior must share one scale")
        prior_scale = float(sc.reshape(-1)[0])
    if prior_scale <= 0:
        raise ValueError("prior scales must be positive")
    s = _const_param(yrv.scale, "likelihood scale", bindings)
    if np.any(s != s.reshape(-1)[0]) or s.reshape(-1)[0] <= 0:
        raise UnsupportedModel("the likelihood scale must be one positive constant")
    noise = float(s.reshape(-1)[0])
    X = const_value(Xn, bindings)
    batch = None
    if X is None:
        if not isinstance(Xn, Placeholder):
            raise UnsupportedModel("the network input must be data (an array or a placeholder)")
        if Xn.shape is None or len(Xn.shape) != 2 or Xn.shape[1] != D or Xn.shape[0] is None:
            raise UnsupportedModel("an unbound X placeholder needs the static shape [M, D]")
        batch = int(Xn.shape[0])
    else:
        X = np.ascontiguousarray(X, np.float32)
        if X.ndim != 2 or X.shape[1] != D:
            raise ValueError(f"X has shape {X.shape}; expected [N, {D}]")
    y = None
    if isinstance(yval, Placeholder):
        y = const_value(yval, bindings)
    elif not isinstance(yval, (RandomVariable, Node)):
        y = np.asarray(yval, np.float32).reshape(-1)
    if y is not None and X is not None and y.shape[0] != X.shape[0]:
        raise ValueError(f"y has {y.shape[0]} rows but X has {X.shape[0]}")
    blocks, off = [], 0
    for z, w in zip(order, want):
        n = int(np.prod(w))
        blocks.append(LatentBlock(z, off, n, tuple(z.shape)))
        off += n
    return MLPSpec(D=D, H1=H1, H2=H2, noise=noise, prior_scale=prior_scale, X=X, y=y,
                   X_node=Xn, y_node=yval if isinstance(yval, Placeholder) else None,
                   blocks=blocks, observed=yrv, batch=batch)


# ------------------------------------------------------------- sigmoid belief network

@dataclass
class SBNSpec:
    """Two-layer sigmoid belief network with its recognition network
    (``examples/sigmoid_belief_network.py:54-86``, hidden_sizes = [H0, H1]).
    ``weights`` holds the eight (kernel, bias) Variables in the order
    Wq0, bq0, Wq1, bq1, Wp1, bp1, Wp0, bp0."""
    V: int
    H0: int
    H1: int
    prior_logits: np.ndarray
    weights: list
    X: np.ndarray = None          # bound data [N, V] (uint8 or float), else None
    x_node: Node = None           # the placeholder fed per update
    batch: int = None             # rows per step of a placeholder with static shape
    observed: RandomVariable = None
    z0: RandomVariable = None
    z1: RandomVariable = None


def _strip_cast(node):
    while isinstance(node, Op) and node.op == "cast":
        node = node.args[0]
    return node


def _dense_parts(node, what):
    """matmul(a, W) + b with Variables W, b  ->  (a, W, b)."""
    terms = flatten_add(node)
    mm = [t for t in terms if isinstance(t, Op) and t.op == "matmul"]
    bs = [t for t in terms if isinstance(t, Variable)]
    if len(terms) != 2 or len(mm) != 1 or len(bs) != 1:
        raise UnsupportedModel(f"{what}: logits must be a dense layer matmul(h, W) + b")
    a, W = mm[0].args
    if not isinstance(W, Variable):
        raise UnsupportedModel(f"{what}: the dense kernel must be a Variable")
    return _strip_cast(a), W, bs[0]


def compile_sbn(latent_vars, data):
    """``latent_vars``: {z0: qz0, z1: qz1}; ``data``: {x: x_ph or array}."""
    observed, bindings = _split_data(data)
    if len(observed) != 1 or len(latent_vars) != 2:
        raise UnsupportedModel("the sigmoid belief network has one observed and two latent layers")
    (xrv, xval), = observed.items()
    if not (isinstance(xrv, Bernoulli) and xrv.logits is not None):
        raise UnsupportedModel("the sigmoid belief network needs x ~ Bernoulli(logits=...)")
    z0, Wp0, bp0 = _dense_parts(xrv.logits, "x")
    if not (isinstance(z0, Bernoulli) and z0 in latent_vars and z0.logits is not None):
        raise UnsupportedModel("x's logits must be a dense layer of a latent Bernoulli layer")
    z1, Wp1, bp1 = _dense_parts(z0.logits, "z0")
    if not (isinstance(z1, Bernoulli) and z1 in latent_vars and z1.logits is not None):
        raise UnsupportedModel("z0's logits must be a dense layer of the top latent layer")
    pl = const_value(z1.logits, bindings)
    if pl is None:
        raise UnsupportedModel("the top layer's logits must be constant")
    pl = np.asarray(pl, np.float32)
    pl2 = pl.reshape(-1, pl.shape[-1]) if pl.ndim else pl.reshape(1, 1)
    if not np.all(pl2 == pl2[:1]):
        raise UnsupportedModel("the top layer's logits must be the same for every row")
    qz0, qz1 = latent_vars[z0], latent_vars[z1]
    for q in (qz0, qz1):
        if not (isinstance(q, Bernoulli) and q.logits is not None):
            raise UnsupportedModel("the recognition network must be Bernoulli(logits=...) layers")
    xin, Wq0, bq0 = _dense_parts(qz0.logits, "q(z0)")
    a1, Wq1, bq1 = _dense_parts(qz1.logits, "q(z1)")
    if a1 is not qz0:
        raise UnsupportedModel("q(z1)'s logits must be a dense layer of q(z0)")
    x_node = xval if isinstance(xval, Node) else None
    if x_node is not None and xin is not x_node:
        raise UnsupportedModel("q(z0)'s logits must be a dense layer of the data bound to x")
    V = int(Wq0.shape[0])
    H0, H1 = int(Wq0.shape[1]), int(Wq1.shape[1])
    want = {"Wq0": (Wq0, (V, H0)), "bq0": (bq0, (H0,)), "Wq1": (Wq1, (H0, H1)), "bq1": (bq1, (H1,)),
            "Wp1": (Wp1, (H1, H0)), "bp1": (bp1, (H0,)), "Wp0": (Wp0, (H0, V)), "bp0": (bp0, (V,))}
    for k, (var, shp) in want.items():
        if tuple(var.shape) != shp:
            raise UnsupportedModel(f"{k} has shape {tuple(var.shape)}; the network needs {shp}")
    if pl2.shape[-1] != H1:
        raise UnsupportedModel(f"the top layer's logits have width {pl2.shape[-1]}; expected {H1}")
    weights = [v for v, _ in want.values()]
    if len(set(map(id, weights))) != 8:
        raise UnsupportedModel("every dense layer needs its own kernel and bias")
    X, batch = None, None
    if x_node is None:
        X = np.asarray(xval)
    else:
        bound = const_value(x_node, bindings) if isinstance(x_node, Placeholder) else None
        if bound is not None:
            X = np.asarray(bindings[x_node])
        elif isinstance(x_node, Placeholder) and x_node.shape and x_node.shape[0] is not None:
            batch = int(x_node.shape[0])
        else:
            raise UnsupportedModel("the data placeholder needs the static shape [B, V]")
    if X is not None:
        if X.ndim != 2 or X.shape[1] != V:
            raise ValueError(f"x data has shape {X.shape}; expected [N, {V}]")
        X = np.ascontiguousarray(X if X.dtype == np.uint8 else X.astype(np.float32))
    return SBNSpec(V=V, H0=H0, H1=H1, prior_logits=pl2[0].astype(np.float32), weights=weights,
                   X=X, x_node=x_node, batch=batch, observed=xrv, z0=z0, z1=z1)


# ------------------------------------------------------------- constrained latent family

@dataclass
class ExpFamSpec:
    """One latent with constrained support and i.i.d. observations of it:
    Beta + Bernoulli(probs=z), Gamma + Poisson(rate=z), Dirichlet +
    Categorical(probs=z).  Worked in the unconstrained space of the bijector
    auto_transform picks for the support (``util/random_variables.py:856-917``):
    sigmoid, softplus, SoftmaxCentered.  ``K`` is the unconstrained dimension."""
    family: int
    K: int
    prior: np.ndarray
    stats: np.ndarray
    z: RandomVariable
    observed: RandomVariable
    blocks: List[LatentBlock] = field(default_factory=list)

    @property
    def P(self):
        return self.K


def compile_expfam(latents, data):
    from scipy.special import gammaln
    from .models import Beta, Categorical, Dirichlet, Gamma, Poisson
    observed, bindings = _split_data(data)
    if len(latents) != 1 or len(observed) > 1:
        raise UnsupportedModel("the constrained-latent family has one latent and at most one "
                               "observed variable")
    z = latents[0]
    if observed:
        (x, xval), = observed.items()
        if isinstance(xval, (RandomVariable, Node)):
            xval = const_value(xval, bindings) if isinstance(xval, Node) else None
            if xval is None:
                raise UnsupportedModel("observed values must be bound to an array")
        xv = np.asarray(xval)
    else:
        # the latent alone (its prior is the target): no observations
        x, xv = None, np.zeros(0)
        if not isinstance(z, (Beta, Gamma, Dirichlet)):
            raise UnsupportedModel("not a Beta, Gamma or Dirichlet latent")
    none = x is None
    if isinstance(z, Beta) and (none or (isinstance(x, Bernoulli) and x.probs is z)):
        if np.any((xv != 0) & (xv != 1)):
            raise ValueError("Bernoulli observations must be 0 or 1")
        a = _const_param(z.concentration1, "Beta concentration1", bindings)
        b = _const_param(z.concentration0, "Beta concentration0", bindings)
        n1 = float((xv == 1).sum())
        fam, K, prior, stats = 0, 1, [float(a), float(b)], [n1, float(xv.size) - n1]
    elif isinstance(z, Gamma) and (none or (isinstance(x, Poisson) and x.rate is z)):
        if np.any(xv < 0) or np.any(xv != np.round(xv)):
            raise ValueError("Poisson observations must be non-negative integers")
        a = _const_param(z.concentration, "Gamma concentration", bindings)
        r = _const_param(z.rate, "Gamma rate", bindings)
        fam, K = 1, 1
        prior = [float(a), float(r)]
        stats = [float(xv.sum()), float(xv.size), float(gammaln(xv.astype(np.float64) + 1).sum())]
    elif isinstance(z, Dirichlet) and (none or (isinstance(x, Categorical) and x.probs is z)):
        alpha = _const_param(z.concentration, "Dirichlet concentration", bindings).reshape(-1)
        Kc = alpha.size
        if Kc < 2 or Kc > 33:
            raise UnsupportedModel("the Dirichlet latent needs 2 to 33 categories")
        if np.any(xv < 0) or np.any(xv >= Kc) or np.any(xv != np.round(xv)):
            raise ValueError(f"Categorical observations must be integers in [0, {Kc})")
        fam, K = 2, Kc - 1
        prior = list(alpha.astype(float))
        stats = list(np.bincount(xv.astype(np.int64).reshape(-1), minlength=Kc).astype(float))
    else:
        raise UnsupportedModel("not a Beta-Bernoulli, Gamma-Poisson or Dirichlet-Categorical model")
    if np.any(np.asarray(prior) <= 0):
        raise ValueError("prior parameters must be positive")
    spec = ExpFamSpec(fam, K, np.asarray(prior, np.float64), np.asarray(stats, np.float64), z, x)
    spec.blocks = [LatentBlock(z, 0, K, (K,) if fam == 2 else tuple(z.shape))]
    return spec
