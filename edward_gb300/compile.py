"""Model compiler: recognises the model families the CUDA kernels implement.

Edward evaluates arbitrary models by cloning their TF subgraph per Monte
Carlo sample / leapfrog step (``copy``, ``edward/util/random_variables.py:
139-445``).  The GB300 build instead compiles the model once into a dense
description of a supported family and evaluates it with fused kernels:

* ``GLMSpec`` -- y ~ Bernoulli(logits = X.w [+ b]) or Normal(loc = X.w [+ b], s)
  with Normal priors on w and b.  Covers ``ed.dot`` regressions
  (``tests/inferences/hmc_test.py:48-91``) and the Normal-Normal model
  (``tests/inferences/klqp_test.py:14-44``: x ~ Normal(mu, 1), X = ones).

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
    rv: RandomVariable      # prior random variable
    offset: int             # first coordinate in the flat parameter vector z
    size: int
    shape: Tuple[int, ...]


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


def compile_glm(latents, data):
    """``latents``: list of prior RandomVariables; ``data``: Edward data dict.
    Returns a GLMSpec or raises UnsupportedModel."""
    observed, bindings = _split_data(data)
    if len(observed) != 1:
        raise UnsupportedModel("the GLM family has exactly one observed random variable")
    (yrv, yval), = observed.items()
    if isinstance(yval, RandomVariable):
        raise UnsupportedModel("observed values must be arrays, not random variables")
    if isinstance(yval, (list, tuple)) and yval and np.ndim(yval[0]) > 0:
        raise UnsupportedModel("a list of observed arrays (ragged instances) is not a GLM")
    y = np.asarray(yval, np.float32).reshape(-1)
    if isinstance(yrv, Bernoulli):
        if yrv.logits is None:
            raise UnsupportedModel("Bernoulli likelihood must be parameterised by logits")
        eta, lik, lik_scale = yrv.logits, LIK_BERNOULLI, 1.0
    elif isinstance(yrv, Normal):
        eta, lik = yrv.loc, LIK_NORMAL
        s = _const_param(yrv.scale, "likelihood scale", bindings)
        if s.size > 1 and not np.all(s == s.reshape(-1)[0]):
            raise UnsupportedModel("Normal likelihood scale must be one constant")
        lik_scale = float(s.reshape(-1)[0])
    else:
        raise UnsupportedModel(f"unsupported likelihood {type(yrv).__name__}")

    latent_set = set(id(z) for z in latents)
    dot_terms, bias_terms = [], []
    for term in flatten_add(eta):
        if isinstance(term, Op) and term.op == "dot":
            Xn, w = term.args
            if not isinstance(w, RandomVariable) or id(w) not in latent_set:
                raise UnsupportedModel("ed.dot(X, w) needs w to be a latent random variable")
            if isinstance(Xn, Placeholder) and isinstance(bindings.get(Xn), (list, tuple)):
                raise UnsupportedModel("X bound to a list (ragged instances) is not a GLM")
            X = const_value(Xn, bindings)
            if X is None:
                raise UnsupportedModel("X in ed.dot(X, w) must be data (an array or a bound placeholder)")
            dot_terms.append((np.asarray(X, np.float32), w))
        elif isinstance(term, RandomVariable) and id(term) in latent_set:
            bias_terms.append(term)
        else:
            raise UnsupportedModel(f"term {term!r} of the linear predictor is not supported")
    if len(dot_terms) > 1 or len(bias_terms) > 1:
        raise UnsupportedModel("the GLM family supports one ed.dot term and one intercept")
    used = [w for _, w in dot_terms] + bias_terms
    if set(id(z) for z in used) != latent_set or len(used) != len(latent_set):
        raise UnsupportedModel("every latent variable must appear once in the linear predictor")

    N = y.shape[0]
    blocks, locs, scales = [], [], []
    if dot_terms:
        X, w = dot_terms[0]
        if X.ndim != 2 or X.shape[0] != N:
            raise ValueError(f"X has shape {X.shape}; expected [{N}, D]")
        loc, scale, shp = _prior(w, bindings)
        if int(np.prod(shp)) != X.shape[1]:
            raise ValueError(f"w has {int(np.prod(shp))} elements but X has {X.shape[1]} columns")
        blocks.append(LatentBlock(w, 0, X.shape[1], shp))
        locs.append(loc)
        scales.append(scale)
        bias = bool(bias_terms)
        if bias:
            b = bias_terms[0]
            loc, scale, shp = _prior(b, bindings)
            if int(np.prod(shp)) != 1:
                raise UnsupportedModel("the intercept must be a scalar (or shape [1]) latent")
            blocks.append(LatentBlock(b, X.shape[1], 1, shp))
            locs.append(loc)
            scales.append(scale)
    else:
        # x ~ Lik(mu): a scalar latent broadcast over all rows (Normal-Normal)
        mu = bias_terms[0]
        loc, scale, shp = _prior(mu, bindings)
        if int(np.prod(shp)) != 1:
            raise UnsupportedModel("a latent used without ed.dot must be a scalar")
        X = np.ones((N, 1), np.float32)
        blocks.append(LatentBlock(mu, 0, 1, shp))
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
