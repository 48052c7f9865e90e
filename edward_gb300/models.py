"""Random variables: the ``edward.models`` surface used by the hot path.

Edward generates one RandomVariable class per ``tf.contrib.distributions``
class (``edward/models/random_variables.py:13-28``) on top of the
``RandomVariable`` mixin (``edward/models/random_variable.py:18-323``), adds a
``support`` tag to some of them (``random_variables.py:29-43``) and defines
``Empirical`` for MCMC sample stores (``edward/models/empirical.py:16-125``).
Here they are symbolic nodes whose arguments the model compiler reads; the
densities themselves are evaluated by the CUDA kernels.  ``mean`` /
``stddev`` / ``variance`` of the variational and empirical families are
provided for users (they read the current parameter tensors).
"""
import numpy as np
import torch

from .expr import Node, Variable, Op, as_node, const_value


class RandomVariable(Node):
    """Base class.  ``support`` follows ``edward/models/random_variables.py:29-43``."""

    support = None
    reparameterizable = False
    _count = 0

    def __init__(self, sample_shape=(), name=None, value=None):
        if isinstance(sample_shape, int):
            sample_shape = (sample_shape,)
        self.sample_shape = tuple(sample_shape)
        RandomVariable._count += 1
        self.name = name or f"{type(self).__name__}_{RandomVariable._count}"
        self._value = value

    @property
    def batch_shape(self):
        return ()

    @property
    def event_shape(self):
        return ()

    @property
    def shape(self):
        return tuple(self.sample_shape) + tuple(self.batch_shape) + tuple(self.event_shape)

    def get_variables(self):
        out = []
        for a in self.params().values():
            out += _variables_in(a)
        return out

    def params(self):
        return {}

    def __repr__(self):
        return f"<ed.RandomVariable '{self.name}' shape={self.shape}>"

    def __hash__(self):
        return id(self)

    def __eq__(self, other):
        return self is other


def _variables_in(node):
    if isinstance(node, Variable):
        return [node]
    if isinstance(node, Op):
        out = []
        for a in node.args:
            out += _variables_in(a)
        return out
    return []


def _eval(node):
    """Current numeric value (torch) of a parameter expression of Variables/constants."""
    if isinstance(node, Variable):
        return node.value.detach().float()
    if isinstance(node, Op):
        args = [_eval(a) for a in node.args]
        if node.op == "softplus":
            return torch.nn.functional.softplus(args[0])
        if node.op == "add":
            return args[0] + args[1].to(args[0].device)
        if node.op == "mul":
            return args[0] * args[1].to(args[0].device)
        if node.op == "neg":
            return -args[0]
        if node.op == "sigmoid":
            return torch.sigmoid(args[0])
        if node.op == "tanh":
            return torch.tanh(args[0])
    v = const_value(node)
    if v is None:
        raise TypeError(f"cannot evaluate {node!r} outside inference")
    return torch.as_tensor(v)


class Normal(RandomVariable):
    support = "real"
    reparameterizable = True

    def __init__(self, loc=0.0, scale=1.0, sample_shape=(), name=None, value=None):
        super().__init__(sample_shape, name, value)
        self.loc = as_node(loc)
        self.scale = as_node(scale)

    @property
    def batch_shape(self):
        a, b = self.loc.shape, self.scale.shape
        if a is None or b is None:
            return ()
        return tuple(np.broadcast_shapes(a, b))

    def params(self):
        return {"loc": self.loc, "scale": self.scale}

    def mean(self):
        return _eval(self.loc).expand(self.batch_shape).clone()

    def stddev(self):
        return _eval(self.scale).expand(self.batch_shape).clone()

    def variance(self):
        return self.stddev() ** 2


class HalfNormal(RandomVariable):
    """HalfNormal(scale).  As in the reference, it carries no support tag
    (``edward/models/random_variables.py:29-43``): set
    ``rv.support = 'nonnegative'`` to have it auto-transformed."""

    support = None
    reparameterizable = True

    def __init__(self, scale=1.0, sample_shape=(), name=None, value=None):
        super().__init__(sample_shape, name, value)
        self.scale = as_node(scale)

    @property
    def batch_shape(self):
        return tuple(self.scale.shape or ())

    def params(self):
        return {"scale": self.scale}


class Bernoulli(RandomVariable):
    support = "binary"
    reparameterizable = False

    def __init__(self, logits=None, probs=None, sample_shape=(), name=None, value=None):
        super().__init__(sample_shape, name, value)
        if (logits is None) == (probs is None):
            raise ValueError("Bernoulli needs exactly one of logits or probs")
        self.logits = as_node(logits) if logits is not None else None
        self.probs = as_node(probs) if probs is not None else None

    @property
    def batch_shape(self):
        n = self.logits if self.logits is not None else self.probs
        return tuple(n.shape or ())

    def params(self):
        return {"logits": self.logits} if self.logits is not None else {"probs": self.probs}

    def mean(self):
        if self.logits is not None:
            return torch.sigmoid(_eval(self.logits))
        return _eval(self.probs)


class Empirical(RandomVariable):
    """MCMC sample store.  ``params`` has shape [T, *event] for one chain,
    or [T, C, *event] with ``n_chains=C`` for C independent chains
    (the reference runs exactly one chain, ``edward/inferences/hmc.py:81-85``).
    Statistics reduce over the sample axis only, as in
    ``edward/models/empirical.py:87-93``."""

    support = "points"

    def __init__(self, params, n_chains=None, name=None):
        super().__init__((), name)
        if not isinstance(params, Variable):
            params = Variable(params, trainable=False)
        self.params_var = params
        self.n_chains = n_chains
        shp = params.shape
        if n_chains is not None and (len(shp) < 2 or shp[1] != n_chains):
            raise ValueError(f"Empirical params with n_chains={n_chains} must have shape [T, C, ...]")
        self.n = shp[0]
        self._constrain = None

    @property
    def params(self):
        """Samples [T, ...]; for a latent sampled in an unconstrained space the
        stored values are mapped back through the transform, as
        ``qz_constrained.params = bijector.inverse(params)`` does in the reference
        (``edward/inferences/inference.py:247-253``)."""
        v = self.params_var.value
        return self._constrain(v) if self._constrain is not None else v

    @property
    def event_shape(self):
        shp = self.params_var.shape
        return tuple(shp[2:]) if self.n_chains is not None else tuple(shp[1:])

    def get_variables(self):
        return [self.params_var]

    def mean(self):
        return self.params.double().mean(0).float()

    def variance(self):
        return self.params.double().var(0, unbiased=False).float()

    def stddev(self):
        return self.variance().sqrt()


class PointMass(RandomVariable):
    """Point mass (``edward/models/point_mass.py:16``); only its ``support``
    tag matters to auto_transform here."""

    support = "point"

    def __init__(self, params, name=None):
        super().__init__((), name)
        self.params_node = as_node(params)


class Beta(RandomVariable):
    """Beta(concentration1, concentration0) (support '01')."""

    support = "01"
    reparameterizable = True

    def __init__(self, concentration1=1.0, concentration0=1.0, sample_shape=(), name=None,
                 value=None):
        super().__init__(sample_shape, name, value)
        self.concentration1 = as_node(concentration1)
        self.concentration0 = as_node(concentration0)

    @property
    def batch_shape(self):
        return tuple(np.broadcast_shapes(self.concentration1.shape or (),
                                         self.concentration0.shape or ()))

    def params(self):
        return {"concentration1": self.concentration1, "concentration0": self.concentration0}


class Gamma(RandomVariable):
    """Gamma(concentration, rate) (support 'nonnegative')."""

    support = "nonnegative"
    reparameterizable = True

    def __init__(self, concentration=1.0, rate=1.0, sample_shape=(), name=None, value=None):
        super().__init__(sample_shape, name, value)
        self.concentration = as_node(concentration)
        self.rate = as_node(rate)

    @property
    def batch_shape(self):
        return tuple(np.broadcast_shapes(self.concentration.shape or (), self.rate.shape or ()))

    def params(self):
        return {"concentration": self.concentration, "rate": self.rate}


class Dirichlet(RandomVariable):
    """Dirichlet(concentration [K]) (support 'simplex'; event shape [K])."""

    support = "simplex"
    reparameterizable = True

    def __init__(self, concentration, sample_shape=(), name=None, value=None):
        super().__init__(sample_shape, name, value)
        self.concentration = as_node(concentration)

    @property
    def event_shape(self):
        return tuple(self.concentration.shape[-1:]) if self.concentration.shape else ()

    @property
    def batch_shape(self):
        return tuple(self.concentration.shape[:-1]) if self.concentration.shape else ()

    def params(self):
        return {"concentration": self.concentration}


class Poisson(RandomVariable):
    """Poisson(rate) (support 'countable')."""

    support = "countable"

    def __init__(self, rate, sample_shape=(), name=None, value=None):
        super().__init__(sample_shape, name, value)
        self.rate = as_node(rate)

    @property
    def batch_shape(self):
        return tuple(self.rate.shape or ())

    def params(self):
        return {"rate": self.rate}


class Categorical(RandomVariable):
    """Categorical(logits or probs [..., K]) (support 'countable')."""

    support = "countable"

    def __init__(self, logits=None, probs=None, sample_shape=(), name=None, value=None):
        super().__init__(sample_shape, name, value)
        if (logits is None) == (probs is None):
            raise ValueError("Categorical needs exactly one of logits or probs")
        self.logits = as_node(logits) if logits is not None else None
        self.probs = as_node(probs) if probs is not None else None

    @property
    def batch_shape(self):
        n = self.logits if self.logits is not None else self.probs
        return tuple(n.shape[:-1]) if n.shape else ()

    def params(self):
        return {"logits": self.logits} if self.logits is not None else {"probs": self.probs}
