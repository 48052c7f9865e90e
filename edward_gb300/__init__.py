"""edward_gb300: Edward's inference hot path (KLqp, ScoreKLqp, HMC and the
log densities they evaluate) on hand-written sm_103a CUDA kernels.

Usage mirrors ``import edward as ed``::

    import edward_gb300 as ed
    from edward_gb300.models import Normal, Bernoulli, Empirical
    w = Normal(loc=ed.zeros(D), scale=ed.ones(D))
    b = Normal(loc=0.0, scale=1.0)
    y = Bernoulli(logits=ed.dot(X, w) + b)
    ed.KLqp([w, b], data={y: y_train}).run(n_samples=5, n_iter=1000)
"""
__version__ = "1.3.5+gb300.0.1"

from . import layers, models, train
from .criticisms import copy, evaluate, ppc
from .expr import (Variable, placeholder, dot, matmul, tanh, sigmoid, softplus, reshape, cast,
                   zeros, ones)
from .inferences import (Inference, VariationalInference, KLqp, ReparameterizationKLqp,
                         ReparameterizationKLKLqp, ScoreKLqp, ScoreRBKLqp, MonteCarlo, HMC,
                         SGLD, SGHMC, MetropolisHastings)
from .util import set_seed, Progbar
