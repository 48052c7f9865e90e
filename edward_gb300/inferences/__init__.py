"""Inference classes of the hot path (``edward/inferences/__init__.py``)."""
from .inference import Inference
from .variational_inference import VariationalInference
from .klqp import (KLqp, ReparameterizationKLqp, ReparameterizationKLKLqp, ScoreKLqp,
                   ScoreRBKLqp)
from .monte_carlo import MonteCarlo
from .hmc import HMC
from .sgmcmc import SGLD, SGHMC, MetropolisHastings
