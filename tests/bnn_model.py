"""Model-building helpers shared by the Bayesian-NN tests: the model of
``examples/bayesian_nn.py:120-150`` written against the package's Edward
surface."""
import numpy as np

import edward_gb300 as ed
from edward_gb300.models import Normal


def example_model(D, H1, H2, X=None, noise=0.1, prior_scale=1.0):
    """Returns (latents list in W0, b0, W1, b1, W2, b2 order, X node, y rv).
    ``X`` is an array / node, or None for an [M, D] placeholder."""
    W0 = Normal(loc=ed.zeros([D, H1]), scale=prior_scale * ed.ones([D, H1]), name="W_0")
    W1 = Normal(loc=ed.zeros([H1, H2]), scale=prior_scale * ed.ones([H1, H2]), name="W_1")
    W2 = Normal(loc=ed.zeros([H2, 1]), scale=prior_scale * ed.ones([H2, 1]), name="W_2")
    b0 = Normal(loc=ed.zeros(H1), scale=prior_scale * ed.ones(H1), name="b_0")
    b1 = Normal(loc=ed.zeros(H2), scale=prior_scale * ed.ones(H2), name="b_1")
    b2 = Normal(loc=ed.zeros(1), scale=prior_scale * ed.ones(1), name="b_2")
    Xn = X if X is not None else ed.placeholder(shape=[None, D], name="X")
    h = ed.tanh(ed.matmul(Xn, W0) + b0)
    h = ed.tanh(ed.matmul(h, W1) + b1)
    h = ed.matmul(h, W2) + b2
    y = Normal(loc=ed.reshape(h, [-1]), scale=noise, name="y")
    return [W0, b0, W1, b1, W2, b2], Xn, y


def example_q(latents, rng):
    """Mean-field q with free loc and softplus scale per latent (as the example)."""
    out = {}
    for z in latents:
        loc = ed.Variable((rng.standard_normal(z.shape) * 0.2).astype(np.float32))
        rho = ed.Variable((rng.standard_normal(z.shape) * 0.2 - 2.0).astype(np.float32))
        out[z] = Normal(loc=loc, scale=ed.softplus(rho))
    return out


def flat_q(qs, latents, attr):
    """Flat (mu or rho) vector of a q dict in the W0, b0, W1, b1, W2, b2 order."""
    vs = []
    for z in latents:
        q = qs[z]
        node = q.loc if attr == "loc" else q.scale.args[0]
        vs.append(node.numpy().reshape(-1))
    return np.concatenate(vs)
