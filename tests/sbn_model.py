"""The two-layer sigmoid belief network of
``examples/sigmoid_belief_network.py:54-86`` (hidden_sizes = [H0, H1]) written
against the package's Edward surface, for the score-function tests."""
import numpy as np

import edward_gb300 as ed
from edward_gb300.models import Bernoulli


def example_sbn(V, H0, H1, B, x=None, prior_logit=0.0):
    """Returns (latent_vars {z: qz}, x_rv, x_node, weights in the kernel's
    order Wq0, bq0, Wq1, bq1, Wp1, bp1, Wp0, bp0).  ``x`` is the data node of
    the recognition network (default: a float placeholder [B, V])."""
    x_ph = x if x is not None else ed.placeholder(shape=[B, V], name="x")
    z1 = Bernoulli(logits=prior_logit + ed.zeros([B, H1]), name="z1")
    lp1 = ed.layers.dense(ed.cast(z1), H0)
    z0 = Bernoulli(logits=lp1, name="z0")
    lp0 = ed.layers.dense(ed.cast(z0), V)
    xr = Bernoulli(logits=lp0, name="x")
    lq0 = ed.layers.dense(ed.cast(x_ph), H0)
    qz0 = Bernoulli(logits=lq0, name="qz0")
    lq1 = ed.layers.dense(ed.cast(qz0), H1)
    qz1 = Bernoulli(logits=lq1, name="qz1")
    weights = [lq0.args[0].args[1], lq0.args[1], lq1.args[0].args[1], lq1.args[1],
               lp1.args[0].args[1], lp1.args[1], lp0.args[0].args[1], lp0.args[1]]
    return {z0: qz0, z1: qz1}, xr, x_ph, weights


def flat_theta(weights):
    """The flat parameter vector (four [in + 1, out] blocks) of the weights."""
    out = []
    for i in range(4):
        W, b = weights[2 * i].numpy(), weights[2 * i + 1].numpy()
        out += [W.reshape(-1), b.reshape(-1)]
    return np.concatenate(out).astype(np.float64)
