"""Log densities, KL and bijector math restated from the TF 1.x distribution
definitions that Edward's RandomVariables inherit
(``edward/models/random_variables.py:13-28``).  Test infrastructure: see
``oracle/__init__.py``.  All functions are elementwise NumPy and run in the
dtype of their inputs.
"""
import numpy as np

HALF_LOG_2PI = 0.5 * np.log(2.0 * np.pi)


def softplus(x):
    """log(1 + exp(x)), overflow-safe (tf.nn.softplus)."""
    x = np.asarray(x)
    return np.maximum(x, 0) + np.log1p(np.exp(-np.abs(x)))


def softplus_inverse(y):
    """log(exp(y) - 1): the Softplus bijector's inverse
    (``edward/util/random_variables.py:903-904`` maps nonnegative support to
    the real line with tf.contrib.distributions.bijectors.Softplus)."""
    y = np.asarray(y)
    return y + np.log(-np.expm1(-y))


def sigmoid(x):
    x = np.asarray(x)
    return 0.5 * (1.0 + np.tanh(0.5 * x))


def normal_log_prob(x, loc, scale):
    """Normal log density: -0.5 z^2 - log(scale) - 0.5 log(2 pi)."""
    z = (x - loc) / scale
    return -0.5 * z * z - np.log(scale) - HALF_LOG_2PI


def normal_grad_x(x, loc, scale):
    """d/dx of normal_log_prob."""
    return -(x - loc) / (scale * scale)


def bernoulli_logits_log_prob(x, logits):
    """Bernoulli(logits) log pmf as the negated sigmoid cross-entropy:
    -(max(l, 0) - l x + log1p(exp(-|l|)))."""
    return -(np.maximum(logits, 0) - logits * x + np.log1p(np.exp(-np.abs(logits))))


def bernoulli_logits_grad_logits(x, logits):
    """d/dlogits of bernoulli_logits_log_prob = x - sigmoid(logits)."""
    return x - sigmoid(logits)


def half_normal_log_prob(x, scale):
    """HalfNormal(scale) log density on x >= 0: 0.5 log(2/pi) - log(scale) - x^2/(2 scale^2)."""
    return 0.5 * np.log(2.0 / np.pi) - np.log(scale) - 0.5 * (x / scale) ** 2


def kl_normal_normal(loc_q, scale_q, loc_p, scale_p):
    """KL(N(loc_q, scale_q) || N(loc_p, scale_p)), the analytic term used by
    ``build_reparam_kl_loss_and_gradients`` (``klqp.py:751-753``)."""
    ratio = (scale_q / scale_p) ** 2
    return 0.5 * ((loc_q - loc_p) / scale_p) ** 2 + 0.5 * (ratio - 1.0 - np.log(ratio))


def kl_normal_normal_grads(loc_q, scale_q, loc_p, scale_p):
    """(dKL/dloc_q, dKL/dscale_q)."""
    return (loc_q - loc_p) / scale_p ** 2, scale_q / scale_p ** 2 - 1.0 / scale_q
