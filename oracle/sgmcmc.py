"""SGLD and SGHMC chains over a GLM (FP64).  Test infrastructure: see
``oracle/__init__.py``.

SGLD, ``edward/inferences/sgld.py:63-88``: at iteration t (0-based) the
state is params[max(t - 1, 0)], lr = step_size / (t + 1)^0.55 and
z <- z + 0.5 lr grad log p(x, z) + sqrt(lr) e.
SGHMC, ``edward/inferences/sghmc.py:67-102``: lr = 0.01 step_size,
z <- z + v, v <- (1 - 0.5 friction) v + lr grad + sqrt(lr friction) e (v from
before the step).  log p(x, z) = log p(z) + scale * log p(x | z), the
reference's ``_log_joint`` with ``scale``.  e ~ N(0, 1): Philox stream 5 at
iteration t, counter row = chain, element = coordinate.
"""
import numpy as np

from .philox import normals

KIND_SGMCMC = 5


def grad_log_joint(model, Z):
    """Prior + data_scale * likelihood gradient, [C, P]."""
    return model.grad_log_prior(Z) + model.grad_log_lik(Z, scaled=True)


def run(model, z0, n_iter, step_size, method="sgld", friction=0.1, seed=0, t0=0,
        noise_fn=None):
    """Returns (samples [n_iter, C, P], final z, final v)."""
    z = np.array(z0, np.float64)
    v = np.zeros_like(z)
    C, P = z.shape
    out = []
    for i in range(n_iter):
        t = t0 + i
        e = noise_fn(t) if noise_fn else normals(seed, KIND_SGMCMC, t, C, P)
        g = grad_log_joint(model, z)
        if method == "sgld":
            lr = step_size / (t + 1.0) ** 0.55
            z = z + 0.5 * lr * g + np.sqrt(lr) * e
        else:
            lr = step_size * 0.01
            z, v = z + v, (1.0 - 0.5 * friction) * v + lr * g + np.sqrt(lr * friction) * e
        out.append(z.copy())
    return np.array(out), z, v
