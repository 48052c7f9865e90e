"""Metropolis-Hastings with Normal proposals over a GLM (FP64).  Test
infrastructure: see ``oracle/__init__.py``.

``edward/inferences/metropolis_hastings.py:64-156``: z' from the proposal
(random walk N(z, s) or independence N(m, s)), ratio = log p(x, z') -
log p(x, z) - log g(z' | z) + log g(z | z'), accept if log u < ratio; the kept
state goes to params[t].  log p(x, z) = log p(z) + log p(x | z) (no scale).
Draws: e from Philox stream 6 (iteration t, row = chain, element = coordinate),
u from stream 7 (one FP64 uniform per chain).
"""
import numpy as np

from .philox import normals, uniforms64

KIND_PROPOSAL, KIND_UNIFORM = 6, 7


def step(model, z, t, scale, loc=None, seed=0, e=None, u=None):
    """One iteration for all chains.  Returns (z_new, accepted [C], ratio [C])."""
    z = np.asarray(z, np.float64)
    C, P = z.shape
    if e is None:
        e = normals(seed, KIND_PROPOSAL, t, C, P)
    if u is None:
        u = uniforms64(seed, KIND_UNIFORM, t, C)
    scale = np.asarray(scale, np.float64)
    zp = (z if loc is None else np.asarray(loc, np.float64)[None]) + scale[None] * e
    ratio = model.log_joint(zp) - model.log_joint(z)
    if loc is not None:
        a = (z - loc[None]) / scale[None]
        b = (zp - loc[None]) / scale[None]
        ratio = ratio + (-0.5 * a * a + 0.5 * b * b).sum(axis=1)
    acc = np.log(u) < ratio
    return np.where(acc[:, None], zp, z), acc, ratio
