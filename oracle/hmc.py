"""HMC leapfrog + Metropolis update for many independent chains.
Test infrastructure: see ``oracle/__init__.py``.

Restates ``HMC.build_update`` (``edward/inferences/hmc.py:61-130``) and
``leapfrog`` (``hmc.py:195-210``) per chain:

    r0 ~ N(0, I)                                   (hmc.py:88-91)
    g = grad L(z0)
    repeat n_steps:  r += 0.5 eps g;  z += eps r;  g = grad L(z);  r += 0.5 eps g
    ratio = 0.5|r0|^2 - 0.5|r|^2 + L(z) - L(z0)    (hmc.py:100-105)
    accept = log(u) < ratio,  u ~ U(0, 1)          (hmc.py:108-109)
    params[t] = accept ? z : z0;  n_accept += accept  (hmc.py:110-129)

``L`` is the unscaled log joint in the unconstrained space
(``_log_joint_unconstrained``, hmc.py:132-159).  The reference runs one
chain; the batched form treats every row of ``z`` as an independent chain,
each with its own momentum and its own uniform.  The gradient and log joint
at the current state are carried between iterations (the reference recomputes
them; the values are the same).

The energy difference is formed in FP64 (as the GPU kernel does); per-step
arithmetic runs in ``dtype``.
"""
import numpy as np


def hmc_step(lj_grad, z0, g0, lj0, r0, u, step_size, n_steps, dtype=np.float64):
    """One HMC iteration for C chains.

    lj_grad(Z) -> (lj [C] float64, g [C, P]); z0/g0/r0: [C, P]; lj0: [C];
    u: [C] uniforms in (0, 1).  Returns dict with z, g, lj, accept, ratio,
    z_prop, r_prop."""
    dt = dtype
    eps = dt(step_size)
    half = dt(0.5) * eps
    z = np.asarray(z0, dt).copy()
    r = np.asarray(r0, dt).copy()
    g = np.asarray(g0, dt)
    lj = lj0
    for _ in range(n_steps):
        r = r + half * g
        z = z + eps * r
        lj, g = lj_grad(z)
        g = np.asarray(g, dt)
        r = r + half * g
    r0d = np.asarray(r0, np.float64)
    rd = r.astype(np.float64)
    ratio = 0.5 * (r0d * r0d).sum(axis=1) - 0.5 * (rd * rd).sum(axis=1) \
        + np.asarray(lj, np.float64) - np.asarray(lj0, np.float64)
    accept = np.log(np.asarray(u, np.float64)) < ratio
    a = accept[:, None]
    return {
        "z": np.where(a, z, np.asarray(z0, dt)),
        "g": np.where(a, g, np.asarray(g0, dt)),
        "lj": np.where(accept, lj, lj0),
        "accept": accept,
        "ratio": ratio,
        "z_prop": z,
        "r_prop": r,
    }


def glm_lj_grad(model, dtype=np.float64):
    """(lj, grad) closure over an oracle.glm.GLM for ``hmc_step``."""
    def f(Z):
        return model.log_joint(Z, dtype=dtype), model.grad_log_joint(Z, dtype=dtype)
    return f


def run_hmc(lj_grad, z_init, n_iter, step_size, n_steps, seed, t0=0,
            r_fn=None, u_fn=None, dtype=np.float64):
    """n_iter iterations; returns (samples [n_iter, C, P], n_accept [C])."""
    from .philox import normals, uniforms64, KIND_MOMENTUM, KIND_UNIFORM
    z = np.asarray(z_init, np.float64)
    C, P = z.shape
    lj, g = lj_grad(z)
    samples = np.empty((n_iter, C, P))
    n_acc = np.zeros(C, np.int64)
    for i in range(n_iter):
        t = t0 + i
        r0 = r_fn(t) if r_fn else normals(seed, KIND_MOMENTUM, t, C, P)
        u = u_fn(t) if u_fn else uniforms64(seed, KIND_UNIFORM, t, C)
        out = hmc_step(lj_grad, z, g, lj, r0, u, step_size, n_steps, dtype)
        z, g, lj = out["z"], out["g"], out["lj"]
        n_acc += out["accept"]
        samples[i] = z
    return samples, n_acc
