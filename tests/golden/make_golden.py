"""Generates the golden fixtures under tests/golden/ from the FP64 oracle.

The reference (TensorFlow 1.x) cannot run in this environment, so these
fixtures freeze the oracle's outputs on small seeded cases: they pin the GPU
kernels and guard the oracle itself against regressions.  The oracle's own
pins are the Philox known-answer vectors, FP64 finite differences and the
closed-form posteriors of the reference's tests (see tests/test_oracle.py).

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.glm import GLM, NORMAL, synthetic_logreg  # noqa: E402
from oracle.hmc import glm_lj_grad, hmc_step  # noqa: E402
from oracle.klqp import REPARAM, REPARAM_KL, SCORE, TFAdam, default_learning_rate, \
    klqp_glm_loss_and_grads  # noqa: E402
from oracle.philox import KIND_MOMENTUM, KIND_UNIFORM, normals, raw_u32, uniforms64  # noqa: E402


def main():
    rng = np.random.default_rng(1234)
    out = {}
    # Philox streams (seed with both key words non-zero)
    seed = 0x0123456789ABCDEF
    out["philox_u32"] = raw_u32(seed, 1, 7, 5, 10)
    out["philox_normal"] = normals(seed, 1, 7, 5, 10)
    out["philox_uniform64"] = uniforms64(seed, 2, 7, 5)

    # logistic regression, ragged N, bias
    X, y, _, _ = synthetic_logreg(37, 5, seed=3)
    m = GLM(X, y, bias=True, prior_loc=0.25, prior_scale=1.5)
    Z = rng.standard_normal((3, 6))
    out["lr_X"], out["lr_y"], out["lr_Z"] = X, y, Z
    out["lr_lp"] = m.log_joint(Z)
    out["lr_grad"] = m.grad_log_joint(Z)
    out["lr_ll"] = m.log_lik(Z, scaled=False)
    out["lr_gll"] = m.grad_log_lik(Z, scaled=False)

    # Normal-Normal (klqp_test.py:14-44): X = ones(50, 1), no bias
    mn = GLM(np.ones((50, 1)), np.zeros(50), bias=False, lik=NORMAL, lik_scale=1.0)
    Zn = rng.standard_normal((4, 1))
    out["nn_Z"] = Zn
    out["nn_lp"] = mn.log_joint(Zn)
    out["nn_grad"] = mn.grad_log_joint(Zn)

    # KLqp loss / gradients for the three estimators
    mu = rng.standard_normal(6) * 0.5
    rho = rng.standard_normal(6) * 0.5
    eps = rng.standard_normal((4, 6))
    out["kq_mu"], out["kq_rho"], out["kq_eps"] = mu, rho, eps
    for name, meth in (("kl", REPARAM_KL), ("re", REPARAM), ("sc", SCORE)):
        loss, gmu, grho, _ = klqp_glm_loss_and_grads(m, mu, rho, eps, meth)
        out[f"kq_{name}_loss"] = np.array(loss)
        out[f"kq_{name}_gmu"] = gmu
        out[f"kq_{name}_grho"] = grho
    # three Adam steps with the default schedule (analytic KL)
    opt = TFAdam(12)
    th = np.concatenate([mu, rho])
    traj = []
    for t in range(3):
        _, gmu, grho, _ = klqp_glm_loss_and_grads(m, th[:6], th[6:], eps, REPARAM_KL)
        th = opt.apply(th, np.concatenate([gmu, grho]), default_learning_rate(t))
        traj.append(th.copy())
    out["kq_adam_traj"] = np.array(traj)

    # one HMC iteration, 3 chains, 3 leapfrog steps
    z0 = rng.standard_normal((3, 6)) * 0.3
    f = glm_lj_grad(m)
    lj0, g0 = f(z0)
    r0 = normals(99, KIND_MOMENTUM, 0, 3, 6)
    u = uniforms64(99, KIND_UNIFORM, 0, 3)
    res = hmc_step(f, z0, g0, lj0, r0, u, 0.05, 3)
    out["hmc_z0"], out["hmc_r0"], out["hmc_u"] = z0, r0, u
    out["hmc_zprop"], out["hmc_ratio"] = res["z_prop"], res["ratio"]
    out["hmc_accept"] = res["accept"].astype(np.int32)
    out["hmc_z"] = res["z"]
    np.savez_compressed(os.path.join(HERE, "oracle_small.npz"), **out)
    print("wrote", os.path.join(HERE, "oracle_small.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
