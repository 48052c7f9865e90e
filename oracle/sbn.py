"""Sigmoid belief network under the score-function gradient, FP64.
Test infrastructure: see ``oracle/__init__.py``.

Model of ``examples/sigmoid_belief_network.py:54-86`` with two stochastic
layers (hidden_sizes = [H0, H1]):

    p:  z1 ~ Bern(prior_logits),  z0 ~ Bern(z1 Wp1 + bp1),  x ~ Bern(z0 Wp0 + bp0)
    q:  z0 ~ Bern(x Wq0 + bq0),   z1 ~ Bern(z0 Wq1 + bq1)

The gradient is ``build_score_loss_and_gradients`` (``edward/inferences/
klqp.py:840-906``): loss = -mean_s F_s with F_s = sum_b [log p(x_b, z_sb) -
log q(z_sb | x_b)]; the q-gradient is -mean_s grad(log q(z_s)) * F_s (the
learning signal is stop-gradient), the p-gradient is grad(loss).  With a
baseline the learning signal becomes per row, f_sb - b(x_b), with the learned
b(x) = c + sigma * mlp(2x - 1) (tanh hidden layer).

Parameters are four [in + 1, out] blocks (bias as the last row):
Wq0 [V+1, H0], Wq1 [H0+1, H1], Wp1 [H1+1, H0], Wp0 [H0+1, V].
"""
import itertools

import numpy as np

from . import densities as dn
from .philox import uniforms24

NONE, MEAN, MLP = 0, 1, 2
KIND_BERNOULLI = 3


def layout(V, H0, H1):
    shapes = [(V + 1, H0), (H0 + 1, H1), (H1 + 1, H0), (H0 + 1, V)]
    offs = np.concatenate([[0], np.cumsum([a * b for a, b in shapes])])
    return shapes, offs


def n_params(V, H0, H1):
    return int(layout(V, H0, H1)[1][-1])


def unpack(theta, V, H0, H1):
    shapes, offs = layout(V, H0, H1)
    return [np.asarray(theta[offs[i]:offs[i + 1]], np.float64).reshape(shapes[i])
            for i in range(4)]


def baseline_layout(V, BH):
    return [(V + 1, BH), (BH + 1, 1)]


def n_baseline_params(V, BH):
    return (V + 1) * BH + BH + 1


def aug(a):
    """Append the ones column."""
    return np.concatenate([a, np.ones(a.shape[:-1] + (1,))], axis=-1)


def bern_logp(z, logits):
    """log Bern(z | logits), elementwise."""
    return z * logits - dn.softplus(logits)


def draw_uniforms(seed, t, S, B, H0, H1):
    """Philox stream 3 at iteration t: counter row s*B + b, element j (z0) or
    round_up(H0, 4) + j (z1)."""
    H0p = (H0 + 3) // 4 * 4
    u = uniforms24(seed, KIND_BERNOULLI, t, S * B, H0p + H1)
    return u[:, :H0].reshape(S, B, H0), u[:, H0p:H0p + H1].reshape(S, B, H1)


def sample_z(theta, X, u0, u1, V, H0, H1):
    """z = u < sigmoid(logit), layer by layer (z1's logits depend on z0)."""
    Wq0, Wq1, _, _ = unpack(theta, V, H0, H1)
    Xa = aug(np.asarray(X, np.float64))
    p0 = dn.sigmoid(Xa @ Wq0)
    z0 = (u0 < p0[None]).astype(np.float64)
    p1 = dn.sigmoid(aug(z0) @ Wq1)
    z1 = (u1 < p1).astype(np.float64)
    return z0, z1, (p0, p1)


def mlp_forward(bparams, X, V, BH):
    """The baseline network on the centred input 2x - 1: (hidden [B, BH], out [B])."""
    w0 = np.asarray(bparams[:(V + 1) * BH], np.float64).reshape(V + 1, BH)
    w1 = np.asarray(bparams[(V + 1) * BH:], np.float64)
    Hb = np.tanh(aug(2.0 * np.asarray(X, np.float64) - 1.0) @ w0)
    return Hb, Hb @ w1[:BH] + w1[BH]


def score_step(theta, X, prior_logits, z0, z1, V, H0, H1, mode=NONE, stats=None,
               bparams=None, BH=0, rb=False):
    """One score-function gradient at fixed draws.  Returns a dict with loss,
    grad [P] (w.r.t. theta), f [S, B], A [S, B] (the learning signal used for
    q(z0 | x)), F [S] and (MLP mode) Hb, mlp_out.  ``rb``: the Rao-Blackwellised
    estimator of ``build_score_rb_loss_and_gradients`` (``klqp.py:1058-1152``):
    the Markov blanket of z1 in p is {z1, z0} and in q {qz1, qz0}, so q(z1 | z0)'s
    signal is F_s - sum_b log p(x_b | z0_sb); q(z0 | x)'s blanket covers every
    factor (q(z1 | z0) descends from its parameters), so its signal stays F_s."""
    theta = np.asarray(theta, np.float64)
    X = np.asarray(X, np.float64)
    pl = np.asarray(prior_logits, np.float64)
    Wq0, Wq1, Wp1, Wp0 = unpack(theta, V, H0, H1)
    S = z0.shape[0]
    Xa = aug(X)
    Lq0 = Xa @ Wq0                                     # [B, H0]
    lq0 = bern_logp(z0, Lq0[None]).sum(-1)             # [S, B]
    R0 = z0 - dn.sigmoid(Lq0)[None]
    Z0a = aug(z0)
    Lq1 = Z0a @ Wq1                                    # [S, B, H1]
    lq1 = bern_logp(z1, Lq1).sum(-1)
    R1 = z1 - dn.sigmoid(Lq1)
    lp1 = bern_logp(z1, pl[None, None]).sum(-1)
    Z1a = aug(z1)
    Lp1 = Z1a @ Wp1                                    # [S, B, H0]
    lp0 = bern_logp(z0, Lp1).sum(-1)
    Rp1 = z0 - dn.sigmoid(Lp1)
    Lp0 = Z0a @ Wp0                                    # [S, B, V]
    lx = bern_logp(X[None], Lp0).sum(-1)
    Rx = X[None] - dn.sigmoid(Lp0)
    f = lp1 + lp0 + lx - lq0 - lq1
    F = f.sum(axis=1)
    out = {"loss": float(-F.mean()), "f": f, "F": F}
    if mode == NONE:
        A = np.broadcast_to(F[:, None], f.shape)
    elif stats[2] <= 0:
        A = f
    elif mode == MEAN:
        A = f - stats[0]
    else:
        Hb, o = mlp_forward(bparams, X, V, BH)
        out.update(Hb=Hb, mlp_out=o)
        A = f - (stats[0] + stats[1] * o)[None]
    if mode == MLP and "mlp_out" not in out:
        Hb, o = mlp_forward(bparams, X, V, BH)
        out.update(Hb=Hb, mlp_out=o)
    out["A"] = np.array(A)
    A1 = A
    if rb:
        if mode != NONE:
            raise ValueError("the Rao-Blackwellised estimator takes no baseline")
        A1 = np.broadcast_to((F - lx.sum(axis=1))[:, None], f.shape)
    gq0 = Xa.T @ (A[..., None] * R0).sum(axis=0)
    gq1 = np.einsum("sbi,sbj->ij", Z0a, A1[..., None] * R1)
    gp1 = np.einsum("sbi,sbj->ij", Z1a, Rp1)
    gp0 = np.einsum("sbi,sbj->ij", Z0a, Rx)
    out["grad"] = -np.concatenate([g.reshape(-1) for g in (gq0, gq1, gp1, gp0)]) / S
    return out


def baseline_update(out, X, stats, bparams, bslots, V, BH, mode, decay, lr, beta1=0.9,
                    beta2=0.999, epsilon=1e-8):
    """The baseline's own step after a score step: one Adam step of the MLP
    regression of (mean_s f_sb - c) / sigma on x_b (MLP mode, from the second
    update on), then the running mean / scale.  Returns new (stats, bparams,
    bslots) as float64 arrays."""
    stats = np.array(stats, np.float64)
    f = out["f"]
    fbar = f.mean(axis=0)
    B = fbar.shape[0]
    if mode == MLP:
        bparams = np.array(bparams, np.float64)
        bslots = np.array(bslots, np.float64)
    if mode == MLP and stats[2] > 0:
        c, sig = stats[0], stats[1]
        t = (fbar - c) / sig
        o, Hb = out["mlp_out"], out["Hb"]
        d = 2.0 * (o - t) / B
        w1 = bparams[(V + 1) * BH:]
        dw1 = aug(Hb).T @ d
        dHb = d[:, None] * w1[None, :BH] * (1.0 - Hb * Hb)
        dw0 = aug(2.0 * np.asarray(X, np.float64) - 1.0).T @ dHb
        g = np.concatenate([dw0.reshape(-1), dw1])
        PB = g.size
        m, v = bslots[:PB], bslots[PB:]
        b1p, b2p = stats[3], stats[4]
        lr_t = lr * np.sqrt(1 - b2p) / (1 - b1p)
        m = beta1 * m + (1 - beta1) * g
        v = beta2 * v + (1 - beta2) * g * g
        bparams = bparams - lr_t * m / (np.sqrt(v) + epsilon)
        bslots = np.concatenate([m, v])
        stats[5] = np.mean((o - t) ** 2)
        stats[3] *= beta1
        stats[4] *= beta2
    mean = fbar.mean()
    var = max((fbar ** 2).mean() - mean ** 2, 0.0)
    if stats[2] <= 0:
        stats[0] = mean
        stats[1] = np.sqrt(max(var, 1e-6))
    else:
        c0 = stats[0]
        s2 = decay * stats[1] ** 2 + (1 - decay) * (var + (mean - c0) ** 2)
        stats[0] = decay * c0 + (1 - decay) * mean
        stats[1] = np.sqrt(max(s2, 1e-6))
    stats[2] += 1
    return stats, bparams, bslots


def exact_elbo(theta, X, prior_logits, V, H0, H1):
    """sum_b E_q[log p(x_b, z) - log q(z | x_b)] by enumerating every z0, z1
    (tiny widths only)."""
    theta = np.asarray(theta, np.float64)
    Wq0, Wq1, Wp1, Wp0 = unpack(theta, V, H0, H1)
    pl = np.asarray(prior_logits, np.float64)
    total = 0.0
    for x in np.asarray(X, np.float64):
        xa = np.append(x, 1.0)
        Lq0 = xa @ Wq0
        for z0 in itertools.product((0.0, 1.0), repeat=H0):
            z0 = np.array(z0)
            lq0 = bern_logp(z0, Lq0).sum()
            Lq1 = np.append(z0, 1.0) @ Wq1
            Lp0 = np.append(z0, 1.0) @ Wp0
            lx = bern_logp(x, Lp0).sum()
            for z1 in itertools.product((0.0, 1.0), repeat=H1):
                z1 = np.array(z1)
                lq = lq0 + bern_logp(z1, Lq1).sum()
                lp = bern_logp(z1, pl).sum() + bern_logp(z0, np.append(z1, 1.0) @ Wp1).sum() + lx
                total += np.exp(lq) * (lp - lq)
    return total


def exact_grad(theta, X, prior_logits, V, H0, H1, h=1e-6):
    """d(-ELBO)/d theta by central differences of the enumerated ELBO."""
    theta = np.asarray(theta, np.float64)
    g = np.empty_like(theta)
    for p in range(theta.size):
        a, b = theta.copy(), theta.copy()
        a[p] += h
        b[p] -= h
        g[p] = -(exact_elbo(a, X, prior_logits, V, H0, H1) -
                 exact_elbo(b, X, prior_logits, V, H0, H1)) / (2 * h)
    return g


def synthetic(N, V, H0, H1, seed=0):
    """Binary data [N, V] (uint8) from a random SBN H1 -> H0 -> V with
    W ~ N(0, 1) / sqrt(fan_in), zero biases and z1 ~ Bern(1/2)."""
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((H1, H0)) / np.sqrt(H1)
    W0 = rng.standard_normal((H0, V)) / np.sqrt(H0)
    z1 = (rng.random((N, H1)) < 0.5).astype(np.float64)
    z0 = (rng.random((N, H0)) < dn.sigmoid(z1 @ W1)).astype(np.float64)
    return (rng.random((N, V)) < dn.sigmoid(z0 @ W0)).astype(np.uint8)
