"""Criticism on the device sample store: ``ed.copy`` (posterior predictive
nodes), ``ed.evaluate`` and ``ed.ppc`` (``edward/criticisms/evaluate.py:20-233``,
``ppc.py:13-104``, ``edward/util/random_variables.py:139-445``) for the GLM
family.

The posterior draws come straight from the inference's device buffers (an
``Empirical`` store [T, (C,) ...] or a Normal q's parameters); the predictive
means, linear predictors and replicated data are computed by
``edg_glm_predict`` and the log-likelihood metric by the log-joint kernel, so
nothing is copied to the host but the metric values.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .compile import compile_glm, parse_normal_q
from .expr import Placeholder
from .models import Bernoulli, Empirical, Normal, RandomVariable
from .ops import GLMDevice, glm_logjoint_grad


class PosteriorPredictive(RandomVariable):
    """``ed.copy(x, {z: qz, ...})``: the observed variable x with its latent
    parents replaced by their posterior approximations."""

    def __init__(self, org, dict_swap):
        super().__init__((), name=f"{org.name}_post")
        self.org = org
        self.dict_swap = dict(dict_swap)
        self.support = org.support

    @property
    def shape(self):
        return self.org.shape


def copy(org, dict_swap=None, scope="copied", replace_itself=False, copy_q=False,
         copy_parent_rvs=True):
    """Posterior predictive of ``org`` under ``dict_swap`` (latent -> q)."""
    if not isinstance(org, RandomVariable):
        raise NotImplementedError("copy is implemented for random variables")
    if not dict_swap:
        return org
    return PosteriorPredictive(org, dict_swap)


def _draws(spec, swap, n, gen, device):
    """n parameter vectors [n, P] drawn from the approximations in ``swap``
    (an Empirical: uniformly among its stored samples, as Empirical.sample;
    a Normal(loc, softplus(rho)) q: loc + scale * N(0, 1))."""
    Z = torch.empty(n, spec.P, dtype=torch.float32, device=device)
    for blk in spec.blocks:
        q = swap.get(blk.rv)
        if q is None:
            raise KeyError(f"no posterior approximation for {blk.rv.name} in dict_swap")
        sl = slice(blk.offset, blk.offset + blk.size)
        if isinstance(q, Empirical):
            v = q.params.to(device, torch.float32).reshape(-1, blk.size)
            idx = torch.randint(0, v.shape[0], (n,), device=device, generator=gen)
            Z[:, sl] = v[idx]
        elif isinstance(q, Normal):
            nq = parse_normal_q(q)
            loc = nq.loc_var.value.to(device, torch.float32).reshape(-1)
            scale = torch.nn.functional.softplus(nq.rho_var.value.to(device, torch.float32)).reshape(-1)
            e = torch.randn(n, blk.size, device=device, generator=gen)
            Z[:, sl] = loc + scale * e
        else:
            raise NotImplementedError(f"posterior approximation {type(q).__name__}")
    return Z


def _setup(data, output_key):
    if output_key is None:
        keys = [k for k in data if isinstance(k, RandomVariable)]
        if len(keys) != 1:
            raise KeyError("User must specify output_key.")
        output_key = keys[0]
    elif not isinstance(output_key, RandomVariable):
        raise TypeError("output_key must have type RandomVariable.")
    post = output_key if isinstance(output_key, PosteriorPredictive) else None
    if post is None:
        raise NotImplementedError("evaluate / ppc need ed.copy(x, {z: qz, ...}) as the output")
    y_true = np.asarray(data[output_key], np.float32).reshape(-1)
    model_data = {post.org: y_true}
    model_data.update({k: v for k, v in data.items() if isinstance(k, Placeholder)})
    spec = compile_glm(list(post.dict_swap.keys()), model_data)
    return post, spec, y_true


def evaluate(metrics, data, n_samples=500, output_key=None, seed=None):
    """``ed.evaluate`` for the GLM family: 'binary_accuracy', 'log_loss' /
    'binary_crossentropy', 'mse', 'mae', 'log_lik' (and their aliases)."""
    if isinstance(metrics, (str, tuple)) or callable(metrics):
        metrics = [metrics]
    elif not isinstance(metrics, list):
        raise TypeError("metrics must have type str or list, or be callable.")
    if not isinstance(n_samples, int):
        raise TypeError("n_samples must have type int.")
    _lib.require_cuda()
    dev = torch.device("cuda")
    post, spec, y_true = _setup(data, output_key)
    glm = GLMDevice(spec, dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed) if seed is not None else int(np.random.randint(0, 2 ** 31 - 1)))
    Z = _draws(spec, post.dict_swap, n_samples, gen, dev)
    yt = glm.y
    N = spec.N
    need_pred = any((m[0] if isinstance(m, tuple) else m) not in ("log_lik", "log_likelihood")
                    for m in metrics)
    y_pred = None
    if need_pred:
        mean = torch.empty(N, dtype=torch.float32, device=dev)
        _lib.call("edg_glm_predict", glm.ref(), _lib.ptr(Z), n_samples, _lib.PREDICT_MEAN, 0, 0,
                  _lib.ptr(mean), _lib.stream_ptr())
        if isinstance(post.org, Bernoulli):
            # round the averaged probabilities, ties broken at random (evaluate.py:152-157)
            tie = torch.rand(N, device=dev, generator=gen)
            y_pred = torch.round(torch.where(mean == 0.5, tie, mean))
        else:
            # the average of n_samples predictive draws: mean eta + noise averaged over the draws
            noise = torch.randn(N, device=dev, generator=gen) * (spec.lik_scale / np.sqrt(n_samples))
            y_pred = mean + noise
    out = []
    for m in metrics:
        name = m[0] if isinstance(m, tuple) else m
        if callable(name):
            out.append(float(name(yt, y_pred)))
        elif name == "binary_accuracy":
            out.append(float((y_pred == yt).float().mean()))
        elif name in ("log_loss", "binary_crossentropy"):
            # tf.nn.sigmoid_cross_entropy_with_logits(logits=y_pred, labels=y_true)
            x = y_pred
            out.append(float((torch.clamp(x, min=0) - x * yt + torch.log1p(torch.exp(-x.abs()))).mean()))
        elif name in ("mse", "MSE", "mean_squared_error"):
            out.append(float(((y_pred - yt) ** 2).mean()))
        elif name in ("mae", "MAE", "mean_absolute_error"):
            out.append(float((y_pred - yt).abs().mean()))
        elif name in ("log_lik", "log_likelihood"):
            lp, _ = glm_logjoint_grad(glm, Z, include_prior=False, data_scale=1.0, want_grad=False)
            out.append(float(lp.mean() / N))
        else:
            raise NotImplementedError("Metric is not implemented: {}".format(name))
    return out[0] if len(out) == 1 else out


def ppc(T, data, latent_vars=None, n_samples=100):
    """``ed.ppc`` for the GLM family.  ``T(xs, zs)`` receives device tensors:
    ``xs`` maps the output to replicated (or observed) data and placeholders to
    their values, ``zs`` maps each latent to a posterior draw.  Returns
    [T(x_rep, z) for each replication, T(x_obs, z) for each], as NumPy arrays."""
    if not callable(T):
        raise TypeError("T must be a callable function.")
    if not isinstance(n_samples, int):
        raise TypeError("n_samples must have type int.")
    _lib.require_cuda()
    dev = torch.device("cuda")
    post, spec, y_true = _setup(data, None)
    glm = GLMDevice(spec, dev)
    swap = dict(post.dict_swap)
    if latent_vars:
        swap.update(latent_vars)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(np.random.randint(0, 2 ** 31 - 1)))
    Z = _draws(spec, swap, 2 * n_samples, gen, dev)
    yrep = torch.empty(n_samples, spec.N, dtype=torch.float32, device=dev)
    _lib.call("edg_glm_predict", glm.ref(), _lib.ptr(Z), n_samples, _lib.PREDICT_SAMPLE,
              int(np.random.randint(0, 2 ** 63 - 1, dtype=np.int64)), 0, _lib.ptr(yrep),
              _lib.stream_ptr())
    ph = {k: torch.as_tensor(np.asarray(v, np.float32), device=dev)
          for k, v in data.items() if isinstance(k, Placeholder)}
    yobs = glm.y

    def zdict(z):
        return {blk.rv: z[blk.offset:blk.offset + blk.size].reshape(blk.shape)
                for blk in spec.blocks}

    Treps, Tobs = [], []
    for i in range(n_samples):
        Treps.append(np.asarray(torch.as_tensor(T({post: yrep[i], **ph}, zdict(Z[i]))).cpu()))
        Tobs.append(np.asarray(torch.as_tensor(T({post: yobs, **ph}, zdict(Z[n_samples + i]))).cpu()))
    return [np.stack(Treps), np.stack(Tobs)]
