"""Thin tensor-level wrappers over the C ABI (device buffers in, device
buffers out) and the ``torch.autograd.Function`` that exposes the
hand-written log-joint adjoint in place of TF autodiff
(``tf.gradients`` at ``edward/inferences/klqp.py:702`` and
``edward/inferences/hmc.py:199,206``)."""
import ctypes

import numpy as np
import torch

from . import _lib
from .compile import GLMSpec


class GLMDevice:
    """Device copy of a compiled GLM (data is copied to HBM once, as
    ``Inference.__init__`` copies numpy data into a TF variable once,
    ``edward/inferences/inference.py:88-95``)."""

    def __init__(self, spec: GLMSpec, device="cuda"):
        _lib.require_cuda()
        self.spec = spec
        self.device = torch.device(device)
        self.X = torch.as_tensor(spec.X, dtype=torch.float32).contiguous().to(self.device)
        self.y = torch.as_tensor(spec.y, dtype=torch.float32).contiguous().to(self.device)
        self.prior_loc = torch.as_tensor(spec.prior_loc, dtype=torch.float32).to(self.device)
        self.prior_scale = torch.as_tensor(spec.prior_scale, dtype=torch.float32).to(self.device)
        self.c = _lib.EdgGLM()
        self.c.X = self.X.data_ptr()
        self.c.y = self.y.data_ptr()
        self.c.N = spec.N
        self.c.D = spec.D
        self.c.bias = 1 if spec.bias else 0
        self.c.lik = spec.lik
        self.c.lik_scale = spec.lik_scale
        self.c.prior_loc = self.prior_loc.data_ptr()
        self.c.prior_scale = self.prior_scale.data_ptr()

    @property
    def P(self):
        return self.spec.P

    def ref(self):
        return ctypes.byref(self.c)


def glm_logjoint_grad(glm: GLMDevice, Z, include_prior=True, data_scale=1.0, want_grad=True):
    """(lp [B] float64, grad [B, P] float32) for parameter vectors Z [B, P]."""
    Z = Z.detach().to(torch.float32).contiguous()
    B = Z.shape[0]
    if Z.dim() != 2 or Z.shape[1] != glm.P:
        raise ValueError(f"Z must have shape [B, {glm.P}]")
    lib = _lib.load()
    ws_bytes = lib.edg_glm_logjoint_grad_workspace_bytes(glm.ref(), B)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=Z.device)
    lp = torch.empty(B, dtype=torch.float64, device=Z.device)
    g = torch.empty(B, glm.P, dtype=torch.float32, device=Z.device) if want_grad else None
    _lib.call("edg_glm_logjoint_grad", glm.ref(), _lib.ptr(Z), B, 1 if include_prior else 0,
              float(data_scale), _lib.ptr(lp), _lib.ptr(g), _lib.ptr(ws), ws_bytes, _lib.stream_ptr())
    return lp, g


class GLMLogJoint(torch.autograd.Function):
    """log p(y, z) per row of Z with the hand-written adjoint as backward."""

    @staticmethod
    def forward(ctx, Z, glm, include_prior, data_scale):
        lp, g = glm_logjoint_grad(glm, Z, include_prior, data_scale, want_grad=True)
        ctx.save_for_backward(g)
        return lp.to(Z.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return (grad_out.to(g.dtype)[:, None] * g).to(grad_out.dtype), None, None, None


def glm_log_joint(glm, Z, include_prior=True, data_scale=1.0):
    return GLMLogJoint.apply(Z, glm, include_prior, data_scale)


def philox_normal(seed, kind, iteration, rows, n, device="cuda"):
    out = torch.empty(rows, n, dtype=torch.float32, device=device)
    _lib.call("edg_philox_normal", int(seed), int(kind), int(iteration), rows, n, _lib.ptr(out),
              _lib.stream_ptr())
    return out


def philox_u32(seed, kind, iteration, rows, n, device="cuda"):
    nq4 = (n + 3) // 4 * 4
    out = torch.empty(rows, nq4, dtype=torch.int32, device=device)
    _lib.call("edg_philox_u32", int(seed), int(kind), int(iteration), rows, n, _lib.ptr(out),
              _lib.stream_ptr())
    return out


def philox_uniform64(seed, kind, iteration, rows, device="cuda"):
    out = torch.empty(rows, dtype=torch.float64, device=device)
    _lib.call("edg_philox_uniform64", int(seed), int(kind), int(iteration), rows, _lib.ptr(out),
              _lib.stream_ptr())
    return out


class HierDevice:
    """Device copy of a ragged batch of hierarchical logistic regressions
    (instance i: X_i [N_i, D_i], y_i [N_i]) packed for edg_hmc_hier_run:
    X and y concatenated, per-instance offsets/sizes, and a launch order that
    starts the heaviest instances (N_i * D_i) first."""

    def __init__(self, Xs, ys, mu_loc=0.0, mu_scale=1.0, tau_scale=1.0, device="cuda"):
        _lib.require_cuda()
        if len(Xs) != len(ys) or not Xs:
            raise ValueError("need one y per X and at least one instance")
        Ns = np.array([np.asarray(x).shape[0] for x in Xs], np.int32)
        Ds = np.array([np.asarray(x).shape[1] for x in Xs], np.int32)
        for x, y in zip(Xs, ys):
            if np.asarray(y).reshape(-1).shape[0] != np.asarray(x).shape[0]:
                raise ValueError("each y_i must have N_i entries")
        self.I = len(Xs)
        self.Ns, self.Ds = Ns, Ds
        self.max_D = int(Ds.max())
        x_off = np.concatenate([[0], np.cumsum(Ns.astype(np.int64) * Ds)[:-1]]).astype(np.int64)
        y_off = np.concatenate([[0], np.cumsum(Ns.astype(np.int64))[:-1]]).astype(np.int64)
        self.device = torch.device(device)
        self.X = torch.as_tensor(np.concatenate([np.asarray(x, np.float32).reshape(-1) for x in Xs]),
                                 device=self.device)
        self.y = torch.as_tensor(np.concatenate([np.asarray(y, np.float32).reshape(-1) for y in ys]),
                                 device=self.device)
        self.x_off = torch.as_tensor(x_off, device=self.device)
        self.y_off = torch.as_tensor(y_off, device=self.device)
        self.N_t = torch.as_tensor(Ns, device=self.device)
        self.D_t = torch.as_tensor(Ds, device=self.device)
        work = Ns.astype(np.int64) * Ds
        self.order = torch.as_tensor(np.argsort(-work, kind="stable").astype(np.int32),
                                     device=self.device)
        self.c = _lib.EdgHier()
        self.c.X, self.c.y = self.X.data_ptr(), self.y.data_ptr()
        self.c.x_offset, self.c.y_offset = self.x_off.data_ptr(), self.y_off.data_ptr()
        self.c.N, self.c.D = self.N_t.data_ptr(), self.D_t.data_ptr()
        self.c.I, self.c.max_D = self.I, self.max_D
        self.c.mu_loc, self.c.mu_scale, self.c.tau_scale = mu_loc, mu_scale, tau_scale

    @property
    def SP(self):
        return self.max_D + 2

    def ref(self):
        return ctypes.byref(self.c)
