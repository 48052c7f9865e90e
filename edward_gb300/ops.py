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

    def tc_tiles(self):
        """(tiles, tile_off) for edg_hmc_hier_tc_run: X re-laid once into
        128-row tiles (edg_hmc_hier_tc_prepare), cached."""
        if getattr(self, "_tc", None) is None:
            lib = _lib.load()
            off = np.zeros(self.I, np.int64)
            total = lib.edg_hmc_hier_tc_tile_offsets(self.Ns.ctypes.data, self.Ds.ctypes.data,
                                                     self.I, off.ctypes.data)
            if total < 0:
                raise NotImplementedError("the tensor-core hierarchical engine needs D_i <= 128")
            tiles = torch.empty(max(int(total), 4), dtype=torch.float32, device=self.device)
            off_t = torch.as_tensor(off, device=self.device)
            _lib.call("edg_hmc_hier_tc_prepare", self.ref(), _lib.ptr(off_t), _lib.ptr(tiles),
                      _lib.stream_ptr())
            self._tc = (tiles, off_t)
        return self._tc


class BNNDevice:
    """Device data of a compiled Bayesian NN (``compile.MLPSpec``) and where
    each step's minibatch comes from:

    * X and y bound to arrays, no ``n_minibatch``: every step uses all N rows;
    * X and y bound to arrays with ``n_minibatch=M``: every step gathers M rows
      uniformly with replacement on the device (``edg_minibatch_gather``, Philox
      stream 4 at the step's iteration), replacing the host-side batching of
      ``examples/bayesian_nn.py``-style feed loops;
    * X and/or y placeholders: ``feed`` copies each update's ``feed_dict``
      arrays into fixed device buffers (``inference.update(feed_dict=...)``,
      ``edward/inferences/variational_inference.py:133-164``)."""

    def __init__(self, spec, device="cuda", n_minibatch=None):
        _lib.require_cuda()
        self.spec = spec
        self.device = torch.device(device)
        dev = self.device
        self.gather = False
        self.default_scale = 1.0
        bound_X, bound_y = spec.X is not None, spec.y is not None
        if bound_X and bound_y:
            self.N = spec.X.shape[0]
            self.X_full = torch.as_tensor(spec.X).contiguous().to(dev)
            self.y_full = torch.as_tensor(spec.y, dtype=torch.float32).contiguous().to(dev)
            if n_minibatch is not None:
                if not 0 < int(n_minibatch):
                    raise ValueError("n_minibatch must be positive")
                self.M = int(n_minibatch)
                self.gather = True
                self.default_scale = self.N / self.M
                self.Xb = torch.empty(self.M, spec.D, dtype=torch.float32, device=dev)
                self.yb = torch.empty(self.M, dtype=torch.float32, device=dev)
            else:
                self.M = self.N
                self.Xb, self.yb = self.X_full, self.y_full
            self._fed = {"X": True, "y": True}
        else:
            if n_minibatch is not None:
                raise ValueError("n_minibatch needs X and y bound to arrays in the data dict")
            if bound_X:
                self.M = spec.X.shape[0]
            elif spec.batch is not None:
                self.M = spec.batch
            else:
                raise ValueError("the X placeholder needs a static number of rows")
            self.Xb = (torch.as_tensor(spec.X).contiguous().to(dev) if bound_X else
                       torch.zeros(self.M, spec.D, dtype=torch.float32, device=dev))
            if bound_y:
                if spec.y.shape[0] != self.M:
                    raise ValueError(f"y has {spec.y.shape[0]} rows; X has {self.M}")
                self.yb = torch.as_tensor(spec.y, dtype=torch.float32).contiguous().to(dev)
            else:
                self.yb = torch.zeros(self.M, dtype=torch.float32, device=dev)
            self._fed = {"X": bound_X, "y": bound_y}
        self.seed = None

    @property
    def ready(self):
        return all(self._fed.values())

    def feed(self, feed_dict):
        for k, v in feed_dict.items():
            if k is self.spec.X_node and not self.gather:
                v = np.asarray(v, np.float32)
                if v.shape != (self.M, self.spec.D):
                    raise ValueError(f"fed X has shape {v.shape}; expected {(self.M, self.spec.D)}")
                self.Xb.copy_(torch.from_numpy(np.ascontiguousarray(v)))
                self._fed["X"] = True
            elif k is self.spec.y_node and not self.gather:
                v = np.asarray(v, np.float32).reshape(-1)
                if v.shape[0] != self.M:
                    raise ValueError(f"fed y has {v.shape[0]} rows; expected {self.M}")
                self.yb.copy_(torch.from_numpy(v))
                self._fed["y"] = True
            else:
                raise KeyError(f"{k!r} is not a placeholder of this model")

    def batch(self, state):
        """(X, y) device buffers for the next step; gathers on the device when
        minibatching from bound arrays (stream-ordered, graph-capturable)."""
        if not self.ready:
            raise ValueError("X / y are placeholders: feed them with update(feed_dict=...)")
        if self.gather:
            _lib.call("edg_minibatch_gather", _lib.ptr(self.X_full), _lib.ptr(self.y_full), self.N,
                      self.spec.D, self.M, int(self.seed), _lib.ptr(state), _lib.ptr(self.Xb),
                      _lib.ptr(self.yb), _lib.stream_ptr())
        return self.Xb, self.yb


def bnn_config(D, H1, H2, n_samples, noise, prior_scale=1.0, data_scale=1.0, method=0, seed=0,
               engine=0):
    cfg = _lib.EdgBNN()
    cfg.D, cfg.H1, cfg.H2, cfg.n_samples = D, H1, H2, n_samples
    cfg.noise, cfg.prior_scale, cfg.data_scale = noise, prior_scale, data_scale
    cfg.method, cfg.seed, cfg.gemm_engine = method, seed, engine
    return cfg


def bnn_loglik_grad(cfg, X, y, theta):
    """(ll [S] float64, grad [S, P] float32) of the scaled Gaussian log-likelihood
    of the network for S weight vectors ``theta`` [S, P] over rows X [M, D], y [M]."""
    theta = theta.detach().to(torch.float32).contiguous()
    S, P = theta.shape
    if S != cfg.n_samples:
        cfg = bnn_config(cfg.D, cfg.H1, cfg.H2, S, cfg.noise, cfg.prior_scale, cfg.data_scale,
                         cfg.method, cfg.seed, cfg.gemm_engine)
    lib = _lib.load()
    M = X.shape[0]
    if P != lib.edg_bnn_num_params(cfg.D, cfg.H1, cfg.H2):
        raise ValueError("theta has the wrong number of parameters")
    ws_bytes = lib.edg_bnn_workspace_bytes(ctypes.byref(cfg), M)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=theta.device)
    ll = torch.empty(S, dtype=torch.float64, device=theta.device)
    g = torch.empty(S, P, dtype=torch.float32, device=theta.device)
    _lib.call("edg_bnn_loglik_grad", ctypes.byref(cfg), _lib.ptr(X.contiguous()),
              _lib.ptr(y.contiguous()), M, _lib.ptr(theta), _lib.ptr(ll), _lib.ptr(g),
              _lib.ptr(ws), ws_bytes, _lib.stream_ptr())
    return ll, g


class BNNLogLik(torch.autograd.Function):
    """Per-sample network log-likelihood with the hand-written adjoint as
    backward (replaces ``tf.gradients`` of ``p_log_lik``, ``klqp.py:746-767``)."""

    @staticmethod
    def forward(ctx, theta, cfg, X, y):
        ll, g = bnn_loglik_grad(cfg, X, y, theta)
        ctx.save_for_backward(g)
        return ll.to(theta.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return (grad_out.to(g.dtype)[:, None] * g).to(grad_out.dtype), None, None, None


def bnn_log_lik(cfg, X, y, theta):
    return BNNLogLik.apply(theta, cfg, X, y)


class SBNDevice:
    """Device data of a compiled sigmoid belief network (``compile.SBNSpec``)
    and the source of each step's B rows: all N bound rows, a device gather
    of ``n_minibatch`` rows from the bound data (uint8 on the device, Philox
    stream 4), or the ``feed_dict`` array of the x placeholder."""

    def __init__(self, spec, device="cuda", n_minibatch=None):
        _lib.require_cuda()
        self.spec = spec
        self.device = torch.device(device)
        self.gather = False
        self.seed = None
        if spec.X is not None:
            X = np.asarray(spec.X)
            if X.dtype != np.uint8:
                if not np.all((X == 0) | (X == 1)):
                    raise ValueError("Bernoulli data must be 0 or 1")
                X = X.astype(np.uint8)
            self.N = X.shape[0]
            self.X_u8 = torch.as_tensor(np.ascontiguousarray(X)).to(self.device)
            if n_minibatch is not None:
                if int(n_minibatch) <= 0:
                    raise ValueError("n_minibatch must be positive")
                self.B = int(n_minibatch)
                self.gather = True
                self.Xb = torch.empty(self.B, spec.V, dtype=torch.float32, device=self.device)
            else:
                self.B = self.N
                self.Xb = self.X_u8.float()
            self.fed = True
        else:
            if n_minibatch is not None:
                raise ValueError("n_minibatch needs x bound to an array in the data dict")
            self.B = spec.batch
            self.Xb = torch.zeros(self.B, spec.V, dtype=torch.float32, device=self.device)
            self.fed = False

    def feed(self, feed_dict):
        for k, v in feed_dict.items():
            if k is self.spec.x_node and not self.gather:
                v = np.asarray(v, np.float32)
                if v.shape != (self.B, self.spec.V):
                    raise ValueError(f"fed x has shape {v.shape}; expected {(self.B, self.spec.V)}")
                self.Xb.copy_(torch.from_numpy(np.ascontiguousarray(v)))
                self.fed = True
            else:
                raise KeyError(f"{k!r} is not a placeholder of this model")

    def batch(self, state):
        if not self.fed:
            raise ValueError("x is a placeholder: feed it with update(feed_dict=...)")
        if self.gather:
            _lib.call("edg_minibatch_gather_u8", _lib.ptr(self.X_u8), self.N, self.spec.V, self.B,
                      int(self.seed), _lib.ptr(state), _lib.ptr(self.Xb), _lib.stream_ptr())
        return self.Xb


def gemm(A, B, M, N, K, ta=False, tb=False, lda=None, ldb=None, batch=1, sA=0, sB=0,
         engine="tc", kchunk=0):
    """C[b] = op(A[b]) op(B[b]) through ``edg_gemm`` (FP32 tensors on the GPU,
    flat or shaped; strides in elements).  Returns C [batch, M, N]."""
    lda = lda if lda is not None else (M if ta else K)
    ldb = ldb if ldb is not None else (K if tb else N)
    eng = {"tc": _lib.GEMM_TC, "simt": _lib.GEMM_SIMT}[engine]
    C = torch.empty(batch, M, N, dtype=torch.float32, device=A.device)
    lib = _lib.load()
    wsb = lib.edg_gemm_workspace_bytes(eng, M, N, K, batch, kchunk)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=A.device)
    _lib.call("edg_gemm", eng, int(ta), int(tb), M, N, K, _lib.ptr(A), lda, sA, _lib.ptr(B), ldb,
              sB, _lib.ptr(C), N, M * N, batch, kchunk, _lib.ptr(ws), wsb, _lib.stream_ptr())
    return C
