"""KL(q||p) variational inference (``edward/inferences/klqp.py``).

``KLqp`` dispatches like the reference (``klqp.py:115-163``): Normal q with
Normal priors -> analytic-KL reparameterisation; other reparameterisable q
-> Monte Carlo reparameterisation; otherwise the score-function family.
The explicit variants pin one estimator.  Each step is one launch of a fused
kernel (Philox eps -> z -> log-lik + adjoint over X for all samples -> KL /
log q -> chain rule through softplus -> optimizer apply).
"""
import numpy as np
import torch

from .. import _lib
from ..compile import (UnsupportedModel, compile_expfam, compile_glm, compile_mlp, compile_sbn,
                       parse_normal_q)
from ..expr import Variable, softplus
from ..models import Normal, RandomVariable
from ..ops import BNNDevice, GLMDevice, SBNDevice
from ..util import next_seed, randn
from .variational_inference import VariationalInference

_CONTINUOUS = ("01", "nonnegative", "simplex", "real", "multivariate_real")

AUTO, REPARAM_KL, REPARAM, SCORE = None, _lib.KLQP_REPARAM_KL, _lib.KLQP_REPARAM, _lib.KLQP_SCORE
SCORE_RB = "score_rb"


class KLqp(VariationalInference):
    """Variational inference with KL(q(z; lambda) || p(z | x))."""

    _method = AUTO

    def __init__(self, latent_vars=None, data=None):
        if isinstance(latent_vars, list):
            d = {}
            for z in latent_vars:
                if not hasattr(z, "support") or z.support not in _CONTINUOUS:
                    raise AttributeError(
                        "Random variable {} is not continuous or a random "
                        "variable with supported continuous support.".format(z))
                shape = tuple(z.batch_shape) + tuple(z.event_shape)
                loc = Variable(randn(shape))
                scale = softplus(Variable(randn(shape)))
                d[z] = Normal(loc=loc, scale=scale)
            latent_vars = d
        super().__init__(latent_vars, data)

    def initialize(self, n_samples=1, kl_scaling=None, n_minibatch=None, gemm_engine="tc",
                   *args, **kwargs):
        """``n_samples`` / ``kl_scaling`` as in ``klqp.py:86-113``.  ``n_minibatch``
        (network families, data bound to arrays): each step draws that many
        rows uniformly with replacement on the device instead of using the
        whole data set; for the Bayesian NN ``scale`` for the observed variable
        then defaults to N / n_minibatch.  ``gemm_engine`` (network families):
        ``"tc"`` runs the layer GEMMs on the tensor cores (tcgen05, 3xTF32),
        ``"simt"`` on the FP32 CUDA cores."""
        if gemm_engine not in ("tc", "simt"):
            raise ValueError(f"gemm_engine must be 'tc' or 'simt'; got {gemm_engine!r}")
        self.gemm_engine = _lib.GEMM_TC if gemm_engine == "tc" else _lib.GEMM_SIMT
        if kl_scaling is None:
            kl_scaling = {}
        if n_samples <= 0:
            raise ValueError("n_samples should be greater than zero: {}".format(n_samples))
        self.n_samples = n_samples
        self.kl_scaling = kl_scaling
        self.n_minibatch = n_minibatch
        return super().initialize(*args, **kwargs)

    # ------------------------------------------------------------ dispatch
    def _choose_method(self):
        is_reparameterizable = all(q.reparameterizable for q in self.latent_vars.values())
        is_analytic_kl = all(isinstance(z, Normal) and isinstance(q, Normal)
                             for z, q in self.latent_vars.items())
        if not is_analytic_kl and self.kl_scaling:
            raise TypeError("kl_scaling must be None when using non-analytic KL term")
        if self._method is not AUTO:
            if self._method == REPARAM_KL and not is_analytic_kl:
                raise TypeError("analytic KL needs Normal priors and Normal q")
            return self._method
        if is_reparameterizable:
            return REPARAM_KL if is_analytic_kl else REPARAM
        return SCORE_RB

    def _validate(self):
        method = self._choose_method()
        latents = list(self.latent_vars.keys())
        discrete = bool(self.latent_vars) and all(not q.reparameterizable
                                                  for q in self.latent_vars.values())
        self._rao_blackwell = method == SCORE_RB
        if method == SCORE_RB and not discrete:
            raise NotImplementedError(
                "Rao-Blackwellised score gradients are implemented for the sigmoid belief "
                "network family")
        self._method_id = SCORE if method == SCORE_RB else method
        if self._method_id == SCORE and discrete:
            self._spec = compile_sbn(self.latent_vars, self.data)
            self._family = "sbn"
            if self.kl_scaling or self.scale:
                raise NotImplementedError("scale / kl_scaling for the sigmoid belief network")
            if self._rao_blackwell and getattr(self, "baseline", "none") != "none":
                raise NotImplementedError("ScoreRBKLqp takes no baseline")
            return
        method = self._method_id
        try:
            self._spec = compile_glm(latents, self.data, params=True)
            self._family = "glm"
        except UnsupportedModel as e_glm:
            try:
                self._spec = compile_mlp(latents, self.data)
                self._family = "bnn"
            except UnsupportedModel as e_mlp:
                try:
                    self._spec = compile_expfam(latents, self.data)
                except UnsupportedModel as e_ef:
                    raise UnsupportedModel(f"{e_glm} (GLM family); {e_mlp} (Bayesian NN family); "
                                           f"{e_ef} (constrained-latent family)")
                self._family = "expfam"
                if self._method_id not in (REPARAM,):
                    raise NotImplementedError("the constrained-latent family takes the "
                                              "reparameterisation gradient with Monte Carlo KL")
                if not self.auto_transform and self._spec.family == _lib.EXPFAM_DIRICHLET:
                    raise NotImplementedError("the Dirichlet latent needs auto_transform=True")
                for blk in self._spec.blocks:
                    parse_normal_q(self.latent_vars[blk.rv])
                return
            if method == SCORE:
                raise NotImplementedError("ScoreKLqp for the Bayesian NN family")
            if any(np.any(np.asarray(v) != 1.0) for v in self.kl_scaling.values()):
                raise NotImplementedError("kl_scaling for the Bayesian NN family")
            if any(z in self.scale for z in latents):
                raise NotImplementedError("per-latent scale for the Bayesian NN family")
        if self._family == "glm" and self.n_minibatch is not None:
            raise NotImplementedError("n_minibatch applies to the Bayesian NN family")
        for blk in self._spec.blocks:
            if not getattr(blk, "point", False):
                parse_normal_q(self.latent_vars[blk.rv])

    def build_loss_and_gradients(self, var_list):
        if self._family == "expfam":
            return self._build_expfam(var_list)
        if self._family == "bnn":
            return self._build_bnn(var_list)
        if self._family == "sbn":
            return self._build_sbn(var_list)
        method = self._method_id
        spec = self._spec
        self._glm = GLMDevice(spec, self._device)
        P = spec.P
        dev = self._device
        q_vars = self._bind_q(var_list)
        kls = np.ones(P, np.float32)
        lsc = np.ones(P, np.float32)
        for blk in spec.blocks:
            kls[blk.offset:blk.offset + blk.size] = np.broadcast_to(
                np.asarray(self.kl_scaling.get(blk.rv, 1.0), np.float32), blk.shape).reshape(-1)
            lsc[blk.offset:blk.offset + blk.size] = np.broadcast_to(
                np.asarray(self.scale.get(blk.rv, 1.0), np.float32), blk.shape).reshape(-1)
        dscale = np.asarray(self.scale.get(spec.observed, 1.0), np.float32)
        if dscale.size != 1:
            raise NotImplementedError("per-row data scale is not supported; pass a scalar")
        self._kls = torch.as_tensor(kls, device=dev)
        self._lsc = torch.as_tensor(lsc, device=dev)
        point = np.zeros(P, np.int32)
        for blk in spec.blocks:
            if blk.point:
                point[blk.offset:blk.offset + blk.size] = 1
        self._point = torch.as_tensor(point, device=dev) if point.any() else None
        self._slots = torch.zeros(4 * P, dtype=torch.float32, device=dev)
        self._reset_optimizer()
        cfg = _lib.EdgKLqp()
        cfg.method = method
        cfg.n_samples = self.n_samples
        cfg.data_scale = float(dscale.reshape(-1)[0])
        cfg.kl_scaling = self._kls.data_ptr()
        cfg.latent_scale = self._lsc.data_ptr()
        cfg.point = self._point.data_ptr() if self._point is not None else None
        cfg.seed = next_seed()
        self._cfg = cfg
        self._opt = self.optimizer.to_c()
        lib = _lib.load()
        self._ws_bytes = lib.edg_klqp_glm_workspace_bytes(self._glm.ref(), cfg)
        self._ws = torch.empty(max(self._ws_bytes, 1), dtype=torch.uint8, device=dev)
        self._grad = torch.zeros(2 * P, dtype=torch.float32, device=dev)
        return None, [(None, v) for v in q_vars]

    def _bind_q(self, var_list):
        """Rebinds every q parameter Variable to its slice of the flat device
        buffers (mu, rho) so that the fused kernels update them in place."""
        spec, dev = self._spec, self._device
        self._mu = torch.empty(spec.P, dtype=torch.float32, device=dev)
        self._rho = torch.empty(spec.P, dtype=torch.float32, device=dev)
        q_vars = []
        for blk in spec.blocks:
            if getattr(blk, "point", False):
                # a model parameter: its value lives in mu (rho is unused)
                var = blk.rv
                var._rebind(self._mu[blk.offset:blk.offset + blk.size].view(var.shape or ()))
                self._rho[blk.offset:blk.offset + blk.size].zero_()
                q_vars.append(var)
                continue
            q = parse_normal_q(self.latent_vars[blk.rv])
            for var, buf in ((q.loc_var, self._mu), (q.rho_var, self._rho)):
                if int(np.prod(var.shape)) != blk.size:
                    raise ValueError(f"q parameter {var.name} has shape {var.shape}; "
                                     f"latent {blk.rv.name} has {blk.size} elements")
                var._rebind(buf[blk.offset:blk.offset + blk.size].view(var.shape or ()))
                q_vars.append(var)
        if var_list is not None and set(map(id, var_list)) != set(map(id, q_vars)):
            raise NotImplementedError("var_list must be the variational parameters of q")
        return q_vars

    def _build_bnn(self, var_list):
        spec, dev = self._spec, self._device
        q_vars = self._bind_q(var_list)
        P = spec.P
        self._bnn = BNNDevice(spec, dev, self.n_minibatch)
        dscale = self.scale.get(spec.observed)
        if dscale is None:
            dscale = self._bnn.default_scale
        dscale = np.asarray(dscale, np.float32)
        if dscale.size != 1:
            raise NotImplementedError("per-row data scale is not supported; pass a scalar")
        cfg = _lib.EdgBNN()
        cfg.D, cfg.H1, cfg.H2, cfg.n_samples = spec.D, spec.H1, spec.H2, self.n_samples
        cfg.noise, cfg.prior_scale = spec.noise, spec.prior_scale
        cfg.data_scale = float(dscale.reshape(-1)[0])
        cfg.method = self._method_id
        cfg.gemm_engine = self.gemm_engine
        cfg.seed = next_seed()
        self._bnn.seed = next_seed()
        self._cfg = cfg
        self._opt = self.optimizer.to_c()
        self._slots = torch.zeros(4 * P, dtype=torch.float32, device=dev)
        self._reset_optimizer()
        lib = _lib.load()
        self._ws_bytes = lib.edg_bnn_workspace_bytes(cfg, self._bnn.M)
        if self._ws_bytes == 0:
            _lib.call("edg_bnn_workspace_bytes", cfg, self._bnn.M)
        self._ws = torch.empty(self._ws_bytes, dtype=torch.uint8, device=dev)
        self._grad = torch.zeros(2 * P, dtype=torch.float32, device=dev)
        return None, [(None, v) for v in q_vars]

    def _build_expfam(self, var_list):
        spec, dev = self._spec, self._device
        q_vars = self._bind_q(var_list)
        K = spec.K
        self._ef_prior = torch.as_tensor(spec.prior, device=dev)
        self._ef_stats = torch.as_tensor(spec.stats, device=dev)
        m = _lib.EdgExpFam()
        m.family, m.K = spec.family, K
        m.prior, m.stats = self._ef_prior.data_ptr(), self._ef_stats.data_ptr()
        # auto_transform=False: q is fitted on the latent's support itself, and
        # draws outside it give a NaN loss (inference_auto_transform_test.py:46-63)
        m.transform = 1 if self.auto_transform else 0
        self._ef = m
        self._ef_seed = next_seed()
        self._slots = torch.zeros(4 * K, dtype=torch.float32, device=dev)
        self._reset_optimizer()
        self._opt = self.optimizer.to_c()
        self._grad = torch.zeros(2 * K, dtype=torch.float32, device=dev)
        z = spec.z
        if not self.auto_transform:
            self.transformations = {}
        elif spec.family == _lib.EXPFAM_BETA:
            self.transformations = {z: torch.sigmoid}
        elif spec.family == _lib.EXPFAM_GAMMA:
            self.transformations = {z: torch.nn.functional.softplus}
        else:
            self.transformations = {z: lambda u: torch.softmax(
                torch.cat([u, torch.zeros_like(u[..., :1])], dim=-1), dim=-1)}
        return None, [(None, v) for v in q_vars]

    def _build_sbn(self, var_list):
        spec, dev = self._spec, self._device
        lib = _lib.load()
        V, H0, H1 = spec.V, spec.H0, spec.H1
        P = lib.edg_sbn_num_params(V, H0, H1)
        self._theta = torch.empty(P, dtype=torch.float32, device=dev)
        off = 0
        for i, (fin, fout) in enumerate(((V, H0), (H0, H1), (H1, H0), (H0, V))):
            W, b = spec.weights[2 * i], spec.weights[2 * i + 1]
            W._rebind(self._theta[off:off + fin * fout].view(fin, fout))
            b._rebind(self._theta[off + fin * fout:off + (fin + 1) * fout])
            off += (fin + 1) * fout
        if var_list is not None and set(map(id, var_list)) != set(map(id, spec.weights)):
            raise NotImplementedError("var_list must be every trainable weight of the network")
        self._sbn = SBNDevice(spec, dev, self.n_minibatch)
        self._sbn.seed = next_seed()
        self._prior = torch.as_tensor(spec.prior_logits, device=dev)
        from .. import train
        if not hasattr(self, "baseline"):        # KLqp / ScoreRBKLqp: no control variate
            self.baseline, self.baseline_hidden, self.baseline_decay = "none", 1, 0.9
            self.baseline_optimizer = train.AdamOptimizer(1e-2)
        mode = {"none": _lib.BASELINE_NONE, "mean": _lib.BASELINE_MEAN,
                "mlp": _lib.BASELINE_MLP}[self.baseline]
        cfg = _lib.EdgSBN()
        cfg.V, cfg.H0, cfg.H1, cfg.n_samples = V, H0, H1, self.n_samples
        cfg.baseline, cfg.baseline_hidden = mode, self.baseline_hidden
        cfg.baseline_decay = self.baseline_decay
        cfg.gemm_engine = self.gemm_engine
        cfg.rao_blackwell = 1 if self._rao_blackwell else 0
        cfg.seed = next_seed()
        self._cfg = cfg
        self._opt = self.optimizer.to_c()
        self._bopt = self.baseline_optimizer.to_c()
        self._slots = torch.zeros(2 * P, dtype=torch.float32, device=dev)
        self._P = P
        self._reset_optimizer()
        BH = self.baseline_hidden
        PB = lib.edg_sbn_baseline_num_params(V, BH)
        lim = np.sqrt(6.0 / (V + BH))
        bp = np.zeros(PB, np.float32)
        bp[:V * BH] = np.random.uniform(-lim, lim, V * BH)
        self._bparams = torch.as_tensor(bp, device=dev)
        self._bslots = torch.zeros(2 * PB, dtype=torch.float32, device=dev)
        a, b = self.baseline_optimizer.slot_init()
        self._bslots[:PB].fill_(a)
        self._bslots[PB:].fill_(b)
        bo = self.baseline_optimizer
        self._bstats = torch.tensor([0.0, 1.0, 0.0, getattr(bo, "beta1", 0.9),
                                     getattr(bo, "beta2", 0.999), 0.0, 0.0, 0.0],
                                    dtype=torch.float32, device=dev)
        self._ws_bytes = lib.edg_sbn_workspace_bytes(cfg, self._sbn.B)
        if self._ws_bytes == 0:
            _lib.call("edg_sbn_workspace_bytes", cfg, self._sbn.B)
        self._ws = torch.empty(self._ws_bytes, dtype=torch.uint8, device=dev)
        self._grad = torch.zeros(P, dtype=torch.float32, device=dev)
        return None, [(None, v) for v in spec.weights]

    def _feed(self, feed_dict):
        if self._family == "bnn":
            return self._bnn.feed(feed_dict)
        if self._family == "sbn":
            return self._sbn.feed(feed_dict)
        return super()._feed(feed_dict)

    def _run_loop(self):
        if self._family == "bnn" and not self._bnn.ready:
            raise ValueError("X / y are placeholders: feed them with update(feed_dict=...)")
        if self._family == "sbn" and not self._sbn.fed:
            raise ValueError("x is a placeholder: feed it with update(feed_dict=...)")
        super()._run_loop()

    def _reset_optimizer(self):
        if self._family == "sbn":
            a, b = self.optimizer.slot_init()
            self._slots[:self._P].fill_(a)
            self._slots[self._P:].fill_(b)
            return
        a, b = self.optimizer.slot_init()
        P = self._spec.P
        self._slots[: 2 * P].fill_(a)
        self._slots[2 * P:].fill_(b)

    def _step(self, apply=True, eps=None, grad_out=None, signal_out=None):
        import ctypes
        if self._family == "expfam":
            _lib.call("edg_expfam_klqp_step", ctypes.byref(self._ef), self.n_samples,
                      self._ef_seed, ctypes.byref(self._opt), _lib.ptr(self._mu),
                      _lib.ptr(self._rho), _lib.ptr(self._slots), _lib.ptr(self._state),
                      _lib.ptr(eps), _lib.ptr(grad_out), 1 if apply else 0, _lib.stream_ptr())
            return
        if self._family == "sbn":
            X = self._sbn.batch(self._state)
            _lib.call("edg_sbn_score_step", ctypes.byref(self._cfg), ctypes.byref(self._opt),
                      ctypes.byref(self._bopt), _lib.ptr(X), self._sbn.B, _lib.ptr(self._prior),
                      _lib.ptr(self._theta), _lib.ptr(self._slots), _lib.ptr(self._state),
                      _lib.ptr(self._bparams), _lib.ptr(self._bslots), _lib.ptr(self._bstats),
                      _lib.ptr(eps), _lib.ptr(grad_out), _lib.ptr(signal_out), 1 if apply else 0,
                      _lib.ptr(self._ws), self._ws_bytes, _lib.stream_ptr())
            return
        if self._family == "bnn":
            X, y = self._bnn.batch(self._state)
            _lib.call("edg_bnn_klqp_step", ctypes.byref(self._cfg), ctypes.byref(self._opt),
                      _lib.ptr(X), _lib.ptr(y), self._bnn.M, _lib.ptr(self._mu),
                      _lib.ptr(self._rho), _lib.ptr(self._slots), _lib.ptr(self._state),
                      _lib.ptr(eps), _lib.ptr(grad_out), 1 if apply else 0, _lib.ptr(self._ws),
                      self._ws_bytes, _lib.stream_ptr())
            return
        _lib.call("edg_klqp_glm_step", self._glm.ref(), ctypes.byref(self._cfg),
                  ctypes.byref(self._opt), _lib.ptr(self._mu), _lib.ptr(self._rho),
                  _lib.ptr(self._slots), _lib.ptr(self._state), _lib.ptr(eps), _lib.ptr(grad_out),
                  1 if apply else 0, _lib.ptr(self._ws), self._ws_bytes, _lib.stream_ptr())

    def loss_and_gradients(self, eps=None):
        """(loss, dloss/dmu, dloss/drho) at the current parameters without
        applying the optimizer; ``eps`` [n_samples, P] overrides the draws."""
        if eps is not None:
            eps = torch.as_tensor(eps, dtype=torch.float32, device=self._device).contiguous()
        self._step(apply=False, eps=eps, grad_out=self._grad)
        st = self._read_state()
        P = self._spec.P
        g = self._grad.detach().clone()
        return float(st.loss), g[:P], g[P:]

    def score_gradients(self, z=None, signal=False):
        """(loss, grad [P]) at the current parameters without applying the
        optimizer (sigmoid belief network); ``z`` = (z0 [S, B, H0], z1 [S, B, H1])
        overrides the draws; ``signal=True`` also returns f [S, B] and the
        learning signal [S, B]."""
        if self._family != "sbn":
            raise NotImplementedError("score_gradients is for the sigmoid belief network")
        zo = None
        if z is not None:
            zo = torch.cat([torch.as_tensor(np.asarray(a, np.float32)).reshape(-1) for a in z])
            zo = zo.to(self._device)
        S, B = self.n_samples, self._sbn.B
        sig = torch.empty(2 * S * B, dtype=torch.float32, device=self._device) if signal else None
        self._step(apply=False, eps=zo, grad_out=self._grad, signal_out=sig)
        st = self._read_state()
        out = (float(st.loss), self._grad.detach().clone())
        if signal:
            out += (sig[:S * B].view(S, B).clone(), sig[S * B:].view(S, B).clone())
        return out

    @property
    def seed(self):
        return int(self._cfg.seed)

    @seed.setter
    def seed(self, v):
        self._cfg.seed = int(v)
        self._graphs = {}


class ReparameterizationKLqp(KLqp):
    """Monte Carlo KL with the reparameterisation gradient (klqp.py:166-226, 642-704)."""
    _method = REPARAM


class ReparameterizationKLKLqp(KLqp):
    """Analytic KL with the reparameterisation gradient (klqp.py:229-303, 707-769)."""
    _method = REPARAM_KL


class ScoreKLqp(KLqp):
    """Score-function gradient (klqp.py:370-430, 840-906).

    ``baseline`` (sigmoid belief network family): ``None`` / ``"none"`` is the
    reference's estimator (no control variate); ``"mean"`` subtracts a running
    mean of the per-row learning signal; ``"mlp"`` subtracts
    c + sigma * mlp(2x - 1), a ``baseline_hidden``-unit tanh network trained online
    on the (x, learning signal) pairs the estimator produces, with
    ``baseline_optimizer`` (default Adam, learning rate 1e-2)."""
    _method = SCORE

    def initialize(self, n_samples=1, kl_scaling=None, n_minibatch=None, gemm_engine="tc",
                   baseline=None, baseline_hidden=100, baseline_optimizer=None, baseline_decay=0.9,
                   *args, **kwargs):
        from .. import train
        self.baseline = baseline or "none"
        if self.baseline not in ("none", "mean", "mlp"):
            raise ValueError(f"baseline must be None, 'mean' or 'mlp'; got {baseline!r}")
        self.baseline_hidden = int(baseline_hidden)
        self.baseline_optimizer = (train.AdamOptimizer(1e-2) if baseline_optimizer is None
                                   else train.resolve(baseline_optimizer, None))
        if not 0.0 <= baseline_decay < 1.0:
            raise ValueError("baseline_decay must be in [0, 1)")
        self.baseline_decay = float(baseline_decay)
        return super().initialize(n_samples, kl_scaling, n_minibatch, gemm_engine, *args, **kwargs)

    def _validate(self):
        super()._validate()
        if self._family != "sbn" and self.baseline != "none":
            raise NotImplementedError("baselines are implemented for the sigmoid belief network")


class ScoreRBKLqp(KLqp):
    """Score-function gradient with Rao-Blackwellisation across stochastic nodes
    (``klqp.py:572-639``, ``build_score_rb_loss_and_gradients`` 1058-1152): each
    variational factor's learning signal keeps only the log densities in the
    Markov blanket of its latent variable.  ``ed.KLqp`` dispatches here for
    non-reparameterisable (discrete) latent variables (``klqp.py:153-163``)."""
    _method = SCORE_RB
