"""Stochastic-gradient MCMC: ``SGLD`` (``edward/inferences/sgld.py:19-88``) and
``SGHMC`` (``edward/inferences/sghmc.py:19-102``) for the GLM family.

Same surface as the reference (``Empirical`` stores, ``initialize(step_size)``
and ``initialize(step_size, friction)``, ``update`` / ``run``, ``n_accept``);
the log joint uses ``scale`` as the reference's ``_log_joint`` does.  Two
engines: the tensor-core HMC kernel in its SG-MCMC form (one 3xTF32
gradient evaluation per iteration, the update fused into its owner phase,
``edg_sgmcmc_glm_tc_run``; P <= 64), and the SIMT form (the batched log-joint
gradient plus a fused update kernel, ``edg_sgmcmc_glm_run``).  ``engine`` in
``initialize`` picks one ("tc", "simt"); "auto" times both once per model
shape.
"""
import ctypes

import numpy as np
import torch

from .. import _lib, autotune
from ..compile import compile_glm
from ..ops import GLMDevice
from ..util import next_seed
from .monte_carlo import MonteCarlo


def _check_override(t, numel, dtype, name):
    """A per-iteration draw / output buffer must hold exactly the elements
    the launch reads or writes."""
    if t is None:
        return
    if not isinstance(t, torch.Tensor) or t.dtype != dtype or t.numel() != numel:
        raise ValueError(f"{name} must be a {dtype} tensor of {numel} elements")


class _SGMCMC(MonteCarlo):
    _method = None

    def _validate(self):
        self._spec = compile_glm(list(self.latent_vars.keys()), self.data)
        for z in self.latent_vars:
            if getattr(z, "support", "real") not in (None, "real", "multivariate_real"):
                raise NotImplementedError(
                    f"latent support '{z.support}' for stochastic-gradient MCMC")
        C = self.n_chains or 1
        for qz in self.latent_vars.values():
            if (qz.n_chains or 1) != C:
                raise ValueError("every Empirical must hold the same number of chains")
        if any(z in self.scale for z in self.latent_vars):
            raise NotImplementedError("scale on latent variables")
        dscale = np.asarray(self.scale.get(self._spec.observed, 1.0), np.float32)
        if dscale.size != 1:
            raise NotImplementedError("per-row data scale is not supported; pass a scalar")
        self._data_scale = float(dscale.reshape(-1)[0])

    def build_update(self):
        spec = self._spec
        dev = self._device
        self._glm = GLMDevice(spec, dev)
        C = self._bind_glm_store(spec)
        self._v = torch.zeros(C, spec.P, dtype=torch.float32, device=dev)
        self._n_accept = torch.zeros(C, dtype=torch.int32, device=dev)
        cfg = _lib.EdgSGMCMC()
        cfg.method = self._method
        cfg.step_size = float(self.step_size)
        cfg.friction = float(getattr(self, "friction", 0.0))
        cfg.data_scale = self._data_scale
        cfg.seed = next_seed()
        self._cfg = cfg
        lib = _lib.load()
        self._ws_bytes = lib.edg_sgmcmc_glm_workspace_bytes(self._glm.ref(), C)
        self._ws = torch.empty(max(self._ws_bytes, 1), dtype=torch.uint8, device=dev)
        # tensor-core form: X re-laid into operand tiles once, and a cache of
        # the current state's gradient carried between launches
        self._g = torch.zeros(C, spec.P, dtype=torch.float32, device=dev)
        self._cache_valid = 0
        self._tiles = None
        req = getattr(self, "_engine_req", "auto")
        if req not in ("auto", "tc", "simt"):
            raise ValueError("engine must be 'auto', 'tc' or 'simt'")
        if req != "simt" and spec.P <= 64:
            nbytes = lib.edg_hmc_glm_tc_tiles_bytes(self._glm.ref())
            self._tiles = torch.empty(nbytes, dtype=torch.uint8, device=dev)
            _lib.call("edg_hmc_glm_tc_prepare", self._glm.ref(), _lib.ptr(self._tiles), nbytes,
                      _lib.stream_ptr())
        if req == "tc":
            if self._tiles is None:
                raise NotImplementedError("the tensor-core engine needs P <= 64")
            self.engine = "tc"
        elif req == "simt" or self._tiles is None:
            self.engine = "simt"
        else:
            self.engine = self._autotune()
        self.train = self.update
        return self.train

    def _run_engine(self, engine, n_iter, z, v, g, n_accept, state, samples, noise,
                    cache_valid):
        if engine == "tc":
            _lib.call("edg_sgmcmc_glm_tc_run", self._glm.ref(), ctypes.byref(self._cfg), self.C,
                      int(n_iter), _lib.ptr(self._tiles), _lib.ptr(z), _lib.ptr(v), _lib.ptr(g),
                      cache_valid, _lib.ptr(n_accept), _lib.ptr(state), _lib.ptr(samples),
                      samples.shape[0] if samples is not None else 0, _lib.ptr(noise),
                      _lib.stream_ptr())
        else:
            _lib.call("edg_sgmcmc_glm_run", self._glm.ref(), ctypes.byref(self._cfg), self.C,
                      int(n_iter), _lib.ptr(z), _lib.ptr(v), _lib.ptr(n_accept),
                      _lib.ptr(state), _lib.ptr(samples),
                      samples.shape[0] if samples is not None else 0, _lib.ptr(noise),
                      _lib.ptr(self._ws), self._ws_bytes, _lib.stream_ptr())

    def _autotune(self):
        """The faster engine for this model shape, one launch of each on
        scratch copies of the state (cached per shape and device)."""
        z, v, g = self._z.clone(), self._v.clone(), torch.zeros_like(self._g)
        nacc = torch.zeros_like(self._n_accept)
        st = _lib.new_state(self._device)

        def run(engine):
            z.copy_(self._z)
            v.copy_(self._v)
            self._run_engine(engine, 1, z, v, g, nacc, st, None, None, 0)
        spec = self._spec
        key = f"N{spec.N}_P{spec.P}_C{self.C}_m{self._method}"
        return autotune.choose("sgmcmc_engine", key, ["tc", "simt"], run)

    def _launch(self, n_iter, noise=None):
        self._run_engine(self.engine, n_iter, self._z, self._v, self._g, self._n_accept,
                         self._state, self._samples, noise, self._cache_valid)
        self._cache_valid = 1

    def update(self, feed_dict=None):
        """One iteration for every chain; returns ``{'t', 'accept_rate'}``
        (every proposal is kept, as in the reference)."""
        if feed_dict:
            raise NotImplementedError("feed_dict is not supported for this model family")
        self._launch(1)
        t = self.t
        acc = float(self._n_accept.sum().item()) / (max(t, 1) * self._n_accept.numel())
        return {"t": t, "accept_rate": acc}

    def _run_loop(self):
        chunk = self.n_print if self.n_print else self.n_iter
        done = 0
        while done < self.n_iter:
            k = min(chunk, self.n_iter - done)
            self._launch(k)
            done += k
            t = self.t
            acc = float(self._n_accept.sum().item()) / (max(t, 1) * self._n_accept.numel())
            self.print_progress({"t": t, "accept_rate": acc})

    def run_iterations(self, k, noise=None):
        """k iterations without host synchronisation; ``noise`` [k, C, P]
        overrides the Philox draws."""
        if noise is not None:
            noise = torch.as_tensor(noise, dtype=torch.float32, device=self._device).contiguous()
            _check_override(noise, k * self.C * self._spec.P, torch.float32, "noise")
        self._launch(k, noise)

    @property
    def n_accept(self):
        if self._n_accept.numel() == 1:
            return int(self._n_accept[0].item())
        return self._n_accept

    def reset(self):
        super().reset()
        self._n_accept.zero_()
        self._z.copy_(self._samples[0])
        self._v.zero_()
        self._cache_valid = 0


class SGLD(_SGMCMC):
    """Stochastic gradient Langevin dynamics (``sgld.py:52-88``):
    lr = step_size / (t + 1)^0.55, z <- z + lr/2 grad log p + N(0, lr)."""
    _method = _lib.SGMCMC_SGLD

    def initialize(self, step_size=0.25, *args, engine="auto", **kwargs):
        self.step_size = step_size
        self._engine_req = engine
        return super().initialize(*args, **kwargs)


class SGHMC(_SGMCMC):
    """Stochastic gradient Hamiltonian Monte Carlo (``sghmc.py:58-102``):
    lr = step_size * 0.01, z <- z + v, v <- (1 - friction/2) v + lr grad log p
    + N(0, lr * friction)."""
    _method = _lib.SGMCMC_SGHMC

    def initialize(self, step_size=0.25, friction=0.1, *args, engine="auto", **kwargs):
        self.step_size = step_size
        self.friction = friction
        self._engine_req = engine
        return super().initialize(*args, **kwargs)


class MetropolisHastings(MonteCarlo):
    """Metropolis-Hastings (``edward/inferences/metropolis_hastings.py:19-156``)
    with the reference's surface: ``MetropolisHastings(latent_vars,
    proposal_vars, data)``.  Proposals for the GLM family are Normal random
    walks ``Normal(loc=z, scale=s)`` or independence proposals
    ``Normal(loc=m, scale=s)`` (constant m, s), per latent.  Two engines, as
    for SG-MCMC: the tensor-core HMC kernel in its Metropolis-Hastings form
    (``edg_mh_glm_tc_run``, P <= 64) and the SIMT form (``edg_mh_glm_run``);
    ``initialize(engine=...)`` picks one, "auto" times both once per shape."""

    def __init__(self, latent_vars, proposal_vars, data=None, n_chains=None):
        from ..inferences.inference import check_latent_vars
        check_latent_vars(proposal_vars)
        self.proposal_vars = proposal_vars
        super().__init__(latent_vars, data, n_chains=n_chains)

    def _validate(self):
        from ..compile import _const_param
        from ..models import Normal
        self._spec = compile_glm(list(self.latent_vars.keys()), self.data)
        C = self.n_chains or 1
        for qz in self.latent_vars.values():
            if (qz.n_chains or 1) != C:
                raise ValueError("every Empirical must hold the same number of chains")
        P = self._spec.P
        loc = np.zeros(P, np.float32)
        scale = np.ones(P, np.float32)
        walk = None
        for blk in self._spec.blocks:
            g = self.proposal_vars.get(blk.rv)
            if not isinstance(g, Normal):
                raise NotImplementedError(
                    f"the proposal of {blk.rv.name} must be a Normal random variable")
            is_walk = g.loc is blk.rv
            if walk is None:
                walk = is_walk
            elif walk != is_walk:
                raise NotImplementedError("mixing random-walk and independence proposals")
            sl = slice(blk.offset, blk.offset + blk.size)
            scale[sl] = np.broadcast_to(_const_param(g.scale, "proposal scale", {}),
                                        blk.shape).reshape(-1)
            if not is_walk:
                loc[sl] = np.broadcast_to(_const_param(g.loc, "proposal loc", {}),
                                          blk.shape).reshape(-1)
        if np.any(scale <= 0):
            raise ValueError("proposal scales must be positive")
        self._walk, self._prop_loc, self._prop_scale = walk, loc, scale

    def build_update(self):
        spec = self._spec
        dev = self._device
        self._glm = GLMDevice(spec, dev)
        C = self._bind_glm_store(spec)
        self._lj = torch.zeros(C, dtype=torch.float64, device=dev)
        self._cache_valid = 0
        self._n_accept = torch.zeros(C, dtype=torch.int32, device=dev)
        self._loc_t = torch.as_tensor(self._prop_loc, device=dev)
        self._scale_t = torch.as_tensor(self._prop_scale, device=dev)
        cfg = _lib.EdgMH()
        cfg.proposal_loc = None if self._walk else self._loc_t.data_ptr()
        cfg.proposal_scale = self._scale_t.data_ptr()
        cfg.seed = next_seed()
        self._cfg = cfg
        lib = _lib.load()
        self._ws_bytes = lib.edg_mh_glm_workspace_bytes(self._glm.ref(), C)
        self._ws = torch.empty(max(self._ws_bytes, 1), dtype=torch.uint8, device=dev)
        # tensor-core form: X re-laid into operand tiles once; `_g` is the
        # kernel's gradient scratch
        self._g = torch.zeros(C, spec.P, dtype=torch.float32, device=dev)
        self._tiles = None
        req = getattr(self, "_engine_req", "auto")
        if req not in ("auto", "tc", "simt"):
            raise ValueError("engine must be 'auto', 'tc' or 'simt'")
        if req != "simt" and spec.P <= 64:
            nbytes = lib.edg_hmc_glm_tc_tiles_bytes(self._glm.ref())
            self._tiles = torch.empty(nbytes, dtype=torch.uint8, device=dev)
            _lib.call("edg_hmc_glm_tc_prepare", self._glm.ref(), _lib.ptr(self._tiles), nbytes,
                      _lib.stream_ptr())
        if req == "tc":
            if self._tiles is None:
                raise NotImplementedError("the tensor-core engine needs P <= 64")
            self.engine = "tc"
        elif req == "simt" or self._tiles is None:
            self.engine = "simt"
        else:
            self.engine = self._autotune()
        self.train = self.update
        return self.train

    def initialize(self, *args, engine="auto", **kwargs):
        self._engine_req = engine
        return super().initialize(*args, **kwargs)

    def _run_engine(self, engine, n_iter, z, lj, cache_valid, n_accept, state, samples,
                    e_override=None, u_override=None, ratio_out=None):
        T_cap = samples.shape[0] if samples is not None else 0
        if engine == "tc":
            _lib.call("edg_mh_glm_tc_run", self._glm.ref(), ctypes.byref(self._cfg), self.C,
                      int(n_iter), _lib.ptr(self._tiles), _lib.ptr(z), _lib.ptr(self._g),
                      _lib.ptr(lj), cache_valid, _lib.ptr(n_accept), _lib.ptr(state),
                      _lib.ptr(samples), T_cap, _lib.ptr(e_override), _lib.ptr(u_override),
                      _lib.ptr(ratio_out), _lib.stream_ptr())
        else:
            _lib.call("edg_mh_glm_run", self._glm.ref(), ctypes.byref(self._cfg), self.C,
                      int(n_iter), _lib.ptr(z), _lib.ptr(lj), cache_valid, _lib.ptr(n_accept),
                      _lib.ptr(state), _lib.ptr(samples), T_cap, _lib.ptr(e_override),
                      _lib.ptr(u_override), _lib.ptr(ratio_out), _lib.ptr(self._ws),
                      self._ws_bytes, _lib.stream_ptr())

    def _autotune(self):
        """The faster engine for this model shape, one launch of each on
        scratch copies of the state (cached per shape and device)."""
        z, lj = self._z.clone(), torch.zeros_like(self._lj)
        nacc = torch.zeros_like(self._n_accept)
        st = _lib.new_state(self._device)

        def run(engine):
            z.copy_(self._z)
            self._run_engine(engine, 1, z, lj, 0, nacc, st, None)
        spec = self._spec
        key = f"N{spec.N}_P{spec.P}_C{self.C}_walk{int(bool(self._walk))}"
        return autotune.choose("mh_engine", key, ["tc", "simt"], run)

    def _launch(self, n_iter, e_override=None, u_override=None, ratio_out=None):
        self._run_engine(self.engine, n_iter, self._z, self._lj, self._cache_valid,
                         self._n_accept, self._state, self._samples, e_override, u_override,
                         ratio_out)
        self._cache_valid = 1

    update = _SGMCMC.update
    _run_loop = _SGMCMC._run_loop
    n_accept = _SGMCMC.n_accept

    def run_iterations(self, k, e_override=None, u_override=None, ratio_out=None):
        """k iterations without host synchronisation (optional draws / ratios)."""
        _check_override(e_override, k * self.C * self._spec.P, torch.float32, "e_override")
        _check_override(u_override, k * self.C, torch.float64, "u_override")
        _check_override(ratio_out, k * self.C, torch.float64, "ratio_out")
        self._launch(k, e_override, u_override, ratio_out)

    def reset(self):
        MonteCarlo.reset(self)
        self._n_accept.zero_()
        self._z.copy_(self._samples[0])
        self._cache_valid = 0
