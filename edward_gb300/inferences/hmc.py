"""Hamiltonian Monte Carlo (``edward/inferences/hmc.py``).

Per iteration and chain (``hmc.py:61-130,195-210``): momentum r0 ~ N(0, I);
``n_steps`` leapfrog steps (half kick, drift, gradient, half kick); FP64 log
acceptance ratio 0.5|r0|^2 - 0.5|r|^2 + L(z) - L(z0); accept if
log u < ratio; the kept state goes to ``Empirical.params[t]``.  All chains
and all ``n_iter`` iterations of one ``update``/``run`` chunk run in one
persistent kernel launch; the log joint and its gradient at the current
state are carried between iterations instead of being recomputed.
"""
import ctypes

import numpy as np
import torch

from .. import _lib, autotune
from ..compile import UnsupportedModel, compile_expfam, compile_glm, compile_hier
from ..ops import GLMDevice, HierDevice
from ..util import next_seed
from .monte_carlo import MonteCarlo


class HMC(MonteCarlo):
    def initialize(self, step_size=0.25, n_steps=2, engine="auto", chains_per_block=0,
                   cluster_size=0, *args, **kwargs):
        """``step_size`` / ``n_steps`` as in ``hmc.py:45-59``.

        engine: "tc" (tcgen05 tensor cores: P <= 64 for a single GLM, max D_i
        <= 128 for a ragged hierarchical batch), "simt" (CUDA cores) or "auto"
        (autotuned between them); ``chains_per_block`` (SIMT) and
        ``cluster_size`` (tensor cores) pin a launch shape, 0 = autotuned."""
        if engine not in ("auto", "tc", "simt"):
            raise ValueError("engine must be 'auto', 'tc' or 'simt'")
        self.step_size = step_size
        self.n_steps = n_steps
        self._engine_req = engine
        self._cpb = chains_per_block
        self._cluster = cluster_size
        return super().initialize(*args, **kwargs)

    def _validate(self):
        if not self.auto_transform:
            raise ValueError("This implementation of HMC requires that all "
                             "variables have unconstrained support. Please "
                             "initialize with auto_transform=True to ensure "
                             "this. (if your variables already have unconstrained "
                             "support then doing this is a no-op).")
        try:
            self._spec = compile_glm(list(self.latent_vars.keys()), self.data)
            self._family = "glm"
        except UnsupportedModel as e_glm:
            try:
                self._spec = compile_hier(list(self.latent_vars.keys()), self.data)
                self._family = "hier"
            except UnsupportedModel as e_hier:
                try:
                    self._spec = compile_expfam(list(self.latent_vars.keys()), self.data)
                    self._family = "expfam"
                except UnsupportedModel as e_ef:
                    raise UnsupportedModel(
                        f"model is not in the GLM family ({e_glm}), the hierarchical family "
                        f"({e_hier}) or the constrained-latent family ({e_ef})") from None
        if self._family == "glm":
            for z in self.latent_vars:
                if getattr(z, "support", "real") not in (None, "real", "multivariate_real"):
                    raise NotImplementedError(
                        f"auto_transform of support '{z.support}' for this model family")
        if self._family == "glm":
            C = self.n_chains or 1
            for qz in self.latent_vars.values():
                if (qz.n_chains or 1) != C:
                    raise ValueError("every Empirical must hold the same number of chains")

    def build_update(self):
        if self._family == "hier":
            return self._build_hier()
        if self._family == "expfam":
            return self._build_expfam()
        spec = self._spec
        self._glm = GLMDevice(spec, self._device)
        C = self._bind_glm_store(spec)
        P = spec.P
        dev = self._device
        self._g = torch.zeros(C, P, dtype=torch.float32, device=dev)
        self._lj = torch.zeros(C, dtype=torch.float64, device=dev)
        self._cache_valid = 0
        self._n_accept = torch.zeros(C, dtype=torch.int32, device=dev)
        cfg = _lib.EdgHMC()
        cfg.step_size = float(self.step_size)
        cfg.n_steps = int(self.n_steps)
        cfg.seed = next_seed()
        cfg.chains_per_block = int(self._cpb)
        cfg.cluster_size = int(self._cluster)
        self._cfg = cfg
        self._tiles = None
        tc_ok = spec.P <= 64 and self.n_steps > 0
        if self._engine_req == "tc" and not tc_ok:
            raise NotImplementedError("the tensor-core engine needs P <= 64 and n_steps > 0")
        if tc_ok and self._engine_req in ("auto", "tc"):
            lib = _lib.load()
            nbytes = lib.edg_hmc_glm_tc_tiles_bytes(self._glm.ref())
            self._tiles = torch.empty(nbytes, dtype=torch.uint8, device=dev)
            _lib.call("edg_hmc_glm_tc_prepare", self._glm.ref(), _lib.ptr(self._tiles), nbytes,
                      _lib.stream_ptr())
        if self._engine_req == "tc":
            self.engine = "tc"
        elif self._engine_req == "simt" or self._tiles is None:
            self.engine = "simt"
        else:
            self.engine = None
        if self.engine is None or (self.engine == "simt" and cfg.chains_per_block == 0):
            best = self._autotune()
            if best == "tc":
                self.engine = "tc"
            else:
                self.engine = "simt"
                cfg.chains_per_block = int(best)
        self.train = self.update
        return self.train

    def _autotune(self):
        C = self.C
        z = self._z.clone()
        g = torch.zeros_like(self._g)
        lj = torch.zeros_like(self._lj)
        st = _lib.new_state(self._device)
        cands = ([8, 16, 32] if C > 8 else [8]) if self._engine_req != "tc" else []
        if self._tiles is not None and self._engine_req != "simt":
            cands = ["tc"] + cands

        def run(c):
            cfg = _lib.EdgHMC()
            cfg.step_size, cfg.n_steps, cfg.seed = self._cfg.step_size, self._cfg.n_steps, 1
            cfg.cluster_size = self._cfg.cluster_size
            z.copy_(self._z)
            if c == "tc":
                _lib.call("edg_hmc_glm_tc_run", self._glm.ref(), ctypes.byref(cfg), C, 1,
                          _lib.ptr(self._tiles), _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), 0, None,
                          _lib.ptr(st), None, 0, None, None, None, None, _lib.stream_ptr())
            else:
                cfg.chains_per_block = c
                _lib.call("edg_hmc_glm_run", self._glm.ref(), ctypes.byref(cfg), C, 1,
                          _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), 0, None, _lib.ptr(st),
                          None, 0, None, None, None, None, _lib.stream_ptr())

        key = f"N{self._spec.N}_D{self._spec.D}_b{int(self._spec.bias)}_C{C}_L{self.n_steps}"
        return autotune.choose("hmc_glm", key, cands, run)

    def _build_hier(self):
        """Ragged batch of hierarchical logistic regressions (edg_hmc_hier_run).
        Samples live in one [T, I*C, max_D + 2] store (w, zeros, mu, u); the
        Empiricals are views of it (tau is shown as softplus(u))."""
        spec = self._spec
        hd = HierDevice(spec.Xs, spec.ys, spec.mu_loc, spec.mu_scale, spec.tau_scale,
                        self._device)
        self._hier = hd
        C = self.n_chains or 1
        self.C = C
        I, SP, T = hd.I, hd.SP, self.n_iter
        dev = self._device
        self._samples = torch.zeros(T, I * C, SP, dtype=torch.float32, device=dev)
        view = self._samples.view(T, I, C, SP)
        lead = (T, I) if I > 1 else (T,)
        lead = lead + ((C,) if self.n_chains else ())
        Dmax = hd.max_D
        parts = {spec.w: view[..., :Dmax], spec.mu: view[..., SP - 2], spec.tau: view[..., SP - 1]}
        for z, v in parts.items():
            qz = self.latent_vars[z]
            init = qz.params_var.value
            tgt = v[0]
            if init[0].numel() == tgt.numel():
                tgt.copy_(init[0].to(dev).reshape(tgt.shape))
            # else (ragged w declared with another width): the chains start from zeros
            shape = lead + ((Dmax,) if z is spec.w else ())
            qz.params_var._value = v.view(shape)
            qz.params_var.shape = shape
            qz.n = T
        self.latent_vars[spec.tau]._constrain = torch.nn.functional.softplus
        self._z = self._samples[0].clone()
        self._g = torch.zeros_like(self._z)
        self._lj = torch.zeros(I * C, dtype=torch.float64, device=dev)
        self._cache_valid = 0
        self._n_accept = torch.zeros(I * C, dtype=torch.int32, device=dev)
        cfg = _lib.EdgHMC()
        cfg.step_size = float(self.step_size)
        cfg.n_steps = int(self.n_steps)
        cfg.seed = next_seed()
        self._cfg = cfg
        self.engine = "hier"
        self._graphs = {}
        best = self._autotune_hier()
        cfg.launch, cfg.chains_per_block = best & 1, 16 if best & 2 else 32
        self.hier_engine = "tc" if best & 4 else "simt"
        if best & 4:
            self._hier_tiles = self._hier.tc_tiles()
        else:
            self._hier_tiles = None
            self._hier._tc = None  # the re-laid copy of X is only the tensor-core engine's
        self.train = self.update
        return self.train

    def _autotune_hier(self):
        """Engine, launch form (persistent work-queue grid or one CTA per
        (instance, chain tile)) and, for the SIMT engine, the tile shape (32
        chains x 64 rows or 16 chains x 128 rows) of the ragged batch, timed on
        scratch copies of the state and cached per model shape.  Candidate c
        encodes launch = c & 1, 16 chains per block when c & 2, and the
        tensor-core engine (64 chains x 128 rows, max_D <= 128) when c & 4."""
        hd, C = self._hier, self.C
        req = self._engine_req
        tc_ok = hd.max_D <= 128
        if req == "tc" and not tc_ok:
            raise NotImplementedError("the tensor-core hierarchical engine needs max_D <= 128")
        cands = ([0, 1, 2, 3] if req != "tc" else []) + ([4, 5] if tc_ok and req != "simt" else [])
        z = self._z.clone()
        g = torch.zeros_like(self._g)
        lj = torch.zeros_like(self._lj)

        def run(c):
            cfg = _lib.EdgHMC()
            cfg.step_size, cfg.n_steps, cfg.seed = self._cfg.step_size, self._cfg.n_steps, 1
            cfg.launch, cfg.chains_per_block = c & 1, 16 if c & 2 else 32
            z.copy_(self._z)
            st = _lib.new_state(self._device)
            if c & 4:
                tiles, toff = hd.tc_tiles()
                _lib.call("edg_hmc_hier_tc_run", hd.ref(), ctypes.byref(cfg), C, 1,
                          _lib.ptr(hd.order), _lib.ptr(tiles), _lib.ptr(toff), _lib.ptr(z),
                          _lib.ptr(g), _lib.ptr(lj), 0, None, _lib.ptr(st), None, 0, None, None,
                          None, None, _lib.stream_ptr())
            else:
                _lib.call("edg_hmc_hier_run", hd.ref(), ctypes.byref(cfg), C, 1,
                          _lib.ptr(hd.order), _lib.ptr(z), _lib.ptr(g), _lib.ptr(lj), 0, None,
                          _lib.ptr(st), None, 0, None, None, None, None, _lib.stream_ptr())

        work = int((hd.Ns.astype(np.int64) * hd.Ds).sum())
        key = f"I{hd.I}_work{work}_maxD{hd.max_D}_C{C}_L{self.n_steps}"
        return autotune.choose("hmc_hier_engine_shape", key, cands, run)

    def _build_expfam(self):
        """Chains of the unconstrained latent u (FP32, as the reference's
        chains); the Empirical shows the constrained values
        (``inference.py:247-253``) while ``params_var`` holds u."""
        spec = self._spec
        dev = self._device
        C = self.n_chains or 1
        self.C = C
        T, K = self.n_iter, spec.K
        self._ef_prior = torch.as_tensor(spec.prior, device=dev)
        self._ef_stats = torch.as_tensor(spec.stats, device=dev)
        m = _lib.EdgExpFam()
        m.family, m.K = spec.family, K
        m.prior, m.stats = self._ef_prior.data_ptr(), self._ef_stats.data_ptr()
        m.transform = 1
        self._ef = m
        self._samples = torch.zeros(T, C, K, dtype=torch.float32, device=dev)
        qz = self.latent_vars[spec.z]
        init = qz.params_var.value
        if init[0].numel() == C * K:
            self._samples[0] = init[0].to(dev, torch.float32).reshape(C, K)
        lead = (T, C) if self.n_chains else (T,)
        shape = lead + ((K,) if spec.family == _lib.EXPFAM_DIRICHLET else ())
        qz.params_var._value = self._samples.view(shape)
        qz.params_var.shape = shape
        qz.n = T
        if spec.family == _lib.EXPFAM_BETA:
            qz._constrain = torch.sigmoid
        elif spec.family == _lib.EXPFAM_GAMMA:
            qz._constrain = torch.nn.functional.softplus
        else:
            qz._constrain = lambda u: torch.softmax(
                torch.cat([u, torch.zeros_like(u[..., :1])], dim=-1), dim=-1)
        self._z = self._samples[0].clone()
        self._g = torch.zeros_like(self._z)
        self._lj = torch.zeros(C, dtype=torch.float64, device=dev)
        self._cache_valid = 0
        self._n_accept = torch.zeros(C, dtype=torch.int32, device=dev)
        cfg = _lib.EdgHMC()
        cfg.step_size = float(self.step_size)
        cfg.n_steps = int(self.n_steps)
        cfg.seed = next_seed()
        self._cfg = cfg
        self.engine = "expfam"
        self.train = self.update
        return self.train

    def _launch(self, n_iter, r_override=None, u_override=None, ratio_out=None):
        if self.engine == "expfam":
            if r_override is not None:
                r_override = r_override.to(torch.float32).contiguous()
            if u_override is not None:
                u_override = u_override.to(torch.float64).contiguous()
            _lib.call("edg_expfam_hmc_run", ctypes.byref(self._ef), ctypes.byref(self._cfg),
                      self.C, int(n_iter), _lib.ptr(self._z), _lib.ptr(self._g),
                      _lib.ptr(self._lj), self._cache_valid, _lib.ptr(self._n_accept),
                      _lib.ptr(self._state), _lib.ptr(self._samples), self._samples.shape[0],
                      _lib.ptr(r_override), _lib.ptr(u_override), _lib.stream_ptr())
            self._cache_valid = 1
            return
        if self.engine == "hier":
            def launch():
                if self._hier_tiles is not None:
                    fn = "edg_hmc_hier_tc_run"
                    lead = (_lib.ptr(self._hier.order), _lib.ptr(self._hier_tiles[0]),
                            _lib.ptr(self._hier_tiles[1]))
                else:
                    fn, lead = "edg_hmc_hier_run", (_lib.ptr(self._hier.order),)
                _lib.call(fn, self._hier.ref(), ctypes.byref(self._cfg), self.C,
                          int(n_iter), *lead, _lib.ptr(self._z),
                          _lib.ptr(self._g), _lib.ptr(self._lj), self._cache_valid,
                          _lib.ptr(self._n_accept), _lib.ptr(self._state),
                          _lib.ptr(self._samples), self._samples.shape[0], None,
                          _lib.ptr(r_override), _lib.ptr(u_override), _lib.ptr(ratio_out),
                          _lib.stream_ptr())
            plain = r_override is not None or u_override is not None or ratio_out is not None
            if plain or not self._cache_valid:
                launch()
                self._cache_valid = 1
                return
            # the k-iteration launch with a valid cache is replayed from a CUDA
            # graph (its arguments are fixed; t and the work counter live on
            # the device)
            gph = self._graphs.get(int(n_iter))
            if gph is None:
                gph = torch.cuda.CUDAGraph()
                s = torch.cuda.Stream()
                s.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(s):
                    with torch.cuda.graph(gph, stream=s):
                        launch()
                torch.cuda.current_stream().wait_stream(s)
                self._graphs[int(n_iter)] = gph
            gph.replay()
            return
        if self.engine == "tc":
            _lib.call("edg_hmc_glm_tc_run", self._glm.ref(), ctypes.byref(self._cfg), self.C,
                      int(n_iter), _lib.ptr(self._tiles), _lib.ptr(self._z), _lib.ptr(self._g),
                      _lib.ptr(self._lj), self._cache_valid, _lib.ptr(self._n_accept),
                      _lib.ptr(self._state), _lib.ptr(self._samples), self._samples.shape[0],
                      None, _lib.ptr(r_override), _lib.ptr(u_override), _lib.ptr(ratio_out),
                      _lib.stream_ptr())
        else:
            _lib.call("edg_hmc_glm_run", self._glm.ref(), ctypes.byref(self._cfg), self.C,
                      int(n_iter), _lib.ptr(self._z), _lib.ptr(self._g), _lib.ptr(self._lj),
                      self._cache_valid, _lib.ptr(self._n_accept), _lib.ptr(self._state),
                      _lib.ptr(self._samples), self._samples.shape[0], None,
                      _lib.ptr(r_override), _lib.ptr(u_override), _lib.ptr(ratio_out),
                      _lib.stream_ptr())
        self._cache_valid = 1

    def check_errors(self):
        """Raises if a kernel recorded a bounded-wait timeout (reads the device state)."""
        st = self._read_state()
        if st.error:
            raise TimeoutError("an HMC kernel gave up a bounded device-side wait")

    def update(self, feed_dict=None):
        """One HMC iteration for every chain; returns ``{'t', 'accept_rate'}``
        (``monte_carlo.py:111-150``), accept_rate = n_accept / t averaged over chains."""
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

    def run_iterations(self, k, r_override=None, u_override=None, ratio_out=None):
        """k iterations in one launch, no host synchronisation."""
        self._launch(k, r_override, u_override, ratio_out)

    @property
    def n_accept(self):
        if self._n_accept.numel() == 1:
            return int(self._n_accept[0].item())
        return self._n_accept

    def reset(self):
        """Zeroes t and n_accept (``inference.py:283-285``, ``monte_carlo.py:104``);
        the next iteration restarts from params[0] as the reference's
        ``params[max(t - 1, 0)]`` does."""
        super().reset()
        self._n_accept.zero_()
        self._z.copy_(self._samples[0])
        self._cache_valid = 0
