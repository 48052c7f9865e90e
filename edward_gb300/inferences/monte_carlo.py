"""``MonteCarlo`` (``edward/inferences/monte_carlo.py:16-170``): Empirical
sample stores, ``n_iter`` = the shortest store, an ``n_accept`` counter and
an update that advances ``t`` by one.

Extension for the GB300 build: ``n_chains=C`` runs C independent chains in
one launch; Empirical params then have shape [T, C, *event] and ``n_accept``
is per chain.
"""
import numpy as np
import torch

from .. import _lib
from ..expr import Variable
from ..models import Empirical
from .inference import Inference


class MonteCarlo(Inference):
    def __init__(self, latent_vars=None, data=None, n_chains=None):
        if isinstance(latent_vars, list):
            lv = {}
            for z in latent_vars:
                shape = [int(1e4)] + ([n_chains] if n_chains else []) + \
                    list(z.batch_shape) + list(z.event_shape)
                lv[z] = Empirical(Variable(np.zeros(shape, np.float32), trainable=False),
                                  n_chains=n_chains)
            latent_vars = lv
        elif isinstance(latent_vars, dict):
            for qz in latent_vars.values():
                if not isinstance(qz, Empirical):
                    raise TypeError("Posterior approximation must consist of only "
                                    "Empirical random variables.")
        self.n_chains = n_chains
        super().__init__(latent_vars, data)

    def initialize(self, *args, **kwargs):
        kwargs["n_iter"] = int(np.amin([qz.n for qz in self.latent_vars.values()]))
        super().initialize(*args, **kwargs)
        self._validate()
        _lib.require_cuda()
        self._device = torch.device("cuda")
        self._state = _lib.new_state(self._device)
        self.build_update()

    def _validate(self):
        """Host-only model checks run before any device work."""

    def _bind_glm_store(self, spec):
        """One device sample store [T, C, P] for all latents of a compiled GLM;
        every Empirical's params Variable becomes a strided view of it (its
        initial values are copied in), and the chain state starts at
        params[0].  Returns the number of chains C."""
        C = self.n_chains or 1
        self.C = C
        T = self.n_iter
        dev = self._device
        self._samples = torch.zeros(T, C, spec.P, dtype=torch.float32, device=dev)
        for blk in spec.blocks:
            qz = self.latent_vars[blk.rv]
            var = qz.params_var
            src = var.value.to(dev).reshape(qz.n, C, blk.size)[:T]
            self._samples[:, :, blk.offset:blk.offset + blk.size] = src
            view = self._samples[:, :, blk.offset:blk.offset + blk.size]
            shape = (T, C) + tuple(blk.shape) if qz.n_chains else (T,) + tuple(blk.shape)
            var._value = view.view(shape)
            var.shape = tuple(shape)
            qz.n = T
        self._z = self._samples[0].clone()
        return C

    def build_update(self):
        raise NotImplementedError()

    def print_progress(self, info_dict):
        if self.n_print != 0:
            t = info_dict["t"]
            if t == 1 or t % self.n_print == 0:
                self.progbar.update(t, {"Acceptance Rate": info_dict["accept_rate"]})
