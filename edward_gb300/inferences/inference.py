"""``Inference``: the root of the drop-in surface
(``edward/inferences/inference.py:20-376``).

Same constructor (``latent_vars`` / ``data`` dicts), ``run`` /
``initialize`` / ``update`` / ``print_progress`` / ``finalize``, the
``scale`` / ``auto_transform`` / ``debug`` keyword arguments and the
iteration counter ``t`` with ``reset``.  Instead of a TF session, the
subclasses drive fused CUDA kernels through the C ABI.
"""
import abc

import numpy as np

from ..expr import Node, Placeholder
from ..models import RandomVariable
from ..util import Progbar


def check_latent_vars(latent_vars):
    """Type checks of ``edward/util/random_variables.py:64-83``."""
    for key, value in latent_vars.items():
        if not isinstance(key, RandomVariable):
            raise TypeError("Latent variable key has an invalid type: {}".format(type(key)))
        if not isinstance(value, RandomVariable):
            raise TypeError("Latent variable value has an invalid type: {}".format(type(value)))


def check_data(data):
    """Type checks of ``edward/util/random_variables.py:21-61``."""
    for key, value in data.items():
        if isinstance(key, Placeholder):
            if isinstance(value, RandomVariable):
                raise TypeError("Data value has an invalid type: {}".format(type(value)))
        elif isinstance(key, RandomVariable):
            if not isinstance(value, (RandomVariable, Node, np.ndarray, list, float, int,
                                      np.number)) and not hasattr(value, "shape"):
                raise TypeError("Data value has an invalid type: {}".format(type(value)))
        else:
            raise TypeError("Data key has an invalid type: {}".format(type(key)))


class Inference(abc.ABC):
    def __init__(self, latent_vars=None, data=None):
        if latent_vars is None:
            latent_vars = {}
        if data is None:
            data = {}
        check_latent_vars(latent_vars)
        self.latent_vars = latent_vars
        check_data(data)
        self.data = {}
        for k, v in data.items():
            if hasattr(v, "detach"):
                v = v.detach().cpu().numpy()
            self.data[k] = v
        self._initialized = False

    # ------------------------------------------------------------ run loop
    def run(self, variables=None, use_coordinator=True, *args, **kwargs):
        """initialize -> n_iter x (update, print_progress) -> finalize
        (``inference.py:97-154``).  ``variables`` and ``use_coordinator``
        are accepted for signature compatibility (there is no TF session)."""
        self.initialize(*args, **kwargs)
        self._run_loop()
        self.finalize()

    def _run_loop(self):
        for _ in range(self.n_iter):
            info = self.update()
            self.print_progress(info)

    @abc.abstractmethod
    def initialize(self, n_iter=1000, n_print=None, scale=None, auto_transform=True,
                   logdir=None, log_timestamp=True, log_vars=None, debug=False):
        self.n_iter = n_iter
        self.n_print = int(n_iter / 100) if n_print is None else n_print
        self.progbar = Progbar(self.n_iter)
        if scale is None:
            scale = {}
        elif not isinstance(scale, dict):
            raise TypeError("scale must be a dict object.")
        self.scale = scale
        self.auto_transform = auto_transform
        self.transformations = {}
        self.logging = logdir is not None
        self.logdir = logdir
        self.debug = debug
        self._initialized = True

    @abc.abstractmethod
    def update(self, feed_dict=None):
        raise NotImplementedError()

    def print_progress(self, info_dict):
        if self.n_print != 0:
            t = info_dict["t"]
            if t == 1 or t % self.n_print == 0:
                self.progbar.update(t)

    def finalize(self):
        pass

    # ------------------------------------------------------------ state
    @property
    def t(self):
        """Iterations run since initialize / reset (``inference.py:195-197``)."""
        return int(self._read_state().t)

    def _read_state(self):
        from .. import _lib
        return _lib.read_state(self._state)

    def reset(self):
        """Re-initialises ``t`` and the subclass state, as running the
        reference's ``inference.reset`` ops does (``inference.py:283-285``)."""
        from .. import _lib
        self._state.copy_(_lib.new_state(self._state.device))
