"""``VariationalInference`` (``edward/inferences/variational_inference.py:16-185``):
optimizer / learning-rate resolution and the update loop around a fused
ELBO-gradient + optimizer-apply kernel."""
import abc

import torch

from .. import _lib
from .. import train
from .inference import Inference


class VariationalInference(Inference):
    def initialize(self, optimizer=None, var_list=None, use_prettytensor=False, global_step=None,
                   *args, **kwargs):
        super().initialize(*args, **kwargs)
        if use_prettytensor:
            raise NotImplementedError("PrettyTensor optimizers are not supported")
        self.optimizer = train.resolve(optimizer, global_step)
        self._validate()
        _lib.require_cuda()
        self._device = torch.device("cuda")
        self._state = _lib.new_state(self._device, getattr(self.optimizer, "beta1", 0.9),
                                     getattr(self.optimizer, "beta2", 0.999))
        self._graphs = {}
        self.loss, self.grads_and_vars = self.build_loss_and_gradients(var_list)

    def _validate(self):
        """Host-only model checks run before any device work."""

    @abc.abstractmethod
    def build_loss_and_gradients(self, var_list):
        raise NotImplementedError()

    # Subclasses provide _step(apply) launching one fused step on the current stream.
    def update(self, feed_dict=None):
        """One ELBO-gradient step + optimizer apply; returns ``{'t', 'loss'}``
        (``variational_inference.py:133-164``).  Reads the loss back to the host."""
        if feed_dict:
            self._feed(feed_dict)
        self._step(apply=True)
        st = self._read_state()
        if self.debug and st.nonfinite:
            raise FloatingPointError("non-finite loss or gradient detected (debug=True)")
        return {"t": int(st.t), "loss": float(st.loss)}

    def _feed(self, feed_dict):
        raise NotImplementedError("feed_dict is not supported for this model family")

    def print_progress(self, info_dict):
        if self.n_print != 0:
            t = info_dict["t"]
            if t == 1 or t % self.n_print == 0:
                self.progbar.update(t, {"Loss": info_dict["loss"]})

    def _run_loop(self):
        """n_iter steps with one host read-back per print interval.  The
        steps between prints are replayed from a CUDA graph."""
        done = 0
        chunk = self.n_print if self.n_print else self.n_iter
        chunk = max(1, min(chunk, 100))
        while done < self.n_iter:
            k = min(chunk, self.n_iter - done)
            self.steps(k)
            done += k
            st = self._read_state()
            if self.debug and st.nonfinite:
                raise FloatingPointError("non-finite loss or gradient detected (debug=True)")
            self.print_progress({"t": int(st.t), "loss": float(st.loss)})

    def steps(self, k, use_graph=True):
        """Runs k fused steps without host synchronisation."""
        if not use_graph or k < 4:
            for _ in range(k):
                self._step(apply=True)
            return
        g = self._graphs.get(k)
        if g is None:
            self._step(apply=True)  # warm-up outside capture (sets kernel attributes)
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    for _ in range(k):
                        self._step(apply=True)
            torch.cuda.current_stream().wait_stream(s)
            self._graphs[k] = g
            # capture does not execute the steps: the warm-up did one, replay
            # the graph minus one step's worth is not expressible, so run the
            # remaining k - 1 steps directly this time
            for _ in range(k - 1):
                self._step(apply=True)
            return
        g.replay()

    def reset(self):
        from .. import _lib as lib
        self._state.copy_(lib.new_state(self._state.device, getattr(self.optimizer, "beta1", 0.9),
                                        getattr(self.optimizer, "beta2", 0.999)))
        self._reset_optimizer()

    def _reset_optimizer(self):
        pass
