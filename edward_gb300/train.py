"""Optimizer descriptions: the ``tf.train.*Optimizer`` choices that
``VariationalInference.initialize`` accepts
(``edward/inferences/variational_inference.py:83-116``).  They are applied
inside the fused KLqp kernels; these classes only carry hyper-parameters."""
from dataclasses import dataclass

from . import _lib


@dataclass
class ExponentialDecay:
    """``tf.train.exponential_decay(lr0, global_step, decay_steps, decay_rate, staircase)``."""
    learning_rate: float
    decay_steps: int
    decay_rate: float
    staircase: bool = False


def exponential_decay(learning_rate, global_step=None, decay_steps=100, decay_rate=0.9,
                      staircase=False):
    return ExponentialDecay(learning_rate, decay_steps, decay_rate, staircase)


class Optimizer:
    kind = None

    def __init__(self, learning_rate=0.001):
        self.learning_rate = learning_rate

    def slot_init(self):
        """Initial values of the two slot arrays (TF slot initialisers)."""
        return 0.0, 0.0

    def to_c(self):
        o = _lib.EdgOpt()
        o.optimizer = self.kind
        lr = self.learning_rate
        if isinstance(lr, ExponentialDecay):
            o.lr0 = lr.learning_rate
            o.decay_steps = int(lr.decay_steps)
            o.decay_rate = lr.decay_rate
            o.staircase = 1 if lr.staircase else 0
        else:
            o.lr0 = float(lr)
            o.decay_steps = 0
            o.decay_rate = 1.0
            o.staircase = 0
        o.beta1, o.beta2, o.epsilon = 0.9, 0.999, 1e-8
        o.momentum, o.rho = 0.0, 0.95
        self._fill(o)
        return o

    def _fill(self, o):
        pass


class AdamOptimizer(Optimizer):
    kind = _lib.OPT_ADAM

    def __init__(self, learning_rate=0.001, beta1=0.9, beta2=0.999, epsilon=1e-8):
        super().__init__(learning_rate)
        self.beta1, self.beta2, self.epsilon = beta1, beta2, epsilon

    def _fill(self, o):
        o.beta1, o.beta2, o.epsilon = self.beta1, self.beta2, self.epsilon


class GradientDescentOptimizer(Optimizer):
    kind = _lib.OPT_SGD


class MomentumOptimizer(Optimizer):
    kind = _lib.OPT_MOMENTUM

    def __init__(self, learning_rate, momentum=0.9):
        super().__init__(learning_rate)
        self.momentum = momentum

    def _fill(self, o):
        o.momentum = self.momentum


class AdagradOptimizer(Optimizer):
    kind = _lib.OPT_ADAGRAD

    def __init__(self, learning_rate, initial_accumulator_value=0.1):
        super().__init__(learning_rate)
        self.initial_accumulator_value = initial_accumulator_value

    def slot_init(self):
        return self.initial_accumulator_value, 0.0


class RMSPropOptimizer(Optimizer):
    kind = _lib.OPT_RMSPROP

    def __init__(self, learning_rate, decay=0.9, momentum=0.0, epsilon=1e-10):
        super().__init__(learning_rate)
        self.decay, self.momentum, self.epsilon = decay, momentum, epsilon

    def slot_init(self):
        return 1.0, 0.0

    def _fill(self, o):
        o.rho, o.momentum, o.epsilon = self.decay, self.momentum, self.epsilon


class AdadeltaOptimizer(Optimizer):
    kind = _lib.OPT_ADADELTA

    def __init__(self, learning_rate=0.001, rho=0.95, epsilon=1e-8):
        super().__init__(learning_rate)
        self.rho, self.epsilon = rho, epsilon

    def _fill(self, o):
        o.rho, o.epsilon = self.rho, self.epsilon


_BY_NAME = {
    "gradientdescent": GradientDescentOptimizer,
    "adadelta": AdadeltaOptimizer,
    "adagrad": AdagradOptimizer,
    "momentum": lambda lr: MomentumOptimizer(lr, 0.9),
    "adam": AdamOptimizer,
    "rmsprop": RMSPropOptimizer,
}


def resolve(optimizer, global_step):
    """The optimizer/learning-rate choice of variational_inference.py:83-116."""
    use_decay = (optimizer is None and global_step is None) or global_step is not None
    lr = exponential_decay(0.1, None, 100, 0.9, staircase=True) if use_decay else 0.01
    if optimizer is None:
        return AdamOptimizer(lr)
    if isinstance(optimizer, str):
        if optimizer == "ftrl":
            raise NotImplementedError("the ftrl optimizer is not fused into the KLqp kernels")
        if optimizer not in _BY_NAME:
            raise ValueError("Optimizer class not found:", optimizer)
        return _BY_NAME[optimizer](lr)
    if isinstance(optimizer, Optimizer):
        return optimizer
    raise TypeError("Optimizer must be str, tf.train.Optimizer, or None.")
