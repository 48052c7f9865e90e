"""``tf.layers.dense`` analogue for model and recognition networks written as
in ``examples/sigmoid_belief_network.py:60-80``: it creates a kernel
Variable [in, units] (Glorot-uniform, TF's default initializer) and a bias
Variable [units] (zeros) and returns ``matmul(inputs, kernel) + bias``.
The model compiler finds the Variables in the expression; inference rebinds
them to its flat device parameter buffer."""
import numpy as np

from .expr import Variable, as_node, matmul


def dense(inputs, units, activation=None, use_bias=True, name=None):
    x = as_node(inputs)
    shp = getattr(x, "shape", None)
    if not shp or shp[-1] is None:
        raise ValueError("dense needs inputs with a static last dimension")
    fan_in = int(shp[-1])
    lim = np.sqrt(6.0 / (fan_in + units))
    kernel = Variable(np.random.uniform(-lim, lim, (fan_in, units)).astype(np.float32),
                      name=f"{name or 'dense'}/kernel")
    out = matmul(x, kernel)
    if use_bias:
        out = out + Variable(np.zeros(units, np.float32), name=f"{name or 'dense'}/bias")
    if activation is not None:
        out = activation(out)
    return out
