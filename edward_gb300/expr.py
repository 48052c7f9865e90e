"""Symbolic model expressions.

Edward builds models as TensorFlow graphs: ``ed.dot(X, w) + b``,
``tf.matmul``, ``tf.tanh``, ``tf.nn.softplus``, placeholders and variables
(``edward/util/tensorflow.py:10-47``; ``examples/bayesian_nn.py:121-125``).
Here the same expressions build a small symbolic DAG that the model compiler
(``edward_gb300.compile``) pattern-matches into one of the families the CUDA
kernels implement.  Nothing here computes on the hot path.
"""
import numbers

import numpy as np
import torch


class Node:
    """Base of every symbolic value (constants, variables, ops, random variables)."""

    shape = ()

    def __add__(self, o):
        return Op("add", self, as_node(o))

    def __radd__(self, o):
        return Op("add", as_node(o), self)

    def __sub__(self, o):
        return Op("add", self, Op("neg", as_node(o)))

    def __rsub__(self, o):
        return Op("add", as_node(o), Op("neg", self))

    def __mul__(self, o):
        return Op("mul", self, as_node(o))

    def __rmul__(self, o):
        return Op("mul", as_node(o), self)

    def __neg__(self):
        return Op("neg", self)

    def __matmul__(self, o):
        return matmul(self, o)


class Const(Node):
    def __init__(self, value, dtype=np.float32):
        if isinstance(value, torch.Tensor):
            value = value.detach().cpu().numpy()
        self.value = np.asarray(value, dtype=dtype)
        self.shape = tuple(self.value.shape)

    def __repr__(self):
        return f"Const(shape={self.shape})"


class Variable(Node):
    """A trainable (or not) parameter, the analogue of ``tf.Variable``.

    The value is a torch tensor.  After ``KLqp.initialize`` the tensor is a
    view into the flat device buffer that the fused kernel updates, so
    ``var.value`` always shows the current parameter."""

    _count = 0

    def __init__(self, initial_value, trainable=True, name=None, dtype=torch.float32):
        if isinstance(initial_value, Node):
            raise TypeError("Variable initial value must be numeric")
        t = torch.as_tensor(np.asarray(initial_value), dtype=dtype).clone()
        self._value = t
        self._initial = t.clone()
        self.trainable = trainable
        Variable._count += 1
        self.name = name or f"Variable_{Variable._count}"
        self.shape = tuple(t.shape)

    @property
    def value(self):
        return self._value

    def assign(self, v):
        self._value.copy_(torch.as_tensor(np.asarray(v), dtype=self._value.dtype))

    def _rebind(self, tensor_view):
        tensor_view.copy_(self._value.to(tensor_view.device).reshape(tensor_view.shape))
        self._value = tensor_view

    def numpy(self):
        return self._value.detach().cpu().numpy()

    def __repr__(self):
        return f"Variable({self.name}, shape={self.shape})"


class Placeholder(Node):
    """``tf.placeholder`` analogue: bound to an array through the data dict."""

    def __init__(self, dtype=np.float32, shape=None, name=None):
        self.dtype = dtype
        self.shape = tuple(shape) if shape is not None else None
        self.name = name or "Placeholder"

    def __repr__(self):
        return f"Placeholder({self.name}, shape={self.shape})"


class Op(Node):
    def __init__(self, op, *args, **attrs):
        self.op = op
        self.args = args
        self.attrs = attrs
        self.shape = _infer_shape(op, args, attrs)

    def __repr__(self):
        return f"Op({self.op}, {', '.join(map(repr, self.args))})"


def _shape(n):
    return n.shape if n.shape is not None else None


def _infer_shape(op, args, attrs):
    try:
        if op in ("add", "mul"):
            a, b = (_shape(x) for x in args)
            if a is None or b is None:
                return None
            return tuple(np.broadcast_shapes(a, b))
        if op in ("neg", "tanh", "sigmoid", "softplus", "cast"):
            return _shape(args[0])
        if op == "dot":
            a = _shape(args[0])
            return None if a is None else (a[0],)
        if op == "matmul":
            a, b = (_shape(x) for x in args)
            if a is None or b is None:
                return None
            return (a[0], b[1])
        if op == "reshape":
            shp = tuple(attrs["shape"])
            if -1 in shp:
                a = _shape(args[0])
                if a is None or None in a:
                    return None
                known = int(np.prod([d for d in shp if d != -1]))
                shp = tuple(int(np.prod(a)) // known if d == -1 else d for d in shp)
            return shp
    except (ValueError, IndexError, TypeError):
        pass
    return None


def as_node(x):
    if isinstance(x, Node):
        return x
    if isinstance(x, (numbers.Number, np.ndarray, list, tuple, torch.Tensor, np.number)):
        return Const(x)
    raise TypeError(f"cannot use {type(x).__name__} in a model expression")


def dot(x, y):
    """``ed.dot``: matrix-vector product (``edward/util/tensorflow.py:10-47``)."""
    return Op("dot", as_node(x), as_node(y))


def matmul(a, b):
    return Op("matmul", as_node(a), as_node(b))


def tanh(x):
    return Op("tanh", as_node(x))


def sigmoid(x):
    return Op("sigmoid", as_node(x))


def softplus(x):
    """``tf.nn.softplus``; ``Normal(loc=v1, scale=softplus(v2))`` is the
    mean-field family the KLqp kernels optimise."""
    return Op("softplus", as_node(x))


def reshape(x, shape):
    return Op("reshape", as_node(x), shape=tuple(shape))


def cast(x, dtype=np.float32):
    return Op("cast", as_node(x), dtype=dtype)


def zeros(shape):
    return Const(np.zeros(shape, np.float32))


def ones(shape):
    return Const(np.ones(shape, np.float32))


def placeholder(dtype=np.float32, shape=None, name=None):
    return Placeholder(dtype, shape, name)


def flatten_add(node):
    """Terms of a (possibly nested) sum."""
    if isinstance(node, Op) and node.op == "add":
        return flatten_add(node.args[0]) + flatten_add(node.args[1])
    return [node]


def const_value(node, bindings=None):
    """NumPy value of a constant / bound placeholder / non-trainable expression, else None."""
    bindings = bindings or {}
    if isinstance(node, Const):
        return node.value
    if isinstance(node, Placeholder):
        v = bindings.get(node)
        return None if v is None else np.asarray(v, np.float32)
    if isinstance(node, Op):
        vals = [const_value(a, bindings) for a in node.args]
        if any(v is None for v in vals):
            return None
        if node.op == "add":
            return vals[0] + vals[1]
        if node.op == "mul":
            return vals[0] * vals[1]
        if node.op == "neg":
            return -vals[0]
        if node.op == "cast":
            return vals[0].astype(node.attrs.get("dtype", np.float32))
        if node.op == "reshape":
            return vals[0].reshape(node.attrs["shape"])
    return None
