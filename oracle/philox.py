"""Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
easy as 1, 2, 3", SC 2011) and the value mappings shared with the CUDA
kernels.  Test infrastructure: see ``oracle/__init__.py``.

The reference draws its randomness from stateful TF ops:
``tf.random_normal`` for HMC momenta (``edward/inferences/hmc.py:88-91``),
``tf.random_uniform`` for the Metropolis test (``hmc.py:108``) and the
reparameterised q sample ``loc + scale * eps`` inside ``copy(qz)``
(``edward/inferences/klqp.py:727-731``).  The GPU build replaces them with a
counter-based generator so that every draw is a pure function of
(seed, stream kind, iteration, row, element).

Counter layout (one 128-bit counter per 4 outputs):
    ctr = (quad, row, iteration, kind)    key = (seed_lo, seed_hi)
where ``quad`` = element // 4 and ``row`` is the Monte Carlo sample or the
chain.  Normal draws use Box-Muller on output pairs (0,1) and (2,3);
uniforms use one 32-bit output each.
"""
import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)

KIND_EPS = 0        # reparameterisation noise for KLqp
KIND_MOMENTUM = 1   # HMC momentum
KIND_UNIFORM = 2    # HMC Metropolis uniform
KIND_BERNOULLI = 3  # Bernoulli latent draws (score-function path)
KIND_MINIBATCH = 4  # minibatch row selection


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32 with 10 rounds. All inputs are uint32 arrays
    (broadcastable); returns four uint32 arrays."""
    c0 = np.asarray(c0, np.uint32).astype(np.uint64)
    c1 = np.asarray(c1, np.uint32).astype(np.uint64)
    c2 = np.asarray(c2, np.uint32).astype(np.uint64)
    c3 = np.asarray(c3, np.uint32).astype(np.uint64)
    k0 = np.asarray(k0, np.uint32).astype(np.uint64)
    k1 = np.asarray(k1, np.uint32).astype(np.uint64)
    c0, c1, c2, c3, k0, k1 = np.broadcast_arrays(c0, c1, c2, c3, k0, k1)
    c0, c1, c2, c3 = c0.copy(), c1.copy(), c2.copy(), c3.copy()
    k0, k1 = k0.copy(), k1.copy()
    for rnd in range(10):
        if rnd:
            k0 = (k0 + np.uint64(W0)) & MASK32
            k1 = (k1 + np.uint64(W1)) & MASK32
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return tuple(x.astype(np.uint32) for x in (c0, c1, c2, c3))


def _key(seed):
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return np.uint32(seed & 0xFFFFFFFF), np.uint32(seed >> 32)


def raw_u32(seed, kind, iteration, rows, n_elem, row0=0):
    """uint32 stream laid out [rows, round_up(n_elem, 4)] for one iteration
    (rows row0 .. row0 + rows - 1)."""
    k0, k1 = _key(seed)
    nq = (n_elem + 3) // 4
    q = np.arange(nq, dtype=np.uint32)[None, :]
    r = (np.arange(rows, dtype=np.uint64) + np.uint64(row0)).astype(np.uint32)[:, None]
    o = philox4x32_10(q, r, np.uint32(iteration & 0xFFFFFFFF), np.uint32(kind), k0, k1)
    out = np.stack(o, axis=-1).reshape(rows, nq * 4)
    return out


def u32_to_open01_f32(a):
    """(2 (a >> 9) + 1) * 2^-24: 23-bit uniform strictly inside (0, 1), exact in FP32."""
    k = (np.asarray(a, np.uint32) >> np.uint32(9)).astype(np.float64)
    return (2.0 * k + 1.0) * (2.0 ** -24)


def u32_to_open01_f64(a):
    """(a + 0.5) * 2^-32: 32-bit uniform strictly inside (0, 1), exact in FP64."""
    return (np.asarray(a, np.uint32).astype(np.float64) + 0.5) * (2.0 ** -32)


def normals(seed, kind, iteration, rows, n_elem, row0=0):
    """Box-Muller normals [rows, n_elem] (computed in FP64; the kernels use
    FP32 logf/sqrtf/sincospif, so agreement is to a few FP32 ulps)."""
    raw = raw_u32(seed, kind, iteration, rows, n_elem, row0).reshape(rows, -1, 4)
    out = np.empty(raw.shape, np.float64)
    for a, b in ((0, 1), (2, 3)):
        u1 = u32_to_open01_f32(raw[..., a])
        u2 = u32_to_open01_f32(raw[..., b])
        rad = np.sqrt(-2.0 * np.log(u1))
        out[..., a] = rad * np.cos(2.0 * np.pi * u2)
        out[..., b] = rad * np.sin(2.0 * np.pi * u2)
    return out.reshape(rows, -1)[:, :n_elem]


def uniforms64(seed, kind, iteration, rows, row0=0):
    """One FP64 uniform in (0,1) per row (the Metropolis ``u``)."""
    raw = raw_u32(seed, kind, iteration, rows, 1, row0)
    return u32_to_open01_f64(raw[:, 0])


def uniforms24(seed, kind, iteration, rows, n_elem):
    """FP32-exact uniforms [rows, n_elem] (Bernoulli latent draws)."""
    raw = raw_u32(seed, kind, iteration, rows, n_elem)
    return u32_to_open01_f32(raw)[:, :n_elem]
