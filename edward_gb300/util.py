"""Seeding and progress printing (``edward/util/graphs.py:59-73``,
``edward/util/progbar.py``)."""
import sys
import time

import numpy as np

_SEED = None
_stream_counter = 0


def set_seed(x):
    """Seeds NumPy (used for Variable initialisation) and the Philox key of
    every inference created afterwards (``ed.set_seed``, graphs.py:59-73)."""
    global _SEED, _stream_counter
    _SEED = int(x)
    _stream_counter = 0
    np.random.seed(_SEED % (2 ** 32))


def next_seed():
    """A fresh 64-bit Philox key: derived from set_seed's value when one was
    set (deterministic), else from NumPy's global generator."""
    global _stream_counter
    _stream_counter += 1
    if _SEED is not None:
        return (_SEED * 0x9E3779B97F4A7C15 + _stream_counter * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    return int(np.random.randint(0, 2 ** 63 - 1, dtype=np.int64))


def randn(shape):
    return np.random.standard_normal(shape).astype(np.float32)


class Progbar:
    """Minimal text progress bar with the reference's update(t, values) API."""

    def __init__(self, target, width=30, interval=0.05):
        self.target = target
        self.width = width
        self.interval = interval
        self.start = time.time()
        self.last = 0.0

    def update(self, current, values=None):
        now = time.time()
        if now - self.last < self.interval and current < self.target:
            return
        self.last = now
        frac = current / float(self.target) if self.target else 1.0
        filled = int(self.width * min(frac, 1.0))
        bar = "[" + "=" * filled + " " * (self.width - filled) + "]"
        info = "".join(f" {k}: {v:.3f}" if isinstance(v, float) else f" {k}: {v}"
                       for k, v in (values or {}).items())
        elapsed = now - self.start
        sys.stdout.write(f"\r{current}/{self.target} {int(100 * frac):3d}% {bar} "
                         f"Elapsed: {int(elapsed)}s |{info}")
        if current >= self.target:
            sys.stdout.write("\n")
        sys.stdout.flush()
