"""Readers for the golden fixtures in tests/golden/ (made by make_golden.py)."""
import gzip
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def stdout_text(test):
    with gzip.open(os.path.join(GOLDEN, f"{test}.stdout.gz"), "rb") as f:
        return f.read().decode()


def f32(name, shape=None):
    with gzip.open(os.path.join(GOLDEN, name), "rb") as f:
        a = np.frombuffer(f.read(), dtype=np.float32).copy()
    return a.reshape(shape) if shape is not None else a


def hexfloats(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return [float.fromhex(t) for t in f.read().split()]


def dump_text(arr, fmt="%f"):
    """The reference tests' dump(): one printf per element, x fastest."""
    flat = np.asarray(arr).reshape(-1)
    if fmt == "%d":
        return "".join("%d\n" % int(v) for v in flat)
    return "".join(fmt % float(v) + "\n" for v in flat)
