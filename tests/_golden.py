"""Helpers to read the committed golden fixtures (tests/golden/)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

QUAD_CASES = ["cfg0", "grid", "testparams", "n1", "n3", "n37"]


def quad(name):
    d = np.load(os.path.join(GOLDEN, f"quad_{name}.npz"))
    return {k: d[k] for k in d.files}


def dropin(name):
    d = np.load(os.path.join(GOLDEN, f"dropin_{name}.npz"))
    return {k: d[k] for k in d.files}


def dropin_cv(name):
    d = np.load(os.path.join(GOLDEN, f"cv_{name}.npz"))
    return {k: d[k] for k in d.files}


def debug8():
    with open(os.path.join(GOLDEN, "debug8.json")) as f:
        return json.load(f)


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)
