"""Shared test helpers: the reference's binomial acceptance bounds and
loaders for the golden known-answer tests."""
import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vectorstate_kats.json")


def erfinv(y):
    from scipy.special import erfinv as _e
    return float(_e(y))


def get_bounds(nr_shots, p, tol):
    """Binomial quantile bounds of src/stats.rs:10-19."""
    mu = nr_shots * p
    sigma = math.sqrt(nr_shots * p * (1.0 - p))
    quantile = mu + sigma * math.sqrt(2.0) * erfinv(2.0 * tol - 1.0)
    low = math.floor(quantile)
    high = math.ceil(mu + (mu - quantile))
    return low, high


def measurement_ok(count, nr_shots, p, tol=1e-5):
    """src/stats.rs:26-32"""
    low, high = get_bounds(nr_shots, p, tol)
    return low < count < high


def kats():
    with open(GOLDEN) as f:
        return json.load(f)


def dec(a):
    """[[re, im], ...] nested -> complex ndarray"""
    a = np.asarray(a, dtype=np.float64)
    return a[..., 0] + 1j * a[..., 1]


# the reference's assert_complex_matrix_eq! tolerance (src/cmatrix.rs:54-120)
KAT_TOL = 1e-15
