"""Per-order precision of integrand values against the oracle's long double truth.

TEST INFRASTRUCTURE (a checker): imported by tests/ and by bench.py's
precision leg; the product package never imports it.

An integrand value of order n is a difference of two connected sums
(twisted - 2 ordinary), each an inclusion-exclusion over 2^n principal-minor
products. Its relative error is ill-posed at high order: the sum cancels by
factors up to 1e19 at order 10 on the 8x8 lattice, so an FP64 evaluation
that makes a round-off of 1e-16 in every term is off by a percent. Three
error forms are reported, each as median, 90th percentile and maximum over
the configurations of an order:

* ``relative``: |x - truth| / |truth|;
* ``combine_scaled``: |x - truth| / (|twisted| + 2 |ordinary|), which removes
  the cancellation of the final combine only (it matters at order 1, where
  twisted - 2 ordinary cancels to round-off);
* ``condition_scaled``: |x - truth| / (M_twisted + 2 M_ordinary), M_set = the
  set's prefactor times the connected recursion run on absolute values (the
  magnitudes of every term that enters the value). This is the well-posed
  form: an evaluation whose every term is right to a relative 1e-10 is right
  to 1e-10 here, at any order.
"""
from __future__ import annotations

from typing import Dict

import numpy as np


def quantiles(e: np.ndarray):
    e = e[np.isfinite(e)]
    if e.size == 0:
        return None
    return {"median": float(np.median(e)), "p90": float(np.percentile(e, 90)), "max": float(e.max())}


def error_forms(value: np.ndarray, truth: np.ndarray, parts: np.ndarray, ok: np.ndarray) -> Dict:
    """The three error forms of `value` against the truth, over the
    configurations where `ok` holds. parts[c] = (twisted, ordinary,
    twisted magnitude, ordinary magnitude) of the truth."""
    d = np.abs(value[ok] - truth[ok])
    p = parts[ok]
    return {"relative": quantiles(d / np.maximum(np.abs(truth[ok]), 1e-300)),
            "combine_scaled": quantiles(d / np.maximum(np.abs(p[:, 0]) + 2 * np.abs(p[:, 1]), 1e-300)),
            "condition_scaled": quantiles(d / np.maximum(p[:, 2] + 2 * p[:, 3], 1e-300))}
