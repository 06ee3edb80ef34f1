"""Shared helpers of the test suite: golden fixtures and parameter sets."""
from __future__ import annotations

import json
import os

import numpy as np

from cdet_gb300.params import CdetParams, named_mask

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KINDS = ("twisted_up", "twisted_down", "ordinary_up", "ordinary_down")
KEYS = ("upper", "lower", "upper_corners", "lower_corners")


def load_case(name: str):
    """(params, tables, data) of a golden parameter set. Kinds whose arrays are
    identical are returned as the same dict object (the reference aliases
    them when ALPHA_UP == ALPHA_DOWN)."""
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        args = json.load(f)[name]
    data = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    params = params_from_reference_args(args)
    tables = {}
    for kind in KINDS:
        tables[kind] = {k: data[f"table.{kind}.{k}"] for k in KEYS}
    if params.alpha_equal:
        tables["twisted_down"] = tables["twisted_up"]
        tables["ordinary_down"] = tables["ordinary_up"]
    return params, tables, data


def params_from_reference_args(args: dict, **overrides) -> CdetParams:
    p = CdetParams(n1=args["n1"], n2=args["n2"], beta=args["beta"], mu=args["mu"], u=args["u"],
                   alpha_up=args["alpha_up"], alpha_down=args["alpha_down"], pbc=args["pbc"],
                   mask_sites=named_mask(args["mask_name"], args["n1"], args["n2"], args["radius"]),
                   cheb_nu=args["nu"], cheb_nv=args["nv"])
    import dataclasses
    return dataclasses.replace(p, **overrides)


def bits_equal(a, b) -> bool:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))
