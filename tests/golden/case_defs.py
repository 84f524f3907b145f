"""Golden-case definitions shared by the fixture generator and the tests:
rebuilds the run directory of a named case from tests/golden/cases.json."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import cases  # noqa: E402


def load_defs():
    with open(os.path.join(HERE, "cases.json")) as fp:
        return json.load(fp)


def make_case(name: str) -> "cases.Case":
    d = dict(load_defs()[name])
    lam_seed = d.pop("lambda_seed", None)
    lam = None
    if lam_seed is not None:
        rng = np.random.default_rng(lam_seed)
        lam = [rng.uniform(-0.5, 0.5, (3, 3)) for _ in range(4)]
    d["kk"] = tuple(d["kk"])
    return cases.Case(lambdas=lam, suffix=name, **d)


def write(name: str, dirpath: str) -> "cases.Case":
    c = make_case(name)
    cases.write_case(c, dirpath)
    return c
