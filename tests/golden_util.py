"""Helpers to regenerate the inputs of a golden fixture."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden import digest, golden_inputs  # noqa: E402


def inputs_of(case):
    ref, q = golden_inputs(str(case["name"]), str(case["dtype"]), int(case["d"]), int(case["n"]),
                           int(case["nq"]), str(case["kind"]))
    assert digest(ref, q) == str(case["input_sha"]), "input generator drifted from the fixture"
    return ref, q


def rows(case):
    return case["dists"].shape[0]
