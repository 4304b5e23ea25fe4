import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def reference_test_settings(**over):
    """The .rc written by the reference's regression driver (test/testElliptic.py:34-59)
    for a 3D hex run; LAMBDA is not among the written keys, so its default 1.0 applies."""
    d = {"FORMAT": "2.0", "DATA FILE": "ellipticSine3D.h", "MESH FILE": "BOX",
         "MESH DIMENSION": 3, "ELEMENT TYPE": 12, "BOX NX": 10, "BOX NY": 10, "BOX NZ": 10,
         "BOX DIMX": 1, "BOX DIMY": 1, "BOX DIMZ": 1, "BOX BOUNDARY FLAG": 1,
         "POLYNOMIAL DEGREE": 4, "DISCRETIZATION": "CONTINUOUS", "LINEAR SOLVER": "PCG",
         "PRECONDITIONER": "MULTIGRID", "MULTIGRID SMOOTHER": "CHEBYSHEV",
         "PARALMOND CYCLE": "VCYCLE", "PARALMOND STRENGTH": "SYMMETRIC",
         "PARALMOND AGGREGATION": "UNSMOOTHED", "PARALMOND SMOOTHER": "CHEBYSHEV"}
    d.update(over)
    return d


def golden_case_settings(case):
    """Translate a reference golden case's keyword settings into .rc keys."""
    s = case["settings"]
    over = {}
    if "precon" in s:
        over["PRECONDITIONER"] = s["precon"]
    if "degree" in s:
        over["POLYNOMIAL DEGREE"] = s["degree"]
    if "boundary_flag" in s:
        over["BOX BOUNDARY FLAG"] = s["boundary_flag"]
    if "discretization" in s:
        over["DISCRETIZATION"] = s["discretization"]
    if "paralmond_aggregation" in s:
        over["PARALMOND AGGREGATION"] = s["paralmond_aggregation"]
    return reference_test_settings(**over)


@pytest.fixture(scope="session")
def reference_norms():
    import json
    return json.load(open(os.path.join(ROOT, "tests", "golden", "reference_norms.json")))
