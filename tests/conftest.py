import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "ie-solver_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def solver_lib():
    from rskel import capi

    return capi


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return {k: d[k] for k in d.files}


def golden_geometry(d):
    from rskel.geometry import Geometry

    return Geometry(d["points"], d["normals"], d["weights"], d["curvatures"], d["hole_centers"],
                    d["hole_radii"], 0)


GOLDEN_CASES = ["laplace_circle_512", "stokes_circle_512", "laplace_annulus_512",
                "stokes_annulus_512", "laplace_unit_circle_4096", "laplace_star_8192_2rhs",
                "stokes_ellipses_4096"]
