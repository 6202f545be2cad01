import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GEO = os.path.join(ROOT, "tests", "golden", "geo")
SPHERE = os.path.join(GEO, "sphere.dat")
TORUS = os.path.join(GEO, "torus.dat")
# The analytic cube sphere (six x/|x| images of the cube faces): the product
# builds it with Geometry.cube_sphere(), the oracle under this name.
CUBE = "analytic:cube_sphere"


def geometry(bg, geo, ctx):
    """The product's geometry for a test geometry name or file."""
    return bg.Geometry.cube_sphere(ctx) if geo == CUBE else bg.Geometry(geo, ctx)


# The unit-square screen of the reference's unit tests (z = 0, bilinear map).
SCREEN_DAT = """# nurbs mesh v.2.1
# screen
# unit square in the plane z = 0
#
2 3 1 0 0
PATCH 0
1 1
2 2
0 0 1 1
0 0 1 1
0 1 0 1
0 0 1 1
0 0 0 0
1 1 1 1
"""


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def screen_path(tmp_path_factory):
    p = tmp_path_factory.mktemp("geo") / "screen.dat"
    p.write_text(SCREEN_DAT)
    return str(p)


@pytest.fixture(scope="session")
def oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.lib()
    return O
