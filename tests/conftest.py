import ast
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_WORLDS = ["c0_seed0", "c1_poisson", "falling_blocks", "bilinear_cantilever", "large_angle", "partial_fix", "bc_regions",
                 "single_voxel", "one_link", "collide_creature", "ref_zoo_basic", "ref_example", "ref_signaling",
                 "ref_memleaking", "ref_circle_push", "ref_target_only"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return dict(z), str(z["vxa"]), ast.literal_eval(str(z["ext"]))


@pytest.fixture(scope="session")
def ctx():
    import gpuvoxels_gb300 as g
    c = g.Context(0, 8 << 30)
    yield c
    c.close()
