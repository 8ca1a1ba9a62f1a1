import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a library)")


@pytest.fixture(scope="session")
def cornell():
    from sparkle_gb300 import scenes
    return scenes.cornell_box(0)


@pytest.fixture(scope="session")
def small_terrain():
    """Stress-scene generator at reduced size: 64x64 grid (8192 tris) + 8 level-2 icospheres."""
    from sparkle_gb300 import scenes
    return scenes.terrain_spheres(seed=3, grid=64, num_spheres=8, sphere_level=2, size=40.0, cube_size=16)
