import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def scene_dir(tmp_path_factory):
    """Seeded procedural jobs shared by the tests (generated once per session)."""
    from hastyrenderer_gb300 import scenes
    base = tmp_path_factory.mktemp("scenes")
    jobs = {
        "cornell": scenes.cornell_box(str(base / "cornell"), seed=0, width=32, height=32, spp=4,
                                      max_depth=8, roulette_start_depth=3),
        "field": scenes.sphere_field(str(base / "field"), seed=1, n_spheres=12, subdiv=1, width=24, height=24, spp=4,
                                     env_size=(64, 32), vary_glass_ior=True, box=4.0),
        "room": scenes.textured_room(str(base / "room"), seed=2, width=32, height=24, spp=4),
        "room_nomis": scenes.textured_room(str(base / "room_nomis"), seed=3, width=32, height=24, spp=4, use_mis=False),
    }
    return jobs
