import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the library's kernels")


@pytest.fixture(scope="session")
def built():
    """Build libhc3d.so (sm_103a) and the CPU oracle once per session."""
    from hochunk3d_gb300.build import build_library, build_oracle

    build_library()
    build_oracle()
    return True


@pytest.fixture(scope="session")
def fixtures_dir(tmp_path_factory, built):
    return tmp_path_factory.mktemp("hc3d_models")


@pytest.fixture(scope="session")
def model_factory(fixtures_dir):
    from tests.helpers import make_model

    cache = {}

    def get(name, warm=True, **over):
        key = (name, warm, tuple(sorted(over.items())))
        if key not in cache:
            cache[key] = make_model(fixtures_dir / f"{name}_{len(cache)}", name, warm=warm, **over)
        return cache[key]

    return get
