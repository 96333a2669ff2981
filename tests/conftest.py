import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def native_lib():
    """Build (if stale) and load the CUDA library."""
    from btrc_gb300 import _build
    _build.build()
    import btrc_gb300
    return btrc_gb300.load_library()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    return oracle.lib()


@pytest.fixture(scope="session")
def scene_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("scenes")
    os.environ.setdefault("BTRC_SCENE_CACHE", str(d))
    return d


@pytest.fixture(scope="session")
def gpu_ctx(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import btrc_gb300
    ctx = btrc_gb300.Context(0)
    yield ctx
    ctx.close()
