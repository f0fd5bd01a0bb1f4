import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def built():
    """Library and oracle built in-tree (no-op when up to date)."""
    from toucangpurt_gb300 import build

    build.build()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def small_design(tmp_path_factory, built):
    from toucangpurt_gb300 import sim, workloads

    d = tmp_path_factory.mktemp("small")
    dp, sp = d / "design.bin", d / "symbols.bin"
    info = sim.generate(dp, sp, **workloads.design_config("small"))
    return dp, sp, info
