import os
import shutil
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


# Files the tests write (host builds of lowered fields, fuzz modules, OBJ
# files) stay inside the repository, in a git-ignored build folder that each
# run starts empty and removes when it ends.
SCRATCH = ROOT / "_build" / "tests"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    if not hasattr(config, "workerinput"):  # the controlling process only
        shutil.rmtree(SCRATCH, ignore_errors=True)
    SCRATCH.mkdir(parents=True, exist_ok=True)
    if not config.option.basetemp:
        config.option.basetemp = str(SCRATCH / ("pytest-" + getattr(config, "workerinput", {}).get("workerid", "main")))


def pytest_unconfigure(config):
    if not hasattr(config, "workerinput"):
        shutil.rmtree(SCRATCH, ignore_errors=True)


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def lib():
    from linon_gb300 import _abi
    return _abi.load()


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def engine():
    if not _has_gpu():
        pytest.fail("GPU test run without a CUDA device")
    os.environ.setdefault("LINON_CACHE_DIR", str(ROOT / "_build_cache"))
    Path(os.environ["LINON_CACHE_DIR"]).mkdir(exist_ok=True)
    from linon_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()
