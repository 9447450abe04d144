import importlib
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pkg_module(name: str = ""):
    """Import the package (its directory name has a hyphen) or one of its submodules."""
    return importlib.import_module("boundary-lab_gb300" + (("." + name) if name else ""))


def cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def native():
    """The CUDA library binding; GPU tests fail loudly if it is missing."""
    mod = pkg_module("native")
    mod.load()
    return mod


@pytest.fixture(scope="session")
def gpu_ctx(native):
    ctx = native.Context(0)
    yield ctx
    ctx.close()
