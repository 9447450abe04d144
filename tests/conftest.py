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


def reference_checkout() -> Path | None:
    """A Boundary Lab source checkout, for the CPU tests that import or read the
    reference's own files: the directory named by BOUNDARY_LAB_REFERENCE, else a
    ``reference`` directory beside this repository.  None when neither exists."""
    import os

    for cand in (os.environ.get("BOUNDARY_LAB_REFERENCE"), ROOT.parent / "reference"):
        if cand and (Path(cand) / "src" / "blab").is_dir():
            return Path(cand)
    return None
