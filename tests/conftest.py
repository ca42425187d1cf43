import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
PKG = ROOT / "fluid-simulation-3d_gb300"
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def built_lib():
    """Compile libsph_gb300.so (cached by mtime) and return its path."""
    import build_lib
    return build_lib.build()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fluidsim
    return fluidsim.load()


def load_fixture(name):
    d = np.load(GOLDEN / name, allow_pickle=False)
    return {k: d[k] for k in d.files}


def fixture_params(fx):
    import json
    from fluidsim.scenes import SimParams
    p = json.loads(str(fx["params"]))
    p["bound"] = tuple(p["bound"])
    return SimParams(**p)


def substep_fixtures():
    return sorted(p.name for p in GOLDEN.glob("substep_*.npz")
                  if "sample" not in p.name)
