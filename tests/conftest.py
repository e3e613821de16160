import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build_oracle, pyoracle
    build_oracle.build_oracle()
    return pyoracle.load()


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library (built here if missing: nvcc cross-compiles)."""
    from chm_gb300 import build, capi
    build.build_cuda()
    return capi.load()


def load_golden_mesh(name: str):
    import numpy as np
    from chm_gb300 import synth
    d = np.load(GOLDEN / name)
    return synth.mesh_from_arrays(d["vertex"], d["elem"], d["neigh"], area=d["area"]), d
