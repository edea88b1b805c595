import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "parallelstencil.jl_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libps_b200.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def golden():
    import json

    here = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(here, "golden.json")) as fh:
        meta = json.load(fh)
    arrays = dict(np.load(os.path.join(here, "golden.npz")))
    return meta, arrays


@pytest.fixture(scope="session")
def ps():
    """The initialised GB300 package (GPU tests only)."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ps_gb300._build import build

    build()
    import ps_gb300

    if not ps_gb300.is_initialized():
        ps_gb300.init_parallel_stencil(ps_gb300.GB300, "Float64", 3)
    return ps_gb300


DT = {"f64": np.float64, "f32": np.float32}
