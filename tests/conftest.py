import contextlib
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
def built():
    """libfbp.so and the oracle libraries, built in-tree if missing."""
    from fasterbackprojection_gb300 import _build

    _build.build()
    _build.build_oracle()
    return True


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def ctx(built, cuda):
    from fasterbackprojection_gb300 import Context

    c = Context(0)
    yield c
    c.close()


def rel_l2(a, b) -> float:
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


@contextlib.contextmanager
def reference_weights(ctx):
    """Run the gathers with the reference's own reciprocal per pair (bitwise
    single-scan parity) and restore the context's weight mode afterwards."""
    from fasterbackprojection_gb300 import FBP_WEIGHTS_REFERENCE

    old = ctx.weight_mode
    ctx.weight_mode = FBP_WEIGHTS_REFERENCE
    try:
        yield ctx
    finally:
        ctx.weight_mode = old
