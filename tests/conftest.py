import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_CASES = ["m5p10_4_4_0", "cfg1_4_4_0", "m5p20_4_4_2", "m5p16_4_6_3", "cube6_8_3_0", "m9p24_8_4_2m"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Build the product library and the oracle once per session."""
    from mpk_gb300 import build as B
    B.build()
    from oracle import oracle as O
    O.build()
    return True


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def golden_matrix(name):
    """The loop matrix (with diagonal) each golden case was generated from."""
    import mpk_gb300 as M
    if name.startswith("cube"):
        return M.Csr.stencil("cube", int(name[4:].split("_")[0]))
    if name.startswith("m9p"):  # gen2's 9-point mesh
        return M.Csr.stencil("m9p", int(name[3:].split("_")[0]))
    size = {"m5p10": 10, "cfg1": 100, "m5p20": 20, "m5p16": 16}[name.split("_")[0]]
    return M.Csr.laplacian(size, size, 1, diag=4.0, off=-1.0)


@pytest.fixture
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu-marked test run without a CUDA device")
    return torch.device("cuda:0")
