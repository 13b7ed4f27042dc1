import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "fast-rbd-gradients_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "iiwa_golden.npz")

# The reference tree, read by the tests that regenerate fixtures from it
# (they skip where it is absent, e.g. on GPU hosts): FRG_REFERENCE_DIR, else
# its path in the build container.
REFERENCE_DIR = os.environ.get("FRG_REFERENCE_DIR", "/root/reference")

# Parity bar: max Frobenius-relative error per output matrix and knot against
# the FP64 oracle / the reference's own FP64 outputs.
TOL = 1e-4


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def built_lib():
    from frg import build
    return build.build()


def max_err(a, b):
    import frg_oracle
    return float(frg_oracle.frob_rel(a, b).max())
