import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA kernels)")


# The reference tree, for the CPU tests that read or compile it (named by
# LUSTRINE_REFERENCE_DIR; those tests skip when it is unset).
REF = os.environ.get("LUSTRINE_REFERENCE_DIR") or ""
HAVE_REF = bool(REF) and os.path.isdir(os.path.join(REF, "src"))


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name)))


def csr_sets(off, flat):
    """Neighbour lists of a CSR fixture as a list of sorted arrays."""
    return [np.sort(flat[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def rows_sets(cnt, idx):
    return [np.sort(idx[i, :cnt[i]]) for i in range(len(cnt))]


def phys_params(p):
    """The physical parameters of the golden fixtures (tests/golden/make_golden.py)."""
    p.rest_density = 1.0
    p.mass = 1.0
    p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, -9.81, 0.0
    p.relaxation_epsilon = 10.0
    p.s_corr_dq = 0.2
    p.s_corr_k = 0.1
    p.s_corr_n = 4.0
    return p


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.build()
    return O
