import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library through its C ABI")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build, pyoracle

    build.build()
    return pyoracle


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library, built if needed; GPU tests fail loudly without it."""
    import torch

    from pelec_gb300 import build, mol

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    build.build()
    return mol


def rel_maxnorm(a, b):
    """Per-component max|a-b| / max|b| (components on axis 0); 0/0 -> 0."""
    import numpy as np

    out = []
    for n in range(b.shape[0]):
        den = np.abs(b[n]).max()
        num = np.abs(a[n] - b[n]).max()
        out.append(0.0 if num == 0 else (num / den if den > 0 else float("inf")))
    return np.array(out)


def divergence_scale(F, vol):
    """Per component, the sum over cells of |each face-flux term| / V that
    enters the divergence (each face feeds two cells): the scale against
    which the round-off of a domain total of the RHS is measured.  The
    reference sums the six face terms left to right (Diffterm.H:475-481),
    so the total of a periodic RHS is exact only to round-off of the large
    uniform terms (the pressure in the momentum fluxes), not of the RHS."""
    import numpy as np

    return np.array([2.0 * sum(np.abs(np.asarray(F[d][n])).sum() for d in range(3)) / vol
                     for n in range(np.asarray(F[0]).shape[0])])
