"""Shared pytest configuration: the ``gpu`` marker and import paths."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in (ROOT, os.path.join(ROOT, "oracle")):
    if sub not in sys.path:
        sys.path.insert(0, sub)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU oracle case")


@pytest.fixture(scope="session")
def oracle():
    import tnr_oracle
    return tnr_oracle


def _flat_spectrum_tensor(d, step, seed):
    """A d^4 tensor whose ((1,2),(3,4)) matricization has sigma_i = 1 - step * i for i < 100 and a
    geometric tail below: at truncrank(24) the subspace iteration's oversampled rank (72) sits in
    the flat part, so the gap at the cut (step, relative) is far too small to iterate on."""
    import numpy as np
    rng = np.random.default_rng(seed)
    n = d * d
    U, _ = np.linalg.qr(rng.standard_normal((n, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    i = np.arange(n)
    s = np.where(i < 100, 1.0 - step * i, (1.0 - step * 100) * 0.5 ** (i - 99))
    return ((U * s) @ V.T).reshape(d, d, d, d)


@pytest.fixture(scope="session")
def flat_spectrum_tensor():
    return _flat_spectrum_tensor
