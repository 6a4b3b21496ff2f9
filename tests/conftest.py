import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "app-kilonova_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle_lib():
    import knc_oracle
    knc_oracle.build()
    return knc_oracle.load()


@pytest.fixture(scope="session")
def trained_mlp():
    """Learned c2p guess trained on the device once per session (1M solver
    pairs over W in [1, 1000], p/rho in [1e-6, 1e2])."""
    from knc import learned
    pairs = learned.generate_pairs(4.0 / 3.0, 1_000_000, seed=21)
    w, loss = learned.train(pairs, steps=3000, seed=21)
    return w, loss
