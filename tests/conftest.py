import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
HERE = Path(__file__).resolve().parent
if str(HERE) not in sys.path:
    sys.path.insert(0, str(HERE))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session", autouse=True)
def _oracle_threads():
    os.environ.setdefault("OMP_NUM_THREADS", str(min(8, os.cpu_count() or 1)))
    yield


@pytest.fixture(autouse=True)
def _initialise_on_the_oracle_without_a_gpu(monkeypatch):
    """Without a GPU, SEIR_ABM's device initialisation (init.fill) is done
    by the oracle's restatement of it, which makes the same draws: the tests
    that build sims on the CPU then see the table the device would build."""
    import torch

    if not torch.cuda.is_available():
        from laser_polio_gb300 import init as dinit
        from oracle_backend import oracle_fill

        monkeypatch.setattr(dinit, "fill", oracle_fill)
    yield
