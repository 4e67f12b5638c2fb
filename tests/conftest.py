import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


def has_gpu():
    try:
        from sem2dpack_gb300 import _lib
        return _lib.lib().sem2d_gpu_device_count() > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


def watch_launches(nsteps, members=1, every=100):
    """Launches of the max|v|, max|d| check in a run of nsteps steps from
    step 0 (one kernel every `every` steps, the default info_every; a batch
    checks all its members in that one launch)."""
    return nsteps // every


def example_deck(golden, name, folder):
    """ParDeck of the example deck `name` of the fixtures, its tables
    (file=...) written to `folder` first."""
    from sem2dpack_gb300.parinp import deck_from_parinp
    prefix = "exfile_%s__" % name
    for k in golden.files:
        if k.startswith(prefix):
            with open(os.path.join(str(folder), k[len(prefix):]), "w") as f:
                f.write(str(golden[k]))
    return deck_from_parinp(str(golden["parinp_" + name]), base=str(folder))
