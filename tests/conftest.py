"""Shared fixtures.  `-m gpu` tests run the engine on cuda:0 through the C ABI;
everything else runs on the CPU (oracle, golden vectors, host logic, ABI
exports)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__  # noqa: E402
from oracle import pyoracle  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine on cuda:0")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def oracle():
    return pyoracle.get()


@pytest.fixture(scope="session")
def pkg():
    """The engine's Python binding; builds the library if needed."""
    mod = __graft_entry__.load_package()
    if not os.path.exists(mod.LIB_PATH):
        __graft_entry__.build()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def P():
    return pyoracle.default_params()


@pytest.fixture(scope="session")
def keys(oracle, P):
    """Keys of the default set from seed 0 (oracle keygen)."""
    lwe, tlwe, ks, bk = oracle.gate_keyset(P, [0])
    bk_fft = oracle.bk_to_fft(P, bk)
    return {"lwe": lwe, "tlwe": tlwe, "ks": ks, "bk": bk, "bk_fft": bk_fft}


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # Work on a non-default stream: torch's copies and the engine's launches
    # (given this stream's handle) are then ordered on one stream.  A NULL
    # handle would send the engine's work to its own stream instead.
    torch.cuda.set_stream(torch.cuda.Stream())
    return torch


@pytest.fixture(scope="session")
def engine(pkg, keys, torch_cuda):
    """Engine on cuda:0 with the seed-0 keys uploaded in both forms."""
    eng = pkg.Engine(pkg.default_params(), device=0)
    eng.upload_bootstrapping_key(keys["bk"])
    eng.upload_keyswitch_key(keys["ks"])
    yield eng
    eng.close()

