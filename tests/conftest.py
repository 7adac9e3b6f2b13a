import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session")
def golden_dir():
    return ROOT / "tests" / "golden"


# ---------------------------------------------------------------- seeded configs shared by the GPU tests
def _synth():
    from livespikesorter_gb300 import synth
    return synth


def _make_dataset(cfg, d):
    from lss_testutil import make_dataset
    return make_dataset(cfg, d)


@pytest.fixture(scope="session")
def cfg_small(tmp_path_factory):
    """96 channels, 64 units, one 60000-sample batch (+2*61)."""
    return _make_dataset(_synth().config_small(seed=11), tmp_path_factory.mktemp("cfg1"))


@pytest.fixture(scope="session")
def cfg_stream(tmp_path_factory):
    """384 channels, 500 templates, 6 batches of 1500 new samples with a rigid drift."""
    cfg = _synth().SynthConfig(n_chan=384, n_units=500, n_samples=6 * 1500 + 300, drift_um=20.0,
                               whiten_batch=3000, whiten_batches=3, seed=5)
    return _make_dataset(cfg, tmp_path_factory.mktemp("cfg2"))


@pytest.fixture(scope="session")
def cfg_dense(tmp_path_factory):
    """The dense shape at oracle-friendly size: 128 channels, 200 units firing at 30 Hz with 30 %
    of the spikes forced to overlap a neighbour unit's within 1 ms, one 12000-sample batch."""
    cfg = _synth().SynthConfig(n_chan=128, n_units=200, n_samples=12000 + 122, rate_hz=30.0, overlap_frac=0.3,
                               whiten_batch=4000, whiten_batches=3, seed=21)
    return _make_dataset(cfg, tmp_path_factory.mktemp("cfg3s"))
