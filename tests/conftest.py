"""pytest configuration: the ``gpu`` marker and shared paths/fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "fpga-litho-accel_gb300")
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) and the built CUDA library")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="session")
def golden_optics():
    """The optics of the reference's TCC golden (tb_calc_tcc_correct.cpp:22-34)."""
    from oracle import np_ref as R
    src = R.normalize_source(R.create_annular(101, 0.6, 0.9))
    sig = R.get_outer_sigma(src)
    nx = R.optics_nx(0.8, 512, sig, 193.0)
    tcc = R.calc_tcc(src, sig, 193.0, 0.8, 0.2, 512, 512, nx, nx)
    return dict(src=src, sigma=sig, Nx=nx, tcc=tcc, L=512, NA=0.8, wavelength=193.0, defocus=0.2)
