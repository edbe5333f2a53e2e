"""Shared test set-up: import paths, the `gpu` marker, and fixtures for the library and oracle."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "project-marshmallow_gb300"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the library's kernels")


@pytest.fixture(scope="session")
def mmlib():
    import marshmallow
    return marshmallow.lib.load()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("the gpu tests need a CUDA device")
    return torch


@pytest.fixture(scope="session")
def oracle_textures(orc):
    """Seed-0 textures from the CPU generators (the reference set the GPU generators must match)."""
    import marshmallow.lib as L
    return {
        "low_res": orc.noise(L.NOISE_LOWRES, 0, 128, 128, 128, 4),
        "hi_res": orc.noise(L.NOISE_HIRES, 0, 32, 32, 32, 4),
        "curl": orc.noise(L.NOISE_CURL2D, 0, 128, 128, 1, 2)[0],
        "weather": orc.noise(L.NOISE_WEATHER, 0, 512, 512, 1, 4)[0],
    }
