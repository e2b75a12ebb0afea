"""Shared test set-up: the `gpu` marker, paths to the oracle and fixtures."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
FIXTURES = os.path.join(ROOT, "tests", "fixtures")
for p in (ROOT, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def fixture(name: str) -> str:
    return os.path.join(FIXTURES, name)


def golden(name: str) -> dict:
    """A known answer of the reference's own tests (tests/golden/reference_known_answers.json)."""
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_known_answers.json")) as f:
        return json.load(f)[name]


@pytest.fixture(scope="session")
def has_gpu():
    import torch
    return torch.cuda.is_available()
