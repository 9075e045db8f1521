import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


GOLDEN = os.path.join(TESTS, "golden")


def golden_cases():
    import json
    with open(os.path.join(GOLDEN, "index.json")) as f:
        return json.load(f)


def golden_input(name):
    with open(os.path.join(GOLDEN, name + ".input.txt"), "rb") as f:
        return f.read()


def golden_expected(name):
    with open(os.path.join(GOLDEN, name + ".expected.txt")) as f:
        return f.read()
