import lzma
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300) and the built engine")


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (built on first use)."""
    from oracle import pyoracle
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def golden_deb(tmp_path_factory):
    """Decompressed shipped example inputs: {'Gamma': path, 'UH3': path}."""
    d = tmp_path_factory.mktemp("golden")
    out = {}
    for key, name in (("Gamma", "GammaAl2O3_10nm.deb"), ("UH3", "UH3_7nm.deb")):
        p = str(d / name)
        with open(os.path.join(GOLDEN, name + ".xz"), "rb") as f:
            raw = lzma.decompress(f.read())
        with open(p, "wb") as f:
            f.write(raw)
        out[key] = p
    return out


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def engine():
    """One engine context on cuda:0 for the GPU tests."""
    import __graft_entry__
    __graft_entry__.build()
    from cudebye_gb300 import Engine
    e = Engine(0)
    yield e
    e.close()
