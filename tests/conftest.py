import gzip
import os
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
PKG = os.path.join(ROOT, "bachelor-thesis_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbmm.so")


def golden_cases():
    names = sorted(f[:-6] for f in os.listdir(GOLDEN) if f.endswith(".in.gz"))
    return names


def load_golden(name):
    with gzip.open(os.path.join(GOLDEN, name + ".in.gz"), "rt") as f:
        text = f.read()
    with gzip.open(os.path.join(GOLDEN, name + ".out.gz"), "rt") as f:
        out = f.read()
    return text, out


@pytest.fixture(scope="session")
def built_lib():
    import build as gbuild
    gbuild.build()
    import gbmm
    return gbmm.lib()


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    if not os.path.exists(orc.LIB_PATH):
        orc.build(with_ref=False)
    return orc
