import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "gbd-pcg_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import build_oracle
    build_oracle.build()
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def gb():
    """The product library (built if missing); GPU tests only."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gbdpcg_build", os.path.join(ROOT, "gbd-pcg_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import gbdpcg
    gbdpcg.lib()
    return gbdpcg


@pytest.fixture(scope="session")
def handle(gb):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    h = gb.Handle(0)
    yield h
    h.close()
