import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "sliding-puzzle_gb300")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (PKG, os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden():
    return load_golden


@pytest.fixture(scope="session")
def pdb24_tables():
    import oracle
    return oracle.tables(5)


@pytest.fixture(scope="session")
def pdb15_tables():
    import oracle
    return oracle.tables(4)


_solvers = {}


@pytest.fixture(scope="session")
def gpu_solver():
    """Session-cached GPU solvers keyed by (width, heuristic); PDBs built on the GPU once."""
    import slide

    def get(width, heuristic):
        key = (width, heuristic)
        if key not in _solvers:
            s = slide.Solver(width, heuristic)
            if heuristic == "pdb":
                s.build_pdb()
            _solvers[key] = s
        s = _solvers[key]
        d = slide.default_config()
        s.set_config(**{f: getattr(d, f) for f, _ in slide.SpConfig._fields_})
        return s

    yield get
    for s in _solvers.values():
        s.close()
    _solvers.clear()
