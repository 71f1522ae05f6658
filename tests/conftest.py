import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
PKG = ROOT / "butterfly-osm_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session")
def built():
    """Native libraries built (idempotent, mtime-checked)."""
    import build
    from oracle.build import build_oracle
    build.build_all()
    build_oracle()
    return True


@pytest.fixture(scope="session")
def kats():
    import json
    return json.loads((ROOT / "tests" / "golden" / "reference_kats.json").read_text())


@pytest.fixture(scope="session")
def grid100(built):
    import cchbuild
    return cchbuild.build_synthetic(cchbuild.KIND_GRID, 100, 100, seed=42)


@pytest.fixture(scope="session")
def country_small(built):
    import cchbuild
    return cchbuild.build_synthetic(cchbuild.KIND_COUNTRY, 200, 250, seed=7)
