import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_MESH = os.path.join(GOLDEN, "mesh", "dyad")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103a GPU (GB300)")


def _build():
    import __graft_entry__ as g
    g.build()


@pytest.fixture(scope="session")
def built():
    _build()
    return True


@pytest.fixture(scope="session")
def srs(built):
    import srs_gb300
    return srs_gb300


@pytest.fixture(scope="session")
def oracle(built):
    from oracle import Oracle
    return Oracle()


def params_from_golden(srs, name):
    d = np.load(os.path.join(GOLDEN, "ref_run_%s.npz" % name))
    p = srs.default_parameters()
    for i, v in enumerate(d["ints"]):
        p.ints[i] = int(v)
    for i, v in enumerate(d["reals"]):
        p.reals[i] = float(v)
    return p, d


@pytest.fixture(scope="session")
def box_mesh(srs, tmp_path_factory):
    """The 10,368-element config mesh (12^3 hexahedra, 49 RyRs, 7 LCCs)."""
    base = str(tmp_path_factory.mktemp("box12") / "box12")
    rep = srs.write_box_mesh(base)
    return base, rep
