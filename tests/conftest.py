import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
GOLDEN_MESH = os.path.join(GOLDEN, "mesh", "dyad")


# line scan along x through the golden mesh (PSF of linescan/DefaultScan.xml)
LINESCAN_DESC = dict(axis=0, offset1=0.0, offset2=0.01, x_min=-0.2, x_max=0.2, res=0.02,
                     var_x=0.0289, var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=4.1667,
                     pad_res=0.1, pad_min=-0.6, pad_max=0.6, domain=(-0.2, 0.2, -0.2, 0.2, 0.0, 0.4))


def linescan_weights(grid, d=LINESCAN_DESC, mesh=GOLDEN_MESH):
    """numpy restatement of linescan/main.cpp:160-225 (oracle/linescan.py):
    dense weights W[i][j] = V0_j N(r_ij) (|r_ij|^2 < r_thresh, reference
    numbering) and the padding-voxel sums pad[i], so F = pad + W @ dye."""
    from oracle import linescan
    el = grid.elements()
    return linescan.weights(mesh, el["order"], d)


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
