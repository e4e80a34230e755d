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
    """numpy restatement of linescan/main.cpp:160-225 for an x-axis scan:
    dense weights W[i][j] = V0_j N(r_ij) (|r_ij|^2 < r_thresh, reference
    numbering) and the padding-voxel sums pad[i], so F = pad + W @ dye."""
    nodes = np.loadtxt(mesh + ".node", skiprows=1)[:, 1:4]
    ele = np.loadtxt(mesh + ".ele", skiprows=1, dtype=np.int64)[:, 1:5] - 1
    el = grid.elements()
    cen = nodes[ele[el["order"]]].mean(axis=1)      # reference numbering
    V0 = el["V0"]
    sx, sy, sz = np.sqrt(d["var_x"]), np.sqrt(d["var_y"]), np.sqrt(d["var_z"])
    alpha = 1.0 / (2 * np.pi) ** 1.5
    pdf = lambda r: alpha * np.exp(-0.5 * (r[..., 0] ** 2 / sx ** 2 + r[..., 1] ** 2 / sy ** 2 +  # noqa
                                           r[..., 2] ** 2 / sz ** 2)) / (sx * sy * sz)
    pads = []
    D, a0, a1, h = d["domain"], d["pad_min"], d["pad_max"], d["pad_res"]

    def grid3(x0, x1, y0, y1, z0, z1):
        dx, dy, dz = (h if x1 > x0 else -h), (h if y1 > y0 else -h), (h if z1 > z0 else -h)
        for i in range(int((x1 - x0) / dx)):
            for j in range(int((y1 - y0) / dy)):
                for k in range(int((z1 - z0) / dz)):
                    pads.append((x0 + i * dx + 0.5 * dx, y0 + j * dy + 0.5 * dy,
                                 z0 + k * dz + 0.5 * dz, abs(dx * dy * dz)))
    grid3(a0, a1, a0, a1, D[5], a1)
    grid3(a0, a1, a0, a1, D[4], a0)
    grid3(D[0], a0, a0, a1, D[4], D[5])
    grid3(D[1], a1, a0, a1, D[4], D[5])
    grid3(D[0], D[1], D[2], a0, D[4], D[5])
    grid3(D[0], D[1], D[3], a1, D[4], D[5])
    pads = np.array(pads)
    ns = int((d["x_max"] - d["x_min"]) / d["res"])
    W = np.zeros((ns, grid.n_ele))
    pad = np.zeros(ns)
    for i in range(ns):
        c = np.array([d["x_min"] + i * d["res"], d["offset1"], d["offset2"]])
        r = cen - c
        m = (r ** 2).sum(1) < d["r_thresh"]
        rp = pads[:, :3] - c
        mp = (rp ** 2).sum(1) < d["r_thresh"]
        pad[i] = (pads[mp, 3] * d["f0_pad"] * pdf(rp[mp])).sum()
        W[i, m] = V0[m] * pdf(r[m])
    return W, pad


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
