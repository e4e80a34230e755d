"""Device line scan against a numpy restatement of linescan/main.cpp:160-225."""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, params_from_golden

pytestmark = pytest.mark.gpu

DESC = dict(axis=0, offset1=0.0, offset2=0.01, x_min=-0.2, x_max=0.2, res=0.02, var_x=0.0289,
            var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=4.1667, pad_res=0.1, pad_min=-0.6,
            pad_max=0.6, domain=(-0.2, 0.2, -0.2, 0.2, 0.0, 0.4))


def restated(srs, grid, states_by_r, d=DESC):
    nodes = np.loadtxt(GOLDEN_MESH + ".node", skiprows=1)[:, 1:4]
    ele = np.loadtxt(GOLDEN_MESH + ".ele", skiprows=1, dtype=np.int64)[:, 1:5] - 1
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
    N = grid.n_ele
    out = np.zeros((len(states_by_r), ns))
    for i in range(ns):
        c = np.array([d["x_min"] + i * d["res"], d["offset1"], d["offset2"]])
        r = cen - c
        m = (r ** 2).sum(1) < d["r_thresh"]
        rp = pads[:, :3] - c
        mp = (rp ** 2).sum(1) < d["r_thresh"]
        padsum = (pads[mp, 3] * d["f0_pad"] * pdf(rp[mp])).sum()
        for k, S in enumerate(states_by_r):
            out[k, i] = padsum + (V0[m] * pdf(r[m]) * S[5 * N:6 * N][m]).sum()
    return out


@pytest.mark.parametrize("prec,eng", [(64, 0), (32, 0), (32, 1)])
def test_linescan_matches_restatement(srs, prec, eng):
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, 3, prec, eng, seeds=[1, 2, 3])
    ns = sim.linescan_setup(**DESC)
    F0, rest = sim.linescan()
    want0 = restated(srs, g, [g.initial_states(p)])
    assert np.allclose(rest, want0[0], rtol=1e-12, atol=0)
    assert np.allclose(F0, want0[0][None, :], rtol=1e-6 if prec == 32 else 1e-12)
    sim.explicit_step(2000)
    F, _ = sim.linescan()
    want = restated(srs, g, [sim.get_state(r)["states"] for r in range(3)])
    assert F.shape == (3, ns)
    assert np.allclose(F, want, rtol=1e-12, atol=0)
    assert (F > F0).any()  # the open RyR raised the bound dye somewhere on the line
