"""Confocal line scan of the bound dye (test infrastructure only).

numpy restatement of the reference's post-processing tool
linescan/main.cpp:88-225: for every sample point c_i on a line along one
axis, F_i = sum_j V0_j [CaDye]_j N(r_ij; sigma) over the cells whose
centroid lies within |r_ij|^2 < r_thresh (r_thresh = 1, :194), plus
padding voxels at the resting fluorescence f0_pad outside the mesh
(AddPointGrid, :114-128 and :275-313).  The cell sums are returned as a
weight matrix W (samples x elements, in the element numbering of `order`)
and the padding sums as pad, so that F = pad + W @ dye.

Only tests/ and bench.py's reference leg use this module, to compare with.
"""
import numpy as np


# the tool's constant (linescan/parameters.h: PI = 3.14159, PDF3D_ALPHA)
PI_TOOL = 3.14159


def _pdf3(r, sx, sy, sz):
    """normpdf3d of linescan/parameters.h: the product of three centred
    normals, normalised with the tool's PI."""
    alpha = 1.0 / (2 * PI_TOOL) ** 1.5
    return alpha * np.exp(-0.5 * (r[..., 0] ** 2 / sx ** 2 + r[..., 1] ** 2 / sy ** 2 +
                                  r[..., 2] ** 2 / sz ** 2)) / (sx * sy * sz)


def _pads(d):
    out = []
    D, a0, a1, h = d["domain"], d["pad_min"], d["pad_max"], d["pad_res"]
    if h <= 0:
        return np.zeros((0, 4))

    def grid3(x0, x1, y0, y1, z0, z1):
        dx, dy, dz = (h if x1 > x0 else -h), (h if y1 > y0 else -h), (h if z1 > z0 else -h)
        for i in range(int((x1 - x0) / dx)):
            for j in range(int((y1 - y0) / dy)):
                for k in range(int((z1 - z0) / dz)):
                    out.append((x0 + i * dx + 0.5 * dx, y0 + j * dy + 0.5 * dy,
                                z0 + k * dz + 0.5 * dz, abs(dx * dy * dz)))
    grid3(a0, a1, a0, a1, D[5], a1)
    grid3(a0, a1, a0, a1, D[4], a0)
    grid3(D[0], a0, a0, a1, D[4], D[5])
    grid3(D[1], a1, a0, a1, D[4], D[5])
    grid3(D[0], D[1], D[2], a0, D[4], D[5])
    grid3(D[0], D[1], D[3], a1, D[4], D[5])
    return np.array(out).reshape(-1, 4)


def cells(mesh_base, order):
    """Cell centroids and volumes from the .node / .ele files
    (linescan/main.cpp:95-109: the mean of the four nodes, |det|/6), in the
    numbering where element k is file element order[k]."""
    nodes = np.loadtxt(mesh_base + ".node", skiprows=1)[:, 1:4]
    ele = np.loadtxt(mesh_base + ".ele", skiprows=1, dtype=np.int64)[:, 1:5] - 1
    c = nodes[ele[np.asarray(order)]]
    v1, v2, v3 = c[:, 0] - c[:, 3], c[:, 1] - c[:, 3], c[:, 2] - c[:, 3]
    vol = np.abs(np.einsum("ij,ij->i", v1, np.cross(v2, v3)) / 6.0)
    return (c[:, 0] + c[:, 1] + c[:, 2] + c[:, 3]) / 4.0, vol


def weights(mesh_base, order, d, V0=None):
    """(W[n_samples][N], pad[n_samples]) for the line-scan description d
    (keys of srs_linescan_desc: axis, offset1, offset2, x_min, x_max, res,
    var_x/y/z, r_thresh, f0_pad, pad_res, pad_min, pad_max, domain).  The
    cell volumes are the tool's (from the nodes) unless V0 is given."""
    cen, vol = cells(mesh_base, order)
    V0 = vol if V0 is None else np.asarray(V0)
    axis = int(d.get("axis", 0))
    if axis == 2:
        sx, sy, sz = np.sqrt(d["var_z"]), np.sqrt(d["var_x"]), np.sqrt(d["var_y"])
    else:
        sx, sy, sz = np.sqrt(d["var_x"]), np.sqrt(d["var_y"]), np.sqrt(d["var_z"])
    pads = _pads(d)
    ns = int((d["x_max"] - d["x_min"]) / d["res"])
    W = np.zeros((ns, len(cen)))
    pad = np.zeros(ns)
    for i in range(ns):
        xi = d["x_min"] + i * d["res"]
        c = [[xi, d["offset1"], d["offset2"]], [d["offset1"], xi, d["offset2"]],
             [d["offset1"], d["offset2"], xi]][axis]
        c = np.array(c)
        r = cen - c
        m = (r ** 2).sum(1) < d["r_thresh"]
        W[i, m] = V0[m] * _pdf3(r[m], sx, sy, sz)
        if len(pads):
            rp = pads[:, :3] - c
            mp = (rp ** 2).sum(1) < d["r_thresh"]
            pad[i] = (pads[mp, 3] * d["f0_pad"] * _pdf3(rp[mp], sx, sy, sz)).sum()
    return W, pad


def to_csr(W):
    """Row pointers, columns and values of a dense weight matrix."""
    ptr = np.zeros(W.shape[0] + 1, np.int32)
    cols, vals = [], []
    for i in range(W.shape[0]):
        nz = np.nonzero(W[i])[0]
        cols.append(nz)
        vals.append(W[i, nz])
        ptr[i + 1] = ptr[i] + len(nz)
    return ptr, np.concatenate(cols).astype(np.int32), np.concatenate(vals).astype(np.float64)
