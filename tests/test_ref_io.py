"""The product's input/output path against the reference's own code (CPU).

oracle/_ref/libsrsref_io.so is the reference's cpu/InitFuncs.cpp and
cpu/OutputFuncs.cpp compiled where they lie (oracle/build_ref.sh, with a
single-rank MPI stand-in and the Xerces DOM subset of oracle/shim/), and
oracle/_ref/linescan its line-scan tool linescan/main.cpp.  They exist only
where the reference sources are present; elsewhere these tests skip.

  ReadParameters            all shipped parameter files: ints, reals, chars equal
  ReadGrid + assembly       aij, nij, boundary rates, element and channel
                            arrays, equilibrium states: bit-identical, both
                            meshes, both boundary modes
  OpenRandomRyR             the oracle's restated initial opening draws the
                            same RyR for the same rand() stream
  WriteToGridFiles          srs_grid_write_vtk writes the same bytes
  linescan tool             the line-scan restatement (oracle/linescan.py)
                            gives the tool's output (its %g precision)
"""
import glob
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_MESH, ROOT

REF_ROOT = os.environ.get("SRS_REFERENCE_ROOT", "/root/reference")
REF_IO = os.path.join(ROOT, "oracle", "_ref", "libsrsref_io.so")
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "cpu")),
                                reason="reference sources absent")


@pytest.fixture(scope="module")
def refio(built):
    from oracle import RefIO
    return RefIO()


def test_read_parameters_matches_reference_on_every_shipped_file(srs, refio):
    files = sorted(glob.glob(os.path.join(REF_ROOT, "param", "**", "*.xml"), recursive=True))
    assert len(files) >= 100
    for f in files:
        ints, reals, chars = refio.read_parameters(f)
        p = srs.read_parameters(f)
        assert np.array_equal(np.array(p.ints[:]), ints), f
        assert np.array_equal(np.array(p.reals[:]), reals), f
        assert [bytes(p.chars[i]).split(b"\0")[0] for i in range(4)] == chars, f


@pytest.mark.parametrize("noflux", [1, 0])
@pytest.mark.parametrize("mesh", ["golden", "config"])
def test_grid_and_operator_match_reference(srs, refio, box_mesh, mesh, noflux):
    base = GOLDEN_MESH if mesh == "golden" else box_mesh[0]
    p = srs.default_parameters().set(FLAG_NO_FLUX_BOUNDARY=noflux, T_STEP=9e-6)
    ref = refio.load(base, p.ints[:], p.reals[:])
    g = srs.Grid(p, base)
    assert (g.n_ele, g.n_face, g.n_nodes, g.n_ryr, g.n_lcc) == (ref.N, ref.NF, ref.NN, ref.NR, ref.NL)
    for a, b in zip(g.operator(), ref.operator()):
        assert np.array_equal(a, b)
    el, rel = g.elements(), ref.elements()
    for k in ("V0", "TT", "domain", "tropc"):
        assert np.array_equal(el[k], rel[k]), k
    ch, rch = g.channels(), ref.channels()
    for k in ch:
        assert np.array_equal(ch[k], rch[k]), k
    # ResetDefaultGridStates (cpu/InitFuncs.cpp:928-953) leaves calsequestrin
    # unset in cytosolic elements (whatever the allocation held); the product
    # stores 0 there.  Every other entry must be equal.
    N = g.n_ele
    keep = np.ones(6 * N, bool)
    keep[4 * N:5 * N] = el["domain"] != 0
    S0 = g.initial_states(p)
    assert np.array_equal(S0[keep], ref.states()[keep])          # InitializeDefaultGrid
    assert np.array_equal(S0[keep], ref.reset_states()[keep])    # ResetDefaultGridStates
    assert not S0[~keep].any()


def test_open_random_ryr_matches_reference(srs, refio, box_mesh):
    """The initial opening of cpu/main.cpp:241-246 (INIT_RYR = -1): the
    oracle's restatement, driven by the same rand() stream, opens the RyR the
    reference's OpenRandomRyR opens (the product opens the oracle's choice for
    the same uniform, checked on the GPU)."""
    from oracle import Mesh, Oracle, RNG_REFERENCE
    base = box_mesh[0]
    p = srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=-1, T_FINAL=0.0,
                                     FLAG_RYR_OUT=1)
    ref = refio.load(base, p.ints[:], p.reals[:])
    m = Mesh(Oracle(), base, 1, np.array(p.reals[:]))
    ints = np.array(p.ints[:])
    picked = set()
    for index in range(48):
        k, _ = ref.open_random_ryr(0, index)
        rows, _, _, _ = m.run_simulation(ints, RNG_REFERENCE, 0, index, row_w=7 + m.NR)
        opened = np.nonzero(rows[0, 7:])[0]
        assert list(opened) == [k], (index, k, opened)
        picked.add(k)
    assert len(picked) > 10  # the draws cover the cluster


@pytest.mark.parametrize("mesh", ["golden", "config"])
def test_vtk_writer_matches_reference(srs, refio, box_mesh, tmp_path, mesh):
    base = GOLDEN_MESH if mesh == "golden" else box_mesh[0]
    p = srs.default_parameters().set(T_STEP=9e-6, OUTPUT_GRID_FLAG=1)
    ref = refio.load(base, p.ints[:], p.reals[:])
    g = srs.Grid(p, base)
    rng = np.random.default_rng(3)
    S = g.initial_states(p) * (1.0 + 0.3 * rng.random(6 * g.n_ele))
    ryr = (rng.random(g.n_ryr) < 0.3).astype(np.int32)
    ref.set_states(S)
    want = ref.write_grid(str(tmp_path), ryr=ryr, rank=2, run=5, n=7, t=1.2345678)
    got = str(tmp_path / "product.vtk")
    g.write_vtk(got, S, ryr, run=5, rank=2, n=7, t=1.2345678)
    assert open(got, "rb").read() == open(want, "rb").read()


def _scan_xml(path, d, gridfile_base, outdir, n_scans):
    """A parameter file for the reference's line-scan tool (symbols of
    linescan/main.cpp:455-510) describing the line scan d."""
    vals = dict(scan_n=n_scans, scan_n_per_line=1, scan_x_res_f=d["res"], scan_x_min=d["x_min"],
                scan_x_max=d["x_max"], scan_offset_1=d["offset1"], scan_offset_2=d["offset2"],
                scan_domain_x=d["domain_size"][0], scan_domain_y=d["domain_size"][1],
                scan_domain_z=d["domain_size"][2], scan_padding_min=d["pad_min"],
                scan_padding_max=d["pad_max"], scan_padding_res=d["pad_res"], scan_var_x=d["var_x"],
                scan_var_y=d["var_y"], scan_var_z=d["var_z"], scan_f0=d["f0_pad"], scan_c0=0.1,
                scan_gridfile_base=gridfile_base, outdir=outdir, scan_axis="XYZ"[d["axis"]])
    with open(path, "w") as f:
        f.write("<?xml version=\"1.0\"?>\n<analysis>\n")
        for k, v in vals.items():
            f.write("  <parameter>\n    <symbol>%s</symbol>\n    <value>%s</value>\n  </parameter>\n"
                    % (k, v))
        f.write("</analysis>\n")


def tool_scan_desc():
    """A line scan of the golden mesh that the tool and the restatement both
    describe: the tool's padding domain is centred, [-D/2, D/2] per axis."""
    size = (0.4, 0.4, 0.8)
    return dict(axis=0, offset1=0.01, offset2=0.05, x_min=-0.3, x_max=0.3, res=0.03, var_x=0.0289,
                var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=4.1667, pad_res=0.1, pad_min=-0.6,
                pad_max=0.6, domain_size=size,
                domain=(-size[0] / 2, size[0] / 2, -size[1] / 2, size[1] / 2, -size[2] / 2,
                        size[2] / 2))


def test_linescan_restatement_matches_reference_tool(srs, refio, tmp_path):
    """Three grid files written by the reference's WriteToGridFiles, scanned by
    the reference's line-scan tool, against oracle/linescan.py on the same
    (%f-rounded) states.  The tool prints %g (six significant digits)."""
    from oracle import linescan
    tool = os.path.join(ROOT, "oracle", "_ref", "linescan")
    p = srs.default_parameters().set(T_STEP=9e-6, OUTPUT_GRID_FLAG=1)
    ref = refio.load(GOLDEN_MESH, p.ints[:], p.reals[:])
    g = srs.Grid(p, GOLDEN_MESH)
    N = g.n_ele
    el = g.elements()
    rng = np.random.default_rng(5)
    d = tool_scan_desc()
    W, pad = linescan.weights(GOLDEN_MESH, el["order"], d)
    want = []
    for n in range(3):
        S = g.initial_states(p)
        S[5 * N:] *= 1.0 + 2.0 * rng.random(N)
        S = np.array([float("%f" % x) for x in S])  # the values the grid file holds
        ref.set_states(S)
        ref.write_grid(str(tmp_path), rank=0, run=0, n=n)
        want.append(pad + W @ S[5 * N:])
    xml = str(tmp_path / "scan.xml")
    _scan_xml(xml, d, str(tmp_path / "grid_0_0"), str(tmp_path), 3)
    r = subprocess.run([tool, "-param", xml], capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    got = np.loadtxt(str(tmp_path / "scan_output.txt"))
    assert got.shape == (3, len(pad))
    # %g keeps six significant digits: at most 5e-6 relative
    assert np.allclose(got, np.array(want), rtol=5e-6, atol=0), np.abs(got / np.array(want) - 1).max()
