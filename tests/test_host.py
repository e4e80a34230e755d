"""Host-side logic on the CPU: parameter parsing, mesh loading and
renumbering, operator assembly, mesh generation, C-ABI surface."""
import ctypes
import glob
import os
import re
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from conftest import GOLDEN_MESH, ROOT

# the reference's parameter files, where its source tree is present (the
# same variable oracle/build_ref.sh reads)
REF_PARAM_DIR = os.path.join(os.environ.get("SRS_REFERENCE_ROOT", "/root/reference"), "param")

# XML symbol -> (kind, index, conversion) of cpu/InitFuncs.cpp:191-349
FLAGS = {"flag_noflux": 9, "flag_nogating": 14, "flag_ffwd": 15, "flag_use_clock": 2,
         "flag_output_grid": 0, "flag_output_ryr_states": 16}
INTS = {"sims_per_proc": 17, "ryr_open_max": 10, "seed_base": 3, "seed_A": 4, "seed_B": 5}
REALS = {"c_min": 4, "ryr_open_time": 55, "v_clamp": 54, "t_clamp": 53, "t_final": 0,
         "states_interval": 2, "grid_interval": 3, "CA_I": 13, "CA_O": 17, "V_M": 15, "D_CA": 5,
         "D_CAJSR": 6, "D_ATP": 7, "D_CMDN": 8, "D_DYE": 11, "B_TOT_ATP": 18, "K_OFF_ATP": 19,
         "K_ON_ATP": 20, "B_TOT_CMDN": 21, "K_OFF_CMDN": 22, "K_ON_CMDN": 23, "B_TOT_TRPN": 24,
         "K_OFF_TRPN": 25, "K_ON_TRPN": 26, "B_TOT_SL": 27, "K_D_SL": 28, "B_TOT_DYE": 31,
         "K_OFF_DYE": 32, "K_ON_DYE": 33, "B_TOT_CSQN": 34, "K_OFF_CSQN": 40, "K_ON_CSQN": 39,
         "V_REFILL": 36, "V_RYR": 37, "RYR_ETA": 41, "RYR_A_STAR": 42, "RYR_EPS_CC": 43,
         "RYR_EPS_OO": 44, "RYR_K_MINUS": 46, "RYR_K_PLUS": 45, "RYR_PHI_N": 47, "RYR_PHI_KD": 48,
         "K_D_I": 49, "K_D_SR": 50, "A_P": 51}


def c_atof(s):
    """strtod semantics: longest numeric prefix, 0.0 when there is none."""
    m = re.match(r"\s*[+-]?(\d+\.?\d*([eE][+-]?\d+)?|\.\d+([eE][+-]?\d+)?)", s)
    return float(m.group(0)) if m else 0.0


def c_atoi(s):
    m = re.match(r"\s*[+-]?\d+", s)
    return int(m.group(0)) if m else 0


def independent_parse(srs, path):
    """A second reading of the reference's symbol table with xml.etree."""
    p = srs.default_parameters()
    ints, reals = list(p.ints), list(p.reals)
    for par in ET.parse(path).getroot().iter("parameter"):
        s, v = par.find("symbol"), par.find("value")
        if s is None or v is None:
            continue
        sym, val = s.text or "", v.text or ""
        if sym in FLAGS:
            ints[FLAGS[sym]] = 1 if val == "true" else 0
        elif sym in INTS:
            ints[INTS[sym]] = c_atoi(val)
        elif sym == "ryr_open_init":
            if val != "":
                ints[18] = c_atoi(val)
        elif sym == "protocol":
            ints[13], ints[1] = {"gain": (1, 0), "fidelity": (0, 1)}.get(val, (0, 0))
        elif sym == "t_step":
            reals[1] = c_atof(val) * 1e-6
        elif sym == "CA_SR":
            reals[14] = reals[16] = c_atof(val)
        elif sym in REALS:
            reals[REALS[sym]] = c_atof(val)
    return ints, reals


@pytest.mark.skipif(not os.path.isdir(REF_PARAM_DIR), reason="reference parameter sets absent")
def test_every_reference_parameter_file_parses_identically(srs):
    files = sorted(glob.glob(os.path.join(REF_PARAM_DIR, "**", "*.xml"), recursive=True))
    assert len(files) >= 160
    for f in files:
        p = srs.read_parameters(f)
        ints, reals = independent_parse(srs, f)
        assert list(p.ints) == ints, f
        assert list(p.reals) == reals, f


def test_missing_parameter_file_is_an_error(srs):
    with pytest.raises(srs.SrsError):
        srs.read_parameters("/nonexistent/params.xml")


@pytest.mark.parametrize("which", ["golden", "config"])
def test_loader_matches_oracle_restatement(srs, oracle, box_mesh, which):
    from oracle import Mesh
    base = GOLDEN_MESH if which == "golden" else box_mesh[0]
    for noflux in (1, 0):
        p = srs.default_parameters().set(FLAG_NO_FLUX_BOUNDARY=noflux)
        g = srs.Grid(p, base)
        m = Mesh(oracle, base, noflux, np.array(p.reals[:]))
        for a, b in zip(g.operator(), m.operator()):
            assert np.array_equal(a, b)  # aij, nij, boundary rates: bit-exact
        ge, me = g.elements(), m.elements()
        for k in ge:
            assert np.array_equal(ge[k], me[k]), k
        gc, mc = g.channels(), m.channels()
        for k in gc:
            assert np.array_equal(gc[k], mc[k]), k
        assert np.array_equal(g.initial_states(p), m.initial_states())


def test_config_mesh_geometry(srs, box_mesh):
    base, rep = box_mesh
    assert rep["n_tets"] == 10368 and rep["n_ryr"] == 49 and rep["n_lcc"] == 7
    p = srs.default_parameters().set(T_STEP=9e-6)
    g = srs.Grid(p, base)
    e = g.elements()
    assert abs(e["V0"].sum() - 8.0) < 1e-6           # 2 x 2 x 2 um box
    assert abs(g.vol_jsr - 0.4 * 0.4 * 0.05) < 1e-9  # 50 nm JSR cap over 400 x 400 nm
    assert g.n_jsr == 384
    # explicit stability margin at the parameter file's dt
    assert 0.25 * 9e-6 * g.max_diag < 0.5
    aij, nij, br = g.operator()
    a = aij.reshape(-1, 5)
    # conservative operator: row sums vanish for no-flux meshes
    assert np.max(np.abs(a.sum(1)) / np.abs(a[:, 0])) < 1e-12
    # symmetric flux: V_i a_ij == V_j a_ji
    V = e["V0"]
    n = nij.reshape(-1, 4)
    for i in range(0, g.n_ele, 97):
        for k in range(4):
            j = n[i, k]
            if j != i:
                kk = list(n[j]).index(i)
                assert abs(V[i] * a[i, 1 + k] - V[j] * a[j, 1 + kk]) < 1e-9 * V[i] * a[i, 1 + k]


def test_disconnected_mesh_is_rejected(srs, tmp_path):
    base = str(tmp_path / "m")
    srs.write_box_mesh(base, box_x=0.4, box_y=0.4, box_z=0.4, foot_half_x=0.1, foot_half_y=0.1,
                       n_foot_x=2, n_foot_y=2, n_out_x=1, n_out_y=1, n_above_z=2, ryr_nx=2,
                       ryr_ny=2, n_lcc=1, lcc_half=0.1)
    # cut every face of element 0 so the breadth-first renumbering cannot reach the rest
    fn = base + "_face_properties.txt"
    lines = open(fn).read().splitlines()
    out = lines[:2]
    for ln in lines[2:]:
        t = ln.split()
        if t[0] == "0" or t[1] == "0":
            t[1] = "-2"
            t[-1] = "1"
        out.append(" ".join(t))
    open(fn, "w").write("\n".join(out) + "\n")
    with pytest.raises(srs.SrsError) as e:
        srs.Grid(srs.default_parameters(), base)
    assert e.value.status == -3


def test_unstable_step_is_rejected_before_any_device_work(srs):
    p = srs.default_parameters().set(T_STEP=5e-3)
    g = srs.Grid(p, GOLDEN_MESH)
    with pytest.raises(srs.SrsError) as e:
        srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN)
    assert e.value.status == -4


def test_capi_exports_every_declared_symbol(srs):
    hdr = open(os.path.join(ROOT, "include", "srs_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    names = set(re.findall(r"\b(srs_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) >= 25
    lib = ctypes.CDLL(srs.LIB_PATH)
    for n in sorted(names):
        assert hasattr(lib, n), n
    # and the Python mirror binds each of them
    assert names <= set(srs._SIGS)


def test_config2_meshes_have_the_specified_sizes(srs, tmp_path):
    """Uneven multi-mesh workload: 6k / 15k / 30k / 60k tets, Poisson-disk
    clusters of 10 / 25 / 60 / 100 RyRs, one LCC per 7 RyRs, all stable at
    dt = 9 ns."""
    from srs_gb300 import workloads as wl
    reps = wl.config2_meshes(str(tmp_path))
    tets = [r["n_tets"] for _, r in reps]
    assert tets == [6000, 15288, 29478, 60984]
    assert [r["n_ryr"] for _, r in reps] == [10, 25, 60, 100]
    assert [r["n_lcc"] for _, r in reps] == [1, 4, 9, 14]
    for base, r in reps:
        leak, trig = wl.config2_protocols(r["max_a0"])
        assert leak.reals[srs.R["T_STEP"]] == 9e-6 and trig.reals[srs.R["T_STEP"]] == 9e-6
        g = srs.Grid(leak, base)
        assert g.n_ele == r["n_tets"]


def _small_multisite(srs, base):
    sites = [(-0.5, -0.4, 12, 0.09), (0.45, -0.3, 20, 0.12), (0.0, 0.5, 30, 0.14)]
    spec = srs.multisite_mesh_spec(
        sites, box_x=2.0, box_y=2.0, box_z=1.5, h_fine=0.06, h_max=0.3, growth=1.25,
        cleft_h=0.015, jsr_h=0.050, n_cleft_z=1, n_jsr_z=1, r_trpn=0.2, flag_tt=1,
        foot_margin=0.05, ryr_pitch=0.030, ryr_depth=0.0075, sheet_half=0.025, seed=3)
    return srs.write_multisite_mesh(base, spec), sites


def test_multisite_mesh_layout(srs, oracle, tmp_path):
    """Several footprints over one box: every RyR's cleft tet in the cytosol
    and JSR tet in the JSR, one LCC per 7 RyRs per site, the JSR (caps and
    sheets) one connected region, a conservative symmetric operator, and the
    product loader equal to the oracle's restatement."""
    from oracle import Mesh
    base = str(tmp_path / "ms")
    rep, sites = _small_multisite(srs, base)
    assert rep["n_ryr"] == sum(n for _, _, n, _ in sites)
    assert rep["n_lcc"] == sum(max(1, round(n / 7)) for _, _, n, _ in sites)
    p = srs.default_parameters().set(T_STEP=9e-6)
    g = srs.Grid(p, base)
    e, ch = g.elements(), g.channels()
    assert abs(e["V0"].sum() - 2.0 * 2.0 * 1.5) < 1e-6
    dom = e["domain"]
    assert np.all(dom[ch["ryr_ele"]] == 0) and np.all(dom[ch["ryr_jsr"]] == 1)
    aij, nij, _ = g.operator()
    a, n = aij.reshape(-1, 5), nij.reshape(-1, 4)
    assert np.max(np.abs(a.sum(1)) / np.abs(a[:, 0])) < 1e-12
    jsr = np.flatnonzero(dom == 1)
    seen, stack = {int(jsr[0])}, [int(jsr[0])]
    while stack:
        i = stack.pop()
        for j in n[i]:
            j = int(j)
            if j != i and dom[j] == 1 and j not in seen:
                seen.add(j)
                stack.append(j)
    assert len(seen) == len(jsr)
    m = Mesh(oracle, base, 1, np.array(p.reals[:]))
    for x, y in zip(g.operator(), m.operator()):
        assert np.array_equal(x, y)
    gc, mc = g.channels(), m.channels()
    for k in gc:
        assert np.array_equal(gc[k], mc[k]), k


def test_config4_mesh_has_the_specified_size(srs, tmp_path):
    """Large release site: about a million tets, clusters of 20 / 40 / 60 /
    100 / 150 RyRs with one LCC per 7, stable at dt = 9 ns."""
    from srs_gb300 import workloads as wl
    base, rep = wl.config4_mesh(str(tmp_path))
    assert 0.95e6 < rep["n_tets"] < 1.1e6
    assert rep["n_ryr"] == 370 and rep["n_lcc"] == 3 + 6 + 9 + 14 + 21
    p = wl.default_spark_params()
    g = srs.Grid(p, base)
    d = max(p.reals[srs.R[k]] for k in ("D_CA", "D_ATP", "D_CMDN", "D_DYE"))
    assert d * p.reals[srs.R["T_STEP"]] * g.max_diag < 1.0
    ch = g.channels()
    dom = g.elements()["domain"]
    assert np.all(dom[ch["ryr_ele"]] == 0) and np.all(dom[ch["ryr_jsr"]] == 1)


@pytest.mark.parametrize("field,value", [("n_sites", 0), ("n_sites", 9), ("h_fine", 0.0),
                                         ("h_max", 0.01), ("growth", 1.0), ("n_cleft_z", 0)])
def test_multisite_spec_errors(srs, tmp_path, field, value):
    """Invalid multi-site specifications end in SRS_ERR_INPUT before any file
    is written."""
    spec = srs.multisite_mesh_spec(
        [(0.0, 0.0, 10, 0.09)], box_x=1.0, box_y=1.0, box_z=1.0, h_fine=0.05, h_max=0.2,
        growth=1.25, cleft_h=0.015, jsr_h=0.05, n_cleft_z=1, n_jsr_z=1, r_trpn=0.2, flag_tt=1,
        foot_margin=0.05, ryr_pitch=0.03, ryr_depth=0.0075, sheet_half=0.025, seed=1)
    setattr(spec, field, value)
    base = str(tmp_path / "bad")
    with pytest.raises(srs.SrsError) as e:
        srs.write_multisite_mesh(base, spec)
    assert e.value.status == -1
    assert not os.path.exists(base + ".ele")


def test_oracle_parameter_vectors_match_product(srs):
    """oracle/params.py (ReadParameters defaults and DefaultSpark, used by the
    CPU-only reference leg of bench.py) equals the product's parameters."""
    from oracle import params as op
    from srs_gb300 import workloads as wl
    p = srs.default_parameters()
    assert list(p.ints) == list(op.DEFAULT_INTS)
    assert list(p.reals) == [float(x) for x in op.DEFAULT_REALS]
    assert op.INT_NAMES == tuple(sorted(srs.I, key=srs.I.get))
    assert op.REAL_NAMES == tuple(sorted(srs.R, key=srs.R.get))
    ints, reals = op.default_spark(T_FINAL=3.0)
    q = wl.default_spark_params(T_FINAL=3.0)
    assert list(q.ints) == ints and list(q.reals) == reals


def test_rcb_tiles_cover_every_element_once_within_the_size():
    """The tiling of the temporal-blocking measurement (bench.py): recursive
    coordinate bisection gives disjoint tiles that cover every element, none
    larger than the bound, each spatially compact along the split axes."""
    import bench
    rng = np.random.default_rng(4)
    cen = rng.random((10000, 3)) * np.array([3.0, 1.0, 1.0])
    tiles = bench.rcb_tiles(cen, 700)
    allidx = np.concatenate(tiles)
    assert len(allidx) == len(cen) and len(np.unique(allidx)) == len(cen)
    assert max(len(t) for t in tiles) <= 700 and min(len(t) for t in tiles) >= 300
    # the first cut is along the longest axis (x): every tile lies on one side of it
    xm = np.median(cen[:, 0])
    assert all((cen[t, 0] <= xm).all() or (cen[t, 0] >= xm).all() for t in tiles)
