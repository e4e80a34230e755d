"""Fault injection on the host: corrupted or missing input files and
inconsistent channel data end in an error code and a message (the reference
prints and exits or aborts, cpu/InitFuncs.cpp / cpu/OutputFuncs.cpp); nothing
reaches the device."""
import os
import shutil

import pytest

from conftest import GOLDEN_MESH, params_from_golden

SUFFIXES = ("_tet_properties.txt", "_face_properties.txt", ".node", ".ele", "_ryr.txt", "_lcc.txt")


@pytest.fixture
def mesh_copy(tmp_path):
    base = str(tmp_path / "m")
    for s in SUFFIXES:
        shutil.copy(GOLDEN_MESH + s, base + s)
    return base


def _edit(path, fn):
    lines = open(path).read().splitlines()
    open(path, "w").write("\n".join(fn(lines)) + "\n")


def _load(srs, base):
    p, _ = params_from_golden(srs, "spark")
    with pytest.raises(srs.SrsError) as e:
        srs.Grid(p, base)
    return e.value.status, str(e.value)


def test_missing_file_is_an_io_error(srs, mesh_copy):
    os.remove(mesh_copy + "_ryr.txt")
    st, msg = _load(srs, mesh_copy)
    assert st == -2 and "_ryr.txt" in msg


def test_truncated_element_file_is_an_io_error(srs, mesh_copy):
    _edit(mesh_copy + "_tet_properties.txt", lambda L: L[: len(L) // 2])
    st, _ = _load(srs, mesh_copy)
    assert st == -2


def test_short_face_line_is_rejected(srs, mesh_copy):
    """The files are read field by field across line breaks (as the
    reference's fscanf does), so a short line shifts every later field: the
    result is an inconsistent mesh or a read error, never a silent load."""
    _edit(mesh_copy + "_face_properties.txt", lambda L: L[:5] + [" ".join(L[5].split()[:10])] + L[6:])
    st, _ = _load(srs, mesh_copy)
    assert st in (-2, -3)


@pytest.mark.parametrize("which,value", [("ryr_ele", "100000"), ("ryr_jsr", "-3"), ("lcc", "384")])
def test_channel_index_out_of_range_is_a_mesh_error(srs, mesh_copy, which, value):
    if which == "lcc":
        _edit(mesh_copy + "_lcc.txt", lambda L: L[:1] + [value] + L[2:])
    else:
        col = 0 if which == "ryr_ele" else 1

        def f(L):
            w = L[1].split()
            w[col] = value
            return L[:1] + [" ".join(w)] + L[2:]
        _edit(mesh_copy + "_ryr.txt", f)
    st, msg = _load(srs, mesh_copy)
    assert st == -3 and "out of range" in msg


def test_face_element_out_of_range_is_a_mesh_error(srs, mesh_copy):
    def f(L):
        w = L[2].split()
        w[0] = "99999"
        return L[:2] + [" ".join(w)] + L[3:]
    _edit(mesh_copy + "_face_properties.txt", f)
    st, _ = _load(srs, mesh_copy)
    assert st == -3


def test_non_positive_volume_is_a_mesh_error(srs, mesh_copy):
    def f(L):
        w = L[2].split()
        w[3] = "0"
        return L[:2] + [" ".join(w)] + L[3:]
    _edit(mesh_copy + "_tet_properties.txt", f)
    st, msg = _load(srs, mesh_copy)
    assert st == -3 and "volume" in msg


def test_parameter_file_errors(srs, tmp_path):
    with pytest.raises(srs.SrsError) as e:
        srs.read_parameters(str(tmp_path / "absent.xml"))
    assert e.value.status == -2
    empty = tmp_path / "empty.xml"
    empty.write_text("<?xml version='1.0'?>\\n<simulation>\\n</simulation>\\n")
    with pytest.raises(srs.SrsError) as e:
        srs.read_parameters(str(empty))
    assert e.value.status == -2


@pytest.mark.parametrize("n", [0, -1, 65536])
def test_realization_count_out_of_range_is_an_input_error(srs, n):
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    with pytest.raises(srs.SrsError) as e:
        srs.Simulation(g, p, n, srs.FP32, srs.ENGINE_PLAIN)
    assert e.value.status == -1 and "n_realizations" in str(e.value)


def test_unstable_time_step_is_rejected(srs):
    """D * dt * max|a0| > 1: the explicit step would blow up, refused before
    any device work."""
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    p = p.copy().set(T_STEP=p.reals[srs.R["T_STEP"]] * 1e4)
    for prec, eng in ((srs.FP64, srs.ENGINE_PLAIN), (srs.FP32, srs.ENGINE_RESIDENT)):
        with pytest.raises(srs.SrsError) as e:
            srs.Simulation(g, p, 4, prec, eng)
        assert e.value.status == -4 and "unstable" in str(e.value)


@pytest.mark.gpu
def test_ryr_with_swapped_domains_is_rejected_by_fp32_engines(srs, mesh_copy):
    """The FP32 engines store Ca relative to each domain's rest and take a
    RyR's flux from its JSR element to its cleft element; a RyR whose two
    elements are swapped is refused instead of giving wrong fluxes."""
    def f(L):
        w = L[1].split()
        w[0], w[1] = w[1], w[0]
        return L[:1] + [" ".join(w)] + L[2:]
    _edit(mesh_copy + "_ryr.txt", f)
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, mesh_copy)
    srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN)  # absolute FP64 state: fine
    for eng in (srs.ENGINE_PLAIN, srs.ENGINE_RESIDENT):
        with pytest.raises(srs.SrsError) as e:
            srs.Simulation(g, p, 1, srs.FP32, eng)
        assert e.value.status == -3


NOALLOC_POINTERS = ("aij", "nij", "br4", "v0", "bhi", "blo", "flags", "chan_ptr", "chan_list",
                    "ryr_ele", "ryr_jsr", "ryr_nb", "lcc_ele", "states_in", "states_out",
                    "ryr_states", "lcc_states", "lccv_states", "residuals")


@pytest.mark.parametrize("missing", NOALLOC_POINTERS + ("reals", "seeds"))
def test_noalloc_step_rejects_null_pointers(srs, missing):
    """Host-side validation of srs_explicit_step_fp64_noalloc: every array the
    FP64 step reads for the given counts must be non-null (ryr_nb only with
    coupled gating), and the call returns SRS_ERR_INPUT before any CUDA call.
    The other pointers are placeholders that must never be dereferenced, so
    the test runs only where no GPU is visible."""
    import ctypes as C

    import numpy as np
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("host-only validation test")
    d = srs.NoallocStep()
    d.n_ele, d.n_realizations, d.n_ryr, d.n_lcc = 10, 2, 3, 1
    for k, name in enumerate(NOALLOC_POINTERS):
        setattr(d, name, 0x1000 + 0x100 * k)
    reals = np.zeros(56)
    reals[srs.R["RYR_A_STAR"]] = 1.0 if missing == "ryr_nb" else 0.0
    seeds = np.zeros(2, np.uint64)
    d.reals = reals.ctypes.data_as(C.c_void_p).value
    d.seeds = seeds.ctypes.data_as(C.c_void_p).value
    setattr(d, missing, None)
    with pytest.raises(srs.SrsError) as e:
        srs.explicit_step_fp64_noalloc(d)
    assert e.value.status == -1 and "pointer" in str(e.value)
