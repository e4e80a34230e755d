"""The drop-in CLI (srs_gb300/bin/cru3d, the reference's cpu/main.cpp
interface) on the golden mesh: it reads a reference-format parameter XML and
writes states_<rank>_<index>.out files (float32 rows, cpu/OutputFuncs.cpp:
223-350) that equal the rows srs_run_simulation returns for the same seeds
(93843 + seed_base + rank * seed_A + index * seed_B, cpu/RunSimulation.cpp:446),
and the legacy VTK snapshot of realization 0."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_MESH, ROOT

pytestmark = pytest.mark.gpu

XML = """<?xml version="1.0" encoding="UTF-8" standalone="no"?>
<simulation>
%s
</simulation>
"""


def _xml(path, values):
    body = "\n".join("  <parameter>\n    <symbol>%s</symbol>\n    <value>%s</value>\n  </parameter>"
                     % kv for kv in values.items())
    with open(path, "w") as f:
        f.write(XML % body)


@pytest.mark.parametrize("precision", [32, 64])
def test_cru3d_states_files_match_run_simulation(srs, tmp_path, precision):
    vals = dict(t_final="0.2", t_step="9", states_interval="0.01", sims_per_proc="3",
                ryr_open_init="4", ryr_open_time="0.05", flag_use_clock="false", seed_base="5",
                seed_A="1000", seed_B="7", flag_noflux="true", flag_output_grid="false")
    param = str(tmp_path / "p.xml")
    _xml(param, vals)
    out = str(tmp_path / "out")
    exe = os.path.join(ROOT, "srs_gb300", "bin", "cru3d")
    r = subprocess.run([exe, "-param", param, "-mesh", GOLDEN_MESH, "-out", out, "-rank", "2",
                        "-start", "1", "-precision", str(precision)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    p = srs.read_parameters(param)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [93843 + 5 + 2 * 1000 + i * 7 for i in (1, 2)]
    sim = srs.Simulation(g, p, 2, precision,
                         srs.ENGINE_RESIDENT if precision == 32 else srs.ENGINE_PLAIN, seeds=seeds)
    sim.reset()
    rows, _, _ = sim.run_simulation()
    for k, i in enumerate((1, 2)):
        f = os.path.join(out, "states_2_%d.out" % i)
        got = np.fromfile(f, dtype=np.float32).reshape(-1, sim.row_width())
        assert np.array_equal(got, rows[k]), f
    assert not os.path.exists(os.path.join(out, "states_2_0.out"))  # -start 1


def test_vtk_snapshot_has_reference_layout(srs, tmp_path):
    p = srs.default_parameters().set(FLAG_NO_FLUX_BOUNDARY=1)
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN, seeds=[3])
    sim.reset()
    path = str(tmp_path / "grid_0_0_0.vtk")
    sim.write_grid_vtk(0, path)
    txt = open(path).read().split()
    assert txt[:2] == ["#", "vtk"]
    assert "UNSTRUCTURED_GRID" in txt and "CELL_DATA" in txt
    assert str(g.n_ele) in txt


def test_cru3d_writes_grid_files_during_the_run(srs, tmp_path):
    """flag_output_grid: grid_<rank>_<index>_<n>.vtk at the start (n = 0), at
    every grid interval while the realization runs and at its end, numbered
    as the reference's output_counter (cpu/RunSimulation.cpp:421, 545-549,
    582)."""
    import math
    vals = dict(t_final="0.2", t_step="9", states_interval="0.01", grid_interval="0.045",
                sims_per_proc="2", ryr_open_init="4", ryr_open_time="0.05",
                flag_use_clock="false", flag_noflux="true", flag_output_grid="true")
    param = str(tmp_path / "p.xml")
    _xml(param, vals)
    out = str(tmp_path / "out")
    exe = os.path.join(ROOT, "srs_gb300", "bin", "cru3d")
    r = subprocess.run([exe, "-param", param, "-mesh", GOLDEN_MESH, "-out", out],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    p = srs.read_parameters(param)
    dt, T, I = (p.reals[srs.R[k]] for k in ("T_STEP", "T_FINAL", "OUTPUT_GRID_INTERVAL"))
    t, last, n_grid = 0.0, 0.0, 0
    while t <= T:
        n_grid += math.floor(t / I) > math.floor((t - last) / I)
        t += dt
        last = dt
    assert n_grid >= 3
    for i in range(2):
        names = sorted(f for f in os.listdir(out) if f.startswith("grid_0_%d_" % i))
        assert names == sorted("grid_0_%d_%d.vtk" % (i, n) for n in range(n_grid + 2)), names
