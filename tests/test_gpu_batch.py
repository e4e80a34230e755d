"""Multi-mesh batch (srs_batch_*): members of different grids, parameters and
sizes advanced by one CUDA graph give exactly the results of running each
member on its own."""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, params_from_golden

pytestmark = pytest.mark.gpu


def _members(srs, tmp_path):
    from srs_gb300 import workloads as wl
    tiny = str(tmp_path / "tiny")
    srs.write_box_mesh(tiny, **wl.TINY_DYAD)
    p1, _ = params_from_golden(srs, "spark")
    p2, _ = params_from_golden(srs, "spark_nogating")
    p3 = wl.default_spark_params(T_FINAL=0.5, OUTPUT_STATES_INTERVAL=0.05, INIT_RYR=4)
    return [(GOLDEN_MESH, p1, [1, 2, 3, 4], 2), (GOLDEN_MESH, p2, [5, 6, 7], 1), (tiny, p3, [8, 9], 1)]


def _make(srs, spec):
    base, p, seeds, C = spec
    g = srs.Grid(p, base)
    sim = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds, cluster_size=C)
    sim.reset()
    return sim


def test_batch_advance_equals_members_alone(srs, tmp_path):
    specs = _members(srs, tmp_path)
    batch_sims = [_make(srs, s) for s in specs]
    b = srs.Batch(batch_sims, steps_per_launch=256)
    b.advance_async(700)  # two graph replays and a remainder of 188 steps
    b.synchronize()
    for spec, bs in zip(specs, batch_sims):
        alone = _make(srs, spec)
        alone.explicit_step(700)
        for r in range(bs.R):
            x, y = bs.get_state(r), alone.get_state(r)
            for k in ("states", "ryr", "lcc", "lccv", "residuals"):
                assert np.array_equal(x[k], y[k]), (spec[0], r, k)


def test_batch_run_simulation_equals_members_alone(srs, tmp_path):
    specs = _members(srs, tmp_path)
    for sp in specs:
        sp[1].set(T_FINAL=0.3, OUTPUT_STATES_INTERVAL=0.01)
    batch_sims = [_make(srs, s) for s in specs]
    res = srs.Batch(batch_sims, steps_per_launch=500).run_simulation()
    for spec, (rows, t_end, n_steps) in zip(specs, res):
        alone = _make(srs, spec)
        rows2, t2, n2 = alone.run_simulation()
        assert np.array_equal(n_steps, n2) and np.array_equal(t_end, t2)
        for a, b in zip(rows, rows2):
            assert np.array_equal(a, b)


def test_batch_rejects_non_resident_members(srs):
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    plain = srs.Simulation(g, p, 1, srs.FP32, srs.ENGINE_PLAIN)
    with pytest.raises(srs.SrsError):
        srs.Batch([plain])
