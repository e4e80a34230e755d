"""GPU parity: every engine against the oracle, through the C ABI.

Bars:
  * FP64 plain engine: bit-exact with the oracle (PHILOX gating), and with the
    reference's own golden rows where no random numbers are involved;
  * FP32 plain engine: bit-exact with the oracle's FP32 restatement (gating on);
  * FP32 resident engine: bit-exact with the FP32 plain engine (same per-element
    arithmetic), for every cluster size;
  * FP32 engines vs FP64: relative error <= 1e-5 on concentrations
    (|c32 - c64| / max(|c64|, 1e-3 uM)) over the deterministic part.
"""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, params_from_golden

pytestmark = pytest.mark.gpu
TOL32 = 1e-5


def rel_err(a, b, floor=1e-3):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def golden_params(srs, name="spark"):
    p, _ = params_from_golden(srs, name)
    return p


def oracle_mesh(oracle, p, base=GOLDEN_MESH):
    from oracle import Mesh
    return Mesh(oracle, base, p.ints[9], np.array(p.reals[:]))


def test_fp64_steps_bit_exact_with_oracle(srs, oracle):
    p = golden_params(srs)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [11, 12, 13]
    sim = srs.Simulation(g, p, len(seeds), srs.FP64, srs.ENGINE_PLAIN, seeds=seeds)
    st0 = [sim.get_state(r) for r in range(len(seeds))]
    n = 600
    sim.explicit_step(n)
    m = oracle_mesh(oracle, p)
    for r, sd in enumerate(seeds):
        s0 = st0[r]
        S, ryr, lcc, lccv, res = (s0["states"].copy(), s0["ryr"].copy(), s0["lcc"].copy(),
                                  s0["lccv"].copy(), s0["residuals"].copy())
        m.steps_philox(S, sd, 0, n, ryr, lcc, lccv, res)
        got = sim.get_state(r)
        assert np.array_equal(got["states"], S)
        assert np.array_equal(got["ryr"], ryr)
        assert np.array_equal(got["lcc"], lcc) and np.array_equal(got["lccv"], lccv)
        assert np.array_equal(got["residuals"], res)


def test_fp64_reset_matches_oracle(srs, oracle):
    for name in ["spark", "lcc_trigger", "gain_clamp"]:
        p = golden_params(srs, name)
        g = srs.Grid(p, GOLDEN_MESH)
        sim = srs.Simulation(g, p, 2, srs.FP64, srs.ENGINE_PLAIN, seeds=[5, 6])
        m = oracle_mesh(oracle, p)
        for r, sd in enumerate([5, 6]):
            want = m.reset_philox(np.array(p.ints[:]), sd)
            got = sim.get_state(r)
            for k in ("states", "ryr", "lcc", "lccv", "residuals"):
                assert np.array_equal(got[k], want[k]), (name, k)


def test_fp64_random_initial_ryr_matches_oracle(srs, oracle):
    p = golden_params(srs).set(INIT_RYR=-1)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = list(range(1, 9))
    sim = srs.Simulation(g, p, len(seeds), srs.FP64, srs.ENGINE_PLAIN, seeds=seeds)
    m = oracle_mesh(oracle, p)
    for r, sd in enumerate(seeds):
        want = m.reset_philox(np.array(p.ints[:]), sd)
        assert np.array_equal(sim.get_state(r)["ryr"], want["ryr"])


@pytest.mark.parametrize("name", ["spark", "spark_nogating", "lcc_trigger", "gain_clamp",
                                  "fidelity"])
def test_fp64_run_simulation_bit_exact_with_oracle(srs, oracle, name):
    from oracle import RNG_PHILOX
    p = golden_params(srs, name)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [21, 22]
    sim = srs.Simulation(g, p, len(seeds), srs.FP64, srs.ENGINE_PLAIN, seeds=seeds)
    rows, t_end, n_steps = sim.run_simulation()
    m = oracle_mesh(oracle, p)
    for r, sd in enumerate(seeds):
        want_rows, want_S, want_t, want_n = m.run_simulation(np.array(p.ints[:]), RNG_PHILOX, sd)
        assert rows[r].shape == want_rows.shape, name
        assert np.array_equal(rows[r], want_rows), name
        assert np.array_equal(sim.get_state(r)["states"], want_S), name
        assert t_end[r] == want_t and n_steps[r] == want_n


def test_fp64_deterministic_run_equals_reference_golden(srs):
    """No random numbers enter a run without gating and with a named initial
    RyR, so the GPU FP64 rows equal the reference's own rows bit for bit."""
    p, d = params_from_golden(srs, "spark_nogating")
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN, seeds=[3])
    rows, _, _ = sim.run_simulation()
    assert np.array_equal(rows[0], d["rows"])
    assert np.array_equal(sim.get_state(0)["states"], d["states"])


def test_fp32_plain_bit_exact_with_fp32_oracle(srs, oracle):
    """The plain FP32 engine (Euler compensation terms kept as halves,
    srs_comp.h) against the oracle's FP32 restatement with the same compact
    compensation."""
    p = golden_params(srs)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [51, 52, 53]
    sim = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    st0 = [sim.get_state(r) for r in range(len(seeds))]
    n = 800
    sim.explicit_step(n)
    m = oracle_mesh(oracle, p)
    for r, sd in enumerate(seeds):
        s0 = st0[r]
        st = m.to_fp32(s0["states"])
        ryr, lcc, lccv, res = (s0["ryr"].copy(), s0["lcc"].copy(), s0["lccv"].copy(),
                               s0["residuals"].copy())
        m.steps_fp32(st, sd, 0, n, ryr, lcc, lccv, res, gating=True, compact=True)
        got = sim.get_state(r)
        assert np.array_equal(got["states"], m.from_fp32(st))
        assert np.array_equal(got["ryr"], ryr) and np.array_equal(got["residuals"], res)
        assert np.array_equal(got["lcc"], lcc) and np.array_equal(got["lccv"], lccv)


def test_fp32_plain_split_form_bit_exact_with_fp32_oracle(srs, oracle, tmp_path):
    """Meshes of 65,536 elements and more take the split form of the plain
    FP32 step (element update and gating as two launches): the same results
    as the oracle's FP32 restatement with compact compensation."""
    base = str(tmp_path / "big")
    rep = srs.write_box_mesh(base, box_x=3.0, box_y=3.0, box_z=3.0, foot_half_x=0.3,
                             foot_half_y=0.3, n_foot_x=10, n_foot_y=10, n_out_x=6, n_out_y=6,
                             n_above_z=22)
    assert rep["n_tets"] >= 65536
    p = golden_params(srs)
    g = srs.Grid(p, base)
    seeds = [61, 62]
    sim = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    st0 = [sim.get_state(r) for r in range(len(seeds))]
    n = 48
    sim.explicit_step(n)
    assert sim.config()["kernel_launches"] >= 2 * n
    m = oracle_mesh(oracle, p, base)
    for r, sd in enumerate(seeds):
        s0 = st0[r]
        st = m.to_fp32(s0["states"])
        ryr, lcc, lccv, res = (s0["ryr"].copy(), s0["lcc"].copy(), s0["lccv"].copy(),
                               s0["residuals"].copy())
        m.steps_fp32(st, sd, 0, n, ryr, lcc, lccv, res, gating=True, compact=True)
        got = sim.get_state(r)
        assert np.array_equal(got["states"], m.from_fp32(st))
        assert np.array_equal(got["ryr"], ryr) and np.array_equal(got["residuals"], res)


def test_fp32_split_form_error_vs_fp64_over_2ms(srs, tmp_path):
    """The large-mesh (split) form over 2 ms (222,224 steps)
    of the DefaultSpark source with gating off: within 1e-5 relative of the
    FP64 engine at every 0.5 ms checkpoint."""
    base = str(tmp_path / "big")
    rep = srs.write_box_mesh(base, box_x=3.0, box_y=3.0, box_z=3.0, foot_half_x=0.3,
                             foot_half_y=0.3, n_foot_x=10, n_foot_y=10, n_out_x=6, n_out_y=6,
                             n_above_z=22)
    assert rep["n_tets"] >= 65536
    p = srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=24,
                                     FLAG_NO_GATING=1)
    g = srs.Grid(p, base)
    s64 = srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN)
    s32 = srs.Simulation(g, p, 2, srs.FP32, srs.ENGINE_PLAIN)
    errs = []
    for _ in range(4):
        for s in (s64, s32):
            s.explicit_step(55556)
        ref = s64.get_state(0)["states"]
        errs.append(max(rel_err(s32.get_state(r)["states"], ref) for r in range(2)))
    assert max(errs) <= TOL32, errs
    assert not (s32.status() & 1)


def test_fp32_plain_within_tolerance_of_fp64(srs):
    p = golden_params(srs, "spark_nogating")
    g = srs.Grid(p, GOLDEN_MESH)
    s64 = srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN)
    s32 = srs.Simulation(g, p, 1, srs.FP32, srs.ENGINE_PLAIN)
    for s in (s64, s32):
        s.explicit_step(4000)
    e = rel_err(s32.get_state(0)["states"], s64.get_state(0)["states"])
    assert e <= TOL32, e


@pytest.mark.parametrize("cluster", [1, 2, 4])
def test_fp32_resident_bit_exact_with_plain(srs, cluster):
    p = golden_params(srs)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [31, 32, 33, 34, 35]
    pl = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    rs = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                        cluster_size=cluster, steps_per_launch=97)
    assert rs.config()["cluster_size"] == cluster
    pl.explicit_step(1000)
    rs.explicit_step(1000)
    for r in range(len(seeds)):
        a, b = pl.get_state(r), rs.get_state(r)
        for k in ("states", "ryr", "lcc", "lccv", "residuals"):
            assert np.array_equal(a[k], b[k]), (cluster, r, k)


@pytest.mark.parametrize("proto,cluster,launch", [("fidelity", 2, 500), ("spark", 3, 700),
                                                  ("lcc_trigger", 2, 333)])
def test_fp32_resident_run_simulation_matches_plain(srs, proto, cluster, launch):
    """Rows and final states, with the run ending inside a later launch (the
    launches before it speculate; the fidelity run never does)."""
    p = golden_params(srs, proto)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [41, 42, 43]
    pl = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    rs = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                        cluster_size=cluster, steps_per_launch=launch)
    ra, ta, na = pl.run_simulation()
    rb, tb, nb = rs.run_simulation()
    for r in range(len(seeds)):
        assert ra[r].shape == rb[r].shape
        assert np.array_equal(ra[r], rb[r])
        assert ta[r] == tb[r] and na[r] == nb[r]
        a, b = pl.get_state(r), rs.get_state(r)
        for k in ("states", "ryr", "lcc", "lccv", "residuals"):
            assert np.array_equal(a[k], b[k]), (proto, r, k)


def test_timed_run_simulation_gives_the_same_run(srs):
    """srs_run_simulation_timed: the same rows, times and states as
    srs_run_simulation, one positive device time per launch."""
    p = golden_params(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [51, 52]
    launch = 700
    sims = [srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                           cluster_size=2, steps_per_launch=launch) for _ in range(2)]
    ra, ta, na = sims[0].run_simulation()
    rb, tb, nb, ms = sims[1].run_simulation(timed=True)
    for r in range(len(seeds)):
        assert np.array_equal(ra[r], rb[r])
        assert ta[r] == tb[r] and na[r] == nb[r]
        assert np.array_equal(sims[0].get_state(r)["states"], sims[1].get_state(r)["states"])
    assert len(ms) == -(-int(na.max()) // launch) and np.all(ms > 0)


@pytest.mark.parametrize("engine,prec", [("RESIDENT", 32), ("PLAIN", 32), ("PLAIN", 64)])
def test_grid_snapshots_during_run(srs, engine, prec):
    """OUTPUT_GRID_FLAG: the run stops at the reference's grid-file steps
    (floor(t / OUTPUT_GRID_INTERVAL) increments, cpu/RunSimulation.cpp:545);
    each snapshot is the state of a run that ends at that step, and the run's
    own rows and final states are those of a run without snapshots."""
    import math
    eng = getattr(srs, "ENGINE_" + engine)
    pr = srs.FP32 if prec == 32 else srs.FP64
    p = golden_params(srs, "spark")
    dt, T = p.reals[srs.R["T_STEP"]], p.reals[srs.R["T_FINAL"]]
    I = T / 4.3
    pg = p.copy().set(OUTPUT_GRID_FLAG=1, OUTPUT_GRID_INTERVAL=I)
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [71, 72]
    kw = dict(seeds=seeds, cluster_size=2, steps_per_launch=300) if engine == "RESIDENT" else dict(seeds=seeds)
    sim = srs.Simulation(g, pg, len(seeds), pr, eng, **kw)
    snaps = []

    def cb(n, t, done):
        snaps.append((n, t, [sim.get_state(r)["states"] for r in range(len(seeds))], done.copy()))

    rows, t_end, nst = sim.run_simulation(grid_callback=cb)
    steps, times = [], []
    t, last, n = 0.0, 0.0, 0
    while t <= T:
        if math.floor(t / I) > math.floor((t - last) / I):
            steps.append(n)
            times.append(t)
        t += dt
        last = dt
        n += 1
    assert len(steps) >= 3
    assert [x[0] for x in snaps] == list(range(1, len(steps) + 1))
    assert [x[1] for x in snaps] == times
    for (_, _, states, done), gs in zip(snaps, steps):
        assert not done.any()
        q = srs.Simulation(g, p.copy().set(T_FINAL=(gs - 0.5) * dt), len(seeds), pr, eng, **kw)
        q.run_simulation()
        for r in range(len(seeds)):
            assert np.array_equal(q.get_state(r)["states"], states[r]), (gs, r)
    ref = srs.Simulation(g, p, len(seeds), pr, eng, **kw)
    rows2, t2, n2 = ref.run_simulation()
    for r in range(len(seeds)):
        assert np.array_equal(rows[r], rows2[r]) and t_end[r] == t2[r] and nst[r] == n2[r]
        assert np.array_equal(sim.get_state(r)["states"], ref.get_state(r)["states"])


@pytest.mark.parametrize("cluster,threads", [(0, 0), (5, 320), (6, 256), (8, 192)])
def test_resident_on_config_mesh_matches_plain(srs, box_mesh, cluster, threads):
    """The default placement and the bench's tuned ones (two CTAs of a
    5-CTA cluster per SM, three of an 8-CTA cluster)."""
    base, _ = box_mesh
    p = srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=24,
                                     INIT_RYR_HOLD=10.0)
    g = srs.Grid(p, base)
    seeds = list(range(1, 5))
    pl = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    rs = srs.Simulation(g, p, len(seeds), srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                        cluster_size=cluster, threads_per_cta=threads)
    cfg = rs.config()
    assert cfg["cluster_size"] >= 2  # 10,368 elements do not fit one CTA's shared memory
    pl.explicit_step(600)
    rs.explicit_step(600)
    for r in range(len(seeds)):
        assert np.array_equal(pl.get_state(r)["states"], rs.get_state(r)["states"])


def test_fp32_resident_error_vs_fp64_on_config_mesh(srs, box_mesh):
    base, _ = box_mesh
    p = srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=24,
                                     FLAG_NO_GATING=1)
    g = srs.Grid(p, base)
    s64 = srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN)
    s32 = srs.Simulation(g, p, 2, srs.FP32, srs.ENGINE_RESIDENT)
    s64.explicit_step(3000)
    s32.explicit_step(3000)
    e = rel_err(s32.get_state(0)["states"], s64.get_state(0)["states"])
    assert e <= TOL32, e


def test_fp32_error_vs_fp64_over_2ms_on_config_mesh(srs, box_mesh):
    """The deterministic part over a real horizon: 2 ms (222,224 steps at
    dt = 9 ns) of the DefaultSpark source (RyR 24 held open, gating off) on
    the config mesh.  Both FP32 engines stay within 1e-5 relative of the FP64
    engine at every 0.5 ms checkpoint."""
    base, _ = box_mesh
    p = srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=24,
                                     FLAG_NO_GATING=1)
    g = srs.Grid(p, base)
    s64 = srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN)
    s32 = srs.Simulation(g, p, 2, srs.FP32, srs.ENGINE_RESIDENT)
    p32 = srs.Simulation(g, p, 1, srs.FP32, srs.ENGINE_PLAIN)
    errs = []
    for _ in range(4):
        for s in (s64, s32, p32):
            s.explicit_step(55556)
        ref = s64.get_state(0)["states"]
        errs.append((rel_err(s32.get_state(0)["states"], ref), rel_err(s32.get_state(1)["states"], ref),
                     rel_err(p32.get_state(0)["states"], ref)))
    assert max(max(e) for e in errs) <= TOL32, errs
    assert not (s32.status() & 1) and not (p32.status() & 1)


def test_nonfinite_state_is_reported(srs):
    p = golden_params(srs, "spark_nogating")
    g = srs.Grid(p, GOLDEN_MESH)
    for eng, prec in ((srs.ENGINE_PLAIN, srs.FP64), (srs.ENGINE_PLAIN, srs.FP32),
                      (srs.ENGINE_RESIDENT, srs.FP32)):
        sim = srs.Simulation(g, p, 1, prec, eng)
        st = sim.get_state(0)
        S = st["states"].copy()
        S[7] = np.nan  # a planted bad value (host side): arithmetic only, no fault
        sim.set_state(0, S)
        sim.explicit_step(4)
        assert sim.status() & 1, (eng, prec)
