"""Stochastic parity: distributions of spark metrics against the reference.

tests/golden/ks_reference.npz holds 1000 runs of the reference's own
cpu/RunSimulation.cpp (glibc rand() gating; written by
tests/golden/gen_ks_reference.py).  The same protocol runs here as 1000
realizations of the FP32 resident engine (Philox gating, seeds 1..1000),
and every metric must pass a two-sample Kolmogorov-Smirnov test at
p > 0.01: peak cleft Ca, time to peak, FDHM, maximum open RyRs, RyR open time.
"""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_MESH

pytestmark = pytest.mark.gpu


def _gen_module():
    spec = importlib.util.spec_from_file_location(
        "gen_ks_reference", os.path.join(GOLDEN, "gen_ks_reference.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_spark_metric_distributions_match_reference(srs):
    stats = pytest.importorskip("scipy.stats")
    d = np.load(os.path.join(GOLDEN, "ks_reference.npz"))
    ref = d["metrics"]
    names = [str(x) for x in d["names"]]
    assert len(ref) >= 1000
    p = srs.default_parameters()
    for i, v in enumerate(d["ints"]):
        p.ints[i] = int(v)
    for i, v in enumerate(d["reals"]):
        p.reals[i] = float(v)
    g = srs.Grid(p, GOLDEN_MESH)
    R = len(ref)
    sim = srs.Simulation(g, p, R, srs.FP32, srs.ENGINE_RESIDENT, seeds=list(range(1, R + 1)))
    rows, t_end, n_steps = sim.run_simulation()
    metrics = _gen_module().metrics
    gpu = np.array([metrics(r) for r in rows])
    report = {}
    for k, name in enumerate(names):
        res = stats.ks_2samp(ref[:, k], gpu[:, k])
        report[name] = (float(res.pvalue), float(ref[:, k].mean()), float(gpu[:, k].mean()))
    bad = {n: v for n, v in report.items() if not v[0] > 0.01}
    assert not bad, report
