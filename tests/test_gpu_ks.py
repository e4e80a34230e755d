"""Stochastic parity: distributions of spark metrics against the reference.

tests/golden/ks_reference.npz holds 1000 runs of the reference's own
cpu/RunSimulation.cpp (glibc rand() gating; written by
tests/golden/gen_ks_reference.py).  The same protocol runs here as 1000
realizations of the FP32 resident engine (Philox gating, seeds 1..1000),
and every metric must pass a two-sample Kolmogorov-Smirnov test at
p > 0.01: peak cleft Ca, time to peak, FDHM, maximum open RyRs, RyR open time.

The metric distributions have atoms: about a fifth of the runs reach their
peak at the first output tick with no other RyR open, so their peak is one
deterministic number.  The FP32 engine reproduces it within the deterministic
tolerance (1e-5 relative), not bit for bit, and a KS test would count the two
copies of the atom as different values.  Engine values within that tolerance
of a reference value are therefore taken as that value before the test.
"""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_MESH

def _gen_module():
    spec = importlib.util.spec_from_file_location(
        "gen_ks_reference", os.path.join(GOLDEN, "gen_ks_reference.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


REL_TOL = 1e-5  # deterministic-part tolerance of the FP32 engine


def snap_to_reference(ref, x, rel=REL_TOL):
    """Replace each value of x by the nearest value of ref when they agree
    within rel (relative); other values are left as they are."""
    u = np.unique(ref)
    j = np.clip(np.searchsorted(u, x), 1, len(u) - 1)
    lo, hi = u[j - 1], u[j]
    near = np.where(np.abs(x - lo) <= np.abs(hi - x), lo, hi)
    ok = np.abs(near - x) <= rel * np.maximum(np.abs(near), 1e-12)
    return np.where(ok, near, x)


def test_snap_to_reference_only_merges_within_tolerance():
    ref = np.array([1.0, 2.0, 8.3652])
    x = np.array([8.36520005, 8.3660, 1.0, 0.5])
    out = snap_to_reference(ref, x)
    assert out[0] == 8.3652 and out[1] == 8.3660 and out[2] == 1.0 and out[3] == 0.5


@pytest.mark.gpu
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
        res = stats.ks_2samp(ref[:, k], snap_to_reference(ref[:, k], gpu[:, k]))
        report[name] = (float(res.pvalue), float(ref[:, k].mean()), float(gpu[:, k].mean()))
    bad = {n: v for n, v in report.items() if not v[0] > 0.01}
    assert not bad, report
