"""Stochastic parity: distributions of spark metrics against the reference.

tests/golden/ks_reference.npz holds 1000 runs of the reference's own
cpu/RunSimulation.cpp (glibc rand() gating; written by
tests/golden/gen_ks_reference.py) of a short recruiting protocol on the
golden mesh.  The same protocol runs here as 1000 realizations of the FP32
resident engine (Philox gating, seeds 1..1000), and the metrics are
compared: peak cleft Ca, time to peak, FDHM, maximum open RyRs, RyR open
time.

Runs in which RyR 4 stays open through the window and no other RyR opens
(about a fifth) share one deterministic trajectory: the distributions are a
mixture of that atom and a continuous part, compared in parts
(tests/ks_mixture.py): the atom's mass (Fisher's exact test), every metric
of the other runs (KS, p > 0.01), and the atom's value against the
reference's at the deterministic tolerance (1e-5 relative).
"""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_MESH
from ks_mixture import mixture_ks, plain_ks


def _gen_module():
    spec = importlib.util.spec_from_file_location(
        "gen_ks_reference", os.path.join(GOLDEN, "gen_ks_reference.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


REL_TOL = 1e-5  # deterministic-part tolerance of the FP32 engine


def atom_mask(m):
    """RyR 4 open at every output tick and no other RyR open: one open RyR
    at most and the whole window's open time (both exact tick counts)."""
    full = m[m[:, 3] == 1, 4].max()
    return (m[:, 3] == 1) & (m[:, 4] == full)


@pytest.mark.gpu
def test_spark_metric_distributions_match_reference(srs):
    pytest.importorskip("scipy.stats")
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
    ref_atom, gpu_atom = atom_mask(ref), atom_mask(gpu)
    report, bad = mixture_ks(ref, gpu, ref_atom, gpu_atom, names)
    assert not bad, report
    # the atom's value: the reference's (FP64) and the engine's (FP32) peak
    v_ref = np.unique(ref[ref_atom, 0], return_counts=True)
    v_gpu = np.unique(gpu[gpu_atom, 0], return_counts=True)
    a_ref, a_gpu = v_ref[0][np.argmax(v_ref[1])], v_gpu[0][np.argmax(v_gpu[1])]
    assert abs(a_gpu - a_ref) <= REL_TOL * abs(a_ref), (a_gpu, a_ref)
    print("golden-mesh KS:", report, "plain KS (atoms included):", plain_ks(ref, gpu, names))
