"""Reference ensemble of the batched-dyad workload for the KS test.

Runs the reference's own cpu/RunSimulation.cpp (compiled in oracle/_ref by
oracle/build_ref.sh) on the 10,368-element box dyad (12^3 hexahedra x 6
tets, 49 RyRs at 31 nm, 7 LCCs) with the DefaultSpark parameters unchanged
(dt = 9 ns, RyR 24 opened at t = 0 and held open for 10 ms, glibc rand()
gating) except the window: T_FINAL = WINDOW_MS, with a grid-file tick every
0.01 ms.  Each run r uses ensemble index r, so it draws its own rand() stream
(seed rule of cpu/RunSimulation.cpp:446-450).  At every tick the harness
takes the Fluo-4 line scan along x through the cluster centre (PSF of
linescan/DefaultScan.xml, oracle/linescan.py) from the reference's own state;
the states rows give the RyR open counts.  Metrics per run: ks_metrics.py.

    python tests/golden/gen_ks_config1.py --work DIR [--runs 1000] [--procs N]

Per-run results go to DIR (one small .npz per run, so an interrupted job
resumes where it stopped); when all runs are there the script writes
tests/golden/ks_config1.npz (metrics, the most LCCs open at any tick, which
runs open no channel besides the held RyR and the centre dF/F0 trace they
share, the parameter vectors).  A run takes about 115 s on one
core of a 2.7 GHz x86 host.
"""
import argparse
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, HERE)

WINDOW_MS = 3.0
TICK_MS = 0.01
N_TICKS = int(round(WINDOW_MS / TICK_MS))  # ticks 1..N_TICKS after t = 0
# Fluo-4 line scan along x through the cluster centre, 100 nm above the
# sarcolemma (PSF variances of linescan/DefaultScan.xml; no padding voxels:
# the box is larger than the PSF's reach along the scan)
LINESCAN = dict(axis=0, offset1=0.0, offset2=0.1, x_min=-1.0, x_max=1.0, res=0.05, var_x=0.0289,
                var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=0.0, pad_res=0.0, pad_min=0.0,
                pad_max=0.0, domain=(0, 0, 0, 0, 0, 0))


def params():
    """DefaultSpark with the window and the tick: T_FINAL half a tick past
    the last tick so that every tick falls inside the time loop."""
    from srs_gb300 import workloads as wl
    return wl.default_spark_params(T_FINAL=WINDOW_MS + 0.5 * TICK_MS, OUTPUT_GRID_FLAG=1,
                                   OUTPUT_GRID_INTERVAL=TICK_MS, OUTPUT_STATES_INTERVAL=TICK_MS)


_ctx = {}


def _setup(mesh_base, ints, reals):
    from oracle import Oracle, Mesh, Reference
    from oracle import linescan
    m = Mesh(Oracle(), mesh_base, 1, np.array(reals))
    el = m.elements()
    W, pad = linescan.weights(mesh_base, el["order"], LINESCAN, V0=el["V0"])
    _ctx.update(m=m, W=W, pad=pad, ref=Reference(), ints=np.array(ints, np.int32))


def _run(args):
    idx, mesh_base, ints, reals, work = args
    out = os.path.join(work, "run%05d.npz" % idx)
    if os.path.exists(out):
        return idx
    if not _ctx:
        _setup(mesh_base, ints, reals)
    rows, _, ls = _ctx["ref"].run_simulation_linescan(_ctx["m"], _ctx["ints"], _ctx["W"], _ctx["pad"],
                                                      rank=0, index=idx)
    tmp = out + ".part.npz"
    np.savez(tmp, ls=ls, rows=rows)
    os.replace(tmp, out)
    return idx


def assemble(work, n_runs, dest):
    from ks_metrics import NAMES, spark_metrics
    from ks_mixture import atom_mask
    p = params()
    ns = int((LINESCAN["x_max"] - LINESCAN["x_min"]) / LINESCAN["res"])
    centre, lccs, metrics = [], [], []
    for i in range(n_runs):
        d = np.load(os.path.join(work, "run%05d.npz" % i))
        ls, rows = d["ls"], d["rows"]
        if len(ls) < N_TICKS + 1 or len(rows) < N_TICKS + 1:
            raise SystemExit("run %d: %d line-scan rows, %d states rows" % (i, len(ls), len(rows)))
        c = ls[:N_TICKS + 1, 1 + ns // 2]
        n = rows[:N_TICKS + 1, 2]
        centre.append(c.astype(np.float64))
        lccs.append(int(rows[:N_TICKS + 1, 3].max()))
        metrics.append(spark_metrics(c, n, TICK_MS))
    # The runs in which no channel opens besides the held RyR share one
    # deterministic trajectory, so their line-scan traces are bit-identical:
    # the atom is the set of runs whose trace equals the most frequent one.
    # (The open counts at the ticks cannot tell: a RyR or an LCC may open and
    # close again between two ticks.)
    metrics, lccs, centre = np.array(metrics), np.array(lccs, np.int8), np.array(centre)
    atom = atom_mask(centre)
    mode = centre[np.nonzero(atom)[0][0]]
    np.savez_compressed(dest, metrics=metrics, names=np.array(NAMES), max_lcc_open=lccs, atom=atom,
                        atom_dff0=(mode / mode[0] - 1.0),
                        ints=np.array(list(p.ints)), reals=np.array(list(p.reals)),
                        window_ms=WINDOW_MS, tick_ms=TICK_MS)
    print("wrote", dest, "from", n_runs, "runs")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--work", required=True)
    ap.add_argument("--runs", type=int, default=1000)
    ap.add_argument("--procs", type=int, default=os.cpu_count())
    ap.add_argument("--assemble-only", action="store_true")
    a = ap.parse_args()
    os.makedirs(a.work, exist_ok=True)
    dest = os.path.join(HERE, "ks_config1.npz")
    if not a.assemble_only:
        import srs_gb300 as srs
        base = os.path.join(a.work, "dyad12")
        srs.write_box_mesh(base)  # the generator's defaults are this mesh
        p = params()
        jobs = [(i, base, list(p.ints), list(p.reals), a.work) for i in range(a.runs)]
        t0 = time.time()
        with mp.get_context("spawn").Pool(a.procs) as pool:
            for k, _ in enumerate(pool.imap_unordered(_run, jobs)):
                if k % 25 == 0:
                    print("%d / %d runs, %.0f s" % (k + 1, a.runs, time.time() - t0), flush=True)
    assemble(a.work, a.runs, dest)


if __name__ == "__main__":
    main()
