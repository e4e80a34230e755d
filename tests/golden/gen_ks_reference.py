"""Reference ensemble for the distribution tests (KS) of stochastic outputs.

Runs the reference's own cpu/RunSimulation.cpp (compiled in oracle/_ref)
for many realizations of one protocol on the golden mesh, varying the
ensemble index so each run draws its own glibc rand() stream (seed rule of
cpu/RunSimulation.cpp:446), and stores per-run summary metrics of the
states rows:

  peak_ca      maximum of the mean cleft Ca at the RyRs (row column 6), uM
  t_peak       time of that maximum, ms
  fdhm         full duration at half maximum of (column 6 - its t=0 value), ms
  max_open     maximum number of open RyRs at the output ticks (column 2)
  open_time    sum over ticks of open RyRs x tick interval (RyR open time), ms

    python tests/golden/gen_ks_reference.py [n_runs]

Output: ks_reference.npz (metrics per run + the parameter vectors).
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
MESH = os.path.join(HERE, "mesh", "dyad")


def ks_params():
    """Spark protocol on the golden mesh: RyR 4 opened at t = 0, 1 ms, with
    a RyR opening rate constant 20x the default so that neighbouring RyRs
    are recruited within the window (more stochastic structure to compare)."""
    import srs_gb300 as srs
    return srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=4,
                                        INIT_RYR_HOLD=0.0, T_FINAL=1.0,
                                        OUTPUT_STATES_INTERVAL=0.005, RYR_K_PLUS=2.214e-3)


def metrics(rows):
    """Summary metrics of one run's states rows (see module docstring)."""
    t = rows[:, 0].astype(np.float64)
    ca = rows[:, 6].astype(np.float64)
    n_open = rows[:, 2].astype(np.float64)
    k = int(np.argmax(ca))
    base = ca[0]
    half = base + 0.5 * (ca[k] - base)
    above = np.where(ca >= half)[0]
    fdhm = float(t[above[-1]] - t[above[0]]) if len(above) else 0.0
    dt_tick = float(np.median(np.diff(t[1:-1]))) if len(t) > 3 else 0.0
    return [float(ca[k]), float(t[k]), fdhm, float(n_open.max()), float(n_open[1:-1].sum() * dt_tick)]


def _run(args):
    idx, ints, reals = args
    sys.path.insert(0, ROOT)
    from oracle import Oracle, Mesh, Reference
    m = Mesh(Oracle(), MESH, 1, np.array(reals))
    rows, _ = Reference().run_simulation(m, np.array(ints), rank=0, index=idx)
    return metrics(rows)


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 1000
    p = ks_params()
    ints, reals = list(p.ints), list(p.reals)
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        out = pool.map(_run, [(i, ints, reals) for i in range(n)], chunksize=4)
    np.savez_compressed(os.path.join(HERE, "ks_reference.npz"), metrics=np.array(out),
                        ints=np.array(ints), reals=np.array(reals),
                        names=np.array(["peak_ca", "t_peak", "fdhm", "max_open", "open_time"]))
    print("wrote", len(out), "runs")


if __name__ == "__main__":
    main()
