"""Spark metrics of a line-scan trace.

The reference ships no definition of these metrics (its line-scan tool,
linescan/main.cpp, writes F(x, t) only), so this one definition is applied
to every run here and to the reference ensembles the tests compare with.
Inputs are one run's line scan of the bound dye at the grid-file ticks
t_k = k * interval (k = 0 .. K, t_0 the initial state) and its states-row
RyR open counts at the same ticks (column 2 of the rows of
cpu/OutputFuncs.cpp:241-350).

  amplitude   max_k dF/F0 at the centre sample, dF/F0 = F / F(t_0) - 1
  t_peak      t_k at that maximum, ms
  fdhm        full duration at half maximum of the centre dF/F0, ms: from the
              first to the last half-maximum crossing, each linearly
              interpolated between ticks (the window end when the trace is
              still above half maximum there)
  max_open    maximum number of open RyRs over the ticks
  open_time   sum over ticks of open RyRs x interval (RyR open time), ms
  t_recruit   first tick with more RyRs open than at t_0 (window end + one
              interval when none), ms
"""
import numpy as np

NAMES = ("amplitude", "t_peak", "fdhm", "max_open", "open_time", "t_recruit")


def spark_metrics(centre, n_open, interval):
    """centre: F at the centre sample per tick (k = 0..K); n_open: open RyRs
    per tick (same ticks).  Returns the NAMES values."""
    f = np.asarray(centre, np.float64)
    n = np.asarray(n_open, np.float64)
    K = len(f) - 1
    c = f / f[0] - 1.0
    k = int(np.argmax(c))
    amp = float(c[k])
    half = 0.5 * amp
    above = np.nonzero(c >= half)[0]
    if amp <= 0 or len(above) == 0:
        fdhm = 0.0
    else:
        i0, i1 = int(above[0]), int(above[-1])
        t0 = i0 * interval
        if i0 > 0:
            t0 = (i0 - 1 + (half - c[i0 - 1]) / (c[i0] - c[i0 - 1])) * interval
        t1 = i1 * interval
        if i1 < K:
            t1 = (i1 + (c[i1] - half) / (c[i1] - c[i1 + 1])) * interval
        fdhm = float(t1 - t0)
    more = np.nonzero(n > n[0])[0]
    t_rec = float(more[0] * interval) if len(more) else float((K + 1) * interval)
    return [amp, float(k * interval), fdhm, float(n.max()), float(n.sum() * interval), t_rec]
