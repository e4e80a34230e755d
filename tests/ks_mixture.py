"""Distribution comparison of spark metrics whose distribution has an atom.

Runs in which no channel besides the initially opened RyR changes state
within the window follow one deterministic trajectory, so every metric of
those runs takes one value: the metric distributions are a mixture of that
atom and a continuous part.  The reference computes the atom in FP64, the
FP32 engine within its deterministic tolerance of it, not bit for bit, so a
plain two-sample KS test would see two atoms a hair apart and fail for a
reason that is not stochastic.  The mixture is compared in parts instead:

  mass        the fraction of atom runs, Fisher's exact test, p > 0.01
  continuous  every metric over the non-atom runs, two-sample KS, p > 0.01
  value       the atom runs' trajectory against the reference's (the caller
              checks it at the deterministic tolerance)

Together these test that the two mixtures are the same distribution.  Atom
runs are identified by the same exact criterion in both ensembles: counts of
open channels at the output ticks (golden-mesh test), or a recorded trace
bit-identical to the ensemble's most frequent one (atom_mask; config-1 test,
where a channel may open and close again between two ticks).
"""


def atom_mask(traces):
    """Runs whose trace is bit-identical to the most frequent trace.  The runs
    in which no channel opens besides the held RyR follow one deterministic
    trajectory, which an engine computes the same way in every run."""
    import numpy as np
    keys = [t.tobytes() for t in np.ascontiguousarray(traces)]
    counts = {}
    for k in keys:
        counts[k] = counts.get(k, 0) + 1
    mode = max(counts, key=counts.get)
    return np.array([k == mode for k in keys])


def mixture_ks(ref, gpu, ref_atom, gpu_atom, names, p_min=0.01):
    """ref, gpu: [runs][metrics]; *_atom: boolean masks.  Returns
    (report, failures): report[name] = (p, ref mean, gpu mean) over the
    non-atom runs, report['atom_mass'] = (p, ref fraction, gpu fraction)."""
    from scipy import stats
    report, bad = {}, {}
    table = [[int(ref_atom.sum()), int((~ref_atom).sum())],
             [int(gpu_atom.sum()), int((~gpu_atom).sum())]]
    p_mass = float(stats.fisher_exact(table)[1])
    report["atom_mass"] = (p_mass, float(ref_atom.mean()), float(gpu_atom.mean()))
    if not p_mass > p_min:
        bad["atom_mass"] = report["atom_mass"]
    a, b = ref[~ref_atom], gpu[~gpu_atom]
    for k, name in enumerate(names):
        res = stats.ks_2samp(a[:, k], b[:, k])
        report[name] = (float(res.pvalue), float(a[:, k].mean()), float(b[:, k].mean()))
        if not report[name][0] > p_min:
            bad[name] = report[name]
    return report, bad


def plain_ks(ref, gpu, names):
    """KS p-values of the metrics over all runs, atoms included (reported,
    not asserted: see the module docstring)."""
    from scipy import stats
    return {name: float(stats.ks_2samp(ref[:, k], gpu[:, k]).pvalue) for k, name in enumerate(names)}
