"""Autotuners of the FP32 engines.

tune_resident: the resident engine's cluster size (CTAs sharing one
realization) and threads per CTA for a given grid and batch, by timing short
trial launches of each candidate on the device (CUDA events on the engine's
stream).  The time steps per persistent launch are not searched: they are
the caller's output cadence (the launch ends at every states-row or
grid-file tick).

tune_plain: the L2 prefetch distance of the plain engine's large-mesh form.  Results are cached per (element count, channel count,
realizations, device) in a JSON file next to the package, so later runs start
with the tuned configuration.
"""
import json
import os

import srs_gb300 as srs

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_tuned.json")


def _key(grid, R):
    try:
        import torch
        dev = torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001 - the name only labels the cache entry
        dev = "cuda"
    return "%s|N%d|R%d|L%d|B%d" % (dev, grid.n_ele, grid.n_ryr, grid.n_lcc, R)


def tune_resident(grid, params, R, seeds=None, clusters=(1, 2, 3, 4, 5, 6, 8, 16),
                  threads=(160, 192, 224, 256, 288, 320, 352, 384, 448, 512, 640), trial_steps=200,
                  repeats=2, use_cache=True, verbose=False):
    """Returns dict(cluster_size, threads_per_cta, ms_per_step, trials).
    Clusters of 16 CTAs (non-portable) are among the candidates: they halve
    the partition of meshes that fit eight CTAs only one CTA per SM."""
    key = _key(grid, R)
    cache = {}
    if use_cache and os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except ValueError:
            cache = {}
        if key in cache:
            return cache[key]
    trials = []
    for C in clusters:
        for T in threads:
            try:
                sim = srs.Simulation(grid, params, R, srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                                     threads_per_cta=T, cluster_size=C,
                                     steps_per_launch=trial_steps)
            except srs.SrsError as e:
                if verbose:
                    print("tuner: C=%d T=%d skipped (%s)" % (C, T, e))
                continue
            sim.advance_async(trial_steps)
            sim.synchronize()
            ms = min(sim.time_advance(trial_steps) for _ in range(repeats))
            trials.append(dict(cluster_size=C, threads_per_cta=T, ms_per_step=ms / trial_steps))
            if verbose:
                print("tuner: C=%d T=%d %.4f ms/step" % (C, T, ms / trial_steps))
            del sim
    if not trials and 16 not in clusters:
        # large grids: non-portable 16-CTA clusters
        return tune_resident(grid, params, R, seeds, clusters=(16,), threads=threads,
                             trial_steps=trial_steps, repeats=repeats, use_cache=use_cache,
                             verbose=verbose)
    if not trials:
        raise RuntimeError("no resident configuration fits this grid")
    best = min(trials, key=lambda d: d["ms_per_step"])
    out = dict(best, trials=trials)
    if use_cache:
        cache[key] = out
        try:
            json.dump(cache, open(CACHE, "w"), indent=1)
        except OSError:
            pass
    return out


def tune_plain(grid, params, R, seeds=None, waves=(0.0, 0.5, 1.0, 2.0, 4.0), trial_steps=32,
               repeats=2, use_cache=True, verbose=False):
    """Prefetch distance of the plain FP32 engine's large-mesh form (meshes of
    65,536 elements and more): each update block asks L2 for the state of the
    element block `distance` blocks ahead.  Candidates are fractions of one
    wave (six blocks per SM over the realizations); each is timed over short
    trial advances.  Returns dict(prefetch_blocks, ms_per_step, trials)."""
    import torch
    n_sm = torch.cuda.get_device_properties(0).multi_processor_count
    wave = max(1, (n_sm * 6 + R - 1) // R)
    key = "plain|" + _key(grid, R)
    cache = {}
    if use_cache and os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except ValueError:
            cache = {}
        if key in cache:
            return cache[key]
    sim = srs.Simulation(grid, params, R, srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    sim.advance_async(trial_steps)
    sim.synchronize()
    trials = []
    for w in sorted(set(int(round(f * wave)) for f in waves)):
        sim.set_prefetch(w)
        sim.time_advance(trial_steps)  # new graph for this distance
        ms = min(sim.time_advance(trial_steps) for _ in range(repeats))
        trials.append(dict(prefetch_blocks=w, ms_per_step=ms / trial_steps))
        if verbose:
            print("tuner: prefetch %d blocks %.4f ms/step" % (w, ms / trial_steps))
    del sim
    best = min(trials, key=lambda d: d["ms_per_step"])
    out = dict(best, trials=trials, wave_blocks=wave)
    if use_cache:
        cache[key] = out
        try:
            json.dump(cache, open(CACHE, "w"), indent=1)
        except OSError:
            pass
    return out
