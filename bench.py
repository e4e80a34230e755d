#!/usr/bin/env python
"""Throughput of the batched spark timestep on GB300.

Workload (config 1): the 10,368-element box dyad (12^3 hexahedra, 49 RyRs,
7 LCCs), DefaultSpark parameters at dt = 9 ns, 1024 independent
realizations (Philox seeds 1..1024) with FP32 state, run by the resident
persistent engine under the reference's RunSimulation protocol for
DefaultSpark (RyR 24 held open, output rows).  One bench step = one
persistent launch that advances all realizations by --launch-steps time
steps.

Metric: simulated spark-ms per wall second (sum over realizations).
  value      device-resident: one run of W + K launches from the equilibrium
             state (uploaded before the run); CUDA events on the engine's
             stream around each launch, the last K summed.  The state
             (1024 x 10,368 x 20 B = 212 MB) is larger than the 129 MB L2, so
             no flush is needed.
  e2e        through the public API with host buffers: srs_sim_reset
             (initial state uploaded from pinned host memory) +
             srs_run_simulation (RunSimulation protocol, states rows read
             back) for --launch-steps steps, per bench step.
  roofline   algorithmic bytes of the dominant kernel per launch =
             elements x realizations x steps x (48 + 44/R) B (FP32 state
             read+write of 6 species-slots and shared geometry), divided by
             the measured launch time, against the measured HBM copy peak.
             Values above 1 are "effective": the engine keeps each
             realization on chip for a whole launch.
  cpu_baseline  the oracle port (RunSimulation of the reference, restated in
             C) on the host cores, one realization per process.

--impl reference times the reference's CPU implementation (oracle/_ref when
it was built from the reference sources, else the oracle port) on the host
cores for the same metric.

Multi-GPU (torchrun, N > 1): replicas only — each rank runs its own 1024
realizations (seeds offset by rank); no collective on the data path; timing
is max over ranks.
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DT_MS = 9e-6
METRIC = "simulated spark-ms/s (batched 1024-realization dyad, config 1)"
UNIT = "spark-ms/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--realizations", type=int, default=1024)
    ap.add_argument("--launch-steps", type=int, default=2000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-tune", action="store_true", help="use the default configuration")
    ap.add_argument("--cluster-size", type=int, default=0, help="with --no-tune: this cluster size")
    ap.add_argument("--threads", type=int, default=0, help="with --no-tune: threads per CTA")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint cost leg")
    ap.add_argument("--adjoint-realizations", type=int, default=64)
    ap.add_argument("--adjoint-steps", type=int, default=4096)
    ap.add_argument("--no-config2", action="store_true", help="skip the multi-mesh batch leg")
    ap.add_argument("--no-config4", action="store_true", help="skip the large-site leg")
    ap.add_argument("--no-config0", action="store_true", help="skip the single-spark leg")
    ap.add_argument("--config0-ms", type=float, default=20.0)
    ap.add_argument("--fp64-steps", type=int, default=22222,
                    help="steps of the FP32-vs-FP64 error check of the config-1 engine")
    ap.add_argument("--config4-steps", type=int, default=4096)
    ap.add_argument("--config4-realizations", type=int, default=32,
                    help="realizations of the large-site leg (32: the workload; fewer for profiling)")
    ap.add_argument("--config4-adjoint-steps", type=int, default=1024,
                    help="steps of the large-site adjoint sample (0: skip it)")
    ap.add_argument("--only", choices=["adjoint", "config0", "config2", "config4", "blocking"],
                    default=None,
                    help="run one secondary leg alone and print its JSON (profiling; 'blocking': "
                         "the temporal-blocking measurement of the large site)")
    ap.add_argument("--adjoint-checkpoint", type=int, default=-1,
                    help="with --only adjoint: one checkpoint interval (0: whole trajectory)")
    ap.add_argument("--config2-ms", type=float, default=2.0,
                    help="simulated window of the multi-mesh batch leg (both protocols)")
    ap.add_argument("--config2-no-alone", action="store_true",
                    help="config2: skip the members-one-after-another comparison (long windows)")
    ap.add_argument("--config2-launch-steps", type=int, default=0,
                    help="steps per member launch in one graph replay (0: one states interval)")
    ap.add_argument("--adjoint-threads", type=int, default=0, help="reverse-sweep threads per CTA")
    ap.add_argument("--adjoint-flags", type=int, default=0, help="srs_adjoint_desc flags")
    ap.add_argument("--adjoint-partitions", type=int, default=0,
                    help="forward partitions per reverse-sweep CTA")
    return ap.parse_args()


# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend)
    return dist


def replica_seeds(rank, R):
    """Philox keys of rank `rank`'s replica: disjoint across ranks."""
    return [1 + rank * R + i for i in range(R)]


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(prefix="srs_clocks_", suffix=".csv")
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1].split()[0]))
                smax.append(float(t[2].split()[0]))
            except ValueError:
                continue
            for n, v in zip(names, t[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """dram bytes per launch of the resident kernel from the committed ncu
    summary (profiles/k_resident32_config1.md, line 'dram_bytes_per_launch:')."""
    p = os.path.join(ROOT, "profiles", "k_resident32_config1.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------------------------
def _cpu_worker(args):
    """One realization of RunSimulation (oracle port, reference gating) for
    n steps on the config mesh; returns the wall seconds of the time loop."""
    base, ints, reals, n_steps, rank = args
    sys.path.insert(0, ROOT)
    import numpy as np
    from oracle import Oracle, Mesh, RNG_REFERENCE, Reference
    reals = np.array(reals)
    reals[0] = (n_steps - 0.5) * reals[1]  # t_final: n_steps steps
    m = Mesh(Oracle(), base, 1, reals)
    t0 = time.perf_counter()
    m.run_simulation(np.array(ints), RNG_REFERENCE, rank, 0)
    return time.perf_counter() - t0


def _ref_worker(args):
    """Same sample through the reference's own RunSimulation (oracle/_ref)."""
    base, ints, reals, n_steps, rank = args
    sys.path.insert(0, ROOT)
    import numpy as np
    from oracle import Oracle, Mesh, Reference
    reals = np.array(reals)
    reals[0] = (n_steps - 0.5) * reals[1]
    m = Mesh(Oracle(), base, 1, reals)
    ref = Reference()
    t0 = time.perf_counter()
    ref.run_simulation(m, np.array(ints), rank=rank)
    return time.perf_counter() - t0


def reference_available():
    return os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libsrsref.so"))


def cpu_sample(base, ints, reals, seconds, cores=None, prefer_reference=False):
    """Times RunSimulation on `cores` processes; returns (spark-ms/s, cores, kind, sample)."""
    cores = cores or os.cpu_count() or 1
    ints, reals = list(ints), list(reals)
    # calibrate: ~31M element-steps/s per core -> steps for the requested seconds
    kind = "reference" if (prefer_reference and reference_available()) else "port"
    worker = _ref_worker if kind == "reference" else _cpu_worker
    probe = worker((base, ints, reals, 200, 0))
    n_steps = max(200, int(200 * seconds / max(probe, 1e-3)))
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        loops = pool.map(worker, [(base, ints, reals, n_steps, r) for r in range(cores)])
        wall = time.perf_counter() - t0
    # metric over the time loops (setup excluded like the reference's clock())
    span = max(loops)
    value = cores * n_steps * DT_MS / span
    sample = ("%d processes x 1 realization x %d steps (%.3g ms simulated each) of the config-1 "
              "mesh, RunSimulation with reference gating; loop time %.1f s, wall %.1f s"
              % (cores, n_steps, n_steps * DT_MS, span, wall))
    return value, cores, kind, sample


def write_config_mesh_host(directory):
    """Writes the config-1 box dyad with the host-only mesh writer
    (srs_gb300/bin/srs_meshgen, built from meshgen.cpp alone; compiled here
    with g++ when absent), so that the CPU legs load no CUDA library."""
    exe = os.path.join(ROOT, "srs_gb300", "bin", "srs_meshgen")
    if not os.path.exists(exe):
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "_srs_build", os.path.join(ROOT, "srs_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        exe = mod.build_meshgen(os.path.join(directory, "srs_meshgen"))
    base = os.path.join(directory, "dyad12")
    subprocess.run([exe, "-out", base], check=True, stdout=subprocess.DEVNULL)
    return base


# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference arm: the reference's RunSimulation (oracle/_ref, built
    from the reference sources where they are present, else the oracle's C
    restatement of it, bit-exact with the reference) on the host cores.  It
    loads only the oracle libraries: parameters from oracle/params.py, the
    mesh from the host-only mesh writer."""
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    from oracle import params as op
    tmp = tempfile.mkdtemp(prefix="srs_bench_")
    base = write_config_mesh_host(tmp)
    ints, reals = op.default_spark()
    per_step = max(2.0, 60.0 / max(1, args.steps + args.warmup))
    vals = []
    for i in range(args.warmup + args.steps):
        v, cores, kind, sample = cpu_sample(base, ints, reals, per_step, prefer_reference=True)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "config1 box dyad 10,368 elements, DefaultSpark dt=9ns, "
                               "one realization per host core", "realizations_per_step": cores},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# Parameters of the adjoint leg's target run (+10 %): the diffusion
# coefficients of Ca and dye, calmodulin / troponin / SL-site buffering, RyR
# unit flux and SERCA.
TARGET_PERTURBED = ("D_CA", "D_DYE", "K_ON_CMDN", "K_OFF_CMDN", "K_ON_TRPN", "K_OFF_TRPN",
                    "B_TOT_SL_HI", "K_D_SL_HI", "V_RYR", "A_P")


def adjoint_cost(srs, grid, p, args):
    """Cost of the pathwise adjoint against the forward pass it differentiates
    (config 3, a bounded sample of its 10 ms): the config mesh x R
    realizations, n explicit steps with gating, the x line scan through the
    cluster sampled every 128 steps, the loss the L2 misfit of the
    realizations' mean dF/F0 trace against the mean trace of a run with the
    same seeds and the parameters in TARGET_PERTURBED raised by 10 %; wall
    time of srs_adjoint (forward pass, with checkpoints every 256 steps and
    segment recomputation, or keeping the whole trajectory; reverse sweep)
    over wall time of the same n steps of the resident engine."""
    import numpy as np
    import torch
    Ra, n, te = args.adjoint_realizations, args.adjoint_steps, 128
    from srs_gb300 import tuner
    if args.no_tune:
        t = dict(cluster_size=args.cluster_size, threads_per_cta=args.threads)
    else:
        t = tuner.tune_resident(grid, p, Ra, seeds=list(range(1, Ra + 1)))
    sim = srs.Simulation(grid, p, Ra, srs.FP32, srs.ENGINE_RESIDENT, seeds=list(range(1, Ra + 1)),
                         cluster_size=t["cluster_size"], threads_per_cta=t["threads_per_cta"],
                         steps_per_launch=256)
    ns = sim.linescan_setup(axis=0, offset1=0.0, offset2=0.1, x_min=-1.0, x_max=1.0, res=0.05,
                            var_x=0.0289, var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=0.0,
                            pad_res=0.0, pad_min=0.0, pad_max=0.0, domain=(0, 0, 0, 0, 0, 0))
    sim.reset()
    _, f0 = sim.linescan()
    # target: mean dF/F0 trace of the perturbed run (its own F0), same seeds
    pt = p.copy()
    for name in TARGET_PERTURBED:
        pt.reals[srs.R[name]] *= 1.1
    simt = srs.Simulation(srs.Grid(pt, grid.mesh_base), pt, Ra, srs.FP32, srs.ENGINE_RESIDENT,
                          seeds=list(range(1, Ra + 1)), cluster_size=t["cluster_size"],
                          threads_per_cta=t["threads_per_cta"], steps_per_launch=te)
    simt.reset()
    simt.linescan_setup(axis=0, offset1=0.0, offset2=0.1, x_min=-1.0, x_max=1.0, res=0.05,
                        var_x=0.0289, var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=0.0,
                        pad_res=0.0, pad_min=0.0, pad_max=0.0, domain=(0, 0, 0, 0, 0, 0))
    _, f0t = simt.linescan()
    target = np.zeros((n // te, ns))
    for k in range(n // te):
        simt.advance_async(te)
        Ft, _ = simt.linescan()
        target[k] = Ft.mean(0) / f0t - 1.0
    del simt
    flags = args.adjoint_flags | srs.ADJ_MEAN_TRACE
    sim.adjoint(512, te, f0, target[:512 // te], checkpoint_every=256, flags=flags)  # warm-up
    sim.reset()
    sim.time_advance(512)
    sim.reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.advance_async(n)
    sim.synchronize()
    fwd = time.perf_counter() - t0
    out = {"workload": "adjoint: config mesh x %d realizations, %d steps, line scan of %d samples "
                       "every %d steps" % (Ra, n, ns, te),
           "cluster_size": sim.config()["cluster_size"], "forward_s": fwd}
    # K = 256: checkpoint + recompute; K = n: the forward pass keeps the trajectory
    modes = ((256, "checkpoint_256"), (n, "whole_trajectory"))
    if args.adjoint_checkpoint >= 0:
        K1 = args.adjoint_checkpoint or n
        modes = ((K1, "checkpoint_%d" % K1),)
    for K, key in modes:
        sim.reset()
        kw = dict(checkpoint_every=K, threads_per_cta=args.adjoint_threads,
                  cta_partitions=args.adjoint_partitions, flags=flags)
        sim.adjoint(n, te, f0, target, **kw)  # warm: work buffers of this mode
        sim.reset()
        t0 = time.perf_counter()
        loss, grad, _ = sim.adjoint(n, te, f0, target, **kw)
        adj = time.perf_counter() - t0
        if not np.isfinite(grad).all():
            raise SystemExit("non-finite adjoint gradient")
        g = grad.sum(0)
        out[key] = {"adjoint_s": adj, "cost_ratio": adj / fwd, "loss": float(loss[0]),
                    "grad": {name: float(g[k]) for k, name in enumerate(srs.ADJ_PARAMS)}}
    return out


def plain_one_realization(srs, grid, p, n=4000):
    """The plain form the batched engine is measured against: one realization,
    one fused step kernel per time step (graph-replayed), FP32 and FP64."""
    out = {}
    for name, prec in (("fp32", srs.FP32), ("fp64", srs.FP64)):
        sim = srs.Simulation(grid, p, 1, prec, srs.ENGINE_PLAIN, seeds=[1])
        sim.reset()
        sim.time_advance(256)
        ms = sim.time_advance(n)
        out[name] = {"value": n * DT_MS / (ms / 1e3), "unit": UNIT, "us_per_step": 1e3 * ms / n}
    return out


def config2_batch(srs, args):
    """Uneven multi-mesh batch: four box dyads (6k / 15k / 30k / 60k tets,
    Poisson-disk clusters of 10 / 25 / 60 / 100 RyRs, one LCC per 7 RyRs) x
    two protocols (leak: clamped at rest, no trigger, 100 ms; LCC-triggered:
    clamped at 0 mV, 30 ms, as param/Gain_0mV.xml) x 32 realizations = 256
    realizations, each member at its tuned resident configuration, run by
    srs_batch_run_simulation (the members' resident launches as branches of
    one CUDA graph, the RunSimulation protocol on: LCC gating and clamp,
    states rows on the device) over the first --config2-ms of both protocols
    (a bounded sample of the 30 / 100 ms runs, each protocol capped at its own
    length; the whole runs are projected from it).  Reported against the same members run one after another
    (srs_run_simulation each), with the roofline of the batch (algorithmic
    48 + 44/R B per element-step of every member)."""
    import numpy as np
    from srs_gb300 import tuner
    from srs_gb300 import workloads as wl
    tmp = tempfile.mkdtemp(prefix="srs_c2_")
    W = args.config2_ms
    members, seed0 = [], 1
    for base, rep_ in wl.config2_meshes(tmp):
        for k, p in enumerate(wl.config2_protocols(rep_["max_a0"])):
            full = p.reals[srs.R["T_FINAL"]]
            p.set(T_FINAL=min(W, full))
            g = srs.Grid(p, base)
            seeds = list(range(seed0, seed0 + 32))
            seed0 += 32
            # alone, a member's 32 realizations leave SMs idle, so its best
            # configuration buys parallelism with larger clusters; in the
            # batch the other members fill those SMs, so there the
            # configuration that is fastest per element-step on a full GPU
            # (tuned on 256 realizations) is used
            t = tuner.tune_resident(g, p, 32, seeds=seeds)
            tb = tuner.tune_resident(g, p, 256, seeds=list(range(1, 257)))
            members.append(dict(grid=g, p=p, seeds=seeds, tune=t, tune_batch=tb, n_tets=rep_["n_tets"],
                                protocol=("leak", "lcc_trigger")[k], full_ms=full))

    def make(S, which):
        out = []
        for m in members:
            sim = srs.Simulation(m["grid"], m["p"], 32, srs.FP32, srs.ENGINE_RESIDENT, seeds=m["seeds"],
                                 cluster_size=m[which]["cluster_size"],
                                 threads_per_cta=m[which]["threads_per_cta"], steps_per_launch=S)
            sim.reset()
            out.append(sim)
        return out

    def launch_steps(m):
        p = m["p"]
        return int(round(p.reals[srs.R["OUTPUT_STATES_INTERVAL"]] / p.reals[srs.R["T_STEP"]]))

    S = args.config2_launch_steps or max(launch_steps(m) for m in members)
    # warm-up: one graph replay of every member
    sims = make(S, "tune_batch")
    srs.Batch(sims, steps_per_launch=S).time_advance(S)
    # members one after another, each at its own tuned configuration
    one_rows, one_each = [], []
    if not args.config2_no_alone:
        sims = make(S, "tune")
        torch_sync()
        for sim in sims:
            t0 = time.perf_counter()
            one_rows.append(sim.run_simulation())
            one_each.append(time.perf_counter() - t0)
    one_s = sum(one_each) if one_each else None
    # the batch
    sims = make(S, "tune_batch")
    b = srs.Batch(sims, steps_per_launch=S)
    torch_sync()
    t0 = time.perf_counter()
    outs = b.run_simulation()
    batch_s = time.perf_counter() - t0
    spark_ms, alg, per = 0.0, 0.0, []
    alone = list(zip(one_rows, one_each)) if one_each else [((None, None, None), None)] * len(members)
    for m, sim, (rows, t_end, n_steps), ((rows1, _, n1), t1) in zip(members, sims, outs, alone):
        dt = m["p"].reals[srs.R["T_STEP"]]
        if n1 is not None and not np.array_equal(n_steps, n1):
            raise RuntimeError("batch and one-by-one runs differ in length")
        spark_ms += float(n_steps.sum()) * dt
        alg += float(n_steps.sum()) * m["n_tets"] * (48.0 + 44.0 / sim.R)
        max_open = [float(r[:, 2].max()) for r in rows]
        lcc_open = [float(r[:, 3].max()) for r in rows]
        per.append({"tets": m["n_tets"], "protocol": m["protocol"],
                    "cluster_size": sim.config()["cluster_size"],
                    "threads_per_cta": sim.config()["threads_per_cta"],
                    "alone_cluster_size": m["tune"]["cluster_size"],
                    "alone_threads_per_cta": m["tune"]["threads_per_cta"], "steps": int(n_steps.max()),
                    "alone_s": t1, "alone_ps_per_element_step":
                        1e12 * t1 / (float(n_steps.sum()) * m["n_tets"]) if t1 is not None else None,
                    "runs_with_lcc_opening": int(sum(x > 0 for x in lcc_open)),
                    "runs_with_recruited_ryr": int(sum(x > 0 for x in max_open)),
                    "mean_max_open_ryr": float(np.mean(max_open))})
    peak, peak_kind = measured_peaks()
    rate = spark_ms / batch_s
    return {"workload": "config2: 4 meshes (6000/15288/29478/60984 tets; 10/25/60/100 RyR) x "
                        "2 protocols x 32 realizations, RunSimulation protocol, first %.3g ms" % W,
            "value": rate, "unit": UNIT, "batch_s": batch_s, "members_one_by_one_s": one_s,
            "batch_over_one_by_one": one_s / batch_s if one_s else None, "steps_per_launch": S,
            "roofline": {"bound": "hbm", "achieved": alg / batch_s / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / batch_s / 1e9 / peak,
                         "note": "effective: algorithmic 48 + 44/R B per element-step of every "
                                 "member, wall time of srs_batch_run_simulation; peak %s" % peak_kind},
            # the whole runs (leak 100 ms, LCC-triggered 30 ms) at this window's rate
            "projected_full_runs_s": sum(32 * m["full_ms"] for m in members) / rate,
            "members": per}


def torch_sync():
    import torch
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def fp64_error(srs, grid, p, n, engine, **sim_kw):
    """Error of an FP32 engine against the FP64 engine (the same per-element
    arithmetic in FP64, bit-exact with the FP64 oracle) over the deterministic
    part of the workload: n steps with gating off and the protocol's source
    (RyR 24 held open) from rest, two FP32 realizations against one FP64 run.
    Error: max over elements and species of |c32 - c64| / max(|c64|, 1e-3 uM)."""
    import numpy as np
    pd = p.copy().set(FLAG_NO_GATING=1)
    s64 = srs.Simulation(grid, pd, 1, srs.FP64, srs.ENGINE_PLAIN, seeds=[1])
    s32 = srs.Simulation(grid, pd, 2, srs.FP32, engine, seeds=[1, 2], **sim_kw)
    s64.explicit_step(n)
    s32.explicit_step(n)
    ref = s64.get_state(0)["states"]
    err = max(float(np.max(np.abs(s32.get_state(r)["states"] - ref) / np.maximum(np.abs(ref), 1e-3)))
              for r in range(2))
    return {"max_rel": err, "bar": 1e-5, "steps": n, "simulated_ms": n * DT_MS,
            "engine": "resident" if engine == srs.ENGINE_RESIDENT else "plain",
            "against": "FP64 plain engine, gating off"}


def mass_balance(srs, grid, p, n, engine, **sim_kw):
    """Mass balance of an FP32 engine with every Ca source and sink across the
    compartment boundary off (SERCA A_P = 0, JSR refill V_REFILL = 0, LCCs
    closed and gating off, no-flux boundaries), RyR 24 held open so Ca moves
    from the JSR into the cytosol: over n steps the total Ca of cytosol + JSR
    (free, bound and rapid-buffer Ca, FP64 sums of the state: srs_sim_total_ca)
    must stay constant.  Returns the relative change of the total and the
    moved fraction (the JSR's loss relative to the total)."""
    import numpy as np
    pm = p.copy().set(A_P=0.0, V_REFILL=0.0, FLAG_NO_GATING=1, FLAG_NO_FLUX_BOUNDARY=1)
    sim = srs.Simulation(grid, pm, 2, srs.FP32, engine, seeds=[1, 2], **sim_kw)
    t0 = np.asarray(sim.total_ca())
    sim.explicit_step(n)
    t1 = np.asarray(sim.total_ca())
    tot0, tot1 = t0.sum(1), t1.sum(1)
    return {"steps": n, "total_rel_change": float(np.max(np.abs(tot1 - tot0) / tot0)),
            "moved_rel": float(np.max((t0[:, 1] - t1[:, 1]) / tot0)),
            "sources": "SERCA, refill, LCC and boundary fluxes off; RyR 24 open"}


def config0_spark(srs, args):
    """Plain single spark (config 0, the reference's CPU-runnable case): the
    config mesh, one realization in FP64 on the plain engine under the
    DefaultSpark protocol for --config0-ms, the Fluo-4 line scan along x
    through the cluster centre (linescan/DefaultScan.xml PSF) sampled every
    0.01 ms at the run's grid-file steps (srs_run_simulation_grid), and the
    spark's amplitude (peak F/F0 - 1 at the centre sample), time to peak and
    full duration at half maximum from it."""
    from srs_gb300 import workloads as wl
    import numpy as np
    tmp = tempfile.mkdtemp(prefix="srs_c0_")
    base, _ = wl.config_mesh(tmp)
    T, I = args.config0_ms, 0.01
    p = wl.default_spark_params(T_FINAL=T, OUTPUT_GRID_FLAG=1, OUTPUT_GRID_INTERVAL=I,
                                OUTPUT_STATES_INTERVAL=I)
    g = srs.Grid(p, base)
    sim = srs.Simulation(g, p, 1, srs.FP64, srs.ENGINE_PLAIN, seeds=[1])
    sim.reset()
    ns = sim.linescan_setup(axis=0, offset1=0.0, offset2=0.1, x_min=-1.0, x_max=1.0, res=0.05,
                            var_x=0.0289, var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=0.0,
                            pad_res=0.0, pad_min=0.0, pad_max=0.0, domain=(0, 0, 0, 0, 0, 0))
    _, f0 = sim.linescan()
    ts, F = [0.0], [np.ones(ns)]

    def sample(n, t, done):
        if not done[0]:
            ts.append(t)
            F.append(sim.linescan()[0][0] / f0)

    t0 = time.perf_counter()
    rows, _, n_steps, launch_ms = sim.run_simulation(timed=True, grid_callback=sample)
    wall = time.perf_counter() - t0
    from srs_gb300.metrics import NAMES, spark_metrics
    F = np.array(F)
    K = min(len(F), len(rows[0]))
    met = spark_metrics(F[:K, ns // 2], rows[0][:K, 2], I)
    return {"workload": "config0: config mesh, 1 realization, FP64 plain engine, DefaultSpark, "
                        "%.3g ms, line scan of %d samples every %.3g ms" % (T, ns, I),
            "steps": int(n_steps[0]), "device_s": float(launch_ms.sum()) / 1e3, "wall_s": wall,
            "value": T / wall, "unit": UNIT,
            "spark": dict(zip(NAMES, met)), "spark_metrics": "srs_gb300/metrics.py (centre sample)"}


def rcb_tiles(cen, max_tile):
    """Recursive coordinate bisection of the element centroids cen[N][3]:
    index arrays of compact tiles of at most max_tile elements."""
    import numpy as np
    out, todo = [], [np.arange(len(cen))]
    while todo:
        idx = todo.pop()
        if len(idx) <= max_tile:
            out.append(idx)
            continue
        c = cen[idx]
        ax = int(np.argmax(c.max(0) - c.min(0)))
        order = idx[np.argsort(c[:, ax], kind="stable")]
        h = len(order) // 2
        todo += [order[:h], order[h:]]
    return out


def blocking_probe(srs, args):
    """Temporal blocking of the large release site, measured by emulation.

    A blocked scheme loads a tile of the mesh plus a halo k elements deep,
    runs k time steps on chip (recomputing the halo, whose outer layers go
    stale one per step) and writes the tile back.  Its two factors are
    measured separately:
      halo  the config-4 mesh cut into compact tiles of at most 16,384
            elements (recursive coordinate bisection of the centroids) and
            k-hop halos over the face graph: at step s of a block the
            elements within k - s hops of the tile are updated, so a block
            updates update_factor times the elements it advances;
      chip  the resident engine, which is such a blocked step without a
            halo: each launch loads every realization's state, runs k steps
            on chip and writes the state back.  It runs the 15,288-element
            box of the multi-mesh batch (a tile-sized mesh that one cluster
            holds) with 2016 realizations in flight, the 63 tiles x 32
            realizations of the site, at k steps per launch.
    The blocked cost per advanced element-step is chip x update_factor (the
    halo's extra loads not counted); the plain engine's streaming split form
    on the site is timed alongside."""
    import numpy as np
    from scipy import sparse
    from srs_gb300 import tuner
    from srs_gb300 import workloads as wl
    tmp = tempfile.mkdtemp(prefix="srs_blk_")
    base4, rep4 = wl.config4_mesh(tmp)
    p = wl.default_spark_params()
    g4 = srs.Grid(p, base4)
    N = g4.n_ele
    _, nij, _ = g4.operator()
    fidx = g4.elements()["order"]
    nodes = np.loadtxt(base4 + ".node", skiprows=1, usecols=(1, 2, 3))
    ele = np.loadtxt(base4 + ".ele", skiprows=1, usecols=(1, 2, 3, 4), dtype=np.int64) - 1
    cen = nodes[ele[fidx]].mean(axis=1)
    rows = np.repeat(np.arange(N), 4)
    cols = nij.astype(np.int64)
    ok = (cols >= 0) & (cols < N) & (cols != rows)
    A = sparse.csr_matrix((np.ones(int(ok.sum()), np.float32), (rows[ok], cols[ok])), shape=(N, N))
    tiles = rcb_tiles(cen, 16384)
    K = (1, 2, 4, 8)
    reach = {k: 0 for k in range(max(K) + 1)}  # elements within k hops of a tile, summed over tiles
    for t in tiles:
        v = np.zeros(N, bool)
        v[t] = True
        reach[0] += len(t)
        for k in range(1, max(K) + 1):
            v = v | (A @ v.astype(np.float32) > 0)
            reach[k] += int(v.sum())
    halo = {}
    for k in K:
        upd = sum(reach[k - s] for s in range(1, k + 1)) / (k * reach[0])
        halo[k] = {"halo_elements": reach[k] / reach[0] - 1.0, "update_factor": upd}
    # streaming split form on the site (32 realizations)
    s4 = srs.Simulation(g4, p, 32, srs.FP32, srs.ENGINE_PLAIN, seeds=list(range(1, 33)))
    s4.advance_async(64)
    s4.synchronize()
    n4 = 512
    stream_ps = s4.time_advance(n4) * 1e9 / (n4 * 32 * N)
    del s4
    # the on-chip factor on a tile-sized mesh
    spec = wl.config2_mesh_specs()[1]
    base1 = os.path.join(tmp, "tile")
    rep1 = srs.write_box_mesh(base1, **spec)
    p1 = wl.default_spark_params(T_STEP=wl.stable_dt(p, rep1["max_a0"]))
    g1 = srs.Grid(p1, base1)
    R = 2016
    seeds = list(range(1, R + 1))
    t = tuner.tune_resident(g1, p1, R, seeds=seeds, clusters=(4, 5, 6, 8),
                            threads=(192, 256, 320, 384, 512), use_cache=False)
    chip = {}
    for k in K:
        sim = srs.Simulation(g1, p1, R, srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                             cluster_size=t["cluster_size"], threads_per_cta=t["threads_per_cta"],
                             steps_per_launch=k)
        sim.advance_async(8 * k)
        sim.synchronize()
        n = 64
        chip[k] = sim.time_advance(n) * 1e9 / (n * R * g1.n_ele)
        del sim
    return {"workload": "temporal blocking of the config-4 site (%d tets) emulated: halo factors from "
                        "its mesh, the on-chip step from the resident engine on a %d-tet box with %d "
                        "realizations at k steps per launch" % (N, g1.n_ele, R),
            "tiles": len(tiles), "tile_elements": reach[0] / len(tiles),
            "halo": {str(k): halo[k] for k in K},
            "chip_ps_per_element_step": {str(k): chip[k] for k in K},
            "chip_config": {"cluster_size": t["cluster_size"], "threads_per_cta": t["threads_per_cta"]},
            "blocked_ps_per_advanced_element_step": {str(k): chip[k] * halo[k]["update_factor"] for k in K},
            "streaming_ps_per_element_step": stream_ps}


def config4_site(srs, args):
    """Large release site: the multi-site mesh of about a million tets (five
    clusters of 20 / 40 / 60 / 100 / 150 RyRs, one LCC per 7 RyRs), 32
    realizations under the DefaultSpark protocol in FP32.  A realization does
    not fit on chip, so the plain FP32 engine runs it: one fused kernel per
    time step for all 32 realizations, the state streamed through HBM.  A
    bounded sample of the 30 ms run: one run of 4096 + --config4-steps
    steps; the engine advances it in chunks of up to 4096 steps, the first
    chunk is the warm-up and the others are timed on the device
    (srs_run_simulation_timed); FP64 total Ca per compartment
    (srs_sim_total_ca) at the start and the end."""
    from srs_gb300 import workloads as wl
    import numpy as np
    tmp = tempfile.mkdtemp(prefix="srs_c4_")
    t0 = time.perf_counter()
    base, rep_ = wl.config4_mesh(tmp)
    t_gen = time.perf_counter() - t0
    n, warm = args.config4_steps, 4096
    p = wl.default_spark_params(T_FINAL=(warm + n - 0.5) * DT_MS, OUTPUT_STATES_INTERVAL=warm * DT_MS)
    t0 = time.perf_counter()
    g = srs.Grid(p, base)
    t_load = time.perf_counter() - t0
    R = args.config4_realizations
    from srs_gb300 import tuner
    if args.no_tune:  # the default distance: one wave of blocks
        tuned = dict(prefetch_blocks=-1, trials=[])
    else:
        tuned = tuner.tune_plain(g, p, R, seeds=list(range(1, R + 1)))
    sim = srs.Simulation(g, p, R, srs.FP32, srs.ENGINE_PLAIN, seeds=list(range(1, R + 1)))
    sim.set_prefetch(tuned["prefetch_blocks"])
    sim.reset()
    tot0 = sim.total_ca()
    rows4, _, n_run, launch_ms = sim.run_simulation(timed=True)
    tot1 = sim.total_ca()
    # RyR open counts at the states rows (column 2): how far the sparks spread
    max_open = np.array([float(r[:, 2].max()) if len(r) else 0.0 for r in rows4])
    if len(launch_ms) < 2 or int(n_run.min()) != warm + n:
        raise RuntimeError("config4 run: %d chunks, %d steps" % (len(launch_ms), int(n_run.min())))
    ms = float(launch_ms[1:].sum())
    n_el = rep_["n_tets"]
    alg = n_el * R * n * (48.0 + 44.0 / R)
    peak, peak_kind = measured_peaks()
    del sim
    err64 = fp64_error(srs, g, p, 2048, srs.ENGINE_PLAIN)
    mass = mass_balance(srs, g, p, 2048, srs.ENGINE_PLAIN)
    adj = None
    if args.config4_adjoint_steps > 0:
        adj = config4_adjoint(srs, base, R, args.config4_adjoint_steps, ms / n)
    return {"adjoint": adj, "workload": "config4: multi-site release unit, %d tets (%d RyR in 5 clusters, %d LCC), "
                        "%d realizations, DefaultSpark protocol, FP32 plain engine, %d timed steps"
                        % (n_el, rep_["n_ryr"], rep_["n_lcc"], R, n),
            "value": R * n * DT_MS / (ms / 1e3), "unit": UNIT, "ms_per_time_step": ms / n,
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / peak,
                         "note": "algorithmic 48 + 44/R B per element-step; peak %s" % peak_kind},
            "prefetch_blocks": tuned["prefetch_blocks"],
            "prefetch_trials": [(t["prefetch_blocks"], t["ms_per_step"]) for t in tuned["trials"]],
            "ryr_open_max": {"mean": float(max_open.mean()), "max": float(max_open.max()),
                             "runs_recruiting": int((max_open > 1).sum())},
            "fp64_error": err64, "mass_balance": mass, "mesh_generation_s": t_gen,
            "mesh_load_s": t_load,
            "total_ca_start": np.asarray(tot0)[0].tolist(), "total_ca_end": np.asarray(tot1)[0].tolist()}


def config4_adjoint(srs, base, R, n, fwd_ms_per_step):
    """The adjoint over the start of the large-site run (the plain FP32
    engine's reverse sweep, one launch per step, every array in HBM): n steps
    of the 32 realizations from rest with gating, the x line scan through the
    central cluster every 128 steps, the mean-trace misfit against the run
    with TARGET_PERTURBED raised by 10 %.  Wall time of srs_adjoint with
    segments of 64 steps; the reverse sweep's cost per step follows from it
    and the forward steps of the call's checkpoint plan (srs_adjoint_plan),
    and the plan for the first 5 ms projects the whole sweep."""
    import numpy as np
    te = 128
    ls = dict(axis=0, offset1=0.0, offset2=0.1, x_min=-1.0, x_max=1.0, res=0.05, var_x=0.0289,
              var_y=0.1154, var_z=0.0289, r_thresh=1.0, f0_pad=0.0, pad_res=0.0, pad_min=0.0,
              pad_max=0.0, domain=(0, 0, 0, 0, 0, 0))
    seeds = list(range(1, R + 1))
    from srs_gb300 import workloads as wl
    p = wl.default_spark_params()
    pt = p.copy()
    for name in TARGET_PERTURBED:
        pt.reals[srs.R[name]] *= 1.1
    simt = srs.Simulation(srs.Grid(pt, base), pt, R, srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    simt.reset()
    ns = simt.linescan_setup(**ls)
    _, f0t = simt.linescan()
    target = np.zeros((n // te, ns))
    for k in range(n // te):
        simt.advance_async(te)
        Ft, _ = simt.linescan()
        target[k] = Ft.mean(0) / f0t - 1.0
    del simt
    sim = srs.Simulation(srs.Grid(p, base), p, R, srs.FP32, srs.ENGINE_PLAIN, seeds=seeds)
    sim.linescan_setup(**ls)
    sim.reset()
    _, f0 = sim.linescan()
    K = 64
    kw = dict(checkpoint_every=K, flags=srs.ADJ_MEAN_TRACE)
    sim.adjoint(n, te, f0, target, **kw)  # warm-up (and the work buffers of this size)
    sim.reset()
    seg, lev, fwd_steps = sim.adjoint_plan(n, te, checkpoint_every=K)
    t0 = time.perf_counter()
    loss, grad, _ = sim.adjoint(n, te, f0, target, **kw)
    adj_s = time.perf_counter() - t0
    if not np.isfinite(grad).all():
        raise SystemExit("non-finite adjoint gradient (large site)")
    rev_ms = max(adj_s * 1e3 - fwd_steps * fwd_ms_per_step, 0.0) / n
    n5 = int(round(5.0 / DT_MS))
    seg5, lev5, fwd5 = sim.adjoint_plan(n5, te, checkpoint_every=K)
    gsum = grad.sum(0)
    return {"workload": "adjoint over the first %d steps (%.2f us) of the large site, %d realizations, "
                        "line scan of %d samples every %d steps, mean-trace loss" % (n, n * DT_MS * 1e3, R, ns, te),
            "segment_steps": seg, "levels": lev, "forward_steps": fwd_steps, "adjoint_s": adj_s,
            "forward_ms_per_step": fwd_ms_per_step, "reverse_ms_per_step": rev_ms,
            "cost_ratio": adj_s * 1e3 / (n * fwd_ms_per_step), "loss": float(loss[0]),
            "grad": {name: float(gsum[k]) for k, name in enumerate(srs.ADJ_PARAMS)},
            "first_5ms": {"steps": n5, "segment_steps": seg5, "levels": lev5, "forward_steps": fwd5,
                          "projected_s": (fwd5 * fwd_ms_per_step + n5 * rev_ms) / 1e3,
                          "projected_cost_ratio": (fwd5 * fwd_ms_per_step + n5 * rev_ms) /
                                                  (n5 * fwd_ms_per_step)}}


def run_ours(args):
    ws, rank, local = dist_env()
    dist = dist_init(ws)
    import torch
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    import __graft_entry__ as g
    if rank == 0:
        g.build()
    barrier(dist)
    import srs_gb300 as srs
    from srs_gb300 import workloads as wl
    tmp = tempfile.mkdtemp(prefix="srs_bench_%d_" % rank)
    base, rep = wl.config_mesh(tmp)
    p = wl.default_spark_params()
    grid = srs.Grid(p, base)
    if args.only:
        if rank == 0:
            legs = {"adjoint": adjoint_cost, "config2": lambda srs_, g_, p_, a_: config2_batch(srs_, a_),
                    "config4": lambda srs_, g_, p_, a_: config4_site(srs_, a_),
                    "config0": lambda srs_, g_, p_, a_: config0_spark(srs_, a_),
                    "blocking": lambda srs_, g_, p_, a_: blocking_probe(srs_, a_)}
            leg = legs[args.only](srs, grid, p, args)
            print(json.dumps(dict(leg, leg=args.only)))
        return 0
    R, S = args.realizations, args.launch_steps
    seeds = replica_seeds(rank, R)
    from srs_gb300 import tuner
    if args.no_tune:
        tuned = dict(cluster_size=args.cluster_size, threads_per_cta=args.threads, ms_per_step=None,
                     trials=[])
    else:
        tuned = tuner.tune_resident(grid, p, R, seeds=seeds)
    # One bench step = one launch of S time steps of the reference's
    # RunSimulation under the DefaultSpark protocol (RyR 24 held open, output
    # rows every S steps), from the equilibrium state uploaded by
    # srs_sim_reset before the run.  The run has W + K launches: the first W
    # are the warm-up, the last K the timed region, each launch timed on the
    # device (CUDA events on the engine's stream, srs_run_simulation_timed).
    W, K = args.warmup, args.steps
    pr = wl.default_spark_params(T_FINAL=((W + K) * S - 0.5) * DT_MS, OUTPUT_STATES_INTERVAL=S * DT_MS)
    sim = srs.Simulation(grid, pr, R, srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                         steps_per_launch=S, cluster_size=tuned["cluster_size"],
                         threads_per_cta=tuned["threads_per_cta"])
    cfg = sim.config()
    sim.reset()
    clocks = Clocks(local)
    launches0 = sim.config()["kernel_launches"]
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    _, _, n_run, launch_ms = sim.run_simulation(timed=True)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(dist)
    launches = sim.config()["kernel_launches"] - launches0 - W
    ms = float(launch_ms[W:].sum())
    if len(launch_ms) != W + K or int(n_run.min()) != (W + K) * S or int(n_run.max()) != (W + K) * S:
        raise SystemExit("the run did not make %d launches of %d steps" % (W + K, S))
    ms_max = max_over_ranks(dist, ms)
    sec = ms_max / 1e3
    value = ws * R * args.steps * S * DT_MS / sec
    ms_per_step = ms_max / args.steps

    # roofline of the resident kernel (the only kernel in the timed region)
    n_el = rep["n_tets"]
    alg_bytes = n_el * R * S * (48.0 + 44.0 / R)
    achieved = alg_bytes / (ms / args.steps / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = profiled_traffic()
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic,
            "note": "effective fraction (state resident on chip within a launch); peak %s"
                    % peak_kind}

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        pe = wl.default_spark_params(T_FINAL=(S - 0.5) * DT_MS, OUTPUT_STATES_INTERVAL=S * DT_MS / 4)
        sim_e = srs.Simulation(grid, pe, R, srs.FP32, srs.ENGINE_RESIDENT, seeds=seeds,
                               steps_per_launch=S, cluster_size=tuned["cluster_size"],
                               threads_per_cta=tuned["threads_per_cta"])
        cfg_e = sim_e.config()
        sim_e.run_simulation()  # warm
        clocks_e = Clocks(local)
        barrier(dist)
        torch.cuda.synchronize()
        clocks_e.start()
        t0 = time.perf_counter()
        rows_bytes = 0
        t_reset = 0.0
        for _ in range(args.e2e_steps):
            ta = time.perf_counter()
            sim_e.reset()  # returns after its uploads completed
            t_reset += time.perf_counter() - ta
            rows, t_end, n_steps = sim_e.run_simulation()
            rows_bytes = sum(r.nbytes for r in rows)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(dist, (time.perf_counter() - t0) / args.e2e_steps)
        clk_e = clocks_e.stop()
        reset_ms = 1e3 * t_reset / args.e2e_steps
        e2e_val = ws * R * S * DT_MS / e2e_s
        row_cap = int(pe.reals[0] / pe.reals[2]) + 8
        d2h = R * row_cap * sim_e.row_width() * 4 + 2 * cfg_e["ctl_bytes"]

        e2e = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": cfg_e["reset_h2d_bytes"],
               "d2h_bytes_per_step": d2h,
               "call": "srs_sim_reset + srs_run_simulation (%d steps, rows %d B)" % (S, rows_bytes),
               "reset_ms": reset_ms, "ms_per_step": 1e3 * e2e_s, "clocks": clk_e}

    # secondary legs: a failure is reported in the line, not fatal to it
    err64 = None
    if rank == 0 and args.fp64_steps > 0:
        try:
            err64 = fp64_error(srs, grid, p, args.fp64_steps, srs.ENGINE_RESIDENT,
                               cluster_size=tuned["cluster_size"],
                               threads_per_cta=tuned["threads_per_cta"])
        except Exception as e:  # noqa: BLE001
            err64 = {"error": "%s: %s" % (type(e).__name__, e)}
    mass = None
    if rank == 0 and args.fp64_steps > 0:
        try:
            mass = mass_balance(srs, grid, p, args.fp64_steps, srs.ENGINE_RESIDENT,
                                cluster_size=tuned["cluster_size"],
                                threads_per_cta=tuned["threads_per_cta"])
        except Exception as e:  # noqa: BLE001
            mass = {"error": "%s: %s" % (type(e).__name__, e)}
    adj = None
    if rank == 0 and not args.no_adjoint:
        try:
            adj = adjoint_cost(srs, grid, p, args)
        except Exception as e:  # noqa: BLE001
            adj = {"error": "%s: %s" % (type(e).__name__, e)}
    plain1 = None
    if rank == 0:
        try:
            plain1 = plain_one_realization(srs, grid, p)
            plain1["batched_over_plain_fp32"] = value / ws / plain1["fp32"]["value"]
        except Exception as e:  # noqa: BLE001
            plain1 = {"error": "%s: %s" % (type(e).__name__, e)}
    c2 = None
    if rank == 0 and not args.no_config2:
        try:
            c2 = config2_batch(srs, args)
        except Exception as e:  # noqa: BLE001
            c2 = {"error": "%s: %s" % (type(e).__name__, e)}
    c0 = None
    if rank == 0 and not args.no_config0:
        try:
            c0 = config0_spark(srs, args)
        except Exception as e:  # noqa: BLE001
            c0 = {"error": "%s: %s" % (type(e).__name__, e)}
    c4 = None
    if rank == 0 and not args.no_config4:
        try:
            c4 = config4_site(srs, args)
        except Exception as e:  # noqa: BLE001
            c4 = {"error": "%s: %s" % (type(e).__name__, e)}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        v, cores, kind, sample = cpu_sample(base, list(p.ints), list(p.reals), args.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {
                "workload": "config1: batched box dyad, %d realizations x %d elements "
                            "(12^3 hexahedra, 49 RyR, 7 LCC), DefaultSpark dt=9ns, FP32 state, "
                            "RunSimulation protocol (RyR 24 held open, a states row per launch)"
                            % (R, n_el),
                "realizations_per_gpu": R, "elements": n_el, "steps_per_launch": S,
                "engine": "resident", "cluster_size": cfg["cluster_size"],
                "threads_per_cta": cfg["threads_per_cta"], "smem_bytes": cfg["smem_bytes"],
                "l2": "inputs larger than L2 (212 MB state), no flush",
                "tuner": {"trials": len(tuned["trials"]),
                          "best_ms_per_step": tuned["ms_per_step"]},
                "parallelism": "replicas x%d" % ws},
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": roof,
            "fp64_error": err64,
            "mass_balance": mass,
            "cpu_baseline": cpu,
            "clocks": clk,
            "adjoint": adj,
            "plain_one_realization": plain1,
            "config2": c2,
            "config4": c4,
            "config0": c0,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
