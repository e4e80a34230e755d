"""The adjoint over the whole config-3 horizon, against finite differences.

Not collected by pytest (it takes about ten minutes on a GB300): run it as
    python tests/long/adjoint_config3_horizon.py [n_steps] [PARAM,PARAM,...]
Workload: the 10,368-element config mesh, DefaultSpark with gating off (RyR
24 held open, so the trajectory is deterministic and the loss differentiable),
1,111,040 steps (10 ms at dt = 9 ns) by default, the x line scan through the
cluster every 128 steps, the mean-trace loss against the trace of a run with
the parameters of bench.TARGET_PERTURBED raised by 10 %.  The adjoint runs on
the FP32 resident engine (4 realizations, checkpoints every 256 steps); the
central differences (h = 1e-4 |theta|) on the FP64 plain engine from the same
initial state.  Prints one JSON line: losses and, per parameter, (adjoint,
finite difference, relative difference).
"""
import sys, os, json, time, tempfile
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
import numpy as np
import srs_gb300 as srs
from srs_gb300 import workloads as wl
import bench
N_STEPS = int(sys.argv[1]) if len(sys.argv) > 1 else 1111104
TE = 128
N_STEPS = (N_STEPS // TE) * TE
tmp = tempfile.mkdtemp()
base, rep = wl.config_mesh(tmp)
p0 = wl.default_spark_params(FLAG_NO_GATING=1)
LS = dict(axis=0, offset1=0.0, offset2=0.1, x_min=-1.0, x_max=1.0, res=0.05, var_x=0.0289, var_y=0.1154,
          var_z=0.0289, r_thresh=1.0, f0_pad=0.0, pad_res=0.0, pad_min=0.0, pad_max=0.0, domain=(0, 0, 0, 0, 0, 0))
nt = N_STEPS // TE
def trace(p, prec, eng, R, start=None):
    g = srs.Grid(p, base)
    s = srs.Simulation(g, p, R, prec, eng, seeds=list(range(1, R + 1)))
    s.reset()
    s.linescan_setup(**LS)
    if start is not None:
        for r in range(R):
            s.set_state(r, start["states"], start["ryr"], start["lcc"], start["lccv"], start["residuals"])
    _, f0 = s.linescan()
    out = np.zeros((nt, len(f0)))
    for k in range(nt):
        s.explicit_step(TE)
        F, _ = s.linescan()
        out[k] = F.mean(0)
    return out, f0, s
t0 = time.time()
pt = p0.copy()
for name in bench.TARGET_PERTURBED:
    pt.reals[srs.R[name]] *= 1.1
tgt_F, tgt_f0, _ = trace(pt, srs.FP32, srs.ENGINE_RESIDENT, 1)
target = tgt_F / tgt_f0 - 1.0
print('target', time.time() - t0, flush=True)
g = srs.Grid(p0, base)
R = 4
sim = srs.Simulation(g, p0, R, srs.FP32, srs.ENGINE_RESIDENT, seeds=list(range(1, R + 1)))
sim.reset()
sim.linescan_setup(**LS)
_, f0 = sim.linescan()
start = sim.get_state(0)
t0 = time.time()
loss, grad, _ = sim.adjoint(N_STEPS, TE, f0, target, checkpoint_every=256, flags=srs.ADJ_MEAN_TRACE)
t_adj = time.time() - t0
gsum = grad.sum(0)
print('adjoint', t_adj, 'loss', loss[0], flush=True)
def loss_of(p):
    F, _, _ = trace(p, srs.FP64, srs.ENGINE_PLAIN, 1, start)
    e = F / f0 - 1.0 - target
    return 0.5 * float((e * e).sum())
t0 = time.time()
L0 = loss_of(p0)
print('L0', L0, 'fp32 adjoint loss', loss[0], time.time() - t0, flush=True)
names = sys.argv[2].split(',') if len(sys.argv) > 2 else ["D_CA", "D_DYE", "K_ON_CMDN", "K_OFF_CMDN", "K_ON_TRPN", "K_OFF_TRPN", "V_RYR", "A_P", "B_TOT_SL_HI", "K_D_SL_HI"]
res = {}
for name in names:
    k = srs.ADJ_PARAMS.index(name)
    idx = srs.R[name]
    h = 1e-4 * abs(p0.reals[idx])
    hi, lo = p0.copy(), p0.copy()
    hi.reals[idx] += h
    lo.reals[idx] -= h
    fd = (loss_of(hi) - loss_of(lo)) / (2 * h)
    res[name] = (float(gsum[k]), fd, abs(gsum[k] - fd) / abs(fd))
    print(name, res[name], flush=True)
print(json.dumps({"steps": N_STEPS, "R": R, "adjoint_s": t_adj, "loss_adj": float(loss[0]), "loss_fp64": L0, "grads": res}))
