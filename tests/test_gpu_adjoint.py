"""Device pathwise adjoint (srs_adjoint) against the FP64 oracle adjoint and
against central finite differences of the device FP64 engine.

Workload: the golden mesh, 4 realizations (seeds 11..14) from their reset
state, 600 explicit steps with Philox gating, the x line scan of
linescan/DefaultScan.xml sampled every 100 steps, loss
  L_r = 1/2 sum_k sum_i (F_ki / F0_i - 1 - target_rki)^2,
checkpoints every 200 steps (ticks fall on segment boundaries).
Tolerances: loss 1e-5 relative (FP32 trajectory against FP64), gradients
1e-3 relative (the finite-difference bar).
"""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, LINESCAN_DESC, linescan_weights, params_from_golden

pytestmark = pytest.mark.gpu

N_STEPS, TICK, K = 600, 100, 200
SEEDS = [11, 12, 13, 14]


def _params(srs):
    p, _ = params_from_golden(srs, "spark")
    p.ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]] = 1
    p.ints[srs.I["FLAG_NO_GATING"]] = 0
    return p


def _start(srs, p, precision, engine):
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, len(SEEDS), precision, engine, seeds=SEEDS)
    sim.reset()
    sim.linescan_setup(**LINESCAN_DESC)
    return g, sim


@pytest.fixture(scope="module")
def case(srs):
    p = _params(srs)
    g, sim = _start(srs, p, srs.FP32, srs.ENGINE_RESIDENT)
    _, f0 = sim.linescan()
    start = [sim.get_state(r) for r in range(len(SEEDS))]
    rng = np.random.default_rng(3)
    target = rng.standard_normal((len(SEEDS), N_STEPS // TICK, len(f0))) * 0.01
    loss, grad, gs = sim.adjoint(N_STEPS, TICK, f0, target, checkpoint_every=K, grad_state=True)
    return dict(p=p, g=g, sim=sim, f0=f0, start=start, target=target, loss=loss, grad=grad, gs=gs)


def _check_against_oracle(srs, oracle, case, loss, grad, gs_all):
    from oracle import Mesh
    p, g = case["p"], case["g"]
    W, pad = linescan_weights(g)
    noflux = int(p.ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]])
    m = Mesh(oracle, GOLDEN_MESH, noflux, np.array(p.reals[:]))
    ints = np.array(p.ints[:], np.int32)
    N = g.n_ele
    for r, seed in enumerate(SEEDS):
        st = case["start"][r]
        L, go, lam0 = m.adjoint(ints, st["states"], st, seed, N_STEPS, TICK, W, pad, case["f0"],
                                case["target"][r], grad_state=True)
        assert abs(loss[r] - L) <= 1e-5 * L
        scale = np.abs(go)
        for k in range(srs.N_ADJ):
            if scale[k] == 0:
                continue
            assert abs(grad[r, k] - go[k]) <= 1e-3 * scale[k], (r, srs.ADJ_PARAMS[k], grad[r, k], go[k])
        # dL/dS0: species by species, relative to the largest sensitivity
        gs = gs_all[r].reshape(-1)
        for sp in range(6):
            a, b = gs[sp * N:(sp + 1) * N], lam0[sp * N:(sp + 1) * N]
            ref = np.abs(b).max()
            if ref > 0:
                assert np.abs(a - b).max() <= 1e-3 * ref, (r, sp)


def test_adjoint_matches_fp64_oracle(srs, oracle, case):
    _check_against_oracle(srs, oracle, case, case["loss"], case["grad"], case["gs"])


@pytest.fixture(scope="module")
def plain_case(srs, case):
    """The same adjoint on the plain FP32 engine (one launch per reverse step,
    every array in HBM): the form for meshes too large for the resident one."""
    _, sim = _start(srs, case["p"], srs.FP32, srs.ENGINE_PLAIN)
    loss, grad, gs = sim.adjoint(N_STEPS, TICK, case["f0"], case["target"], checkpoint_every=K,
                                 grad_state=True)
    return dict(sim=sim, loss=loss, grad=grad, gs=gs)


def test_plain_engine_adjoint_matches_fp64_oracle(srs, oracle, case, plain_case):
    _check_against_oracle(srs, oracle, case, plain_case["loss"], plain_case["grad"], plain_case["gs"])


def test_plain_engine_adjoint_with_dirichlet_faces_matches_fp64_oracle(srs, oracle, case):
    """The plain engine also runs meshes with Dirichlet faces (on cytosolic
    elements; the resident engine needs no-flux boundaries): their rate kb
    joins the diagonal of the transposed operator and the diffusion
    gradients."""
    p = case["p"].copy()
    p.ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]] = 0
    g, sim = _start(srs, p, srs.FP32, srs.ENGINE_PLAIN)
    _, f0 = sim.linescan()
    start = [sim.get_state(r) for r in range(len(SEEDS))]
    loss, grad, gs = sim.adjoint(N_STEPS, TICK, f0, case["target"], checkpoint_every=K, grad_state=True)
    _check_against_oracle(srs, oracle, dict(case, p=p, g=g, f0=f0, start=start), loss, grad, gs)


def test_plain_engine_adjoint_agrees_with_resident(srs, case, plain_case):
    """Both FP32 engines run the same trajectory (bit-exact with the FP32
    restatement); the line-scan sums and the gradient's FP32 partial sums are
    grouped differently (1e-12 on the loss, 1e-5 on the gradients)."""
    assert np.allclose(plain_case["loss"], case["loss"], rtol=1e-12, atol=0)
    scale = np.abs(case["grad"]).max(0)
    assert np.all(np.abs(plain_case["grad"] - case["grad"]) <= 1e-5 * scale[None, :])
    N = case["g"].n_ele
    for r in range(len(SEEDS)):
        a, b = plain_case["gs"][r].reshape(-1), case["gs"][r].reshape(-1)
        for sp in range(6):
            ref = np.abs(b[sp * N:(sp + 1) * N]).max()
            assert np.abs(a[sp * N:(sp + 1) * N] - b[sp * N:(sp + 1) * N]).max() <= 1e-5 * ref, (r, sp)


@pytest.mark.parametrize("engine", ["RESIDENT", "PLAIN"])
@pytest.mark.parametrize("K2,max_ck,levels", [(50, 6, 2), (25, 6, 3), (25, 0, 1)])
def test_multilevel_checkpoints_give_the_same_result(srs, case, plain_case, engine, K2, max_ck, levels):
    """Fewer snapshots than segments: the sweep takes snapshots on several
    levels and recomputes the forward run more often, from the same states
    with the same gating draws, so the trajectory, the loss and dL/dS0 are
    bit-identical to the one-level sweep (the plain engine's gradient too: its
    per-step block sums do not depend on the segmentation)."""
    ref = case if engine == "RESIDENT" else plain_case
    _, sim = _start(srs, case["p"], srs.FP32, getattr(srs, "ENGINE_" + engine))
    seg, lev, fwd = sim.adjoint_plan(N_STEPS, TICK, checkpoint_every=K2, max_checkpoints=max_ck)
    assert (seg, lev) == (K2, levels)
    assert fwd > N_STEPS if levels > 1 else fwd == N_STEPS + (N_STEPS // K2 - 1) * K2
    loss, grad, gs = sim.adjoint(N_STEPS, TICK, case["f0"], case["target"], checkpoint_every=K2,
                                 max_checkpoints=max_ck, grad_state=True)
    assert np.array_equal(loss, ref["loss"])
    assert np.array_equal(gs, ref["gs"])
    if engine == "PLAIN":
        assert np.array_equal(grad, ref["grad"])
    else:
        assert np.allclose(grad, ref["grad"], rtol=1e-5, atol=0)
    # the state after the call is the one after n_steps
    for r in range(len(SEEDS)):
        assert np.array_equal(sim.get_state(r)["states"], ref["sim"].get_state(r)["states"])


def test_too_few_checkpoints_are_rejected(srs, case):
    _, sim = _start(srs, case["p"], srs.FP32, srs.ENGINE_PLAIN)
    with pytest.raises(srs.SrsError) as e:
        sim.adjoint(N_STEPS, TICK, case["f0"], case["target"], checkpoint_every=50, max_checkpoints=2)
    assert e.value.status == -10  # SRS_ERR_NOMEM: no plan with 3 snapshots covers 12 segments


def test_adjoint_matches_fp64_finite_differences(srs, case):
    """Central differences of the FP64 plain engine from the same start state
    with the same seeds (common random numbers), h = 1e-4 |theta|."""
    p0, f0, target = case["p"], case["f0"], case["target"]

    def loss_of(p):
        _, sim = _start(srs, p, srs.FP64, srs.ENGINE_PLAIN)
        for r, st in enumerate(case["start"]):
            sim.set_state(r, st["states"], st["ryr"], st["lcc"], st["lccv"], st["residuals"])
        L = np.zeros(len(SEEDS))
        for k in range(N_STEPS // TICK):
            sim.explicit_step(TICK)
            F, _ = sim.linescan()
            e = F / f0[None, :] - 1.0 - target[:, k, :]
            L += 0.5 * (e * e).sum(axis=1)
        return L

    L0 = loss_of(p0)
    assert np.allclose(L0, case["loss"], rtol=1e-5)
    checked = []
    for k, name in enumerate(srs.ADJ_PARAMS):
        idx = srs.R[name]
        h = 1e-4 * abs(p0.reals[idx])
        hi, lo = p0.copy(), p0.copy()
        hi.reals[idx] += h
        lo.reals[idx] -= h
        Lp, Lm = loss_of(hi), loss_of(lo)
        if np.abs(Lp - Lm).sum() < 1e-9 * L0.sum():
            continue  # below the loss's rounding
        fd = (Lp - Lm).sum() / (2 * h)
        adj = case["grad"][:, k].sum()
        assert abs(adj - fd) <= 1e-3 * abs(fd), (name, adj, fd)
        checked.append(name)
    # the line scan over 600 steps resolves these at least
    assert {"D_CA", "K_ON_DYE", "K_OFF_DYE", "V_RYR"} <= set(checked), checked


@pytest.mark.parametrize("K2,C", [(0, 1), (600, 2), (150, 3)])
def test_adjoint_segmentation_and_cluster_size_do_not_change_the_result(srs, case, K2, C):
    """The trajectory and lambda are bit-identical for any checkpoint interval
    and cluster size; only the grouping of the FP32 partial sums of the
    gradient changes (1e-5)."""
    p = case["p"]
    g = srs.Grid(p, GOLDEN_MESH)
    sim = srs.Simulation(g, p, len(SEEDS), srs.FP32, srs.ENGINE_RESIDENT, seeds=SEEDS, cluster_size=C)
    assert sim.config()["cluster_size"] == C
    sim.reset()
    sim.linescan_setup(**LINESCAN_DESC)
    loss, grad, gs = sim.adjoint(N_STEPS, TICK, case["f0"], case["target"], checkpoint_every=K2,
                                 grad_state=True)
    assert np.array_equal(loss, case["loss"])
    assert np.array_equal(gs, case["gs"])
    assert np.allclose(grad, case["grad"], rtol=1e-5, atol=0)


@pytest.mark.parametrize("flags,threads", [("LAMBDA_GLOBAL", 0), ("NO_STAGE", 0),
                                          ("LAMBDA_GLOBAL|NO_STAGE", 512), ("", 256),
                                          ("STAGE", 256), ("STAGE|LAMBDA_GLOBAL", 512)])
def test_adjoint_memory_placements_give_the_same_result(srs, case, flags, threads):
    """lambda's owner state on chip or in global memory, the trajectory staged
    in shared memory by bulk copies or read from global memory, 256 or 512
    threads: the same arithmetic, so loss and dL/dS0 are bit-identical and the
    gradient differs only by the grouping of its FP32 partial sums."""
    p = case["p"]
    f = 0
    for name in filter(None, flags.split("|")):
        f |= getattr(srs, "ADJ_" + name)
    _, sim = _start(srs, p, srs.FP32, srs.ENGINE_RESIDENT)
    loss, grad, gs = sim.adjoint(N_STEPS, TICK, case["f0"], case["target"], checkpoint_every=K,
                                 grad_state=True, flags=f, threads_per_cta=threads)
    assert np.array_equal(loss, case["loss"])
    assert np.array_equal(gs, case["gs"])
    assert np.allclose(grad, case["grad"], rtol=1e-5, atol=0)


def test_adjoint_leaves_the_state_after_n_steps(srs, case):
    p = case["p"]
    _, ref = _start(srs, p, srs.FP32, srs.ENGINE_RESIDENT)
    ref.explicit_step(N_STEPS)
    for r in range(len(SEEDS)):
        a, b = case["sim"].get_state(r), ref.get_state(r)
        for key in ("states", "ryr", "lcc", "lccv", "residuals"):
            assert np.array_equal(a[key], b[key]), key


def test_adjoint_rejects_unsupported_configurations(srs, case):
    p = case["p"]
    _, plain = _start(srs, p, srs.FP64, srs.ENGINE_PLAIN)
    with pytest.raises(srs.SrsError) as e:
        plain.adjoint(10, 5, case["f0"])
    assert e.value.status == -6  # SRS_ERR_UNSUPPORTED
    g = srs.Grid(p, GOLDEN_MESH)
    s2 = srs.Simulation(g, p, 1, srs.FP32, srs.ENGINE_RESIDENT, seeds=[1])
    with pytest.raises(ValueError):
        s2.adjoint(10, 5, case["f0"])  # no line scan set up
    s2.reset()
    s2.linescan_setup(**LINESCAN_DESC)
    with pytest.raises(srs.SrsError) as e:
        s2.adjoint(0, 5, case["f0"])
    assert e.value.status == -1  # SRS_ERR_INPUT


def test_mean_trace_loss_matches_fp64_oracle(srs, oracle, case):
    """SRS_ADJ_MEAN_TRACE: L = 1/2 sum (mean_r F_r / F0 - 1 - target)^2.  Its
    gradient is the sum over realizations of per-realization gradients whose
    targets are shifted so that each residual is the mean residual / R; the
    oracle computes those, with F from the FP64 engine (bit-exact with it)."""
    from oracle import Mesh
    p, g, f0 = case["p"], case["g"], case["f0"]
    R, nt = len(SEEDS), N_STEPS // TICK
    tgt = np.random.default_rng(5).standard_normal((nt, len(f0))) * 0.01
    _, sim = _start(srs, p, srs.FP32, srs.ENGINE_RESIDENT)
    loss, grad, _ = sim.adjoint(N_STEPS, TICK, f0, tgt, checkpoint_every=K,
                                flags=srs.ADJ_MEAN_TRACE)
    assert np.all(loss[1:] == 0.0)
    _, s64 = _start(srs, p, srs.FP64, srs.ENGINE_PLAIN)
    for r, st in enumerate(case["start"]):
        s64.set_state(r, st["states"], st["ryr"], st["lcc"], st["lccv"], st["residuals"])
    F = np.zeros((R, nt, len(f0)))
    for k in range(nt):
        s64.explicit_step(TICK)
        F[:, k, :], _ = s64.linescan()
    e = F.mean(0) / f0[None, :] - 1.0 - tgt
    L = 0.5 * float((e * e).sum())
    assert abs(loss[0] - L) <= 1e-5 * L
    W, pad = linescan_weights(g)
    m = Mesh(oracle, GOLDEN_MESH, 1, np.array(p.reals[:]))
    ints = np.array(p.ints[:], np.int32)
    go = np.zeros(srs.N_ADJ)
    scale = np.zeros(srs.N_ADJ)
    for r, seed in enumerate(SEEDS):
        st = case["start"][r]
        shifted = F[r] / f0[None, :] - 1.0 - e / R
        _, gr = m.adjoint(ints, st["states"], st, seed, N_STEPS, TICK, W, pad, f0, shifted)
        go += gr
        scale += np.abs(gr)
    got = grad.sum(0)
    for k in range(srs.N_ADJ):
        if scale[k] > 0:
            assert abs(got[k] - go[k]) <= 1e-3 * scale[k], (srs.ADJ_PARAMS[k], got[k], go[k])
