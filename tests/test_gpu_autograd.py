"""torch.autograd binding of the adjoint (srs_gb300.autograd) against central
finite differences of the FP64 engine with common random numbers."""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, LINESCAN_DESC, params_from_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("engine", ["RESIDENT", "PLAIN"])
def test_autograd_gradient_matches_finite_differences(srs, engine):
    torch = pytest.importorskip("torch")
    from srs_gb300.autograd import AdjointProblem, LinescanLoss
    p, _ = params_from_golden(srs, "spark")
    p.ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]] = 1
    rng = np.random.default_rng(5)
    prob = AdjointProblem(GOLDEN_MESH, p, [21, 22], LINESCAN_DESC, 400, 100,
                          target=rng.standard_normal((2, 4, 20)) * 0.01, checkpoint_every=128,
                          engine=getattr(srs, "ENGINE_" + engine))
    theta = prob.theta0().requires_grad_()
    loss = LinescanLoss.apply(theta, prob)
    (g,) = torch.autograd.grad(loss, theta)
    assert abs(loss.item() - prob.loss_fp64(theta.detach().numpy())) <= 1e-5 * loss.item()
    th = theta.detach().numpy()
    checked = []
    for k, name in enumerate(srs.ADJ_PARAMS):
        h = 1e-4 * abs(th[k])
        hi, lo = th.copy(), th.copy()
        hi[k] += h
        lo[k] -= h
        Lp, Lm = prob.loss_fp64(hi), prob.loss_fp64(lo)
        if abs(Lp - Lm) < 1e-9 * loss.item():
            continue
        fd = (Lp - Lm) / (2 * h)
        assert abs(g[k].item() - fd) <= 1e-3 * abs(fd), (name, g[k].item(), fd)
        checked.append(name)
    assert {"D_CA", "K_ON_DYE", "K_OFF_DYE", "V_RYR"} <= set(checked), checked


def test_mean_trace_gradient_matches_finite_differences(srs):
    """Config-3 form of the loss on the golden mesh: the misfit of the
    realizations' mean dF/F0 trace against the mean trace of the same
    realizations with D_Ca, D_dye, the dye kon/koff and V_RYR raised by 10 %,
    shifted by 0.01 so that over this short run the residual stays well above
    the FP32 trajectory's rounding (the loss is checked to 1e-5)."""
    torch = pytest.importorskip("torch")
    from srs_gb300.autograd import AdjointProblem, LinescanLoss
    p, _ = params_from_golden(srs, "spark")
    p.ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]] = 1
    prob = AdjointProblem(GOLDEN_MESH, p, [31, 32, 33], LINESCAN_DESC, 400, 100,
                          checkpoint_every=128, mean_trace=True)
    th0 = prob.theta0().numpy()
    pert = th0.copy()
    for name in ("D_CA", "D_DYE", "K_ON_DYE", "K_OFF_DYE", "V_RYR"):
        pert[srs.ADJ_PARAMS.index(name)] *= 1.1
    prob.target = prob.mean_trace_fp64(pert) - 0.01
    theta = prob.theta0().requires_grad_()
    loss = LinescanLoss.apply(theta, prob)
    (g,) = torch.autograd.grad(loss, theta)
    assert loss.item() > 0
    assert abs(loss.item() - prob.loss_fp64(th0)) <= 1e-5 * loss.item()
    checked = []
    for k, name in enumerate(srs.ADJ_PARAMS):
        h = 1e-4 * abs(th0[k])
        hi, lo = th0.copy(), th0.copy()
        hi[k] += h
        lo[k] -= h
        Lp, Lm = prob.loss_fp64(hi), prob.loss_fp64(lo)
        if abs(Lp - Lm) < 1e-9 * loss.item():
            continue
        fd = (Lp - Lm) / (2 * h)
        assert abs(g[k].item() - fd) <= 1e-3 * abs(fd), (name, g[k].item(), fd)
        checked.append(name)
    assert {"D_CA", "K_ON_DYE", "V_RYR"} <= set(checked), checked
