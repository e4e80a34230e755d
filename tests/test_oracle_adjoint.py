"""The FP64 pathwise adjoint of the oracle against central finite differences.

The oracle's adjoint (oracle/srs_oracle.c, or_adjoint) is the reference for the
device adjoint, so it is itself pinned here: on the golden mesh, from the
reset state of one realization, 600 explicit steps with Philox gating (or
none), a line-scan loss at every 100th step, and every parameter whose loss
change is resolvable in double precision must agree with
  (L(theta + h) - L(theta - h)) / 2h,  h = 1e-4 |theta|,
to 1e-4 relative.  The perturbed runs use the same seed (common random
numbers) and the same initial state; the mesh is reloaded with the perturbed
parameters, so the boundary rates follow them as they do in the engines.
"""
import numpy as np
import pytest

from conftest import GOLDEN_MESH, params_from_golden

N_STEPS, TICK = 600, 100


def _case(oracle, srs, noflux, gating):
    from oracle import Mesh
    p, _ = params_from_golden(srs, "spark")
    ints = np.array(p.ints[:], np.int32)
    ints[srs.I["FLAG_NO_FLUX_BOUNDARY"]] = noflux
    ints[srs.I["FLAG_NO_GATING"]] = 0 if gating else 1
    reals = np.array(p.reals[:])
    m = Mesh(oracle, GOLDEN_MESH, noflux, reals)
    st = m.reset_philox(ints, 7)
    rng = np.random.default_rng(0)
    ns = 5
    W = np.abs(rng.standard_normal((ns, m.N))) * 1e-3
    pad = np.full(ns, 0.1)
    f0 = pad + W @ st["states"][5 * m.N:6 * m.N]
    target = rng.standard_normal((N_STEPS // TICK, ns)) * 0.01
    return m, ints, reals, st, (W, pad, f0, target)


@pytest.mark.parametrize("noflux,gating", [(0, 1), (1, 0)])
def test_oracle_adjoint_matches_central_differences(oracle, srs, noflux, gating):
    from oracle import Mesh
    m, ints, reals, st, (W, pad, f0, target) = _case(oracle, srs, noflux, gating)
    L0, g = m.adjoint(ints, st["states"], st, 7, N_STEPS, TICK, W, pad, f0, target)
    assert L0 > 0
    checked = 0
    for k, idx in enumerate(oracle.adj_params):
        h = 1e-4 * abs(reals[idx])
        lo, hi = reals.copy(), reals.copy()
        hi[idx] += h
        lo[idx] -= h
        Lp, _ = Mesh(oracle, GOLDEN_MESH, noflux, hi).adjoint(ints, st["states"], st, 7, N_STEPS, TICK,
                                                               W, pad, f0, target, grad=False)
        Lm, _ = Mesh(oracle, GOLDEN_MESH, noflux, lo).adjoint(ints, st["states"], st, 7, N_STEPS, TICK,
                                                               W, pad, f0, target, grad=False)
        if abs(Lp - Lm) < 1e-9 * L0:  # below the loss's own rounding: not resolvable
            continue
        fd = (Lp - Lm) / (2 * h)
        assert abs(g[k] - fd) <= 1e-4 * abs(fd), (srs.ADJ_PARAMS[k], g[k], fd)
        checked += 1
    assert checked >= 14


def test_oracle_parameter_order_matches_c_abi(oracle, srs):
    lib = srs.library()
    assert [lib.srs_adjoint_param_index(k) for k in range(srs.N_ADJ)] == list(oracle.adj_params)
    assert [srs.R[n] for n in srs.ADJ_PARAMS] == list(oracle.adj_params)


def test_oracle_initial_state_gradient_matches_central_differences(oracle, srs):
    m, ints, reals, st, (W, pad, f0, target) = _case(oracle, srs, 1, 1)
    S0 = st["states"]
    L0, _, lam0 = m.adjoint(ints, S0, st, 7, N_STEPS, TICK, W, pad, f0, target, grad_state=True)
    N = m.N
    # the largest Ca, dye and calmodulin sensitivities; the loss is close to
    # linear in the state, so a wide step keeps the difference well above the
    # loss's rounding
    for sp in (0, 5, 2):
        j = int(np.argmax(np.abs(lam0[sp * N:(sp + 1) * N])))
        h = 1e-2 * max(abs(S0[sp * N + j]), 1e-3)
        Sp, Sm = S0.copy(), S0.copy()
        Sp[sp * N + j] += h
        Sm[sp * N + j] -= h
        Lp, _ = m.adjoint(ints, Sp, st, 7, N_STEPS, TICK, W, pad, f0, target, grad=False)
        Lm, _ = m.adjoint(ints, Sm, st, 7, N_STEPS, TICK, W, pad, f0, target, grad=False)
        fd = (Lp - Lm) / (2 * h)
        assert abs(lam0[sp * N + j] - fd) <= 1e-4 * abs(fd), (sp, j, lam0[sp * N + j], fd)
