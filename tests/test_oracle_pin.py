"""The oracle pinned to the reference: golden fixtures written by the
reference's own cpu/RunSimulation.cpp (tests/golden/gen_golden.py) and,
where the reference sources are present, a live comparison."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_MESH

PROTOCOLS = ["spark", "spark_nogating", "lcc_trigger", "gain_clamp", "fidelity"]


def test_oracle_steps_match_reference_golden(oracle):
    from oracle import Mesh
    d = np.load(os.path.join(GOLDEN, "ref_steps.npz"))
    m = Mesh(oracle, GOLDEN_MESH, int(d["ints"][9]), d["reals"])
    S = m.initial_states()
    ryr = np.zeros(m.NR, np.int32)
    ryr[4] = 1
    lcc = np.ones(m.NL, np.int32)
    lccv = 2 * np.ones(m.NL, np.int32)
    for _ in range(int(d["n_steps"])):
        m.explicit_step(S, ryr, lcc, lccv)
    assert np.array_equal(S, d["states"])  # bit-exact


@pytest.mark.parametrize("name", PROTOCOLS)
def test_oracle_run_matches_reference_golden(oracle, name):
    from oracle import Mesh, RNG_REFERENCE
    d = np.load(os.path.join(GOLDEN, "ref_run_%s.npz" % name))
    m = Mesh(oracle, GOLDEN_MESH, int(d["ints"][9]), d["reals"])
    rows, S, t_end, n = m.run_simulation(d["ints"], RNG_REFERENCE, 0, 0)
    assert rows.shape == d["rows"].shape
    assert np.array_equal(rows, d["rows"])
    assert np.array_equal(S, d["states"])


def _reference():
    from oracle import Reference
    try:
        return Reference()
    except FileNotFoundError:
        pytest.skip("reference sources not present")


def test_oracle_matches_live_reference_on_config_mesh(oracle, box_mesh, srs):
    from oracle import Mesh, RNG_REFERENCE
    ref = _reference()
    base, _ = box_mesh
    p = srs.default_parameters().set(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=24, T_FINAL=0.003,
                                     OUTPUT_STATES_INTERVAL=0.001)
    ints, reals = np.array(p.ints[:]), np.array(p.reals[:])
    m = Mesh(oracle, base, 1, reals)
    rows_r, S_r = ref.run_simulation(m, ints)
    rows_o, S_o, _, _ = m.run_simulation(ints, RNG_REFERENCE, 0, 0)
    assert np.array_equal(rows_r, rows_o)
    assert np.array_equal(S_r, S_o)


def test_philox_known_answers(oracle):
    """Philox4x32-10 known-answer vectors published with Random123."""
    import ctypes as C
    cases = [
        ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for ctr, key, want in cases:
        c = np.array(ctr, np.uint32)
        o = np.zeros(4, np.uint32)
        oracle.lib.or_philox4x32_10(c.ctypes.data_as(C.c_void_p), key[0], key[1],
                                    o.ctypes.data_as(C.c_void_p))
        assert [int(x) for x in o] == want


def test_own_log_exp_accuracy(oracle):
    L = oracle.lib
    xs = np.geomspace(1e-6, 1e5, 2001).astype(np.float32)
    got = np.array([L.or_logf(float(x)) for x in xs], np.float64)
    ref = np.log(xs.astype(np.float64))
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1.0)) < 4e-7
    ys = np.linspace(-60, 60, 2001).astype(np.float32)
    got = np.array([L.or_exp2f(float(y)) for y in ys], np.float64)
    ref = np.exp2(ys.astype(np.float64))
    assert np.max(np.abs(got - ref) / ref) < 4e-7
    us = np.random.default_rng(0).random(1000) + 1e-12
    got = np.array([L.or_log(float(u)) for u in us])
    assert np.max(np.abs(got - np.log(us)) / np.maximum(np.abs(np.log(us)), 1e-3)) < 1e-15


def test_linescan_restatement_matches_tool_fixture():
    """oracle/linescan.py against the reference line-scan tool's output
    committed in tests/golden/linescan_tool.npz (%g: 5e-6 relative)."""
    import json

    from conftest import GOLDEN, GOLDEN_MESH
    from oracle import Mesh, Oracle, linescan
    d = np.load(os.path.join(GOLDEN, "linescan_tool.npz"))
    desc = json.loads(str(d["desc"]))
    N = d["states"].shape[1] // 6
    m = Mesh(Oracle(), GOLDEN_MESH, 1, np.zeros(56))
    W, pad = linescan.weights(GOLDEN_MESH, m.elements()["order"], desc)
    got = np.array([pad + W @ S[5 * N:] for S in d["states"]])
    assert np.allclose(got, d["tool_output"], rtol=5e-6, atol=0)


def test_compact_compensation_round_trip_matches_numpy_float16(oracle):
    """The FP32 engines keep Euler compensation terms as IEEE halves of
    c * 2^24 (srs_gb300/csrc/srs_comp.h); the oracle's restatement (the
    compiler's _Float16) against numpy's float16 rounding on values across
    the whole range, subnormal halves, the clamp and a NaN included."""
    rng = np.random.default_rng(1)
    c = np.concatenate([rng.standard_normal(4000) * 10.0 ** rng.uniform(-14, -6, 4000),
                        [0.0, -0.0, 2.0 ** -40, -2.0 ** -30, 2.0 ** -25, 1e-3, -1.0, np.inf, -np.inf,
                         np.nan]]).astype(np.float32)
    want = (np.clip(c * np.float32(2 ** 24), -65504, 65504).astype(np.float16).astype(np.float32)
            * np.float32(2.0 ** -24))
    got = np.array([oracle.lib.or_comp_round_trip(float(x)) for x in c], np.float32)
    assert np.array_equal(got, want, equal_nan=True)
    # every finite half value and every midpoint between neighbours (the
    # round-to-nearest-even ties), scaled back by 2^-24
    h = np.arange(0, 0x7C00, dtype=np.uint16).view(np.float16).astype(np.float32)
    mid = (h[:-1] + h[1:]) / np.float32(2.0)  # exact in float32
    for v in (h, mid, -mid):
        c = v * np.float32(2.0 ** -24)
        want = (np.clip(c * np.float32(2 ** 24), -65504, 65504).astype(np.float16).astype(np.float32)
                * np.float32(2.0 ** -24))
        got = np.array([oracle.lib.or_comp_round_trip(float(x)) for x in c], np.float32)
        assert np.array_equal(got, want)
    # 11 significant bits kept where c * 2^24 is a normal half below the clamp
    big = (np.abs(c) * 2 ** 24 >= 2 ** -14) & (np.abs(c) * 2 ** 24 <= 65504)
    assert np.all(np.abs(got[big] - c[big]) <= np.abs(c[big]) * 2.0 ** -11)
