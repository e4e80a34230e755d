"""The allocation-free step, checked against the regular FP64 engine.

srs_explicit_step_fp64_noalloc exists for callers that cannot allocate
device memory themselves (a host application that owns every device
allocation through its own pool, or a real-time loop in which cudaMalloc must
not run): they hand over their own device buffers and the library uses only
a fixed array compiled into it.
This test builds those buffers with torch, runs two consecutive steps
through the C ABI and requires bit-identical results to two steps of the
regular FP64 engine (srs_explicit_step), whose arithmetic is the
reference's.  It lives in its own file, collected last, and passes both
alone and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import GOLDEN_MESH, params_from_golden

pytestmark = pytest.mark.gpu


def _chan_csr(N, ch):
    per = [[] for _ in range(N)]
    for i, e in enumerate(ch["ryr_ele"]):
        per[e].append((0, i))
    for i, e in enumerate(ch["ryr_jsr"]):
        per[e].append((1, i))
    for i, e in enumerate(ch["lcc_ele"]):
        per[e].append((2, i))
    ptr, lst = [0], []
    for j in range(N):
        for k, c in per[j]:
            lst += [k, c]
        ptr.append(len(lst) // 2)
    return np.array(ptr, np.int32), np.array(lst if lst else [0, 0], np.int32), per


def test_noalloc_step_matches_regular_engine(srs):
    import torch
    p, _ = params_from_golden(srs, "spark")
    g = srs.Grid(p, GOLDEN_MESH)
    seeds = [101, 102, 103]
    R = len(seeds)
    sim = srs.Simulation(g, p, R, srs.FP64, srs.ENGINE_PLAIN, seeds=seeds)
    st0 = [sim.get_state(r) for r in range(R)]
    expect = []
    for _ in range(2):
        sim.explicit_step(1)
        expect.append([sim.get_state(r) for r in range(R)])

    N = g.n_ele
    aij, nij, br = g.operator()
    el = g.elements()
    ch = g.channels()
    reals = np.array(p.reals[:], np.float64)
    br4 = np.concatenate([br[0:N], br[N:2 * N], br[2 * N:3 * N], br[5 * N:6 * N]])
    bhi = el["TT"] * reals[27] / (el["V0"] * 1e-15)
    blo = el["TT"] * reals[29] / (el["V0"] * 1e-15)
    ptr, lst, per = _chan_csr(N, ch)
    flags = (el["domain"] == 1).astype(np.int32) | (el["tropc"] != 0).astype(np.int32) << 1 | \
        np.array([4 if per[j] else 0 for j in range(N)], np.int32)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    bufs = dict(aij=T(aij), nij=T(nij), br4=T(br4), v0=T(el["V0"]), bhi=T(bhi), blo=T(blo),
                flags=T(flags), chan_ptr=T(ptr), chan_list=T(lst), ryr_ele=T(ch["ryr_ele"]),
                ryr_jsr=T(ch["ryr_jsr"]), ryr_nb=T(ch["ryr_nb"]), lcc_ele=T(ch["lcc_ele"]))
    S = [T(np.concatenate([s["states"] for s in st0])),
         torch.zeros(R * 6 * N, dtype=torch.float64, device=dev)]
    ryr = T(np.concatenate([s["ryr"] for s in st0]))
    lcc = T(np.concatenate([s["lcc"] for s in st0]))
    lccv = T(np.concatenate([s["lccv"] for s in st0]))
    res = T(np.concatenate([s["residuals"] for s in st0]))
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    seeds_h = np.array(seeds, np.uint64)
    torch.cuda.synchronize()
    for k in range(2):
        d = srs.NoallocStep()
        d.n_ele, d.n_realizations, d.n_ryr, d.n_lcc = N, R, g.n_ryr, g.n_lcc
        for name, t in bufs.items():
            setattr(d, name, t.data_ptr())
        d.states_in, d.states_out = S[k % 2].data_ptr(), S[(k + 1) % 2].data_ptr()
        d.ryr_states, d.lcc_states = ryr.data_ptr(), lcc.data_ptr()
        d.lccv_states, d.residuals = lccv.data_ptr(), res.data_ptr()
        d.status = status.data_ptr()
        d.reals = reals.ctypes.data_as(C.c_void_p).value
        d.seeds = seeds_h.ctypes.data_as(C.c_void_p).value
        d.step = k
        d.v_m, d.ca_nsr = reals[15], reals[16]
        d.nogating = int(p.ints[14])
        d.stream = torch.cuda.current_stream().cuda_stream
        srs.explicit_step_fp64_noalloc(d)
        torch.cuda.synchronize()
        out = S[(k + 1) % 2].cpu().numpy().reshape(R, 6 * N)
        for r in range(R):
            assert np.array_equal(out[r], expect[k][r]["states"]), (k, r)
            assert np.array_equal(ryr.cpu().numpy().reshape(R, -1)[r], expect[k][r]["ryr"])
            assert np.array_equal(res.cpu().numpy().reshape(R, -1)[r], expect[k][r]["residuals"])
            assert np.array_equal(lcc.cpu().numpy().reshape(R, -1)[r], expect[k][r]["lcc"])
            assert np.array_equal(lccv.cpu().numpy().reshape(R, -1)[r], expect[k][r]["lccv"])
    assert int(status.item()) == 0


def test_noalloc_rejects_oversized_batch(srs):
    d = srs.NoallocStep()
    d.n_ele, d.n_realizations = 10, srs.NOALLOC_MAX_REALIZATIONS + 1
    with pytest.raises(srs.SrsError) as e:
        srs.explicit_step_fp64_noalloc(d)
    assert e.value.status == -1
    assert "realizations" in str(e.value)
