"""ctypes access to the CPU oracles (test infrastructure only).

    Oracle      oracle/_build/liboracle.so — C restatement (srs_oracle.c)
    Reference   oracle/_ref/libsrsref.so   — the reference's own
                cpu/RunSimulation.cpp driven by oracle/ref_harness.cpp

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, and only to compare against.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsrsref.so")
RNG_REFERENCE, RNG_PHILOX = 0, 1


def build():
    subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], check=True)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    def __init__(self):
        if not os.path.exists(ORACLE_SO):
            build()
        self.lib = C.CDLL(ORACLE_SO)
        L = self.lib
        vp = C.c_void_p
        L.or_mesh_load.argtypes = [C.c_char_p, C.c_int, vp, C.POINTER(vp)]
        L.or_mesh_load.restype = C.c_int
        L.or_mesh_free.argtypes = [vp]
        L.or_mesh_counts.argtypes = [vp, vp]
        L.or_mesh_operator.argtypes = [vp, vp, vp, vp]
        L.or_mesh_elements.argtypes = [vp, vp, vp, vp, vp, vp]
        L.or_mesh_channels.argtypes = [vp, vp, vp, vp, vp]
        L.or_initial_states.argtypes = [vp, vp, vp]
        L.or_explicit_step.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.or_gating_philox.argtypes = [vp, vp, C.c_double, vp, C.c_uint64, C.c_int64, vp, vp, vp, vp]
        L.or_steps_philox.argtypes = [vp, vp, vp, vp, C.c_uint64, C.c_int64, C.c_int64, vp, vp, vp, vp]
        L.or_reset_philox.argtypes = [vp, vp, vp, C.c_uint64, vp, vp, vp, vp, vp, vp]
        L.or_run_simulation.argtypes = [vp, vp, vp, C.c_int, C.c_uint64, C.c_int, vp, C.c_int64,
                                        C.c_int, vp, vp, vp]
        L.or_run_simulation.restype = C.c_int64
        L.or_fp32_to_dev.argtypes = [vp, vp, vp, vp, vp]
        L.or_fp32_from_dev.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.or_steps_fp32.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_uint64, C.c_int64, C.c_int64, vp,
                                    vp, vp, vp, C.c_int]
        L.or_logf.argtypes = [C.c_float]
        L.or_logf.restype = C.c_float
        L.or_exp2f.argtypes = [C.c_float]
        L.or_exp2f.restype = C.c_float
        L.or_comp_round_trip.argtypes = [C.c_float]
        L.or_comp_round_trip.restype = C.c_float
        L.or_log.argtypes = [C.c_double]
        L.or_log.restype = C.c_double
        L.or_philox4x32_10.argtypes = [vp, C.c_uint32, C.c_uint32, vp]
        L.or_adjoint.argtypes = [vp] * 8 + [C.c_uint64, C.c_int64, C.c_int, C.c_int] + [vp] * 6
        L.or_adjoint.restype = C.c_double
        L.or_adjoint_loss.argtypes = [vp] * 8 + [C.c_uint64, C.c_int64, C.c_int, C.c_int] + [vp] * 4
        L.or_adjoint_loss.restype = C.c_double
        self.adj_params = np.ctypeslib.as_array((C.c_int * 18).in_dll(L, "or_adj_params")).copy()


class Mesh:
    """Oracle mesh: ReadGrid + operator assembly restated."""

    def __init__(self, oracle, base, flag_noflux, reals):
        self.o = oracle
        self.reals = _f64(reals)
        h = C.c_void_p()
        rc = oracle.lib.or_mesh_load(str(base).encode(), int(flag_noflux), _p(self.reals), C.byref(h))
        if rc != 0:
            raise RuntimeError("oracle mesh load failed (%d)" % rc)
        self.h = h
        c = np.zeros(6, np.int32)
        oracle.lib.or_mesh_counts(h, _p(c))
        self.N, self.NF, self.NN, self.NR, self.NL, self.n_jsr = (int(x) for x in c)

    def __del__(self):
        if getattr(self, "h", None):
            self.o.lib.or_mesh_free(self.h)
            self.h = None

    def operator(self):
        aij = np.zeros(5 * self.N)
        nij = np.zeros(4 * self.N, np.int32)
        br = np.zeros(6 * self.N)
        self.o.lib.or_mesh_operator(self.h, _p(aij), _p(nij), _p(br))
        return aij, nij, br

    def elements(self):
        v0, tt = np.zeros(self.N), np.zeros(self.N)
        dom, trop, order = (np.zeros(self.N, np.int32) for _ in range(3))
        self.o.lib.or_mesh_elements(self.h, _p(v0), _p(tt), _p(dom), _p(trop), _p(order))
        return dict(V0=v0, TT=tt, domain=dom, tropc=trop, order=order)

    def channels(self):
        a, b = np.zeros(self.NR, np.int32), np.zeros(self.NR, np.int32)
        c, d = np.zeros(4 * self.NR, np.int32), np.zeros(self.NL, np.int32)
        self.o.lib.or_mesh_channels(self.h, _p(a), _p(b), _p(c), _p(d))
        return dict(ryr_ele=a, ryr_jsr=b, ryr_nb=c, lcc_ele=d)

    def initial_states(self):
        S = np.zeros(6 * self.N)
        self.o.lib.or_initial_states(self.h, _p(self.reals), _p(S))
        return S

    def explicit_step(self, S, ryr, lcc, lccv, globals_=None):
        g = _f64(globals_ if globals_ is not None else
                 [self.reals[15], self.reals[16]])
        self.o.lib.or_explicit_step(self.h, _p(self.reals), _p(g), _p(S), _p(_i32(ryr)), _p(_i32(lcc)),
                                    _p(_i32(lccv)))
        return S

    def steps_philox(self, S, seed, step0, n, ryr, lcc, lccv, res, globals_=None):
        g = _f64(globals_ if globals_ is not None else [self.reals[15], self.reals[16]])
        self.o.lib.or_steps_philox(self.h, _p(self.reals), _p(g), _p(S), C.c_uint64(seed), step0, n,
                                   _p(ryr), _p(lcc), _p(lccv), _p(res))

    def to_fp32(self, S):
        """Deviation-form FP32 state (U: 4N mobile, Im: N immobile) and zero
        compensation terms (CM, CI)."""
        U = np.zeros(4 * self.N, np.float32)
        Im = np.zeros(self.N, np.float32)
        self.o.lib.or_fp32_to_dev(self.h, _p(self.reals), _p(_f64(S)), _p(U), _p(Im))
        return dict(U=U, Im=Im, CM=np.zeros(4 * self.N, np.float32), CI=np.zeros(self.N, np.float32))

    def from_fp32(self, st):
        S = np.zeros(6 * self.N)
        self.o.lib.or_fp32_from_dev(self.h, _p(self.reals), _p(st["U"]), _p(st["Im"]), _p(st["CM"]),
                                    _p(st["CI"]), _p(S))
        return S

    def steps_fp32(self, st, seed, step0, n, ryr, lcc, lccv, res, gating=True, globals_=None,
                   compact=False):
        """FP32 deviation-form steps; compact: the compensation terms are kept
        in the 16-bit form of the large-mesh engine (srs_comp.h)."""
        g = _f64(globals_ if globals_ is not None else [self.reals[15], self.reals[16]])
        self.o.lib.or_steps_fp32(self.h, _p(self.reals), _p(g), _p(st["U"]), _p(st["Im"]), _p(st["CM"]),
                                 _p(st["CI"]), C.c_uint64(seed), step0, n, _p(ryr), _p(lcc), _p(lccv),
                                 _p(res), int(bool(gating)) | (2 if compact else 0))

    def adjoint(self, ints, S0, ch, seed, n_steps, tick_every, W, pad, f0, target, grad=True,
                grad_state=False):
        """Pathwise adjoint (FP64): line-scan loss L and, if grad, dL/dtheta in
        the order of Oracle.adj_params (and dL/dS0 [6][N] if grad_state).
        ch: dict(ryr, lcc, lccv, residuals) of the initial channel state;
        W: dense [n_samples][N] line-scan weights, pad: [n_samples];
        target: [n_ticks][n_samples]."""
        W = _f64(W)
        args = [self.h, _p(_i32(ints)), _p(self.reals), _p(_f64(S0)), _p(_i32(ch["ryr"])),
                _p(_i32(ch["lcc"])), _p(_i32(ch["lccv"])), _p(_f64(ch["residuals"])),
                C.c_uint64(seed), int(n_steps), int(tick_every), W.shape[0], _p(W), _p(_f64(pad)),
                _p(_f64(f0)), _p(_f64(target))]
        if not grad:
            return self.o.lib.or_adjoint_loss(*args), None
        g = np.zeros(18)
        lam0 = np.zeros(6 * self.N) if grad_state else None
        L = self.o.lib.or_adjoint(*args, _p(g), _p(lam0))
        return (L, g, lam0) if grad_state else (L, g)

    def gating_philox(self, V, ca, seed, step, ryr, lcc, lccv, res):
        self.o.lib.or_gating_philox(self.h, _p(self.reals), float(V), _p(_f64(ca)), C.c_uint64(seed),
                                    step, _p(ryr), _p(lcc), _p(lccv), _p(res))

    def reset_philox(self, ints, seed):
        S = np.zeros(6 * self.N)
        ryr = np.zeros(self.NR, np.int32)
        lcc = np.zeros(self.NL, np.int32)
        lccv = np.zeros(self.NL, np.int32)
        res = np.zeros(self.NR + self.NL)
        step = np.zeros(1, np.int64)
        self.o.lib.or_reset_philox(self.h, _p(_i32(ints)), _p(self.reals), C.c_uint64(seed), _p(S),
                                   _p(ryr), _p(lcc), _p(lccv), _p(res), _p(step))
        return dict(states=S, ryr=ryr, lcc=lcc, lccv=lccv, residuals=res, lcc_close_step=int(step[0]))

    def run_simulation(self, ints, mode, seed_or_rank, index=0, row_capacity=None, row_w=7):
        R = self.reals
        if row_capacity is None:
            row_capacity = int(R[0] / R[2]) + 8
        rows = np.zeros((row_capacity, row_w), np.float32)
        S = np.zeros(6 * self.N)
        t_end = np.zeros(1)
        n_steps = np.zeros(1, np.int64)
        n = self.o.lib.or_run_simulation(self.h, _p(_i32(ints)), _p(R), mode, C.c_uint64(seed_or_rank),
                                         index, _p(rows), row_capacity, row_w, _p(S), _p(t_end),
                                         _p(n_steps))
        return rows[:n].copy(), S, float(t_end[0]), int(n_steps[0])


class Reference:
    """The reference's cpu/RunSimulation.cpp, compiled in oracle/_ref."""

    def __init__(self):
        if not os.path.exists(REF_SO):
            build()
        if not os.path.exists(REF_SO):
            raise FileNotFoundError("reference sources unavailable: %s not built" % REF_SO)
        self.lib = C.CDLL(REF_SO)
        vp = C.c_void_p
        self.lib.ref_explicit_steps.argtypes = [C.c_int] * 3 + [vp] * 18 + [C.c_int64, C.c_uint]
        self.lib.ref_run_simulation.argtypes = [C.c_int] * 3 + [vp] * 14 + [C.c_int, C.c_int, vp,
                                                                             C.c_int64, C.c_int, vp]
        self.lib.ref_run_simulation.restype = C.c_int64
        self.lib.ref_set_linescan.argtypes = [C.c_int] + [vp] * 5 + [C.c_int64]
        self.lib.ref_linescan_rows.restype = C.c_int64

    @staticmethod
    def _mesh_args(m):
        aij, nij, br = m.operator()
        e = m.elements()
        ch = m.channels()
        keep = [aij, nij, br, e["V0"], e["TT"], e["domain"], e["tropc"], ch["ryr_ele"], ch["ryr_jsr"],
                ch["ryr_nb"], ch["lcc_ele"]]
        return keep, [m.N, m.NR, m.NL] + [_p(a) for a in keep]

    def explicit_steps(self, m, ints, S, ryr, lcc, lccv, res, n, srand_seed=1):
        keep, args = self._mesh_args(m)
        ints = _i32(ints)
        self.lib.ref_explicit_steps(*args, _p(ints), _p(m.reals), _p(S), _p(ryr), _p(lcc), _p(lccv),
                                    _p(res), n, srand_seed)

    def run_simulation(self, m, ints, rank=0, index=0, row_capacity=None, row_w=7):
        keep, args = self._mesh_args(m)
        R = m.reals
        if row_capacity is None:
            row_capacity = int(R[0] / R[2]) + 8
        rows = np.zeros((row_capacity, row_w), np.float32)
        S0 = m.initial_states()
        S = np.zeros(6 * m.N)
        ints = _i32(ints)
        n = self.lib.ref_run_simulation(*args, _p(ints), _p(R), _p(S0), rank, index, _p(rows),
                                        row_capacity, row_w, _p(S))
        if n < 0:
            raise ValueError("reference harness needs an explicit initial channel")
        return rows[:n].copy(), S

    def run_simulation_linescan(self, m, ints, W, pad, rank=0, index=0, row_capacity=None, row_w=7,
                                ls_capacity=None):
        """run_simulation with the line scan F = pad + W @ [CaDye] (W dense,
        [n_samples][N] in the mesh's numbering) taken at every grid-file call
        of RunSimulation (t = 0, each grid-file step when OUTPUT_GRID_FLAG is
        set, the end).  Returns (rows, final states, line-scan rows
        [n_calls][1 + n_samples] = t, F_0 .. F_{n-1})."""
        from oracle.linescan import to_csr
        R = m.reals
        if ls_capacity is None:
            ls_capacity = int(R[0] / R[3]) + 8 if R[3] > 0 else 8
        ptr, col, w = to_csr(np.asarray(W, np.float64))
        pad = _f64(pad)
        out = np.zeros((ls_capacity, len(pad) + 1))
        self.lib.ref_set_linescan(len(pad), _p(ptr), _p(col), _p(w), _p(pad), _p(out), ls_capacity)
        try:
            rows, S = self.run_simulation(m, ints, rank, index, row_capacity, row_w)
            n = int(self.lib.ref_linescan_rows())
        finally:
            self.lib.ref_set_linescan(0, None, None, None, None, None, 0)
        return rows, S, out[:n].copy()


REF_IO_SO = os.path.join(HERE, "_ref", "libsrsref_io.so")
REF_LINESCAN = os.path.join(HERE, "_ref", "linescan")


class RefIO:
    """The reference's own cpu/InitFuncs.cpp and cpu/OutputFuncs.cpp
    (oracle/_ref/libsrsref_io.so, driven by oracle/ref_io_harness.cpp)."""

    def __init__(self):
        if not os.path.exists(REF_IO_SO):
            raise FileNotFoundError("reference sources unavailable: %s not built" % REF_IO_SO)
        L = self.lib = C.CDLL(REF_IO_SO)
        vp = C.c_void_p
        L.refio_read_parameters.argtypes = [C.c_char_p, vp, vp, vp]
        L.refio_load.argtypes = [C.c_char_p, vp, vp]
        L.refio_load.restype = vp
        for name in ("refio_counts", "refio_get_states", "refio_set_states", "refio_reset_states"):
            getattr(L, name).argtypes = [vp, vp]
        L.refio_operator.argtypes = [vp] * 4
        L.refio_elements.argtypes = [vp] * 5
        L.refio_channels.argtypes = [vp] * 5
        L.refio_open_random_ryr.argtypes = [vp, C.c_int, C.c_int, vp]
        L.refio_open_random_ryr.restype = C.c_int
        L.refio_write_grid.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double]
        L.refio_free.argtypes = [vp]
        L.refio_set_ryr.argtypes = [vp, vp]

    def read_parameters(self, path):
        """ReadParameters: (ints[19], reals[56], chars[4] as bytes)."""
        ints = np.zeros(19, np.int32)
        reals = np.zeros(56)
        chars = C.create_string_buffer(4 * 255)
        self.lib.refio_read_parameters(str(path).encode(), _p(ints), _p(reals), chars)
        return ints, reals, [chars.raw[i * 255:(i + 1) * 255].split(b"\0")[0] for i in range(4)]

    def load(self, base, ints, reals):
        return RefGrid(self, base, ints, reals)


class RefGrid:
    """ReadGrid + InitializeDefaultGrid + InitializeDomainStruct of the
    reference (cpu/main.cpp:170-189) for one mesh and parameter set."""

    def __init__(self, io, base, ints, reals):
        self.io, self.lib = io, io.lib
        self.ints, self.reals = _i32(ints), _f64(reals)
        self.h = self.lib.refio_load(str(base).encode(), _p(self.ints), _p(self.reals))
        c = np.zeros(5, np.int32)
        self.lib.refio_counts(self.h, _p(c))
        self.N, self.NF, self.NN, self.NR, self.NL = (int(x) for x in c)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.refio_free(self.h)
            self.h = None

    def operator(self):
        aij, nij, br = np.zeros(5 * self.N), np.zeros(4 * self.N, np.int32), np.zeros(6 * self.N)
        self.lib.refio_operator(self.h, _p(aij), _p(nij), _p(br))
        return aij, nij, br

    def elements(self):
        v0, tt = np.zeros(self.N), np.zeros(self.N)
        dom, trop = np.zeros(self.N, np.int32), np.zeros(self.N, np.int32)
        self.lib.refio_elements(self.h, _p(v0), _p(tt), _p(dom), _p(trop))
        return dict(V0=v0, TT=tt, domain=dom, tropc=trop)

    def channels(self):
        a, b = np.zeros(self.NR, np.int32), np.zeros(self.NR, np.int32)
        c, d = np.zeros(4 * self.NR, np.int32), np.zeros(self.NL, np.int32)
        self.lib.refio_channels(self.h, _p(a), _p(b), _p(c), _p(d))
        return dict(ryr_ele=a, ryr_jsr=b, ryr_nb=c, lcc_ele=d)

    def states(self):
        S = np.zeros(6 * self.N)
        self.lib.refio_get_states(self.h, _p(S))
        return S

    def set_states(self, S):
        self.lib.refio_set_states(self.h, _p(_f64(S)))

    def reset_states(self):
        S = np.zeros(6 * self.N)
        self.lib.refio_reset_states(self.h, _p(S))
        return S

    def open_random_ryr(self, rank, index, ryr=None):
        """OpenRandomRyR for (rank, ensemble index); returns (index opened, states)."""
        r = _i32(ryr if ryr is not None else np.zeros(self.NR)).copy()
        k = self.lib.refio_open_random_ryr(self.h, int(rank), int(index), _p(r))
        return k, r

    def write_grid(self, directory, ryr=None, rank=0, run=0, n=0, t=0.0):
        """WriteToGridFiles of the current states (and the RyR states given);
        returns the path <directory>/grid_<rank>_<run>_<n>.vtk."""
        if ryr is not None:
            self.lib.refio_set_ryr(self.h, _p(_i32(ryr)))
        self.lib.refio_write_grid(self.h, str(directory).encode(), int(rank), int(run), int(n), float(t))
        return os.path.join(str(directory), "grid_%d_%d_%d.vtk" % (rank, run, n))
