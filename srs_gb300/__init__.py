"""srs_gb300 — GB300-native (sm_103a) spark timestep of the SRS Ca2+-spark model.

Python mirror of the reference's C++ function set (cpu/parameters.h:252-275)
over the C ABI of include/srs_gb300.h, loaded with ctypes from the in-tree
library srs_gb300/libsrs_gb300.so.  Names follow the reference:

    read_parameters(path)            ReadParameters      cpu/InitFuncs.cpp:25
    Grid(params, mesh_base)          ReadGrid + InitializeDomainStruct
    Simulation(grid, params, ...)    per-realization device state
      .reset()                       cpu/main.cpp:216-257 initial opening
      .explicit_step(n)              ExplicitStep (+UpdateChannelGating)
      .run_simulation(row_capacity)  RunSimulation with states rows

There is no CPU fallback: if the library is missing, importing the module
raises; if no sm_103a GPU is present, creating a Simulation raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsrs_gb300.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "srs_gb300.h")

N_INT, N_REAL, N_CHAR = 19, 56, 4
FP64, FP32 = 64, 32
ENGINE_PLAIN, ENGINE_RESIDENT = 0, 1
STATES_ROW_BASE = 7

# parameter indices (cpu/parameters.h:18-96)
I = dict(OUTPUT_GRID_FLAG=0, FLAG_FIDELITY_SIM=1, FLAG_CLOCK_SEED=2, RAND_SEED_0=3, RAND_ADD_A=4,
         RAND_ADD_B=5, INITIALIZE_FROM_FILE=6, CUDA_DEVICE=7, FLAG_SECONDARY_GRADIENT=8,
         FLAG_NO_FLUX_BOUNDARY=9, N_RYR_FIDELITY=10, FLAG_LCC=11, LCC_INDEX=12, FLAG_V_CLAMP=13,
         FLAG_NO_GATING=14, GATING_FFWD=15, FLAG_RYR_OUT=16, N_SIMS=17, INIT_RYR=18)
R = dict(T_FINAL=0, T_STEP=1, OUTPUT_STATES_INTERVAL=2, OUTPUT_GRID_INTERVAL=3, C_MIN=4, D_CA=5,
         D_CA_JSR=6, D_ATP=7, D_CMDN=8, D_TRPN=9, D_CSQN=10, D_DYE=11, D_EGTA=12, C_0_CA=13,
         C_0_CA_JSR=14, DEFAULT_VM=15, DEFAULT_CA_NSR=16, CA_0=17, B_TOT_ATP=18, K_OFF_ATP=19,
         K_ON_ATP=20, B_TOT_CMDN=21, K_OFF_CMDN=22, K_ON_CMDN=23, B_TOT_TRPN=24, K_OFF_TRPN=25,
         K_ON_TRPN=26, B_TOT_SL_HI=27, K_D_SL_HI=28, B_TOT_SL_LO=29, K_D_SL_LO=30, B_TOT_DYE=31,
         K_OFF_DYE=32, K_ON_DYE=33, B_T_JSR=34, K_M_JSR=35, V_REFILL=36, V_RYR=37, V_CELL=38,
         K_ON_CSQN=39, K_OFF_CSQN=40, RYR_ETA=41, RYR_A_STAR=42, RYR_EPS_CC=43, RYR_EPS_OO=44,
         RYR_K_PLUS=45, RYR_K_MINUS=46, RYR_PHI_M=47, RYR_PHI_B=48, K_D_i=49, K_D_SR=50, A_P=51,
         LCC_DURATION=52, T_CLAMP=53, V_CLAMP=54, INIT_RYR_HOLD=55)
SPECIES = ("CA", "ATP", "CMDN", "TRPN", "CSQN", "DYE")
# parameters of the adjoint gradient, in srs_adjoint order (SRS_ADJ_*)
ADJ_PARAMS = ("D_CA", "D_DYE", "K_ON_CMDN", "K_OFF_CMDN", "K_ON_TRPN", "K_OFF_TRPN", "K_ON_CSQN",
              "K_OFF_CSQN", "K_ON_DYE", "K_OFF_DYE", "V_RYR", "A_P", "B_TOT_SL_HI", "K_D_SL_HI",
              "D_ATP", "D_CMDN", "K_ON_ATP", "K_OFF_ATP")
N_ADJ = len(ADJ_PARAMS)


class SrsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (_lib.srs_status_string(status).decode(), status, msg))
        self.status = status


class Params(C.Structure):
    """ParamStruct (cpu/parameters.h:234-246)."""
    _fields_ = [("ints", C.c_int * N_INT), ("reals", C.c_double * N_REAL),
                ("chars", (C.c_char * 255) * N_CHAR)]

    def copy(self):
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def set(self, **kw):
        for k, v in kw.items():
            if k in I:
                self.ints[I[k]] = int(v)
            elif k in R:
                self.reals[R[k]] = float(v)
            else:
                raise KeyError(k)
        return self


class _GridInfo(C.Structure):
    _fields_ = [("n_ele", C.c_int), ("n_face", C.c_int), ("n_nodes", C.c_int), ("n_ryr", C.c_int),
                ("n_lcc", C.c_int), ("n_jsr", C.c_int), ("vol_jsr", C.c_double),
                ("max_diag", C.c_double)]


class _SimDesc(C.Structure):
    _fields_ = [("n_realizations", C.c_int), ("precision", C.c_int), ("engine", C.c_int),
                ("threads_per_cta", C.c_int), ("cluster_size", C.c_int),
                ("steps_per_launch", C.c_int), ("seeds", C.POINTER(C.c_uint64))]


class _SimConfig(C.Structure):
    _fields_ = [("engine", C.c_int), ("precision", C.c_int), ("threads_per_cta", C.c_int),
                ("cluster_size", C.c_int), ("steps_per_launch", C.c_int), ("smem_bytes", C.c_int),
                ("kernel_launches", C.c_int64), ("reset_h2d_bytes", C.c_int64),
                ("ctl_bytes", C.c_int64), ("engine_elements", C.c_int64)]


class _RunOutput(C.Structure):
    _fields_ = [("rows", C.POINTER(C.c_float)), ("row_capacity", C.c_int64), ("row_width", C.c_int),
                ("n_rows", C.POINTER(C.c_int64)), ("t_end", C.POINTER(C.c_double)),
                ("n_steps", C.POINTER(C.c_int64))]


class BoxMeshSpec(C.Structure):
    """Synthetic box-dyad mesh (see csrc/meshgen.cpp)."""
    _fields_ = [("box_x", C.c_double), ("box_y", C.c_double), ("box_z", C.c_double),
                ("foot_half_x", C.c_double), ("foot_half_y", C.c_double),
                ("n_foot_x", C.c_int), ("n_foot_y", C.c_int), ("n_out_x", C.c_int),
                ("n_out_y", C.c_int), ("cleft_h", C.c_double), ("jsr_h", C.c_double),
                ("n_cleft_z", C.c_int), ("n_jsr_z", C.c_int), ("n_above_z", C.c_int),
                ("r_trpn", C.c_double), ("flag_tt", C.c_int), ("ryr_mode", C.c_int),
                ("ryr_nx", C.c_int), ("ryr_ny", C.c_int), ("ryr_pitch", C.c_double),
                ("ryr_depth", C.c_double), ("ryr_cx", C.c_double), ("ryr_cy", C.c_double),
                ("ryr_count", C.c_int), ("ryr_radius", C.c_double), ("n_lcc", C.c_int),
                ("lcc_half", C.c_double), ("lcc_seed", C.c_uint64), ("seed", C.c_uint64)]


MAX_SITES = 8


_GRID_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_int64, C.c_double, C.POINTER(C.c_int))


class MultiSiteSpec(C.Structure):
    """Synthetic multi-site release unit (srs_multisite_spec, csrc/meshgen.cpp)."""
    _fields_ = [("box_x", C.c_double), ("box_y", C.c_double), ("box_z", C.c_double),
                ("h_fine", C.c_double), ("h_max", C.c_double), ("growth", C.c_double),
                ("cleft_h", C.c_double), ("jsr_h", C.c_double),
                ("n_cleft_z", C.c_int), ("n_jsr_z", C.c_int), ("r_trpn", C.c_double),
                ("flag_tt", C.c_int), ("n_sites", C.c_int),
                ("site_x", C.c_double * MAX_SITES), ("site_y", C.c_double * MAX_SITES),
                ("site_ryr", C.c_int * MAX_SITES), ("site_radius", C.c_double * MAX_SITES),
                ("foot_margin", C.c_double), ("ryr_pitch", C.c_double), ("ryr_depth", C.c_double),
                ("sheet_half", C.c_double), ("seed", C.c_uint64)]


class LinescanDesc(C.Structure):
    """srs_linescan_desc (linescan/main.cpp:160-225)."""
    _fields_ = [("axis", C.c_int), ("offset1", C.c_double), ("offset2", C.c_double),
                ("x_min", C.c_double), ("x_max", C.c_double), ("res", C.c_double),
                ("var_x", C.c_double), ("var_y", C.c_double), ("var_z", C.c_double),
                ("r_thresh", C.c_double), ("f0_pad", C.c_double), ("pad_res", C.c_double),
                ("pad_min", C.c_double), ("pad_max", C.c_double), ("domain", C.c_double * 6)]


NOALLOC_MAX_REALIZATIONS = 256


ADJ_LAMBDA_GLOBAL = 1
ADJ_NO_STAGE = 2
ADJ_STAGE = 4
ADJ_MEAN_TRACE = 8


class _AdjDesc(C.Structure):
    _fields_ = [("n_steps", C.c_int64), ("tick_every", C.c_int), ("checkpoint_every", C.c_int),
                ("f0", C.c_void_p), ("target", C.c_void_p), ("flags", C.c_int),
                ("threads_per_cta", C.c_int), ("cta_partitions", C.c_int),
                ("max_checkpoints", C.c_int)]


class _AdjOut(C.Structure):
    _fields_ = [("loss", C.c_void_p), ("grad", C.c_void_p), ("grad_state", C.c_void_p)]


class NoallocStep(C.Structure):
    """srs_noalloc_step: one FP64 ExplicitStep on caller-owned device buffers."""
    _fields_ = [("n_ele", C.c_int), ("n_realizations", C.c_int), ("n_ryr", C.c_int),
                ("n_lcc", C.c_int)] + [
        (n, C.c_void_p) for n in ("aij", "nij", "br4", "v0", "bhi", "blo", "flags", "chan_ptr",
                                  "chan_list", "ryr_ele", "ryr_jsr", "ryr_nb", "lcc_ele",
                                  "states_in", "states_out", "ryr_states", "lcc_states",
                                  "lccv_states", "residuals", "status", "reals", "seeds")] + [
        ("step", C.c_int64), ("v_m", C.c_double), ("ca_nsr", C.c_double), ("nogating", C.c_int),
        ("stream", C.c_void_p)]


# Every symbol declared in include/srs_gb300.h with its ctypes signature.
_P = C.c_void_p
_SIGS = {
    "srs_status_string": (C.c_char_p, [C.c_int]),
    "srs_last_error": (C.c_char_p, []),
    "srs_version": (C.c_char_p, []),
    "srs_default_parameters": (None, [C.POINTER(Params)]),
    "srs_read_parameters": (C.c_int, [C.POINTER(Params), C.c_char_p]),
    "srs_read_grid": (C.c_int, [C.POINTER(Params), C.c_char_p, C.POINTER(_P)]),
    "srs_free_grid": (None, [_P]),
    "srs_grid_get_info": (C.c_int, [_P, C.POINTER(_GridInfo)]),
    "srs_grid_get_operator": (C.c_int, [_P, _P, _P, _P]),
    "srs_grid_get_elements": (C.c_int, [_P, _P, _P, _P, _P, _P]),
    "srs_grid_get_channels": (C.c_int, [_P, _P, _P, _P, _P]),
    "srs_initial_states": (C.c_int, [_P, C.POINTER(Params), _P]),
    "srs_sim_create": (C.c_int, [_P, C.POINTER(Params), C.POINTER(_SimDesc), C.POINTER(_P)]),
    "srs_sim_destroy": (None, [_P]),
    "srs_sim_get_desc": (C.c_int, [_P, C.POINTER(_SimDesc)]),
    "srs_sim_reset": (C.c_int, [_P]),
    "srs_sim_set_state": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P]),
    "srs_sim_get_state": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P]),
    "srs_sim_set_globals": (C.c_int, [_P, C.c_double, C.c_double]),
    "srs_explicit_step": (C.c_int, [_P, C.c_int64]),
    "srs_run_simulation": (C.c_int, [_P, C.POINTER(_RunOutput)]),
    "srs_run_simulation_timed": (C.c_int, [_P, C.POINTER(_RunOutput), C.POINTER(C.c_float), C.c_int,
                                           C.POINTER(C.c_int)]),
    "srs_run_simulation_grid": (C.c_int, [_P, C.POINTER(_RunOutput), C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_int)]),
    "srs_sim_advance_async": (C.c_int, [_P, C.c_int64]),
    "srs_sim_synchronize": (C.c_int, [_P]),
    "srs_sim_time_advance": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_float)]),
    "srs_sim_status": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "srs_sim_get_config": (C.c_int, [_P, C.POINTER(_SimConfig)]),
    "srs_sim_set_prefetch": (C.c_int, [_P, C.c_int]),
    "srs_write_grid_vtk": (C.c_int, [_P, C.c_int, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double]),
    "srs_grid_write_vtk": (C.c_int, [_P, _P, _P, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double]),
    "srs_box_mesh_default": (None, [C.POINTER(BoxMeshSpec)]),
    "srs_box_mesh_write": (C.c_int, [C.POINTER(BoxMeshSpec), C.c_char_p, _P, _P]),
    "srs_multisite_mesh_write": (C.c_int, [C.POINTER(MultiSiteSpec), C.c_char_p, _P, _P]),
    "srs_explicit_step_fp64_noalloc": (C.c_int, [C.POINTER(NoallocStep)]),
    "srs_linescan_setup": (C.c_int, [_P, C.POINTER(LinescanDesc), C.POINTER(C.c_int)]),
    "srs_linescan": (C.c_int, [_P, _P, _P]),
    "srs_sim_total_ca": (C.c_int, [_P, _P]),
    "srs_comp_round_trip": (C.c_int, [_P, _P, C.c_int64, C.c_int]),
    "srs_batch_create": (C.c_int, [_P, C.c_int, C.c_int, C.POINTER(_P)]),
    "srs_batch_destroy": (None, [_P]),
    "srs_batch_advance": (C.c_int, [_P, C.c_int64]),
    "srs_batch_synchronize": (C.c_int, [_P]),
    "srs_batch_time_advance": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_float)]),
    "srs_batch_run_simulation": (C.c_int, [_P, _P]),
    "srs_adjoint_param_index": (C.c_int, [C.c_int]),
    "srs_adjoint": (C.c_int, [_P, C.POINTER(_AdjDesc), C.POINTER(_AdjOut)]),
    "srs_adjoint_plan": (C.c_int, [_P, C.POINTER(_AdjDesc), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int64)]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("srs_gb300: native library %s is missing; run "
                          "`python -c 'import __graft_entry__ as g; g.build()'` first" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_lib = _load()


def _check(rc):
    if rc != 0:
        raise SrsError(rc, _lib.srs_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def library():
    return _lib


def explicit_step_fp64_noalloc(desc):
    """srs_explicit_step_fp64_noalloc on a filled NoallocStep."""
    _check(_lib.srs_explicit_step_fp64_noalloc(C.byref(desc)))


def comp_round_trip(values, packed=False):
    """The device's round trip of FP32 compensation terms through their stored
    halves (srs_comp_round_trip); returns float32."""
    x = np.ascontiguousarray(values, dtype=np.float32)
    out = np.empty_like(x)
    _check(_lib.srs_comp_round_trip(_ptr(x), _ptr(out), int(x.size), int(bool(packed))))
    return out


def default_parameters():
    p = Params()
    _lib.srs_default_parameters(C.byref(p))
    return p


def read_parameters(path, params=None):
    """ReadParameters (cpu/InitFuncs.cpp:25): defaults overridden by the XML file."""
    p = params.copy() if params is not None else default_parameters()
    _check(_lib.srs_read_parameters(C.byref(p), str(path).encode()))
    return p


def box_mesh_spec(**kw):
    s = BoxMeshSpec()
    _lib.srs_box_mesh_default(C.byref(s))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def write_box_mesh(base, spec=None, **kw):
    """Writes the six reference mesh files for a synthetic box dyad."""
    s = spec if spec is not None else box_mesh_spec(**kw)
    rep = np.zeros(6, np.int32)
    a0 = np.zeros(1, np.float64)
    _check(_lib.srs_box_mesh_write(C.byref(s), str(base).encode(), _ptr(rep), _ptr(a0)))
    keys = ("n_tets", "n_faces", "n_nodes", "n_ryr", "n_lcc", "n_jsr_tets")
    d = {k: int(v) for k, v in zip(keys, rep)}
    d["max_a0"] = float(a0[0])
    return d


def multisite_mesh_spec(sites, **kw):
    """srs_multisite_spec for sites = [(x, y, n_ryr, disc_radius), ...] and
    the scalar fields in kw."""
    s = MultiSiteSpec()
    s.n_sites = len(sites)
    for k, (x, y, n, r) in enumerate(sites):
        s.site_x[k], s.site_y[k], s.site_ryr[k], s.site_radius[k] = x, y, n, r
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def write_multisite_mesh(base, spec):
    """Writes the six reference mesh files for a multi-site release unit."""
    rep = np.zeros(6, np.int32)
    a0 = np.zeros(1, np.float64)
    _check(_lib.srs_multisite_mesh_write(C.byref(spec), str(base).encode(), _ptr(rep), _ptr(a0)))
    keys = ("n_tets", "n_faces", "n_nodes", "n_ryr", "n_lcc", "n_jsr_tets")
    d = {k: int(v) for k, v in zip(keys, rep)}
    d["max_a0"] = float(a0[0])
    return d


class Grid:
    """ReadGrid + InitializeDomainStruct (cpu/InitFuncs.cpp:384, 1005)."""

    def __init__(self, params, mesh_base):
        h = C.c_void_p()
        _check(_lib.srs_read_grid(C.byref(params), str(mesh_base).encode(), C.byref(h)))
        self._h = h
        self.mesh_base = str(mesh_base)
        info = _GridInfo()
        _check(_lib.srs_grid_get_info(h, C.byref(info)))
        self.n_ele, self.n_face, self.n_nodes = info.n_ele, info.n_face, info.n_nodes
        self.n_ryr, self.n_lcc, self.n_jsr = info.n_ryr, info.n_lcc, info.n_jsr
        self.vol_jsr, self.max_diag = info.vol_jsr, info.max_diag

    def operator(self):
        N = self.n_ele
        aij = np.zeros(5 * N, np.float64)
        nij = np.zeros(4 * N, np.int32)
        br = np.zeros(6 * N, np.float64)
        _check(_lib.srs_grid_get_operator(self._h, _ptr(aij), _ptr(nij), _ptr(br)))
        return aij, nij, br

    def elements(self):
        N = self.n_ele
        v0, tt = np.zeros(N), np.zeros(N)
        dom, trop, order = (np.zeros(N, np.int32) for _ in range(3))
        _check(_lib.srs_grid_get_elements(self._h, _ptr(v0), _ptr(tt), _ptr(dom), _ptr(trop),
                                          _ptr(order)))
        return dict(V0=v0, TT=tt, domain=dom, tropc=trop, order=order)

    def channels(self):
        a = np.zeros(self.n_ryr, np.int32)
        b = np.zeros(self.n_ryr, np.int32)
        c = np.zeros(4 * self.n_ryr, np.int32)
        d = np.zeros(self.n_lcc, np.int32)
        _check(_lib.srs_grid_get_channels(self._h, _ptr(a), _ptr(b), _ptr(c), _ptr(d)))
        return dict(ryr_ele=a, ryr_jsr=b, ryr_nb=c, lcc_ele=d)

    def write_vtk(self, path, states, ryr_states=None, run=0, rank=0, n=0, t=0.0):
        """WriteToGridFiles' VTK file from host arrays (states[6N], ryr_states[NR])."""
        S = np.ascontiguousarray(states, dtype=np.float64)
        ryr = np.ascontiguousarray(ryr_states if ryr_states is not None else np.zeros(self.n_ryr),
                                   dtype=np.int32)
        _check(_lib.srs_grid_write_vtk(self._h, _ptr(S), _ptr(ryr), str(path).encode(), run, rank, n,
                                       float(t)))

    def initial_states(self, params):
        S = np.zeros(6 * self.n_ele, np.float64)
        _check(_lib.srs_initial_states(self._h, C.byref(params), _ptr(S)))
        return S

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.srs_free_grid(self._h)
            self._h = None


class Simulation:
    """R independent realizations of one grid on the GPU."""

    def __init__(self, grid, params, n_realizations=1, precision=FP64, engine=ENGINE_PLAIN,
                 seeds=None, threads_per_cta=0, cluster_size=0, steps_per_launch=0):
        self.grid, self.params = grid, params.copy()
        self.R = int(n_realizations)
        d = _SimDesc(self.R, int(precision), int(engine), int(threads_per_cta), int(cluster_size),
                     int(steps_per_launch), None)
        if seeds is not None:
            self._seeds = np.ascontiguousarray(np.asarray(seeds, dtype=np.uint64))
            d.seeds = self._seeds.ctypes.data_as(C.POINTER(C.c_uint64))
        h = C.c_void_p()
        _check(_lib.srs_sim_create(grid._h, C.byref(self.params), C.byref(d), C.byref(h)))
        self._h = h
        self.precision, self.engine = precision, engine

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.srs_sim_destroy(self._h)
            self._h = None

    def config(self):
        c = _SimConfig()
        _check(_lib.srs_sim_get_config(self._h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in _SimConfig._fields_}

    def reset(self):
        _check(_lib.srs_sim_reset(self._h))

    def set_prefetch(self, element_blocks):
        """srs_sim_set_prefetch: L2 prefetch distance of the large-mesh plain
        FP32 engine, in element blocks (negative: the default)."""
        _check(_lib.srs_sim_set_prefetch(self._h, int(element_blocks)))

    def set_state(self, r, states=None, ryr=None, lcc=None, lccv=None, residuals=None):
        conv = lambda a, t: None if a is None else np.ascontiguousarray(a, dtype=t)
        arrs = [conv(states, np.float64), conv(ryr, np.int32), conv(lcc, np.int32),
                conv(lccv, np.int32), conv(residuals, np.float64)]
        _check(_lib.srs_sim_set_state(self._h, r, *[_ptr(a) for a in arrs]))

    def get_state(self, r):
        g = self.grid
        S = np.zeros(6 * g.n_ele)
        ryr = np.zeros(g.n_ryr, np.int32)
        lcc = np.zeros(g.n_lcc, np.int32)
        lccv = np.zeros(g.n_lcc, np.int32)
        res = np.zeros(g.n_ryr + g.n_lcc)
        _check(_lib.srs_sim_get_state(self._h, r, _ptr(S), _ptr(ryr), _ptr(lcc), _ptr(lccv),
                                      _ptr(res)))
        return dict(states=S, ryr=ryr, lcc=lcc, lccv=lccv, residuals=res)

    def set_globals(self, v_m, ca_nsr):
        _check(_lib.srs_sim_set_globals(self._h, float(v_m), float(ca_nsr)))

    def explicit_step(self, n_steps=1):
        _check(_lib.srs_explicit_step(self._h, int(n_steps)))

    def advance_async(self, n_steps):
        _check(_lib.srs_sim_advance_async(self._h, int(n_steps)))

    def synchronize(self):
        _check(_lib.srs_sim_synchronize(self._h))

    def time_advance(self, n_steps):
        ms = C.c_float()
        _check(_lib.srs_sim_time_advance(self._h, int(n_steps), C.byref(ms)))
        return float(ms.value)

    def status(self):
        b = C.c_int()
        _check(_lib.srs_sim_status(self._h, C.byref(b)))
        return int(b.value)

    def row_width(self):
        return STATES_ROW_BASE + (self.grid.n_ryr if self.params.ints[I["FLAG_RYR_OUT"]] else 0)

    def run_simulation(self, row_capacity=None, timed=False, grid_callback=None):
        """RunSimulation for every realization; returns per-realization rows,
        final times and step counts (and, with timed=True, the device time in
        ms of each time-step launch).  grid_callback(n, t, done) is called at
        every grid-file step when OUTPUT_GRID_FLAG is set (done: bool array of
        the realizations already finished); it may read the simulation."""
        p = self.params
        if row_capacity is None:
            row_capacity = int(p.reals[R["T_FINAL"]] / p.reals[R["OUTPUT_STATES_INTERVAL"]]) + 8
        w = self.row_width()
        rows = np.zeros((self.R, row_capacity, w), np.float32)
        n_rows = np.zeros(self.R, np.int64)
        t_end = np.zeros(self.R)
        n_steps = np.zeros(self.R, np.int64)
        out = _RunOutput(rows.ctypes.data_as(C.POINTER(C.c_float)), row_capacity, w,
                         n_rows.ctypes.data_as(C.POINTER(C.c_int64)),
                         t_end.ctypes.data_as(C.POINTER(C.c_double)),
                         n_steps.ctypes.data_as(C.POINTER(C.c_int64)))
        cb = None
        if grid_callback is not None:
            R_ = self.R

            def _cb(user, n, t, done):
                grid_callback(int(n), float(t), np.ctypeslib.as_array(done, shape=(R_,)).astype(bool))
            cb = _GRID_CB(_cb)
        cap = 1 << 16 if timed else 0
        ms = np.zeros(max(cap, 1), np.float32)
        n = C.c_int(0)
        if timed or cb is not None:
            _check(_lib.srs_run_simulation_grid(
                self._h, C.byref(out), C.cast(cb, C.c_void_p) if cb is not None else None, None,
                ms.ctypes.data_as(C.POINTER(C.c_float)) if timed else None, cap, C.byref(n)))
        else:
            _check(_lib.srs_run_simulation(self._h, C.byref(out)))
        res = [rows[r, :n_rows[r]].copy() for r in range(self.R)], t_end, n_steps
        return res + (ms[:min(n.value, cap)].copy(),) if timed else res

    def linescan_setup(self, **kw):
        """Line scan along an axis (see srs_linescan_desc); returns sample count."""
        d = LinescanDesc()
        for k, v in kw.items():
            if k == "domain":
                for i, x in enumerate(v):
                    d.domain[i] = float(x)
            else:
                setattr(d, k, v)
        n = C.c_int()
        _check(_lib.srs_linescan_setup(self._h, C.byref(d), C.byref(n)))
        self._ls_n = n.value
        return n.value

    def linescan(self):
        """(F[R][n_samples], F_rest[n_samples]) of the current state."""
        out = np.zeros((self.R, self._ls_n))
        rest = np.zeros(self._ls_n)
        _check(_lib.srs_linescan(self._h, _ptr(out), _ptr(rest)))
        return out, rest

    def total_ca(self):
        """[R][2] total Ca (uM um^3) of the cytosol and the JSR, FP64 sums."""
        out = np.zeros((self.R, 2))
        _check(_lib.srs_sim_total_ca(self._h, _ptr(out)))
        return out

    def adjoint(self, n_steps, tick_every, f0, target=None, checkpoint_every=0, grad_state=False,
                flags=0, threads_per_cta=0, cta_partitions=0, max_checkpoints=0):
        """srs_adjoint: pathwise gradient of the line-scan dF/F0 loss.

        Returns (loss[R], grad[R][N_ADJ] in ADJ_PARAMS order, and
        dL/d(initial state)[R][6][N] when grad_state is true, else None).
        With flags & ADJ_MEAN_TRACE the loss is that of the realizations'
        mean trace against target[n_ticks][n_samples]: loss[0] holds it and
        grad.sum(0) is its gradient."""
        f0 = np.ascontiguousarray(f0, dtype=np.float64)
        if len(f0) != getattr(self, "_ls_n", -1):
            raise ValueError("f0 needs one value per line-scan sample (call linescan_setup first)")
        n_ticks = int(n_steps) // int(tick_every)
        tg = None
        if target is not None:
            shape = ((n_ticks, len(f0)) if int(flags) & ADJ_MEAN_TRACE
                     else (self.R, n_ticks, len(f0)))
            tg = np.ascontiguousarray(np.broadcast_to(target, shape), dtype=np.float64)
        loss = np.zeros(self.R)
        grad = np.zeros((self.R, N_ADJ))
        gs = np.zeros((self.R, 6, self.grid.n_ele)) if grad_state else None
        d = _AdjDesc(int(n_steps), int(tick_every), int(checkpoint_every), f0.ctypes.data,
                     tg.ctypes.data if tg is not None else None, int(flags), int(threads_per_cta),
                     int(cta_partitions), int(max_checkpoints))
        o = _AdjOut(loss.ctypes.data, grad.ctypes.data, gs.ctypes.data if gs is not None else None)
        _check(_lib.srs_adjoint(self._h, C.byref(d), C.byref(o)))
        return loss, grad, gs

    def adjoint_plan(self, n_steps, tick_every, checkpoint_every=0, max_checkpoints=0):
        """srs_adjoint_plan: (segment steps, checkpoint levels, forward steps)
        that srs_adjoint would use now for these settings."""
        f0 = np.zeros(max(getattr(self, "_ls_n", 1), 1))
        d = _AdjDesc(int(n_steps), int(tick_every), int(checkpoint_every), f0.ctypes.data, None, 0, 0,
                     0, int(max_checkpoints))
        seg, lev, fw = C.c_int(), C.c_int(), C.c_int64()
        _check(_lib.srs_adjoint_plan(self._h, C.byref(d), C.byref(seg), C.byref(lev), C.byref(fw)))
        return seg.value, lev.value, fw.value

    def write_grid_vtk(self, r, path, run=0, rank=0, n=0, t=0.0):
        _check(_lib.srs_write_grid_vtk(self._h, r, str(path).encode(), run, rank, n, float(t)))


class Batch:
    """Several FP32 resident simulations (uneven meshes, protocols and sizes)
    advanced together by replaying one CUDA graph (srs_batch_*)."""

    def __init__(self, sims, steps_per_launch=0):
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[s._h.value for s in self.sims])
        h = C.c_void_p()
        _check(_lib.srs_batch_create(arr, len(self.sims), int(steps_per_launch), C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.srs_batch_destroy(self._h)
            self._h = None

    def advance_async(self, n_steps):
        _check(_lib.srs_batch_advance(self._h, int(n_steps)))

    def synchronize(self):
        _check(_lib.srs_batch_synchronize(self._h))

    def time_advance(self, n_steps):
        ms = C.c_float()
        _check(_lib.srs_batch_time_advance(self._h, int(n_steps), C.byref(ms)))
        return float(ms.value)

    def run_simulation(self, row_capacity=None):
        """srs_run_simulation of every member; returns one
        (rows, t_end, n_steps) tuple per member."""
        outs = (_RunOutput * len(self.sims))()
        keep = []
        for i, sim in enumerate(self.sims):
            p = sim.params
            cap = row_capacity or int(p.reals[R["T_FINAL"]] / p.reals[R["OUTPUT_STATES_INTERVAL"]]) + 8
            w = sim.row_width()
            rows = np.zeros((sim.R, cap, w), np.float32)
            n_rows = np.zeros(sim.R, np.int64)
            t_end = np.zeros(sim.R)
            n_steps = np.zeros(sim.R, np.int64)
            outs[i] = _RunOutput(rows.ctypes.data_as(C.POINTER(C.c_float)), cap, w,
                                 n_rows.ctypes.data_as(C.POINTER(C.c_int64)),
                                 t_end.ctypes.data_as(C.POINTER(C.c_double)),
                                 n_steps.ctypes.data_as(C.POINTER(C.c_int64)))
            keep.append((rows, n_rows, t_end, n_steps))
        _check(_lib.srs_batch_run_simulation(self._h, outs))
        return [([rows[r, :n_rows[r]].copy() for r in range(len(n_rows))], t_end, n_steps)
                for rows, n_rows, t_end, n_steps in keep]
