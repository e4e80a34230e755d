"""Named workloads: mesh specs and parameter sets.

DEFAULT_SPARK reproduces the values of the reference's param/DefaultSpark.xml
(its only differences from the ReadParameters defaults of
cpu/InitFuncs.cpp:28-108 are t_step = 9 ns, ryr_open_init = 24,
ryr_open_time = 10 ms, t_final = 500 ms and the output flags).
"""
import os

import srs_gb300 as srs

DEFAULT_SPARK = dict(T_STEP=9e-6, INIT_RYR=24, INIT_RYR_HOLD=10.0, T_FINAL=500.0,
                     FLAG_CLOCK_SEED=0, OUTPUT_GRID_FLAG=0)

# 2 x 2 x 2 um box of 12^3 hexahedra split into 6 tetrahedra each (10,368
# elements): 15 nm cleft under a 50 nm JSR cap over a 400 x 400 nm
# footprint, 7 x 7 RyRs at 31 nm, 7 LCCs placed at random (seed 1).
CONFIG_DYAD = {}  # the generator defaults are this mesh

# small mesh used by smoke checks and fast tests
TINY_DYAD = dict(box_x=0.4, box_y=0.4, box_z=0.4, foot_half_x=0.1, foot_half_y=0.1, n_foot_x=2,
                 n_foot_y=2, n_out_x=1, n_out_y=1, n_above_z=2, ryr_nx=3, ryr_ny=3, n_lcc=2,
                 lcc_half=0.1)


def default_spark_params(**over):
    p = srs.default_parameters().set(**DEFAULT_SPARK)
    if over:
        p.set(**over)
    return p


def config_mesh(directory):
    base = os.path.join(directory, "dyad12")
    rep = srs.write_box_mesh(base, **CONFIG_DYAD)
    return base, rep


# Uneven multi-mesh batch: four box dyads of 6k / 15k / 30k / 60k tets in
# 1.5 / 2 / 2.5 / 3 um boxes, Poisson-disk RyR clusters (minimum spacing
# 30 nm) of 10 / 25 / 60 / 100 RyRs, one LCC per 7 RyRs.
CONFIG2_MESHES = [
    # box, n_foot, n_out, n_above, n_ryr, cluster radius (um): about a third of
    # the disc covered by the 15 nm exclusion discs
    (1.5, 6, 2, 8, 10, 0.085),
    (2.0, 8, 3, 11, 25, 0.13),
    (2.5, 9, 4, 15, 60, 0.20),
    (3.0, 10, 6, 19, 100, 0.26),
]


def config2_mesh_specs():
    out = []
    for k, (box, nf, no, na, nr, rad) in enumerate(CONFIG2_MESHES):
        half = rad + 0.05
        out.append(dict(box_x=box, box_y=box, box_z=box, foot_half_x=half, foot_half_y=half,
                        n_foot_x=nf, n_foot_y=nf, n_out_x=no, n_out_y=no, n_above_z=na,
                        ryr_mode=1, ryr_count=nr, ryr_radius=rad, ryr_pitch=0.030,
                        n_lcc=max(1, round(nr / 7)),
                        lcc_half=half, seed=11 + k, lcc_seed=21 + k))
    return out


def config2_meshes(directory):
    """Writes the four meshes; returns [(base, report)]."""
    res = []
    for k, spec in enumerate(config2_mesh_specs()):
        base = os.path.join(directory, "c2_mesh%d" % k)
        res.append((base, srs.write_box_mesh(base, **spec)))
    return res


def stable_dt(params, max_a0, dt=9e-6, margin=0.9):
    """dt, reduced below D_max * dt * max|a0| = margin when that bound needs it."""
    d = max(params.reals[srs.R[n]] for n in ("D_CA", "D_ATP", "D_CMDN", "D_DYE"))
    return min(dt, margin / (d * max_a0))


def config2_protocols(max_a0):
    """The two protocols of the batch: leak (voltage clamped at rest, no
    trigger, no forced RyR, 100 ms) and LCC-triggered (clamped at 0 mV,
    30 ms, as param/Gain_0mV.xml)."""
    leak = default_spark_params(INIT_RYR=-1, INIT_RYR_HOLD=0.0, FLAG_V_CLAMP=1, V_CLAMP=-80.0,
                                T_CLAMP=200.0, T_FINAL=100.0)
    trig = default_spark_params(INIT_RYR=-1, INIT_RYR_HOLD=0.0, FLAG_V_CLAMP=1, V_CLAMP=0.0,
                                T_CLAMP=200.0, T_FINAL=30.0)
    for p in (leak, trig):
        p.set(T_STEP=stable_dt(p, max_a0))
    return leak, trig


# Large release site: a 3 x 3 x 4 um box with five cleft footprints holding
# Poisson-disk RyR groups of 20 / 40 / 60 / 100 / 150 channels (30 nm minimum
# spacing, seed 7), one LCC per 7 RyRs, JSR caps joined by 50 nm-thick JSR
# sheets; about a million tets.  The disc radius follows the config-2 rule
# (about a third of the disc covered by the exclusion discs).
CONFIG4_SITES = [(-0.85, -0.80, 20), (0.75, -0.85, 40), (-0.05, 0.05, 60), (-0.80, 0.85, 100),
                 (0.80, 0.70, 150)]


def config4_mesh_spec(h_fine=0.035, h_max=0.2):
    sites = [(x, y, n, 0.026 * n ** 0.5) for (x, y, n) in CONFIG4_SITES]
    return srs.multisite_mesh_spec(
        sites, box_x=3.0, box_y=3.0, box_z=4.0, h_fine=h_fine, h_max=h_max, growth=1.2,
        cleft_h=0.015, jsr_h=0.050, n_cleft_z=2, n_jsr_z=2, r_trpn=0.2, flag_tt=1,
        foot_margin=0.05, ryr_pitch=0.030, ryr_depth=0.0075, sheet_half=0.025, seed=7)


def config4_mesh(directory, **kw):
    base = os.path.join(directory, "c4_site")
    return base, srs.write_multisite_mesh(base, config4_mesh_spec(**kw))
