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
