"""Parameter vectors for the CPU oracles (test infrastructure only).

ParamStruct's Integers[19] / Reals[56] (cpu/parameters.h:18-96) filled with
the defaults of ReadParameters (cpu/InitFuncs.cpp:28-101), and the values
param/DefaultSpark.xml sets on top of them.  These are plain lists, so that
CPU-only callers (bench.py's reference leg) need no product library; a CPU
test pins them to the product's srs_default_parameters.
"""

INT_NAMES = ("OUTPUT_GRID_FLAG", "FLAG_FIDELITY_SIM", "FLAG_CLOCK_SEED", "RAND_SEED_0", "RAND_ADD_A",
             "RAND_ADD_B", "INITIALIZE_FROM_FILE", "CUDA_DEVICE", "FLAG_SECONDARY_GRADIENT",
             "FLAG_NO_FLUX_BOUNDARY", "N_RYR_FIDELITY", "FLAG_LCC", "LCC_INDEX", "FLAG_V_CLAMP",
             "FLAG_NO_GATING", "GATING_FFWD", "FLAG_RYR_OUT", "N_SIMS", "INIT_RYR")
REAL_NAMES = ("T_FINAL", "T_STEP", "OUTPUT_STATES_INTERVAL", "OUTPUT_GRID_INTERVAL", "C_MIN", "D_CA",
              "D_CA_JSR", "D_ATP", "D_CMDN", "D_TRPN", "D_CSQN", "D_DYE", "D_EGTA", "C_0_CA",
              "C_0_CA_JSR", "DEFAULT_VM", "DEFAULT_CA_NSR", "CA_0", "B_TOT_ATP", "K_OFF_ATP",
              "K_ON_ATP", "B_TOT_CMDN", "K_OFF_CMDN", "K_ON_CMDN", "B_TOT_TRPN", "K_OFF_TRPN",
              "K_ON_TRPN", "B_TOT_SL_HI", "K_D_SL_HI", "B_TOT_SL_LO", "K_D_SL_LO", "B_TOT_DYE",
              "K_OFF_DYE", "K_ON_DYE", "B_T_JSR", "K_M_JSR", "V_REFILL", "V_RYR", "V_CELL",
              "K_ON_CSQN", "K_OFF_CSQN", "RYR_ETA", "RYR_A_STAR", "RYR_EPS_CC", "RYR_EPS_OO",
              "RYR_K_PLUS", "RYR_K_MINUS", "RYR_PHI_M", "RYR_PHI_B", "K_D_i", "K_D_SR", "A_P",
              "LCC_DURATION", "T_CLAMP", "V_CLAMP", "INIT_RYR_HOLD")

# cpu/InitFuncs.cpp:28-46
DEFAULT_INTS = (0, 0, 1, 38376427, 12783, 83, 0, 0, 0, 1, 1000, 0, 0, 0, 0, 0, 0, 1, -1)
# cpu/InitFuncs.cpp:48-101
DEFAULT_REALS = (500, 12e-6, 0.01, 1, 1.0, 0.25, 0.25, 0.14, 0.025, 0, 0, 0.042, 0, 0.1, 1000, -80,
                 1000, 2000, 455, 45, 0.225, 24, 0.238, 0.034, 70, 0.02, 0.039, 1.6e-13, 13, 0, 1100,
                 50, 0.110, 0.10, 30000, 638, 0.095, 3e-8, 25.84e3, 0.10, 63.8, 2.1, 0, -0.92, -0.85,
                 0.1107e-3, 0.500, 4.0, 1500, 910, 2240, 150, 0.5, 200, 0, 0)

# param/DefaultSpark.xml on top of the defaults (t_step 9 ns, RyR 24 opened
# and held for 10 ms), with the clock seed and grid files off as every run
# here uses them
DEFAULT_SPARK = dict(T_STEP=9e-6, INIT_RYR=24, INIT_RYR_HOLD=10.0, T_FINAL=500.0, FLAG_CLOCK_SEED=0,
                     OUTPUT_GRID_FLAG=0)


def vectors(**over):
    """(ints[19], reals[56]) of the defaults with `over` applied by name."""
    ints, reals = list(DEFAULT_INTS), [float(x) for x in DEFAULT_REALS]
    for k, v in over.items():
        if k in INT_NAMES:
            ints[INT_NAMES.index(k)] = int(v)
        elif k in REAL_NAMES:
            reals[REAL_NAMES.index(k)] = float(v)
        else:
            raise KeyError(k)
    return ints, reals


def default_spark(**over):
    """DefaultSpark vectors with `over` applied."""
    d = dict(DEFAULT_SPARK)
    d.update(over)
    return vectors(**d)
