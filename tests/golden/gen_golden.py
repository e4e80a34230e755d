"""Generates the golden fixtures of tests/golden from the reference itself.

Run in a tree where the reference sources are present (oracle/build_ref.sh
compiles the reference's cpu/RunSimulation.cpp into oracle/_ref):

    python tests/golden/gen_golden.py

Writes
  mesh/dyad.*            a 384-element box-dyad mesh in the reference's file
                         set (written by the package's mesh generator)
  params.json            the parameter vectors the runs used
  ref_steps.npz          state after 2000 deterministic ExplicitStep calls
  ref_run_*.npz          RunSimulation rows and final state, reference
                         gating (glibc rand), for several protocols
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import srs_gb300 as srs  # noqa: E402
from oracle import Oracle, Mesh, Reference  # noqa: E402

MESH = os.path.join(HERE, "mesh", "dyad")


def mesh_spec():
    return dict(box_x=0.4, box_y=0.4, box_z=0.4, foot_half_x=0.1, foot_half_y=0.1, n_foot_x=2,
                n_foot_y=2, n_out_x=1, n_out_y=1, n_above_z=2, ryr_nx=3, ryr_ny=3, n_lcc=2,
                lcc_half=0.1)


def protocols():
    """name -> parameter overrides on top of the reference defaults."""
    base = dict(T_STEP=9e-6, FLAG_CLOCK_SEED=0, T_FINAL=0.05, OUTPUT_STATES_INTERVAL=0.005)
    return {
        "spark": dict(base, INIT_RYR=4, INIT_RYR_HOLD=0.01),
        "spark_nogating": dict(base, INIT_RYR=4, INIT_RYR_HOLD=0.01, FLAG_NO_GATING=1),
        "lcc_trigger": dict(base, FLAG_LCC=1, LCC_INDEX=0, LCC_DURATION=0.02),
        "gain_clamp": dict(base, FLAG_V_CLAMP=1, V_CLAMP=0.0, T_CLAMP=0.02),
        "fidelity": dict(base, INIT_RYR=4, FLAG_FIDELITY_SIM=1, N_RYR_FIDELITY=3, C_MIN=1.0,
                         T_FINAL=0.2),
    }


def params_for(over):
    p = srs.default_parameters().set(**over)
    return np.array(p.ints[:], np.int32), np.array(p.reals[:], np.float64)


def main():
    os.makedirs(os.path.dirname(MESH), exist_ok=True)
    srs.write_box_mesh(MESH, **mesh_spec())
    o, ref = Oracle(), Reference()
    meta = {}
    # deterministic steps
    ints, reals = params_for(dict(T_STEP=9e-6, FLAG_CLOCK_SEED=0, INIT_RYR=4, FLAG_NO_GATING=1))
    m = Mesh(o, MESH, 1, reals)
    S = m.initial_states()
    ryr = np.zeros(m.NR, np.int32)
    ryr[4] = 1
    lcc = np.ones(m.NL, np.int32)
    lccv = 2 * np.ones(m.NL, np.int32)
    res = -np.ones(m.NR + m.NL)
    ref.explicit_steps(m, ints, S, ryr, lcc, lccv, res, 2000)
    np.savez_compressed(os.path.join(HERE, "ref_steps.npz"), states=S, ints=ints, reals=reals,
                        n_steps=2000, ryr=ryr)
    meta["steps"] = dict(ints=ints.tolist(), reals=reals.tolist())
    for name, over in protocols().items():
        ints, reals = params_for(over)
        m = Mesh(o, MESH, 1, reals)
        rows, Sf = ref.run_simulation(m, ints, rank=0, index=0)
        np.savez_compressed(os.path.join(HERE, "ref_run_%s.npz" % name), rows=rows, states=Sf,
                            ints=ints, reals=reals)
        meta[name] = dict(ints=ints.tolist(), reals=reals.tolist(), n_rows=int(len(rows)))
        print(name, rows.shape)
    with open(os.path.join(HERE, "params.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main()
