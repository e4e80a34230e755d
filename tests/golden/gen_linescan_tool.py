"""Golden output of the reference's line-scan tool for the device line scan.

Writes three grid files of the golden mesh with the reference's own
WriteToGridFiles (cpu/OutputFuncs.cpp, oracle/_ref/libsrsref_io.so), each from
a state whose bound-dye field is perturbed at random and rounded to the %f
values the file holds, runs the reference's line-scan tool
(linescan/main.cpp, oracle/_ref/linescan) on them, and stores the states,
the scan description and the tool's blurred fluorescence (scan_output.txt)
in linescan_tool.npz.  tests/test_gpu_linescan.py compares the device line
scan of the same states with it.

    python tests/golden/gen_linescan_tool.py
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
MESH = os.path.join(HERE, "mesh", "dyad")


def main():
    import srs_gb300 as srs
    from oracle import RefIO
    from test_ref_io import _scan_xml, tool_scan_desc
    p = srs.default_parameters().set(T_STEP=9e-6, OUTPUT_GRID_FLAG=1)
    ref = RefIO().load(MESH, p.ints[:], p.reals[:])
    g = srs.Grid(p, MESH)
    N = g.n_ele
    rng = np.random.default_rng(11)
    tmp = tempfile.mkdtemp(prefix="srs_ls_")
    states = []
    for n in range(3):
        S = g.initial_states(p)
        S[5 * N:] *= 1.0 + 3.0 * rng.random(N) ** 2
        S = np.array([float("%f" % x) for x in S])
        ref.set_states(S)
        ref.write_grid(tmp, rank=0, run=0, n=n)
        states.append(S)
    d = tool_scan_desc()
    xml = os.path.join(tmp, "scan.xml")
    _scan_xml(xml, d, os.path.join(tmp, "grid_0_0"), tmp, len(states))
    subprocess.run([os.path.join(ROOT, "oracle", "_ref", "linescan"), "-param", xml], check=True,
                   cwd=tmp, stdout=subprocess.DEVNULL)
    out = np.loadtxt(os.path.join(tmp, "scan_output.txt"))
    desc = {k: v for k, v in d.items() if k != "domain_size"}
    np.savez_compressed(os.path.join(HERE, "linescan_tool.npz"), states=np.array(states),
                        tool_output=out, desc=json.dumps(desc))
    print("wrote linescan_tool.npz:", out.shape)


if __name__ == "__main__":
    main()
