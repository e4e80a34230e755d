"""Build the sm_103a library and the drop-in CLI in-tree.

Outputs (git-ignored, rebuilt on every box):
  srs_gb300/libsrs_gb300.so   C ABI of include/srs_gb300.h
  srs_gb300/bin/cru3d         drop-in replacement of the reference CLI
  srs_gb300/bin/srs_meshgen   synthetic mesh writer (host code only)

Translation units compile in parallel; the numerics files use -fmad=false so
that every fused multiply-add is an explicit one (bit-reproducible results),
and host code uses -ffp-contract=off for the same reason on both x86-64 and
aarch64 hosts.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INC = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB = os.path.join(HERE, "libsrs_gb300.so")
BIN = os.path.join(HERE, "bin")


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _units():
    common_cu = [nvcc(), *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                 "-Xcompiler", "-ffp-contract=off", "-I", CSRC, "-I", INC]
    common_cc = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-I", CSRC, "-I", INC]
    # Every engine that must match the oracle bit for bit is compiled without
    # FMA contraction; the adjoint (checked to tolerances) contracts.
    return [
        ("k_plain64.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_plain64.cu")]),
        ("k_fp32.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_fp32.cu")]),
        ("k_res_a.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_res_a.cu")]),
        ("k_res_b.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_res_b.cu")]),
        ("k_res_c.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_res_c.cu")]),
        ("k_res_d.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_res_d.cu")]),
        ("srs_capi.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "srs_capi.cu")]),
        ("k_noalloc.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_noalloc.cu")]),
        ("k_linescan.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_linescan.cu")]),
        ("k_adjoint.o", common_cu + ["-c", os.path.join(CSRC, "k_adjoint.cu")]),
        ("k_adjoint_plain.o", common_cu + ["-c", os.path.join(CSRC, "k_adjoint_plain.cu")]),
        ("k_mass.o", common_cu + ["-fmad=false", "-c", os.path.join(CSRC, "k_mass.cu")]),
        ("srs_host.o", common_cc + ["-c", os.path.join(CSRC, "srs_host.cpp")]),
        ("meshgen.o", common_cc + ["-c", os.path.join(CSRC, "meshgen.cpp")]),
    ]


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] + [
        os.path.join(INC, "srs_gb300.h"), __file__]


def _stale(target):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(verbose=False, force=False):
    """Compile everything; returns the path of the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    targets = [LIB, os.path.join(BIN, "cru3d"), os.path.join(BIN, "srs_meshgen")]
    if not force and not any(_stale(t) for t in targets):
        return LIB

    def run(unit):
        out, cmd = unit
        cmd = cmd + ["-o", os.path.join(BUILD, out)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return out

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(run, _units()))
    link = [nvcc(), *ARCH, "-shared", "-o", LIB] + [os.path.join(BUILD, o) for o in objs] + [
        "-lcudart", "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    cmd = ["g++", "-std=c++17", "-O2", "-I", CSRC, "-I", INC, os.path.join(CSRC, "cru3d_main.cpp"),
           "-o", os.path.join(BIN, "cru3d"), "-L", HERE, "-lsrs_gb300", "-Wl,-rpath,$ORIGIN/.."]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link of cru3d failed:\n%s\n%s" % (r.stdout, r.stderr))
    build_meshgen(os.path.join(BIN, "srs_meshgen"))
    return LIB


def build_meshgen(dest):
    """The mesh writer as a host-only executable (meshgen.cpp alone, no CUDA
    library), so that CPU-only runs can write their input files."""
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC, "-I", INC,
           os.path.join(CSRC, "meshgen.cpp"), os.path.join(CSRC, "meshgen_main.cpp"), "-o", dest]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build of %s failed:\n%s\n%s" % (dest, r.stdout, r.stderr))
    return dest


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
