"""Build libpdg.so (the C-ABI CUDA library) in-tree with nvcc for sm_103a.

Translation units compile in parallel; the result lands in
``dune-pdelab_gb300/_build/libpdg.so``.  Host code is portable C++17 (no
x86 intrinsics), so the same recipe builds on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpdg.so")
PROBE_LIB = os.path.join(OUT, "libpdg_probe.so")   # bench-only FMA peak probe
SOURCES = ["pdg_abi.cu", "pdg_apply.cu", "pdg_prec.cu", "pdg_rhs.cu", "pdg_vec.cu",
           "pdg_noalloc.cu", "pdg_conv.cu", "pdg_assemble.cu",
           "pdg_blocksolve.cu", "pdg_apply32.cu",
           "pdg_nonlinear.cu", "pdg_basis.cu", "pdg_general.cu", "pdg_apply_fp.cu", "pdg_apply_m.cu"]
PROBE_SOURCES = ["probe_peak.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-O3"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _compile(src, extra):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(SRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False, extra=None, force=False):
    os.makedirs(OUT, exist_ok=True)
    extra = list(extra or [])
    deps = [os.path.join(SRC, f) for f in os.listdir(SRC)] + [
        os.path.join(HERE, "..", "include", "pdg.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(d) for d in deps)):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + len(PROBE_SOURCES)) as ex:
        res = list(ex.map(lambda s: _compile(s, extra), SOURCES + PROBE_SOURCES))
    objs = [o for o, _ in res[:len(SOURCES)]]
    pobjs = [o for o, _ in res[len(SOURCES):]]
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", PROBE_LIB, *pobjs, "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        for _, err in res:
            if err:
                sys.stderr.write(err)
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
