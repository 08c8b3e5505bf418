"""Build recipe of the solver library (libdrot_gb300.so) for sm_103a.

nvcc compiles the translation units csrc/drot_api.cu (single-instance
solver and C ABI), csrc/drot_batch.cu (batched solver) and
csrc/drot_adjoint.cu (implicit QR adjoint), csrc/drot_gl_adjoint.cu
(unrolled GL adjoint) and csrc/drot_cost.cu (tensor-core cost matrices) in
parallel and links them into
reg_drot/libdrot_gb300.so, in tree.  Device code is compiled with
--fmad=false: the kernels spell out every fused multiply-add they need
(the ones the reference's kernels compile to), so nothing else is contracted.
Host code is compiled with -ffp-contract=off so the parameter mapping rounds
the same on x86-64 and aarch64 hosts.

Usage: python regularized-drot_gb300/build.py [--force] [-v]
"""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT = os.path.join(PKG, "reg_drot", "libdrot_gb300.so")
SOURCES = [os.path.join(CSRC, f)
           for f in ("drot_api.cu", "drot_batch.cu", "drot_adjoint.cu",
                     "drot_gl_adjoint.cu", "drot_cost.cu")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
    [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17", "--fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
]


def nvcc():
    cand = os.environ.get("NVCC") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"),
                                                   "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force=False, verbose=False, extra=()):
    """Compile libdrot_gb300.so if missing or stale; return its path."""
    newest = max(os.path.getmtime(f) for f in DEPS)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= newest:
        return OUT
    objs, procs = [], []
    for src in SOURCES:
        obj = os.path.join(os.path.dirname(OUT), os.path.basename(src) + ".o")
        cmd = [nvcc(), *NVCC_FLAGS, *extra, "-I", INCLUDE, "-I", CSRC, "-c", "-o", obj, src]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((subprocess.Popen(cmd), cmd))
        objs.append(obj)
    for proc, cmd in procs:
        if proc.wait() != 0:
            raise subprocess.CalledProcessError(proc.returncode, cmd)
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", OUT + ".tmp", *objs]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    for obj in objs:
        os.remove(obj)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    extra = ["-Xptxas", "-v"] if "-v" in sys.argv else []
    print(build(force="--force" in sys.argv or bool(extra), verbose=True, extra=extra))
