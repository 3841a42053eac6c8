"""Build librflu_gpu.so (sm_103a) in-tree: rocflu_gb300/_build/.

Translation units, compiled in parallel:
  setup.cpp          host set-up (g++, OpenMP)
  capi.cu            C ABI, renumbering, CSR construction
  kernels_fp64.cu    FP64 kernels, FMA contraction allowed
  kernels_fp64x.cu   FP64 kernels without FMA contraction (reference order)
  kernels_mixed.cu   FP32/FP64 mixed kernels
Host code is compiled with -ffp-contract=off everywhere: set-up values
(geometry, least-squares weights) must match the reference's FP64 bit for
bit on x86 and on aarch64, where GCC would otherwise contract into FMAs.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librflu_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librflu_gpu.so")


def _sources():
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC)
                  if f.endswith((".cu", ".cuh", ".cpp", ".h")))


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources() + [os.path.join(HERE, "..", "include", "rflu_gpu.h")])


def build(verbose=False, force=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    host = ["-Xcompiler", "-fPIC,-ffp-contract=off"]
    common = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr"] + ARCH + host
    jobs = {
        "setup.o": ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-c",
                    os.path.join(SRC, "setup.cpp"), "-o", os.path.join(OUT, "setup.o")],
        "capi.o": [nvcc] + common + ["-c", os.path.join(SRC, "capi.cu"), "-o", os.path.join(OUT, "capi.o")],
        "kernels_fp64.o": [nvcc] + common + ["-fmad=true", "-c", os.path.join(SRC, "kernels_fp64.cu"), "-o",
                                            os.path.join(OUT, "kernels_fp64.o")],
        "kernels_fp64x.o": [nvcc] + common + ["-fmad=false", "-c", os.path.join(SRC, "kernels_fp64x.cu"), "-o",
                                             os.path.join(OUT, "kernels_fp64x.o")],
        # FP32 division and square root at full throughput (within 2 ulp)
        # in the mixed mode; its FP64 parts are IEEE regardless
        "kernels_mixed.o": [nvcc] + common + ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-c",
                                             os.path.join(SRC, "kernels_mixed.cu"), "-o",
                                             os.path.join(OUT, "kernels_mixed.o")],
    }
    if verbose:
        for k in jobs:
            if k.startswith("kernels"):
                jobs[k] += ["-Xptxas", "-v"]
    procs = {k: subprocess.Popen(v, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for k, v in jobs.items()}
    failed = []
    for k, p in procs.items():
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(k)
    if failed:
        raise RuntimeError("build of librflu_gpu.so failed: " + ", ".join(failed))
    objs = [os.path.join(OUT, k) for k in jobs]
    tmp = LIB + ".tmp"
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
