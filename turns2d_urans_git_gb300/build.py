"""Build recipe of the native library libturns2d_gb300.so (sm_103a).

Compiles the CUDA kernels and the host runtime in parallel with nvcc / g++
and links them into turns2d_urans_git_gb300/libturns2d_gb300.so next to this
file.  The plain FP64 kernels are compiled with -fmad=false (two roundings
for a*b+c, as the reference Fortran); host code with -ffp-contract=off.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libturns2d_gb300.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")

COMMON_NV = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-I" + os.path.join(ROOT, "include"),
                    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr"]

UNITS = [
    # (source, extra flags)
    ("kernels/kernels_fp64.cu", ["-fmad=false"]),
    # mixed path: f32 arithmetic with approximate division / square root
    # (rcp / rsqrt based, <= 2 ulp) and flush-to-zero; its accuracy is stated
    # against the FP64 oracle, not bitwise
    ("kernels/kernels_fp32.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    # the fused residual, one unit per (precision, tile shape) so that its
    # variants compile in parallel
    ("kernels/resid_f32_16x16.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("kernels/resid_f32_32x8.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("kernels/resid_f32_8x32.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("kernels/resid_f32_32x16.cu", ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]),
    ("kernels/resid_f64_16x16.cu", ["-fmad=false"]),
    ("kernels/resid_f64_32x8.cu", ["-fmad=false"]),
    ("kernels/resid_f64_8x32.cu", ["-fmad=false"]),
    ("kernels/resid_f64_32x16.cu", ["-fmad=false"]),
    ("host/runtime.cu", ["-fmad=false"]),
    ("host/solver.cu", ["-fmad=false"]),
    ("host/dropin.cu", ["-fmad=false"]),
    ("host/noalloc.cu", ["-fmad=false"]),
    ("host/io.cu", ["-fmad=false"]),
    ("host/geom.cpp", None),
    ("host/setup_host.cpp", None),
]


def _compile(src, extra):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
    if extra is None:
        cmd = [CXX, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CSRC, "host"),
               "-c", path, "-o", obj]
    else:
        cmd = [NVCC] + COMMON_NV + extra + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    units = [(s, e) for s, e in UNITS if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), units))
    cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", OUT] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose:
        print("built", OUT)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
