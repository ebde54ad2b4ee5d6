"""Recipe: build the reference's own binning kernels, from its sources, into
oracle/_ref/ (git-ignored).  TEST INFRASTRUCTURE ONLY.

The reference's src/GSCudaKernels.cu cannot be compiled whole here (its
header pulls in Eigen and OpenCV, and other kernels in the file use Eigen in
device code).  The binning path uses none of them, so this recipe takes the
functions of that path out of the file as they are -- quaternionToMatrix
(src/GSCudaKernels.cu:319-334), invert2x2 (1411-1437),
projectGaussiansWorldToScreen_kernel (345-476), countTilesPerGaussian_kernel
(549-593), generateTileHashes_kernel (596-667), computeIndicesRanges_kernel
(669-707) and perTileBucketCount (2074-2090) -- together with the float3
operators of include/f_vigs_slam/CudaMathOperations.cuh, writes them to
oracle/_ref/, and compiles two harnesses around them:

* oracle/_ref/libref_gpu.so: oracle/ref_gpu.cu, by nvcc for sm_103a with the
  reference's own CUDA flags (no fast-math, default FMA contraction), which
  launches the kernels on the GPU as GSSlam::prepareRasterization does
  (src/GSSlam.cu:408-646);
* oracle/_ref/libref_host.so: oracle/ref_host.cpp, by g++ with floating-point
  contraction off, which runs the same kernel bodies on the CPU thread by
  thread.

Where /root/reference is absent (the GPU machine), the harnesses are compiled
from the files a previous run left in oracle/_ref/.  Nothing in the library
uses any of this.

Usage: python oracle/ref_build.py [--force]
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_ROOT = "/root/reference"
REF_KERNELS = os.path.join(REF_ROOT, "src", "GSCudaKernels.cu")
REF_MATH = os.path.join(REF_ROOT, "include", "f_vigs_slam", "CudaMathOperations.cuh")
INC = os.path.join(OUT, "ref_binning_kernels.inc")
MATH = os.path.join(OUT, "CudaMathOperations.cuh")
LIB_GPU = os.path.join(OUT, "libref_gpu.so")
LIB_HOST = os.path.join(OUT, "libref_host.so")

# functions of the binning path, in definition-before-use order
FUNCTIONS = [
    "quaternionToMatrix",
    "invert2x2",
    "projectGaussiansWorldToScreen_kernel",
    "countTilesPerGaussian_kernel",
    "generateTileHashes_kernel",
    "computeIndicesRanges_kernel",
    "perTileBucketCount",
]


def _strip_for_scan(text: str) -> str:
    """The text with comments and string literals blanked (same length), so
    braces inside them are not counted."""
    out = list(text)
    i, n = 0, len(text)
    while i < n:
        if text.startswith("//", i):
            j = text.find("\n", i)
            j = n if j < 0 else j
            for k in range(i, j):
                out[k] = " "
            i = j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            for k in range(i, j):
                if out[k] != "\n":
                    out[k] = " "
            i = j
        elif text[i] in "\"'":
            q = text[i]
            j = i + 1
            while j < n and text[j] != q:
                j += 2 if text[j] == "\\" else 1
            for k in range(i + 1, min(j, n)):
                out[k] = " "
            i = j + 1
        else:
            i += 1
    return "".join(out)


def extract(text: str, name: str) -> str:
    """One function definition of `name` (its qualifiers to its closing
    brace), taken verbatim."""
    scan = _strip_for_scan(text)
    brace = -1
    for m in re.finditer(r"(__global__|__device__)[^;{}]*?\b%s\s*\(" % re.escape(name), scan):
        # the parameter list, then a body (not a declaration)
        depth, i = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(scan[i], 0)
            i += 1
        rest = scan[i:].lstrip()
        if rest.startswith("{"):
            brace = len(scan) - len(rest)
            break
    if brace < 0:
        raise RuntimeError("definition of %s not found in %s" % (name, REF_KERNELS))
    start = scan.rfind("\n", 0, m.start()) + 1
    depth, i = 0, brace
    while True:
        if scan[i] == "{":
            depth += 1
        elif scan[i] == "}":
            depth -= 1
            if depth == 0:
                break
        i += 1
    return text[start:i + 1] + "\n"


def refresh_sources() -> bool:
    """Write oracle/_ref/ref_binning_kernels.inc and the math header from the
    reference sources, if they are present.  Returns whether they were."""
    if not (os.path.exists(REF_KERNELS) and os.path.exists(REF_MATH)):
        return False
    os.makedirs(OUT, exist_ok=True)
    with open(REF_KERNELS, encoding="utf-8", errors="replace") as f:
        text = f.read()
    parts = ["// Generated by oracle/ref_build.py from %s; do not edit.\n" % REF_KERNELS]
    for name in FUNCTIONS:
        parts.append(extract(text, name))
    body = "".join(parts)
    if not os.path.exists(INC) or open(INC, encoding="utf-8").read() != body:
        with open(INC, "w", encoding="utf-8") as f:
            f.write(body)
    shutil.copyfile(REF_MATH, MATH)
    return True


def _stale(target, deps):
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in deps)


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return None


def build(force: bool = False, gpu: bool = True, host: bool = True):
    """Build what can be built; returns {"host": path or None, "gpu": path or None}."""
    refresh_sources()
    out = {"host": None, "gpu": None}
    if not os.path.exists(INC):
        return out
    cuda_inc = "/usr/local/cuda/include"
    if host:
        src = os.path.join(HERE, "ref_host.cpp")
        if force or _stale(LIB_HOST, [src, INC, MATH]):
            tmp = LIB_HOST + ".tmp%d" % os.getpid()
            subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                                   "-shared", "-w", "-I", OUT, "-I", cuda_inc, "-o", tmp, src])
            os.replace(tmp, LIB_HOST)
        out["host"] = LIB_HOST
    nvcc = _nvcc()
    if gpu and nvcc:
        src = os.path.join(HERE, "ref_gpu.cu")
        if force or _stale(LIB_GPU, [src, INC, MATH]):
            tmp = LIB_GPU + ".tmp%d" % os.getpid()
            subprocess.check_call([nvcc, "-gencode=arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w",
                                   "-Xcompiler", "-fPIC", "-shared", "-I", OUT, "-o", tmp, src])
            os.replace(tmp, LIB_GPU)
        out["gpu"] = LIB_GPU
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
