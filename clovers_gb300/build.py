"""Builds the GB300 shared library ``_build/libclovers_gb300.so``.

Three translation units, compiled in parallel:

* ``csrc/clovers_gb300.cu`` -- kernels and the C ABI, by nvcc for sm_103a
  only.  ``-fmad=false`` keeps every multiply and add separately rounded, the
  operation order of the reference's f32 arithmetic (bit-exact hit ids).
* ``csrc/guide.cu`` -- the path guide's tensor-core (tcgen05) kernels and its
  part of the C ABI, by nvcc for sm_103a (multiply-add fusion allowed: the
  guide is not part of the reference's arithmetic).
* ``csrc/scene.cpp`` -- scene flattening and the SAH build, by the host C++
  compiler with ``-ffp-contract=off`` for the same reason.

No x86-specific flags: the same commands build on the aarch64 GPU hosts.
"""

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libclovers_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build clovers_gb300")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".cpp", ".hpp", ".h"))] + [os.path.join(INCLUDE, "clovers_gpu.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build(force=False, verbose=False, ptxas_info=False):
    """Compile the library if any source is newer than it; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = nvcc_path()
    cu_obj = os.path.join(OUT, "clovers_gb300.o")
    guide_obj = os.path.join(OUT, "guide.o")
    cpp_obj = os.path.join(OUT, "scene.o")
    cu_cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-c",
              os.path.join(CSRC, "clovers_gb300.cu"), "-o", cu_obj]
    guide_cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-c",
                 os.path.join(CSRC, "guide.cu"), "-o", guide_obj]
    if ptxas_info:
        cu_cmd[1:1] = ["-Xptxas", "-v"]
        guide_cmd[1:1] = ["-Xptxas", "-v"]
    extra = os.environ.get("CLV_NVCC_FLAGS", "").split()  # e.g. -DCLV_MINB=8 for occupancy experiments
    cu_cmd[1:1] = extra
    guide_cmd[1:1] = extra
    cxx = os.environ.get("CXX", "g++")
    cpp_cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-I", INCLUDE, "-c",
               os.path.join(CSRC, "scene.cpp"), "-o", cpp_obj]
    with ThreadPoolExecutor(3) as ex:
        outs = list(ex.map(_run, [cu_cmd, guide_cmd, cpp_cmd]))
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, cu_obj, guide_obj, cpp_obj, "-lpthread"])
    os.replace(tmp, LIB)
    if verbose or ptxas_info:
        sys.stdout.write("".join(outs))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
