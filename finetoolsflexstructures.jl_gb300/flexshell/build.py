"""Build of the flexshell CUDA library (libflexshell.so) for sm_103a.

nvcc compiles each translation unit of csrc/ in parallel, then links one
shared library into flexshell/_build/.  The library exports the C ABI of
include/flexshell.h.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libflexshell.so")
SOURCES = ["fs_api.cu", "fs_symbolic.cu", "fs_numeric.cu", "fs_elem_t3.cu", "fs_elem_q4.cu", "fs_gather.cu",
           "fs_explicit.cu", "fs_noalloc.cu", "fs_beam.cu", "fs_batch.cu", "fs_resultants.cu",
           "fs_loads.cu", "fs_eigen.cu"]
HEADERS = ["fs_internal.cuh", "fs_elem_math.cuh", "fs_elem_common.cuh", "fs_comp_sum.cuh", "fs_beam_math.cuh",
           "fs_host_prep.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, "include", "flexshell.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-I", os.path.join(ROOT, "include"), "-I", CSRC] + list(extra)
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]

    def comp(i):
        cmd = [nvcc(), "-c", os.path.join(CSRC, SOURCES[i]), "-o", objs[i]] + flags
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        results = list(ex.map(comp, range(len(SOURCES))))
    for cmd, r in results:
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s" % cmd[2])
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("link of libflexshell.so failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
