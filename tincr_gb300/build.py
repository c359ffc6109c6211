"""Build the in-tree CUDA library `tincr_gb300/lib/libtincr_gb300.so` for sm_103a.

    python -m tincr_gb300.build          (or tincr_gb300.build.build())

Each translation unit is compiled in parallel with nvcc, then linked as a shared library whose
exported symbols are exactly the `extern "C"` entry points of include/tincr_gb300.h.
"""

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libtincr_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["abi.cu", "tda.cu", "gradient.cu", "noalloc.cu", "mixed.cu", "batch.cu", "eig_cluster.cu", "digits.cu",
           "exciton.cu", "scc.cu", "rpa.cu", "eigen_host.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _flags(verbose_ptxas=False):
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3,-fopenmp", "--expt-relaxed-constexpr",
         "-I", os.path.join(HERE, "..", "include")] + ARCH
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def build(force=False, verbose_ptxas=False, jobs=None):
    """Compile if any source is newer than the library.  Returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(SRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "tincr_gb300.h"))
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        cmd = [nvcc, "-c", src, "-o", obj] + _flags(verbose_ptxas)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        return obj, r.stderr

    with ThreadPoolExecutor(max_workers=jobs or len(srcs)) as ex:
        for obj, log in ex.map(compile_one, srcs):
            objs.append(obj)
            if verbose_ptxas and log:
                sys.stderr.write(log)
    tmp = LIB + ".tmp"
    # export the extern "C" entry points only
    vscript = os.path.join(OUT, "exports.map")
    with open(vscript, "w") as f:
        f.write("{ global: tincr_*; local: *; };\n")
    cmd = [nvcc, "-shared", "-o", tmp] + objs + ARCH + ["-lcudart", "-Xcompiler", "-fopenmp",
                                                        "-Xlinker", "--version-script=" + vscript]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
