"""In-tree build of the GB300 library: nvcc for sm_103a, no cmake.

    python -m gplum_gb300.build

compiles every gplum_gb300/csrc/*.cu (and the host tree builder) in parallel
and links gplum_gb300/_build/libgplum_p3t.so.  Rebuilds only when a source
or header is newer than the library.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgplum_p3t.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP64 physics kept free of FMA contraction, so it rounds as GPLUM's host build
NO_FMAD = {"engine.cu", "hard.cu", "dtree.cu"}


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    return cu, cpp


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = _sources()
    jobs = []
    for src in cu:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        extra = ["-fmad=false"] if os.path.basename(src) in NO_FMAD else []
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fno-fast-math", "--expt-relaxed-constexpr", *extra, "-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-c", src,
                     "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return cmd[-1]

    with ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 2))) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp", "-lcudart"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
