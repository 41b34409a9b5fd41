"""Build libbeachslope.so in-tree with nvcc for sm_103a.

Each .cu translation unit compiles in its own nvcc process (in parallel),
then one shared-library link.  Output: beach-slope_gb300/_lib/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libbeachslope.so")
INCLUDE = os.path.join(HERE, "..", "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills"]
SOURCES = ["bs_bin.cu", "bs_sweep.cu", "bs_solver.cu", "bs_mg.cu", "bs_static.cu", "bs_probe.cu", "bs_host.cu"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    d = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh"))]
    d.append(os.path.join(INCLUDE, "beachslope.h"))
    return d


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build_library(force=False, verbose=False, extra=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()

    def one(src):
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [cc] + ARCH + FLAGS + list(extra) + ["-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build_library(force=True, verbose=True, extra=["-Xptxas", "-v"])
    print(LIB)
