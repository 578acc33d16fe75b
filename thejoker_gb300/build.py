"""Build libjoker_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel (``nvcc -c``), then linked with
``nvcc -shared``.  A stamp of the sources' contents and the flags skips
rebuilds when nothing changed.
"""
import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(OUT_DIR, "libjoker_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
SOURCES = ["joker_lnl.cu", "joker_lnl_packed.cu", "joker_lnl_fast.cu", "joker_lnl_fused.cu",
           "joker_accept.cu",
           "joker_tier2.cu", "joker_abi.cu",
           "joker_noalloc.cu", "joker_iter.cu", "joker_posterior.cu", "joker_prior.cu"]
HEADERS = ["joker_internal.cuh", "joker_math.cuh", "joker_fp64.cuh", "joker_mixed.cuh",
           "joker_fast.cuh",
           "joker_sincos_table.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libjoker_gb300")


def _stamp():
    h = hashlib.sha256()
    for f in SOURCES + HEADERS:
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(fh.read())
    with open(os.path.join(INCLUDE, "joker_gb300.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH + FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile the CUDA sources into ``thejoker_gb300/_lib/libjoker_gb300.so``."""
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp_path = os.path.join(OUT_DIR, "build.stamp")
    stamp = _stamp()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp_path):
        with open(stamp_path) as fh:
            if fh.read().strip() == stamp:
                return LIB_PATH
    nvcc = _nvcc()
    objs = [os.path.join(OUT_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc] + ARCH + FLAGS + ["-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(compile_one, zip(SOURCES, objs)))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    with open(stamp_path, "w") as fh:
        fh.write(stamp)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
