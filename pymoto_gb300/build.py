"""Build recipe of the CUDA library libpymoto_gb300.so (sm_103a only).

Compiles every translation unit of csrc/ with nvcc in parallel and links them into one shared library
next to this file.  No PyTorch headers are involved: the library exposes a plain C ABI
(include/pymoto_gb300.h) that the Python host layer binds with ctypes.

    python -m pymoto_gb300.build          # or __graft_entry__.build()
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(ROOT, "_build")
LIB_NAME = "libpymoto_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# per-file flags: the MMA update keeps numpy's rounding of every element-wise expression (no FMA contraction)
FILE_FLAGS = {"mma.cu": ["--fmad=false"]}


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pymoto_gb300")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _flags():
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            "-I" + os.path.join(ROOT, "include")]


def _fingerprint():
    h = hashlib.sha256()
    for path in sources() + [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cuh")] + \
            [os.path.join(ROOT, "include", "pymoto_gb300.h")]:
        with open(path, "rb") as f:
            h.update(path.encode() + f.read())
    h.update(" ".join(_flags()).encode())
    h.update(repr(sorted(FILE_FLAGS.items())).encode())
    return h.hexdigest()


def build(force=False, verbose=False):
    """Compile csrc/*.cu into pymoto_gb300/libpymoto_gb300.so; returns the library path."""
    fp = _fingerprint()
    stamp = LIB_PATH + ".stamp"
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == fp:
                return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + _flags() + FILE_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-cudart", "static", "-Xcompiler", "-fPIC", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
