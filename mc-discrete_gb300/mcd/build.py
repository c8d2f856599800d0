"""Build libmcd.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in parallel; the shared library links against
the shared CUDA runtime so it shares the runtime already loaded by PyTorch.
Usage: python -m mcd.build  (from mc-discrete_gb300/) or mcd.build.build().
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libmcd.so")
BUILD_DIR = os.path.join(ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
SOURCES = ["mcd_host.cpp", "mcd_tables.cu", "mcd_transport.cu", "mcd_adjoint.cu", "mcd_detector.cu"]
EXTRA = {
    # FP32 transport: approximate division/sqrt and flush-to-zero; FP64
    # transport is unaffected by these flags.
    "mcd_transport.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false", "-Xptxas", "-v"],
    "mcd_adjoint.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false", "--extended-lambda"],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmcd")


def _compile(src, verbose):
    obj = os.path.join(BUILD_DIR, src + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + COMMON + EXTRA.get(src, [])
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + COMMON
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "..", "include", "mcd.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile and link libmcd.so if any source is newer than it."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-cudart", "shared", "-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
