"""Build libnixis_gb300.so (all CUDA sources in csrc/) for sm_103a, in tree.

    python -m nixis_gb300.build [--verbose] [--ptxas-v]

Each translation unit is compiled by its own nvcc process (in parallel), then
linked into a shared library next to this file.  Rebuilds only when a source
or header is newer than the library.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnixis_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h"))


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


def _compile(src, ptxas_v):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_v else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, obj, r.returncode, r.stdout + r.stderr


def build(force=False, verbose=False, ptxas_v=False):
    """Compile every CUDA source for sm_103a and link the shared library."""
    if not force and not ptxas_v and up_to_date():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_v), srcs))
    errors = [r for r in results if r[2] != 0]
    for src, _, rc, out in results:
        if (verbose or ptxas_v or rc) and out.strip():
            sys.stderr.write(f"--- {os.path.basename(src)}\n{out}\n")
    if errors:
        raise RuntimeError("nvcc failed for: " + ", ".join(os.path.basename(e[0]) for e in errors))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [r[1] for r in results] + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose="--verbose" in sys.argv, ptxas_v="--ptxas-v" in sys.argv)
    print(LIB)
