"""Builds the C-ABI shared library librtcore_gb300.so for sm_103a.

Six translation units (builder, traversal, tuned traversal shapes, proposer,
path tracer, C ABI) are compiled in parallel with nvcc and linked into one
shared object (soname libembree3.so.3, so a program linked against the
reference's library name finds it).  The traversal and builder units use
--fmad=false: the hit-deciding arithmetic spells out every FMA itself.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(REPO, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "librtcore_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["gb_build.cu", "gb_trace.cu", "gb_trace_shapes.cu", "gb_learned.cu", "gb_paths.cu", "rtcore_api.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
            "-I", INC, "-I", CSRC] + ARCH


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return files


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in _deps() + [os.path.abspath(__file__)])


def build(force=False, verbose=False):
    """Compiles and links the library if any source changed; returns its path."""
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [nvcc] + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared"] + ARCH + objs + ["-o", tmp, "-Xlinker", "-soname=libembree3.so.3", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for alias in ("libembree3.so.3", "libembree3.so"):
        p = os.path.join(PKG, alias)
        if os.path.lexists(p):
            os.remove(p)
        os.symlink(os.path.basename(LIB), p)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
