"""Build the CUDA library libatsat_dyn.so in-tree, for sm_103a only.

Each .cu under csrc/ is compiled to an object in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a), then linked into atsat_gb300/_lib/libatsat_dyn.so with
the static CUDA runtime. No cmake, no PyTorch extension machinery.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libatsat_dyn.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "--expt-relaxed-constexpr"]
# Per-file additions. The pressure variants' column residual is a sum of nearly cancelling terms that the
# barotropic solve then amplifies; compiled without multiply-add contraction their arithmetic rounds
# operation by operation as the reference's does (it is not on the default path, so the cost is moot).
FILE_FLAGS = {"press_variants.cu": ["-fmad=false"]}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libatsat_dyn.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(lib: str, deps) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "atsat_dyn.h"))
    deps.append(os.path.abspath(__file__))
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    cc = nvcc()

    def one(src):
        obj = os.path.join(OUT, "obj", os.path.basename(src).replace(".cu", ".o"))
        cmd = [cc, *ARCH, *NVFLAGS, *FILE_FLAGS.get(os.path.basename(src), []), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(one, sources()))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", tmp, *objs, "-lgomp"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
