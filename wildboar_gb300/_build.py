"""Compile the CUDA sources in ``csrc/`` into ``libwbgpu.so`` (sm_103a only).

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library next to this file.  The FP64 parity kernels are compiled with
``-fmad=false`` so that no multiply-add is contracted (the reference's C code
is built by gcc -O2, which never fuses on x86-64).
"""

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwbgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# per-file extra flags; everything not listed gets -fmad=false.  dtw32.cu
# (batched FP32 dtw and its backward) keeps -fmad=false as well: its error
# bounds are stated for separately rounded products.
FILE_FLAGS = {
    "euclid_gemm.cu": ["-fmad=true"],
}


def nvcc():
    cand = os.environ.get("NVCC")
    if cand:
        return cand
    p = shutil.which("nvcc")
    if p:
        return p
    return "/usr/local/cuda/bin/nvcc"


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return sorted(hs)


def _digest():
    h = hashlib.sha256()
    for p in [os.path.join(CSRC, f) for f in _sources()] + _headers() + [__file__]:
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def _compile(src, debug_bounds=False):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    flags = FILE_FLAGS.get(src, ["-fmad=false"])
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "--expt-relaxed-constexpr", "-I", INCLUDE, *flags, "-c",
           os.path.join(CSRC, src), "-o", obj]
    if debug_bounds:
        cmd.insert(1, "-DWB_DEBUG_BOUNDS=1")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False):
    """Build libwbgpu.so if any source changed; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp")
    digest = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
