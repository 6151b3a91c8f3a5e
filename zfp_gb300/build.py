"""Build libzfp_gb300.so in-tree: nvcc for sm_103a, one object per source,
compiled in parallel, linked with the static CUDA runtime."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libzfp_gb300.so")
LOOP_LIB = os.path.join(HERE, "libzfp_gb300_loop.so")   # per-call C client of the API (benchmark arm)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]

SOURCES = ["zfp_api.cpp", "blocks.cpp", "gpu_codec.cu", "batch.cu", "noalloc.cu", "serve.cu", "index.cu"] + [f"kern_{t}_{d}d.cu" for t in ("f32", "f64", "i32", "i64") for d in (1, 2, 3, 4)]


def _deps() -> list[str]:
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", f) for f in os.listdir(os.path.join(HERE, "..", "include"))]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [NVCC, *ARCH, *CFLAGS, *extra, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC, *CFLAGS, *extra, "-x", "cu", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile the CUDA library if any source changed; return its path."""
    deps = _deps()
    if not force and not _newer(LIB, deps):
        if _newer(LOOP_LIB, [LIB, os.path.join(CSRC, "percall_loop.c")]):
            build_loop()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    extra = extra or []
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcuda"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_loop()
    if verbose:
        print("built", LIB)
    return LIB


def build_loop() -> str:
    """libzfp_gb300_loop.so: csrc/percall_loop.c, a C client linked against the library."""
    src = os.path.join(CSRC, "percall_loop.c")
    r = subprocess.run([os.environ.get("CC", "gcc"), "-O2", "-std=c99", "-fPIC", "-shared", "-o", LOOP_LIB, src,
                        "-L", HERE, "-lzfp_gb300", "-Wl,-rpath,$ORIGIN"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return LOOP_LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
