"""Builds the in-tree CUDA library ``libhermes_gb300.so`` for sm_103a.

One nvcc invocation per translation unit (run in parallel), then one link.
The library links the CUDA runtime and cuFFT from the toolkit; nothing is
installed outside this package directory.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(PKG_DIR, "libhermes_gb300.so")
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = os.path.join(cuda_home, "bin", "nvcc")
    if os.path.exists(cand):
        return cand
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found; set CUDA_HOME")
    return found


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src, extra):
    obj = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
    cmd = [nvcc_path(), "-c", os.path.join(CSRC, src), "-o", obj, "-O3", "-lineinfo",
           "-std=c++17", "-Xcompiler", "-fPIC", *ARCH_FLAGS, *extra]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def _stale(objs):
    if not os.path.exists(LIB_PATH):
        return True
    lib_t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(PKG_DIR, "..", "include", "hermes_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > lib_t for d in deps if os.path.exists(d))


def build(force=False, verbose=False, extra_flags=()):
    """Compile every csrc/*.cu for sm_103a and link libhermes_gb300.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = sources()
    if not force and not _stale(srcs):
        return LIB_PATH
    extra = list(extra_flags)
    if verbose:
        extra += ["-Xptxas", "-v"]
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1, len(srcs)))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), srcs))
    if verbose:
        for (_, log), s in zip(results, srcs):
            sys.stderr.write(f"== {s}\n{log}")
    objs = [o for o, _ in results]
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc_path(), "-shared", "-o", tmp, *objs, *ARCH_FLAGS, "-lcufft", "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB_PATH)
