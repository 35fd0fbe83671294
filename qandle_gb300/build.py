"""Build the CUDA library in-tree: qandle_gb300/_build/libqandle_gb300.so.

Every translation unit is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked into
one shared library with a C ABI (include/qandle_gb300.h).  No torch headers
are involved, so a build takes seconds.  A content hash of the sources and
flags decides whether to rebuild.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libqandle_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the qandle_gb300 CUDA library cannot be built")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


# Headers the run-time compiler (csrc/jit.cpp) needs, embedded in the library
# so that it does not depend on the source tree at run time.
JIT_HEADERS = ["devmath.cuh", "engine.h", "planar.cuh", "fwd_kernel.cuh", "bwd_kernel.cuh", "jit_ops.cuh"]


def _write_jit_headers() -> str:
    out = os.path.join(BUILD, "jit_headers.cpp")
    lines = ["// Generated by qandle_gb300/build.py from csrc/: the headers handed to NVRTC.",
             "namespace qg {", f"extern const int kJitHeaderCount = {len(JIT_HEADERS)};",
             "extern const char* const kJitHeaderNames[] = {" +
             ", ".join(f'"{h}"' for h in JIT_HEADERS) + "};",
             "extern const char* const kJitHeaderTexts[] = {"]
    for h in JIT_HEADERS:
        with open(os.path.join(CSRC, h)) as f:
            text = f.read()
        if ")QGJIT" in text:
            raise RuntimeError(f"{h} contains the raw-string delimiter")
        lines.append('R"QGJIT(' + text + ')QGJIT",')
    lines += ["};", "}  // namespace qg", ""]
    body = "\n".join(lines)
    old = None
    if os.path.exists(out):
        with open(out) as f:
            old = f.read()
    if old != body:
        with open(out, "w") as f:
            f.write(body)
    return out


def _cuda_lib_dir() -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    for cand in ("lib64", "lib"):
        d = os.path.join(root, cand)
        if os.path.isdir(d):
            return d
    return "/usr/local/cuda/lib64"


def _digest(extra_flags) -> str:
    h = hashlib.sha256()
    files = _sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh")) +
                                glob.glob(os.path.join(CSRC, "*.h")) +
                                glob.glob(os.path.join(INCLUDE, "*.h")))
    for f in files:
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + list(extra_flags)).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp")
    dig = _digest(extra_flags)
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [cc, *ARCH, *NVCC_FLAGS, f'-DQG_CUDA_LIB_DIR="{_cuda_lib_dir()}"', *extra_flags, "-c", src,
               "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    srcs = _sources() + [_write_jit_headers()]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
