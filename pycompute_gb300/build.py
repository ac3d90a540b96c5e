"""Build the native library in-tree: pycompute_gb300/_build/libpcgb.so.

The library is C++17 + CUDA compiled by nvcc for sm_103a
(``-gencode arch=compute_103a,code=sm_103a``). The device sources that are
compiled at run time by NVRTC (csrc/lm_params.h, csrc/lm_kernel.cuh) are
embedded into it as string literals, so the .so is self-contained.
"""
from __future__ import annotations

import glob
import hashlib
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libpcgb.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
EMBED = ["lm_params.h", "lm_kernel.cuh"]


def _embedded_cpp() -> str:
    out = ["// generated by pycompute_gb300/build.py: device sources compiled at run time"]
    for name in EMBED:
        with open(os.path.join(CSRC, name)) as f:
            text = f.read()
        assert ")PCGBSRC\"" not in text
        sym = "pcgb_embedded_" + name.replace(".", "_")
        out.append(f'extern const char* {sym};\nconst char* {sym} = R"PCGBSRC({text})PCGBSRC";')
    return "\n".join(out) + "\n"


def _sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cpp")) + glob.glob(os.path.join(CSRC, "*.cu")))


def _inputs_hash(extra: str) -> str:
    h = hashlib.sha1(extra.encode())
    for p in _sources() + [os.path.join(CSRC, n) for n in EMBED] + glob.glob(os.path.join(CSRC, "*.h")) + \
            glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> str:
    """Compile libpcgb.so if any source changed; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    flags = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", GENCODE, "-lineinfo", "-Xptxas", "-v",
             f"-I{INCLUDE}", f"-I{CSRC}", "-cudart", "static", "-lnvrtc", f"-L{CUDA_HOME}/lib64",
             f"-Xlinker", f"-rpath,{CUDA_HOME}/lib64"]
    stamp = os.path.join(BUILD, "libpcgb.stamp")
    key = _inputs_hash(" ".join(flags))
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == key:
        return LIB
    emb = os.path.join(BUILD, "pcgb_embedded.cpp")
    with open(emb, "w") as f:
        f.write(_embedded_cpp())
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [NVCC, *flags, *_sources(), emb, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"libpcgb build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stdout.write(r.stdout + r.stderr)
    os.replace(tmp, LIB)
    with open(os.path.join(BUILD, "ptxas.log"), "w") as f:
        f.write(r.stdout + r.stderr)
    with open(stamp, "w") as f:
        f.write(key)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
