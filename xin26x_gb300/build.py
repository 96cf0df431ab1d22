"""Build libxingpu{8,10}.so in-tree with nvcc for sm_103a (and the CPU oracle).

    python -m xin26x_gb300.build          # both bit depths, in parallel
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] + [os.path.join(ROOT, "include", "xingpu.h"),
                                                                       os.path.join(ROOT, "include", "xingpu_me.h"),
                                                                       os.path.join(ROOT, "include", "xingpu_install.h")]


def _stale(out: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in _sources())


def build_lib(bitdepth: int, force: bool = False) -> str:
    out = os.path.join(HERE, f"libxingpu{bitdepth}.so")
    if not force and not _stale(out):
        return out
    tmp = out + ".tmp"
    # -Bsymbolic: calls inside the library bind to its own definitions, so the 8-bit and the
    # 10-bit build (same exported names) can live in one process
    cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-Xlinker", "-Bsymbolic",
           f"-DXG_BITDEPTH={bitdepth}", "-o", tmp, os.path.join(CSRC, "xingpu.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {bitdepth}-bit:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


def build_all(force: bool = False) -> list:
    with ThreadPoolExecutor(2) as ex:
        outs = list(ex.map(lambda b: build_lib(b, force), (8, 10)))
    return outs


if __name__ == "__main__":
    for p in build_all(force="--force" in sys.argv):
        print(p)
