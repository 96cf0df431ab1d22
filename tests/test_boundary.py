"""The C-ABI boundary, checked without a GPU: the libraries load and export every
function include/xingpu.h declares; the ME-state mirror (include/xingpu_me.h and
its ctypes copy) has the reference's xin_me_struct layout."""
import ctypes as C
import os
import subprocess
import tempfile

import pytest

from xin26x_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"


@pytest.mark.parametrize("bd", (8, 10))
def test_library_exports_every_declared_symbol(bd):
    path = _lib.lib_path(bd)
    if not os.path.exists(path):
        pytest.skip("libxingpu not built (run __graft_entry__.build())")
    lib = C.CDLL(path)
    names = _lib.header_functions()
    assert len(names) >= 80, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_loader_fails_loudly_without_library(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "HERE", str(tmp_path))
    monkeypatch.setattr(_lib, "_LIBS", {})
    with pytest.raises(ImportError):
        _lib.load(8)


_FIELDS = ["width", "height", "minMv", "maxMv", "meCand", "candNum", "biMe", "oneDimMe", "bestMv", "predMv", "bestCost",
           "bestSad", "bestPos", "searchWidth", "searchHeight", "iMvMode", "bestRound", "bestDist", "maxLgTZDist",
           "rasterDist", "bestMvX", "bestMvY", "numSearchRound", "searchOffset", "searchRadius", "searchPoints",
           "skippedSR", "refinedSR", "sadLambda", "sseLambda", "refIdx", "listIdx", "input", "inputStride", "input1",
           "input1Stride", "input2", "input2Stride", "ref", "refStride", "ref1", "ref1Stride", "ref2", "ref2Stride",
           "interpBuf", "halfPelH", "halfPelV", "halfPelHv", "integPel", "interpStride", "halfPel", "qBufA", "qBufB"]


def _offsets_c(src: str, incs: list) -> dict:
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "o.c")
        exe = os.path.join(d, "o")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-o", exe, c] + [f"-I{i}" for i in incs], check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


def _probe(struct: str, headers: list) -> str:
    inc = "".join(f'#include "{h}"\n' for h in headers)
    body = "".join(f'printf("{f} %zu\\n", offsetof({struct}, {f}));\n' for f in _FIELDS)
    return f"#include <stdio.h>\n#include <stddef.h>\n#include <stdint.h>\n{inc}int main(void){{\n{body}printf(\"sizeof %zu\\n\", sizeof({struct}));return 0;}}\n"


def test_me_mirror_matches_ctypes_copy():
    mine = _offsets_c(_probe("xin_gpu_me_struct", ["xingpu_me.h"]), [os.path.join(ROOT, "include")])
    for f in _FIELDS:
        assert getattr(_lib.xin_gpu_me_struct, f).offset == mine[f], f
    assert C.sizeof(_lib.xin_gpu_me_struct) == mine["sizeof"]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "h26x_core")), reason="reference tree absent")
def test_me_mirror_matches_reference_layout():
    incs = [os.path.join(REF, p) for p in ("common/include", "video_api/video_common/include", "h26x_core/include")]
    ref = _offsets_c(_probe("xin_me_struct", ["xin_typedef.h", "xin_video_common.h", "h26x_me_struct.h"]), incs)
    mine = _offsets_c(_probe("xin_gpu_me_struct", ["xingpu_me.h"]), [os.path.join(ROOT, "include")])
    assert ref == mine
