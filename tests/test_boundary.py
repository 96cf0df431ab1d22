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
from __graft_entry__ import REFERENCE_DIR as REF


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


_FUNC_MEMBERS = ["pfXinComputeSad", "pfXinComputeSatd", "pfXinComputeDist", "pfXinComputeAvgSad", "pfXinComputeAvgDist",
                 "pfXinComputeWeightDist", "pfXinComputeSadx8", "pfXinComputeAvgSadx8", "pfXinLumaInterp",
                 "pfXinChromaInterp", "pfXinBiliInterp", "pfXinLumaInterpS16", "pfXinChromaInterpS16", "pfXinInterpAvg", "pfXinInterpWeight",
                 "pfXinQuantInvQuant", "pfXinFor2dDct2", "pfXinFor2dSkip", "pfXinInv2dSkip", "pfXinFor1dDct",
                 "pfXinInv2dDct2", "pfXinInv1dDct", "pfXinBlockSubForDct", "pfXinBlockAddForDct", "pfXinComputeHada8x8",
                 "pfXinPreRdoq", "pfXinPreDepQuant", "pfXinDepQuant", "pfXinFilterIntraNB"]


def _func_probe(struct, headers):
    inc = "".join(f'#include "{h}"\n' for h in headers)
    body = "".join(f'printf("{f} %zu\\n", offsetof({struct}, {f}));\n' for f in _FUNC_MEMBERS)
    return f"#include <stdio.h>\n#include <stddef.h>\n#include <stdint.h>\n{inc}int main(void){{\n{body}printf(\"sizeof %zu\\n\", sizeof({struct}));return 0;}}\n"


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "h266_encoder")), reason="reference tree absent")
def test_func_table_mirror_matches_reference_layout():
    hdrs = ["xin_typedef.h", "basic_macro.h", "h26x_definition.h", "h266_definition.h", "h266_constant.h",
            "xin_video_common.h", "h266_picture_struct.h", "h266_intra_pred_context.h", "h266_pred_unit_struct.h",
            "h266_seq_struct.h", "h266_trans_unit_struct.h", "h26x_me_struct.h", "h266_cabac_struct.h",
            "h266_md_buffer_struct.h", "h266_coding_unit_struct.h", "h266_alf_struct.h", "h266_section_struct.h",
            "h26x_trans_context.h", "h266_func_struct.h"]
    incs = [os.path.join(REF, p) for p in ("common/include", "video_api/video_common/include", "video_api/video_encoder/include",
                                           "h26x_core/include", "h266_core/include", "h266_encoder/include")]
    ref = _offsets_c(_func_probe("xin_func_struct", hdrs), incs)
    mine = _offsets_c(_func_probe("xin_gpu_func_struct", ["xingpu_install.h"]), [os.path.join(ROOT, "include")])
    assert ref == mine


@pytest.mark.parametrize("bd", (8, 10))
def test_installer_fills_tables_without_gpu(bd):
    path = _lib.lib_path(bd)
    if not os.path.exists(path):
        pytest.skip("libxingpu not built")
    lib = C.CDLL(path)
    lib.xin_gpu_install.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32]
    # offsets from the mirror header, via a probe program
    offs = _offsets_c(_func_probe("xin_gpu_func_struct", ["xingpu_install.h"]), [os.path.join(ROOT, "include")])
    size = offs["sizeof"]
    fs = (C.c_void_p * (size // 8))()
    satd_slot = offs["pfXinComputeSatd"] // 8 + 3
    dist_slot = offs["pfXinComputeDist"] // 8 + 3
    fs[satd_slot] = fs[dist_slot] = 0x1234        # preset selected SATD for width 8
    me = _lib.xin_gpu_me_struct()
    assert lib.xin_gpu_install(C.addressof(fs), C.addressof(me), 15) == 0
    addr = lambda n: C.cast(getattr(lib, n), C.c_void_p).value  # noqa: E731
    assert fs[offs["pfXinComputeSad"] // 8] == addr("XinGpuComputeSad")
    assert fs[dist_slot] == addr("XinGpuComputeSatd")
    assert fs[offs["pfXinComputeDist"] // 8 + 4] == addr("XinGpuComputeSad")
    assert fs[offs["pfXinLumaInterp"] // 8 + 16 + 3] == addr("XinGpuLumaInterpHor")       # [1][0][3]
    assert fs[offs["pfXinFor1dDct"] // 8 + 2 * 8 + 4] == addr("XinGpuFDst7P16")          # [DST7][16]
    assert fs[offs["pfXinInv1dDct"] // 8 + 6] == addr("XinGpuIDct2P64")
    assert fs[offs["pfXinFor1dDct"] // 8 + 1 * 8 + 6] is None                             # no 64-point DCT8
    assert fs[offs["pfXinQuantInvQuant"] // 8 + 5] == addr("XinGpuQuantInvQuant")
    assert fs[offs["pfXinPreRdoq"] // 8] == addr("XinGpuPreRdoq")
    assert fs[offs["pfXinDepQuant"] // 8] == addr("XinGpuDepQuant")
    assert fs[offs["pfXinBiliInterp"] // 8 + 3 * 8 + 4] == addr("XinGpuBiliInterpHorVet")  # [1][1][4]
    assert fs[offs["pfXinBiliInterp"] // 8 + 1 * 8 + 2] == addr("XinGpuBiliInterpVet")     # [0][1][2]
    assert fs[offs["pfXinFilterIntraNB"] // 8] is None                                    # off the hot path
    assert me.funcSet[0] == addr("XinGpuComputeSad")
    assert lib.xin_gpu_install(None, None, 15) == -2


_REF_HDRS = ["xin_typedef.h", "basic_macro.h", "h26x_definition.h", "h266_definition.h", "h266_constant.h",
             "xin_video_common.h", "h266_picture_struct.h", "h266_intra_pred_context.h", "h266_pred_unit_struct.h",
             "h266_seq_struct.h", "h266_trans_unit_struct.h", "h26x_me_struct.h", "h266_cabac_struct.h",
             "h266_md_buffer_struct.h", "h266_coding_unit_struct.h", "h266_alf_struct.h", "h266_section_struct.h",
             "h266_dep_quant_struct.h"]
_CTX = ["XIN_CO_QT_ROOT_CBF", "XIN_CO_QT_CBF_Y", "XIN_CO_QT_CBF_U", "XIN_CO_QT_CBF_V", "XIN_CO_SIG_COEFF_GROUP_LUMA",
        "XIN_CO_SIG_COEFF_GROUP_CHROMA", "XIN_CO_SIG_FLAG_LUMA", "XIN_CO_SIG_FLAG_CHROMA", "XIN_CO_PAR_FLAG_LUMA",
        "XIN_CO_PAR_FLAG_CHROMA", "XIN_CO_GT2_FLAG_LUMA", "XIN_CO_GT1_FLAG_LUMA", "XIN_CO_LAST_X_LUMA",
        "XIN_CO_LAST_X_CHROMA", "XIN_CO_LAST_Y_LUMA", "XIN_CO_LAST_Y_CHROMA"]
_MINE = ["ROOT_CBF", "CBF_Y", "CBF_U", "CBF_V", "SIGGRP_L", "SIGGRP_C", "SIG_L", "SIG_C", "PAR_L", "PAR_C", "GT2_L",
         "GT1_L", "LASTX_L", "LASTX_C", "LASTY_L", "LASTY_C"]


@pytest.mark.parametrize("tenbit", (False, True))
@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "h266_encoder")), reason="reference tree absent")
def test_dep_quant_boundary_matches_reference(tenbit):
    """The three structure fields XinGpuDepQuant reads, the context layout and
    the context indices of the library and the oracle equal the reference's."""
    import re
    incs = [os.path.join(REF, p) for p in ("common/include", "video_api/video_common/include", "video_api/video_encoder/include",
                                           "h26x_core/include", "h266_core/include", "h266_encoder/include")]
    inc = "".join(f'#include "{h}"\n' for h in _REF_HDRS)
    pre = "#define ENABLE_10BIT_ENCODER\n" if tenbit else ""
    body = ('printf("ctx %zu\\n", offsetof(xin_dep_quant, context));'
            'printf("full %zu\\n", offsetof(xin_fast_md_buf, fullBuf));'
            'printf("type %zu\\n", offsetof(xin_fast_md_buf, type));'
            'printf("tunum %zu\\n", offsetof(xin_full_md_buf, tuNum));'
            'printf("intra %d\\n", (int)XIN_INTRA_MODE);'
            'printf("nctx %d\\n", (int)XIN_NUM_OF_CTX);'
            'printf("prob %zu\\n", sizeof(xin_prob_model));'
            + "".join(f'printf("{m} %d\\n", (int){c});' for m, c in zip(_MINE, _CTX)))
    src = f"{pre}#include <stdio.h>\n#include <stddef.h>\n{inc}int main(void){{{body}return 0;}}\n"
    ref = _offsets_c(src, incs)
    hdr = open(os.path.join(ROOT, "include", "xingpu.h")).read()
    d = {k: int(v) for k, v in re.findall(r"#define (XIN_GPU_\w+)\s+(\d+)", hdr)}
    assert ref["ctx"] == d["XIN_GPU_DQ_CONTEXT_OFFSET"] and ref["full"] == d["XIN_GPU_FASTBUF_FULLBUF_OFFSET"]
    assert ref["type"] == d["XIN_GPU_FASTBUF_TYPE_OFFSET"] and ref["tunum"] == d["XIN_GPU_FULLBUF_TUNUM_OFFSET"]
    assert ref["intra"] == d["XIN_GPU_INTRA_MODE"] and ref["nctx"] == d["XIN_GPU_NUM_CTX"] == _lib.NUM_CTX
    assert ref["prob"] == C.sizeof(_lib.xin_gpu_prob)
    for name in ("csrc/xg_dq.cuh",):
        txt = open(os.path.join(ROOT, "xin26x_gb300", name)).read()
        mine = {k: int(v) for k, v in re.findall(r"XG_DQC_(\w+) = (\d+)", txt)}
        for m in _MINE:
            assert mine[m] == ref[m], m
    txt = open(os.path.join(ROOT, "oracle", "oracle_dq.c")).read()
    mine = {k: int(v) for k, v in re.findall(r"DQC_(\w+) = (\d+)", txt)}
    for m in _MINE:
        assert mine[m] == ref[m], m


# the library's own public structs: the ctypes and numpy mirrors the Python side
# passes across the C ABI have the header's layout (sizes and member offsets)
_MIRRORS = ["xin_gpu_stream_cfg", "xin_gpu_picture", "xin_gpu_cu_result", "xin_gpu_results", "xin_gpu_tq_block",
            "xin_gpu_dq_block", "xin_gpu_server_cfg", "xin_gpu_server_done", "xin_gpu_server_stats"]


@pytest.mark.parametrize("bd", (8, 10))
def test_public_struct_mirrors_match_the_header(bd):
    import numpy as np
    from xin26x_gb300 import frame
    checks = []                                  # (C struct, {member: offset}, size)
    for name in _MIRRORS:
        cls = getattr(_lib, name)
        checks.append((name, {f: getattr(cls, f).offset for f, *_ in cls._fields_ if not f.startswith("reserved")},
                       C.sizeof(cls)))
    for name, dt in (("xin_gpu_cu_result", frame.CU_DTYPE), ("xin_gpu_cu_mts", frame.MTS_DTYPE),
                     ("xin_gpu_cu_bi", frame.BI_DTYPE)):
        checks.append((name, {f: dt.fields[f][1] for f in dt.names if not f.startswith("reserved")}, dt.itemsize))
    inc = '#define ENABLE_10BIT_ENCODER\n' if bd == 10 else ''
    body = ""
    for i, (name, offs, _) in enumerate(checks):
        body += "".join(f'printf("{i}.{f} %zu\\n", offsetof({name}, {f}));\n' for f in offs)
        body += f'printf("{i}.sizeof %zu\\n", sizeof({name}));\n'
    src = (f"#include <stdio.h>\n#include <stddef.h>\n#include <stdint.h>\n{inc}#include \"xingpu.h\"\n"
           f"int main(void){{\n{body}return 0;}}\n")
    got = _offsets_c(src, [os.path.join(ROOT, "include")])
    for i, (name, offs, size) in enumerate(checks):
        assert got[f"{i}.sizeof"] == size, (name, got[f"{i}.sizeof"], size)
        for f, o in offs.items():
            assert got[f"{i}.{f}"] == o, (name, f, got[f"{i}.{f}"], o)
