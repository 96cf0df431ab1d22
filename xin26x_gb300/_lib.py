"""ctypes binding of libxingpu{8,10}.so (include/xingpu.h).

The product path: every call goes to the CUDA library.  There is no CPU
fallback -- if the shared library is missing or cannot load, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "xingpu.h")
HEADERS = [os.path.join(ROOT, "include", f) for f in ("xingpu.h", "xingpu_me.h", "xingpu_install.h")]

i32, u32, u64, ip, vp = C.c_int32, C.c_uint32, C.c_uint64, C.c_ssize_t, C.c_void_p


class xin_gpu_stream_cfg(C.Structure):
    _fields_ = [("width", i32), ("height", i32), ("ctu_size", i32), ("search_range", i32),
                ("level_mask", u32), ("out_flags", u32), ("use_graph", i32), ("device_io", i32),
                ("input_bitdepth", i32), ("search_mode", i32), ("tu_mode", i32), ("refs", i32), ("dpb", i32)]


class xin_gpu_picture(C.Structure):
    _fields_ = [("plane", vp * 3), ("stride", ip * 3), ("qp", i32), ("uv_qp", i32), ("sad_lambda", u32)]


class xin_gpu_cu_result(C.Structure):
    _fields_ = [("mvx", i32), ("mvy", i32), ("cost", u32), ("int_cost", u32), ("nz", u64 * 3), ("ssd", u64 * 3)]


class xin_gpu_results(C.Structure):
    _fields_ = [("cu", vp), ("q", vp * 3), ("rec", vp * 3), ("gpu_ms", C.c_float), ("mts", vp), ("bi", vp)]


class xin_gpu_tq_block(C.Structure):
    _fields_ = [("offset", u32), ("log2w", C.c_uint8), ("log2h", C.c_uint8), ("mts", C.c_uint8), ("flags", C.c_uint8),
                ("qp", i32)]


class xin_gpu_dq_block(C.Structure):
    _fields_ = [("offset", u32), ("stride", C.c_uint16), ("log2_w", C.c_uint8), ("log2_h", C.c_uint8), ("qp", C.c_uint8),
                ("comp", C.c_uint8), ("root_cbf", C.c_uint8), ("reserved", C.c_uint8), ("ctx_set", u32)]


NUM_CTX = 401     # context records per set (xin_gpu_prob, 6 bytes each)


class xin_gpu_prob(C.Structure):
    _fields_ = [("state", C.c_uint16 * 2), ("rate", C.c_uint8)]


class xin_gpu_server_cfg(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("mpix_budget", C.c_double), ("max_inflight", u32), ("max_streams", u32),
                ("max_queue", u32), ("batch_max", u32), ("batch_window_us", u32), ("reserved", u32)]


class xin_gpu_server_done(C.Structure):
    _fields_ = [("stream_id", i32), ("frame_index", u32), ("user_tag", C.c_uint64), ("status", i32),
                ("has_results", i32), ("gpu_ms", C.c_float), ("reserved", C.c_float), ("queue_ms", C.c_double),
                ("latency_ms", C.c_double)]


class xin_gpu_server_stats(C.Structure):
    _fields_ = [("streams", i32), ("running", i32), ("queued", i32), ("reserved", i32), ("hbm_budget", C.c_uint64),
                ("hbm_used", C.c_uint64), ("mpix_used", C.c_double), ("launched", C.c_uint64),
                ("completed", C.c_uint64), ("batches", C.c_uint64), ("batched_pictures", C.c_uint64)]


class xin_gpu_mv(C.Structure):
    _fields_ = [("mvX", C.c_int16), ("mvY", C.c_int16)]


class xin_gpu_me_struct(C.Structure):
    """Layout mirror of the reference's xin_me_struct (h26x_core/include/h26x_me_struct.h:60-131)."""
    _fields_ = [("funcSet", vp * (13 * 8 + 2)),
                ("width", u32), ("height", u32), ("minMv", xin_gpu_mv), ("maxMv", xin_gpu_mv),
                ("meCand", xin_gpu_mv * 12), ("candNum", u32), ("biMe", i32), ("oneDimMe", i32),
                ("bestMv", xin_gpu_mv), ("predMv", xin_gpu_mv), ("bestCost", u32), ("bestSad", u32), ("bestPos", u32),
                ("searchWidth", i32), ("searchHeight", i32), ("iMvMode", i32),
                ("bestRound", i32), ("bestDist", i32), ("maxLgTZDist", i32), ("rasterDist", i32),
                ("bestMvX", i32), ("bestMvY", i32), ("numSearchRound", i32),
                ("searchOffset", xin_gpu_mv * (16 * 13)), ("searchRadius", u32 * 16), ("searchPoints", u32 * 16),
                ("skippedSR", u32), ("refinedSR", u32), ("sadLambda", u32), ("sseLambda", u64),
                ("refIdx", i32), ("listIdx", i32),
                ("input", vp), ("inputStride", ip), ("input1", vp), ("input1Stride", ip),
                ("input2", vp), ("input2Stride", ip), ("ref", vp), ("refStride", ip),
                ("ref1", vp), ("ref1Stride", ip), ("ref2", vp), ("ref2Stride", ip),
                ("interpBuf", vp), ("halfPelH", vp), ("halfPelV", vp), ("halfPelHv", vp), ("integPel", vp),
                ("interpStride", ip), ("halfPel", vp * 9), ("qBufA", vp * 72), ("qBufB", vp * 72)]


_INTERP = [vp, ip, vp, ip, i32, u32, u32, u32]
_F1 = [vp, ip, vp, ip, i32, i32]
_I1 = [vp, ip, vp, ip, i32, i32, i32]
SIGNATURES = {
    "xin_gpu_init": ([C.c_int], C.c_int),
    "xin_gpu_bitdepth": ([], C.c_int),
    "xin_gpu_last_status": ([], C.c_int),
    "xin_gpu_last_error": ([], C.c_char_p),
    "xin_gpu_clear_error": ([], None),
    "xin_gpu_kernel_launches": ([], u64),
    "XinGpuComputeSad": ([vp, ip, vp, ip, u32, u32, vp], None),
    "XinGpuComputeSatd": ([vp, ip, vp, ip, u32, u32, vp], None),
    "XinGpuComputeAvgSad": ([vp, ip, vp, vp, ip, u32, u32, vp], None),
    "XinGpuComputeAvgSatd": ([vp, ip, vp, vp, ip, u32, u32, vp], None),
    "XinGpuComputeWeightSad": ([vp, ip, vp, vp, ip, u32, u32, i32, i32, vp], None),
    "XinGpuComputeWeightSatd": ([vp, ip, vp, vp, ip, u32, u32, i32, i32, vp], None),
    "XinGpuComputeSadx8": ([vp, ip, vp, ip, u32, u32, vp], None),
    "XinGpuComputeSadx5": ([vp, ip, vp, vp, vp, vp, vp, ip, u32, u32, vp], None),
    "XinGpuComputeSadx3": ([vp, ip, vp, vp, vp, ip, u32, u32, vp], None),
    "XinGpuComputeAvgSadx8": ([vp, ip, vp, vp, ip, u32, u32, vp], None),
    "XinGpuComputeVar": ([vp, ip, vp, ip, u32, u32, vp], None),
    "XinGpuComputeAvgVar": ([vp, ip, vp, vp, ip, u32, u32, vp], None),
    "XinGpuComputeHada8x8": ([vp, ip, vp], None),
    "XinGpuInterpAvgS16U8": ([vp, ip, vp, ip, vp, ip, u32, u32], None),
    "XinGpuInterpWeightS16U8": ([vp, ip, vp, ip, vp, ip, u32, u32, i32, i32], None),
    "XinGpuFDct2WxH": ([vp, ip, vp, ip, u32, u32, vp, i32, i32], None),
    "XinGpuIDct2WxH": ([vp, ip, vp, ip, u32, u32, vp, i32, i32], None),
    "XinGpuFSkipWxH": ([vp, ip, vp, ip, u32, u32, vp], None),
    "XinGpuISkipWxH": ([vp, ip, vp, ip, u32, u32], None),
    "XinGpuBlockSubForDct": ([vp, ip, vp, ip, vp, ip, u32, u32], None),
    "XinGpuBlockAddForDct": ([vp, ip, vp, ip, vp, ip, u32, u32], None),
    "XinGpuQuantInvQuant": ([vp, vp, vp, ip, u32, u32, u32, u32, i32, i32, i32, i32, i32, i32, vp], None),
    "XinGpuPreRdoq": ([vp, vp, vp, ip, u32, u32, u32, u32, i32, vp, vp], None),
    "XinGpuMotionEstFull": ([C.POINTER(xin_gpu_me_struct)], None),
    "XinGpuFullSubPelMe": ([C.POINTER(xin_gpu_me_struct)], None),
    "xin_gpu_stream_open": ([C.POINTER(xin_gpu_stream_cfg), C.POINTER(vp)], C.c_int),
    "xin_gpu_stream_close": ([vp], C.c_int),
    "xin_gpu_stream_num_cus": ([vp], C.c_int),
    "xin_gpu_stream_num_levels": ([vp], C.c_int),
    "xin_gpu_stream_level_info": ([vp, C.c_int, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], C.c_int),
    "xin_gpu_frame_submit": ([vp, C.POINTER(xin_gpu_picture)], C.c_int),
    "xin_gpu_frame_submit_refs": ([vp, C.POINTER(xin_gpu_picture), i32, i32], C.c_int),
    "xin_gpu_stream_tune_search": ([vp, vp, vp], C.c_int),
    "xin_gpu_stream_tune_table": ([vp, vp, vp, vp], C.c_int),
    "xin_gpu_stream_tune_tails": ([vp, vp, vp], C.c_int),
    "xin_gpu_frame_wait": ([vp, C.POINTER(xin_gpu_results), i32], C.c_int),
    "xin_gpu_stream_stage_ms": ([vp, C.POINTER(C.c_float)], C.c_int),
    "xin_gpu_stream_set_wait_tries": ([vp, C.c_int64], C.c_int),
    "xin_gpu_stream_device_results": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)], C.c_int),
    "xin_gpu_measure_sad_peak": ([C.POINTER(C.c_double)], C.c_int),
    "xin_gpu_install": ([vp, vp, u32], C.c_int),
    "xin_gpu_fdct2_wxh_noalloc": ([vp, ip, vp, ip, u32, u32, i32, i32, vp], C.c_int),
    "xin_gpu_tq_batch": ([vp, i32, vp, vp, vp, vp, vp, C.c_size_t, i32], C.c_int),
    "xin_gpu_tq_batch_device": ([vp, i32, vp, vp, vp, vp, vp, C.c_size_t, i32, vp, vp], C.c_int),
    "xin_gpu_stream_footprint": ([vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], C.c_int),
    "xin_gpu_server_open": ([vp, C.POINTER(vp)], C.c_int),
    "xin_gpu_server_join": ([vp, vp, C.c_double, C.POINTER(i32)], C.c_int),
    "xin_gpu_server_submit": ([vp, i32, vp, vp, C.c_uint64], C.c_int),
    "xin_gpu_server_submit_planes": ([vp, i32, vp, vp, vp, C.c_uint64], C.c_int),
    "xin_gpu_server_poll": ([vp, vp, i32, i32, C.POINTER(i32)], C.c_int),
    "xin_gpu_server_leave": ([vp, i32, i32], C.c_int),
    "xin_gpu_server_get_stats": ([vp, vp], C.c_int),
    "xin_gpu_server_close": ([vp], C.c_int),
    "xin_gpu_tq_plan_create": ([vp, i32, C.c_size_t, i32, C.POINTER(vp)], C.c_int),
    "xin_gpu_tq_plan_run": ([vp, vp, vp, vp, vp, vp, vp], C.c_int),
    "xin_gpu_tq_plan_tiles": ([vp, vp], C.c_int),
    "xin_gpu_tq_plan_status": ([vp], C.c_int),
    "xin_gpu_stream_set_contexts": ([vp, vp], C.c_int),
    "xin_gpu_tq_plan_set_wait_tries": ([vp, C.c_int64], C.c_int),
    "xin_gpu_tq_plan_destroy": ([vp], None),
    "xin_gpu_dep_quant_batch": ([vp, i32, vp, vp, vp, vp, C.c_size_t, vp, i32], C.c_int),
    "xin_gpu_dep_quant_batch_device": ([vp, i32, vp, vp, vp, vp, C.c_size_t, vp, i32, vp], C.c_int),
    "xin_gpu_dq_plan_create": ([vp, i32, C.c_size_t, i32, C.POINTER(vp)], C.c_int),
    "xin_gpu_dq_plan_run": ([vp, vp, vp, vp, vp, vp, vp], C.c_int),
    "xin_gpu_dq_plan_destroy": ([vp], None),
    "XinGpuBiliInterpCopy": ([vp, C.c_ssize_t, vp, C.c_ssize_t, i32, u32, u32], None),
    "XinGpuBiliInterpHor": ([vp, C.c_ssize_t, vp, C.c_ssize_t, i32, u32, u32], None),
    "XinGpuBiliInterpVet": ([vp, C.c_ssize_t, vp, C.c_ssize_t, i32, u32, u32], None),
    "XinGpuBiliInterpHorVet": ([vp, C.c_ssize_t, vp, C.c_ssize_t, i32, u32, u32], None),
    "XinGpuDownscale2x2": ([vp, C.c_ssize_t, i32, i32, vp, C.c_ssize_t, u32, u32], None),
    "XinGpuMotionSearchHier": ([vp, C.c_ssize_t, vp, C.c_ssize_t, i32, i32, i32, i32, u32, u32, vp], None),
    "XinGpuMotionEstHier": ([vp], None),
    "XinGpuFastSubPelMeVar": ([vp, i32, i32], None),
    "XinGpuInterpoHalfPel": ([vp, C.c_ssize_t, u32, u32, vp, vp, vp, vp, C.c_ssize_t, i32], None),
    "XinGpuLumaMotionCompDmvr": ([vp, vp, C.c_ssize_t, i32, i32, i32, i32, i32, i32, u32, u32, vp, i32, vp, C.c_ssize_t,
                                  vp], None),
    "XinGpuComputeSadS16": ([vp, C.c_ssize_t, vp, C.c_ssize_t, u32, u32, u32, vp], None),
    "XinGpuCopyAndPad": ([vp, C.c_ssize_t, vp, C.c_ssize_t, u32, u32], None),
    "XinGpuCopyAndPadUv": ([vp, vp, C.c_ssize_t, vp, vp, C.c_ssize_t, u32, u32], None),
    "XinGpuDepQuant": ([vp, vp, vp, vp, vp, vp, C.c_ssize_t, u32, i32, i32, vp, u32], None),
}
for _n in ["InterpCopy", "InterpCopyU8S16", "LumaInterpHor", "LumaInterpVet", "LumaInterpHorVet", "LumaInterpHorU8S16",
           "LumaInterpVetU8S16", "LumaInterpHorVetU8S16", "LumaInterpVetS16U8", "LumaInterpVetS16S16",
           "ChromaInterpHor", "ChromaInterpVet", "ChromaInterpHorVet", "ChromaInterpHorU8S16", "ChromaInterpVetU8S16",
           "ChromaInterpHorVetU8S16", "ChromaInterpVetS16U8", "ChromaInterpVetS16S16"]:
    SIGNATURES["XinGpu" + _n] = (_INTERP, None)
for _t, _sizes in (("Dct2", (2, 4, 8, 16, 32, 64)), ("Dst7", (4, 8, 16, 32)), ("Dct8", (4, 8, 16, 32))):
    for _n in _sizes:
        SIGNATURES[f"XinGpuF{_t}P{_n}"] = (_F1, None)
        SIGNATURES[f"XinGpuI{_t}P{_n}"] = (_I1, None)


def header_functions(paths=None) -> list:
    """Every function name the include/*.h headers declare (after macro expansion of the 1-D families)."""
    txt = " ".join(re.sub(r"/\*.*?\*/", " ", open(p).read(), flags=re.S) for p in (paths or HEADERS))
    names = set(re.findall(r"\b(?:void|int|const char \*|uint64_t)\s*\**\s*(\w+)\s*\(", txt))
    names |= set(re.findall(r"XG_[FI]DCT1D\((\w+)\)", txt))
    return sorted(n for n in names if n not in ("XG_FDCT1D", "XG_IDCT1D") and not n.startswith("NAME"))


def lib_path(bitdepth: int = 8) -> str:
    return os.path.join(HERE, f"libxingpu{bitdepth}.so")


_LIBS: dict = {}


def load(bitdepth: int = 8) -> C.CDLL:
    """Load libxingpu for the bit depth; raises if the CUDA library is missing."""
    if bitdepth in _LIBS:
        return _LIBS[bitdepth]
    path = lib_path(bitdepth)
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path, mode=C.RTLD_LOCAL)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _LIBS[bitdepth] = lib
    return lib


def check(lib: C.CDLL, what: str = "") -> None:
    """Raise if the calling thread's last library call failed."""
    st = lib.xin_gpu_last_status()
    if st != 0:
        raise RuntimeError(f"libxingpu {what} failed ({st}): {lib.xin_gpu_last_error().decode()}")
