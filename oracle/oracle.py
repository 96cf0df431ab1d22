"""ctypes access to the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle{8,10}.so`` (the C restatement in xin_oracle.c) and,
where it was built, ``oracle/_ref/libxinref{8,10}.so`` (the reference's open C
compiled in place, see oracle/Makefile).  Both expose the same logical calls,
so a test can run one case through either and compare.  Used only by tests/,
__graft_entry__.smoke() and bench.py's CPU legs, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

i32, u32, u64, ip = C.c_int32, C.c_uint32, C.c_uint64, C.c_ssize_t
vp = C.c_void_p


def build(ref: bool = False) -> None:
    """Compile the oracle (and, with ref=True and the reference tree present, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def ref_available(bitdepth: int = 8) -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", f"libxinref{bitdepth}.so"))


def ptr(a: np.ndarray, off: int = 0) -> int:
    """Address of element ``off`` (flat index, may be negative) of a C-contiguous array."""
    return a.ctypes.data + off * a.itemsize


class orc_me_io(C.Structure):
    _fields_ = [("best_mvx", i32), ("best_mvy", i32), ("best_cost", u32), ("best_sad", u32)]


class orc_qparams(C.Structure):
    _fields_ = [("qmult", i32), ("qadd", i32), ("qshift", i32), ("iqmult", i32), ("iqadd", i32), ("iqshift", i32)]


class orc_frame_desc(C.Structure):
    _fields_ = [("width", i32), ("height", i32), ("ctu", i32),
                ("in_", vp * 3), ("in_stride", ip * 2),
                ("ref", vp * 3), ("ref_stride", ip * 2),
                ("search_range", i32), ("sad_lambda", u32), ("qp", i32), ("uv_qp", i32), ("intra_frame", i32),
                ("search_mode", i32), ("in_lo", vp * 2), ("in_lo_stride", ip * 2),
                ("ref_lo", vp * 2), ("ref_lo_stride", ip * 2), ("tu_mode", i32), ("ctx", vp),
                ("refs", i32), ("ref1", vp * 3), ("ref1_lo", vp * 2)]


class orc_hier_in(C.Structure):
    _fields_ = [("in_", vp * 3), ("in_stride", ip * 3), ("ref", vp * 3), ("ref_stride", ip * 3),
                ("cand", vp), ("ncand", u32)]


class orc_dq_param(C.Structure):
    _fields_ = [("qShift", i32), ("qAdd", i32), ("qScale", i32), ("maxQIdx", i32), ("thresLast", i32),
                ("iqShift", i32), ("iqScale", i32), ("distShift", i32), ("distAdd", i32),
                ("distStepAdd", C.c_int64), ("distOrgFact", C.c_int64)]


class xin_dp_param(C.Structure):
    """the reference's xin_dp_param (h266_encoder/include/h266_seq_struct.h:118-134)"""
    _fields_ = [("qShift", i32), ("qAdd", i32), ("qScale", i32), ("maxQIdx", i32), ("thresLast", i32),
                ("thresSSbb", i32), ("iqAdd", i32), ("iqShift", i32), ("iqScale", i32), ("distShift", i32),
                ("distAdd", i32), ("distStepAdd", C.c_int64), ("distOrgFact", C.c_int64)]


class orc_cu_out(C.Structure):
    _fields_ = [("mvx", i32), ("mvy", i32), ("cost", u32), ("int_cost", u32), ("nz", u64 * 3), ("ssd", u64 * 3),
                ("satd_cost", u32), ("ncand", u32), ("nz_mts", u64 * 5), ("ssd_mts", u64 * 5),
                ("mvx1", i32), ("mvy1", i32), ("cost1", u32), ("int_cost1", u32), ("bmv", i32 * 4), ("bi_cost", u32),
                ("inter_dir", u32)]


# logical name -> (oracle symbol, reference symbol or None, argtypes)
_INTERP8 = [vp, ip, vp, ip, i32, u32, u32, u32]
_SIGS = {
    "interp_copy": ("orc_interp_copy", "Xin266InterpCopy", _INTERP8),
    "interp_copy_s16": ("orc_interp_copy_s16", "Xin266InterpCopyU8S16", _INTERP8),
    "luma_hor": ("orc_luma_hor", "Xin266LumaInterpHor", _INTERP8),
    "luma_vet": ("orc_luma_vet", "Xin266LumaInterpVet", _INTERP8),
    "luma_hv": ("orc_luma_hv", "Xin266LumaInterpHorVet", _INTERP8),
    "luma_hor_s16": ("orc_luma_hor_s16", "Xin266LumaInterpHorU8S16", _INTERP8),
    "luma_vet_s16": ("orc_luma_vet_s16", "Xin266LumaInterpVetU8S16", _INTERP8),
    "luma_hv_s16": ("orc_luma_hv_s16", "Xin266LumaInterpHorVetU8S16", _INTERP8),
    "luma_vet_s16_pix": ("orc_luma_vet_s16_pix", "Xin266LumaInterpVetS16U8", _INTERP8),
    "luma_vet_s16_s16": ("orc_luma_vet_s16_s16", "Xin266LumaInterpVetS16S16", _INTERP8),
    "chroma_hor": ("orc_chroma_hor", "Xin266ChromaInterpHor", _INTERP8),
    "chroma_vet": ("orc_chroma_vet", "Xin266ChromaInterpVet", _INTERP8),
    "chroma_hv": ("orc_chroma_hv", "Xin266ChromaInterpHorVet", _INTERP8),
    "chroma_hor_s16": ("orc_chroma_hor_s16", "Xin266ChromaInterpHorU8S16", _INTERP8),
    "chroma_vet_s16": ("orc_chroma_vet_s16", "Xin266ChromaInterpVetU8S16", _INTERP8),
    "chroma_hv_s16": ("orc_chroma_hv_s16", "Xin266ChromaInterpHorVetU8S16", _INTERP8),
    "chroma_vet_s16_pix": ("orc_chroma_vet_s16_pix", "Xin266ChromaInterpVetS16U8", _INTERP8),
    "chroma_vet_s16_s16": ("orc_chroma_vet_s16_s16", "Xin266ChromaInterpVetS16S16", _INTERP8),
    "interp_avg": ("orc_interp_avg", "Xin266InterpAvgS16U8", [vp, ip, vp, ip, vp, ip, u32, u32]),
    "interp_weight": ("orc_interp_weight", "Xin266InterpWeightS16U8", [vp, ip, vp, ip, vp, ip, u32, u32, i32, i32]),
    "quant_inv_quant": ("orc_quant_inv_quant", "Xin266QuantInvQuant",
                        [vp, vp, vp, ip, u32, u32, u32, u32, i32, i32, i32, i32, i32, i32, vp]),
    "pre_rdoq": ("orc_pre_rdoq", "Xin266PreRdoq", [vp, vp, vp, ip, u32, u32, u32, u32, i32, vp, vp]),
    "iskip_wxh": ("orc_iskip_wxh", "Xin266ISkipWxH", [vp, ip, vp, ip, u32, u32]),
    "fdct_wxh": ("orc_fdct_wxh", "ref_fdct_wxh", [vp, ip, vp, ip, u32, u32, u32, u32, i32, i32]),
    "idct_wxh": ("orc_idct_wxh", "ref_idct_wxh", [vp, ip, vp, ip, u32, u32, i32, u32, u32, i32]),
    "sub_fdct_wxh": ("orc_sub_fdct_wxh", "ref_sub_fdct_wxh", [vp, ip, vp, ip, vp, ip, u32, u32, i32, i32, i32, i32]),
    "idct_add": ("orc_idct_add", "ref_idct_add", [vp, ip, vp, ip, vp, ip, i32, u32, u32, u32, u32, i32]),
    # oracle-only
    "sad": ("orc_sad", None, [vp, ip, vp, ip, u32, u32, vp]),
    "sad_xn": ("orc_sad_xn", None, [vp, ip, vp, C.c_int, ip, u32, u32, vp]),
    "avg_sad": ("orc_avg_sad", None, [vp, ip, vp, vp, ip, u32, u32, vp]),
    "avg_sad_xn": ("orc_avg_sad_xn", None, [vp, ip, vp, vp, C.c_int, ip, u32, u32, vp]),
    "satd": ("orc_satd", None, [vp, ip, vp, ip, u32, u32, vp]),
    "avg_satd": ("orc_avg_satd", None, [vp, ip, vp, vp, ip, u32, u32, vp]),
    "weight_sad": ("orc_weight_sad", None, [vp, ip, vp, vp, ip, u32, u32, i32, i32, vp]),
    "weight_satd": ("orc_weight_satd", None, [vp, ip, vp, vp, ip, u32, u32, i32, i32, vp]),
    "hada8x8": ("orc_hada8x8", None, [vp, ip, vp]),
    "var": ("orc_var", None, [vp, ip, vp, ip, u32, u32, vp]),
    "avg_var": ("orc_avg_var", None, [vp, ip, vp, vp, ip, u32, u32, vp]),
    "fdct1d": ("orc_fdct1d", None, [C.c_int, C.c_int, vp, ip, vp, ip, i32, i32]),
    "idct1d": ("orc_idct1d", None, [C.c_int, C.c_int, vp, ip, vp, ip, i32, i32, i32]),
    "fdct2_wxh": ("orc_fdct2_wxh", None, [vp, ip, vp, ip, u32, u32, i32, i32]),
    "idct2_wxh": ("orc_idct2_wxh", None, [vp, ip, vp, ip, u32, u32, i32, i32]),
    "fskip_wxh": ("orc_fskip_wxh", None, [vp, ip, vp, ip, u32, u32]),
    "block_sub": ("orc_block_sub", None, [vp, ip, vp, ip, vp, ip, u32, u32]),
    "block_add": ("orc_block_add", None, [vp, ip, vp, ip, vp, ip, u32, u32]),
    "luma_interpolation": ("orc_luma_interpolation", None, [vp, ip, vp, ip, i32, u32, u32, u32]),
    "luma_inter_pred": ("orc_luma_inter_pred", None, [vp, ip, vp, ip, i32, i32, i32, i32, i32, i32, i32, i32, u32, u32, u32]),
    "chroma_motion_comp": ("orc_chroma_motion_comp", None, [vp, ip, vp, ip, i32, i32, i32, i32, i32, i32, i32, i32, u32, u32]),
    "luma_motion_comp_bi": ("orc_luma_motion_comp_bi", None, [vp, vp, ip, vp, ip, vp, i32, i32, i32, i32, i32, i32, u32, u32]),
    "chroma_motion_comp_bi": ("orc_chroma_motion_comp_bi", None, [vp, vp, ip, vp, ip, vp, i32, i32, i32, i32, i32, i32,
                                                                  u32, u32]),
    "bi_me_input": ("orc_bi_me_input", None, [vp, ip, vp, ip, vp, ip, u32, u32]),
    "quant_params": ("orc_quant_params", None, [i32, u32, u32, u32, C.c_int, C.c_int, C.POINTER(orc_qparams)]),
    "transform_tu": ("orc_transform_tu", None, [vp, ip, vp, ip, vp, vp, vp, ip, u32, u32, u32, u32, i32, C.c_int, C.c_int,
                                                C.c_int, C.c_int, vp]),
    "tq_block": ("orc_tq_block", None, [vp, ip, u32, u32, u32, u32, i32, C.c_int, C.c_int, C.c_int, C.c_int,
                                        vp, vp, vp, ip, vp]),
    "mvd_bits": ("orc_mvd_bits", None, [i32]),
    "mv_window": ("orc_mv_window", None, [i32] * 7 + [C.POINTER(i32)] * 4),
    "me_full": ("orc_me_full", None, [vp, ip, vp, ip, u32, u32, i32, i32, i32, u32, i32, i32, i32, i32, C.POINTER(orc_me_io)]),
    "full_subpel_me": ("orc_full_subpel_me", None, [vp, ip, vp, ip, u32, u32, i32, i32, u32, i32, i32, i32, i32,
                                                    C.POINTER(orc_me_io)]),
    "downscale2x2": ("orc_downscale2x2", None, [vp, ip, C.c_int, C.c_int, vp, ip, u32, u32]),
    "hier_search": ("orc_hier_search", None, [vp, ip, vp, ip, i32, i32, i32, i32, u32, u32, C.POINTER(i32),
                                              C.POINTER(i32)]),
    "me_hier": ("orc_me_hier", None, [C.POINTER(orc_hier_in), u32, u32, i32, i32, i32, i32, u32, i32, i32, i32, i32,
                                      C.POINTER(orc_me_io)]),
    "interpo_half_pel": ("orc_interpo_half_pel", None, [vp, ip, u32, u32, vp, vp, vp, vp, ip, C.c_int]),
    "qpel_pair": ("orc_qpel_pair", None, [i32, i32, i32, i32, vp]),
    "half_grid_block": ("orc_half_grid_block", None, [vp, ip, i32, i32, u32, u32, u32, vp, ip]),
    "fast_subpel_me_var": ("orc_fast_subpel_me_var", "ref_fast_subpel_me_var",
                           [vp, ip, vp, ip, u32, u32, i32, i32, C.c_uint64, i32, i32, i32, i32, i32, vp]),
    "sad_s16": ("orc_sad_s16", None, [vp, ip, vp, ip, u32, u32, u32, vp]),
    "block_pad": ("orc_block_pad", None, [vp, ip, u32, u32, u32, u32]),
    "copy_and_pad": ("orc_copy_and_pad", "ref_copy_and_pad", [vp, ip, vp, ip, u32, u32]),
    "copy_and_pad_uv": ("orc_copy_and_pad_uv", "ref_copy_and_pad_uv", [vp, vp, ip, vp, vp, ip, u32, u32]),
    "dmvr_luma": ("orc_dmvr_luma", "ref_dmvr_luma", [vp, vp, ip, i32, i32, i32, i32, i32, i32, u32, u32, vp, C.c_int,
                                                     vp, vp, ip]),
    "cu_hotpath": ("orc_cu_hotpath", None, [C.POINTER(orc_frame_desc), i32, i32, i32, vp * 3, ip * 2, vp * 3, ip * 2,
                                            C.POINTER(orc_cu_out)]),
    "tr_matrix": ("orc_tr_matrix", None, [C.c_int, C.c_int]),
    "dep_quant": ("orc_dep_quant", "ref_dep_quant", [vp, ip, C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int,
                                                     vp, vp, vp]),
    "bili_interp": ("orc_bili_interp", "ref_bili_interp", [C.c_int, vp, ip, vp, ip, i32, u32, u32]),
    "dq_params": ("orc_dq_params", None, [C.c_int, C.c_int, C.POINTER(orc_dq_param)]),
    "dq_frac_bits": ("orc_dq_frac_bits", None, [C.c_int, vp]),
    "dq_rice_bits": ("orc_dq_rice_bits", None, [C.c_int, C.c_int]),
    "dq_last_group": ("orc_dq_last_group", None, [C.c_int]),
}
_REF_ONLY = {
    "idct2_wxh_tmp": ("Xin266IDct2WxH", [vp, ip, vp, ip, u32, u32, vp, i32, i32]),
    "full_subpel_me_io": ("ref_full_subpel_me", [vp, ip, vp, ip, u32, u32, i32, i32, u32, i32, i32, i32, i32, vp]),
    "dq_param_ref": ("ref_dq_param", [C.c_int, C.c_int, C.POINTER(xin_dp_param)]),
    "luma_inter_pred_ref": ("ref_luma_inter_pred", [vp, ip, vp, ip, i32, i32, i32, i32, i32, i32, i32, i32, u32, u32,
                                                    i32]),
    "chroma_motion_comp_ref": ("ref_chroma_motion_comp", [vp, vp, vp, vp, ip, vp, vp, ip, vp, i32, i32, u32, i32, i32,
                                                          i32, i32, i32, i32, u32, u32]),
    "luma_motion_comp_ref": ("ref_luma_motion_comp", [vp, vp, ip, vp, ip, vp, i32, i32, i32, i32, i32, i32, u32, u32]),
    "weight_bi_me_input_ref": ("Xin266ConstructWeightBiMeInput", [vp, ip, vp, ip, vp, ip, u32, u32, i32]),
    "transform_tu_ref": ("ref_transform_tu", [vp, ip, vp, ip, vp, vp, vp, ip, u32, u32, u32, u32, i32, i32, u32, i32, i32,
                                              i32, vp, vp]),
}


class _Lib:
    def __init__(self, path: str, which: int, bitdepth: int):
        self.path = path
        self.lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        self.bitdepth = bitdepth
        self.pix = np.uint8 if bitdepth == 8 else np.uint16
        self.coef = np.int16 if bitdepth == 8 else np.int32
        self.max_pix = (1 << bitdepth) - 1
        for name, spec in _SIGS.items():
            sym = spec[which]
            if sym is None:
                continue
            f = getattr(self.lib, sym)
            f.argtypes = spec[2]
            f.restype = None
            setattr(self, name, f)
        if which == 0:
            self.mvd_bits.restype = u32
            self.tr_matrix.restype = C.POINTER(C.c_int16)
            self.dq_rice_bits.restype = i32
            self.dq_last_group.restype = C.c_int
        else:
            for name, (sym, args) in _REF_ONLY.items():
                f = getattr(self.lib, sym)
                f.argtypes = args
                f.restype = None
                setattr(self, name, f)

    def matrix(self, tr_type: int, n: int) -> np.ndarray:
        p = self.tr_matrix(tr_type, n)
        return np.ctypeslib.as_array(p, shape=(n * n,)).reshape(n, n).copy()


_CACHE: dict = {}


def oracle(bitdepth: int = 8) -> _Lib:
    """The C restatement (checker), built on demand."""
    key = ("orc", bitdepth)
    if key not in _CACHE:
        path = os.path.join(HERE, f"liboracle{bitdepth}.so")
        if not os.path.exists(path):
            build()
        _CACHE[key] = _Lib(path, 0, bitdepth)
    return _CACHE[key]


def reference(bitdepth: int = 8) -> _Lib:
    """The reference's open C compiled in place (only where oracle/_ref was built)."""
    key = ("ref", bitdepth)
    if key not in _CACHE:
        path = os.path.join(HERE, "_ref", f"libxinref{bitdepth}.so")
        _CACHE[key] = _Lib(path, 1, bitdepth)
    return _CACHE[key]
