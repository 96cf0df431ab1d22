/*
 * ref_shim.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Links the reference's open hot-path C, compiled in place from the xin26x
 * source tree (see oracle/Makefile, target "ref"), into oracle/_ref/libxinref*.so.
 * The open files call symbols that the reference ships only inside a closed
 * Windows library (h26x_core/h26x_core.lib).  This file supplies those symbols
 * by forwarding to the oracle restatements in xin_oracle.c, so the open 2-D
 * wrappers, quantiser, interpolation and sub-pel search run unmodified around
 * them.  Also supplies the 8-argument Xin266LumaInterpolation that
 * h266_sub_pel_refine.c calls through h266_encoder/include/h266_inter_prediction.h:43
 * (filter index 0), and no-op LMCS chroma scaling (LMCS is off in every harness).
 */
#include "xin_typedef.h"
#include "basic_macro.h"
#include "h26x_definition.h"
#include "h266_definition.h"
#include "h266_constant.h"
#include "xin_video_common.h"
#include "h266_picture_struct.h"
#include "h266_intra_pred_context.h"
#include "h266_pred_unit_struct.h"
#include "h266_seq_struct.h"
#include "h266_trans_unit_struct.h"
#include "h26x_me_struct.h"
#include "h266_cabac_struct.h"
#include "h266_md_buffer_struct.h"
#include "h266_coding_unit_struct.h"
#include "h266_alf_struct.h"
#include "h266_section_struct.h"
#include "h26x_trans_context.h"
#include "h266_func_struct.h"
#include "h266_inter_pred_context.h"
#include "xin_oracle.h"

/* closed tables (h26x_core/include/h26x_common_data.h:23-24, h26x_trans_context.h:67) */
const UINT32 calcLog2[256] = {
    0, 0, 1, 0, 2, 0, 0, 0, 3, 0, 0, 0, 0, 0, 0, 0, 4, [32] = 5, [64] = 6, [128] = 7 };
UINT8 ExpGolombBits[16383 * 2 + 1];
const SINT8 mtsIdx2txType[XIN_MTS_IDX_NUM][2] = {
    { XIN_DCT2, XIN_DCT2 }, { XIN_SKIP, XIN_SKIP }, { XIN_DST7, XIN_DST7 },
    { XIN_DCT8, XIN_DST7 }, { XIN_DST7, XIN_DCT8 }, { XIN_DCT8, XIN_DCT8 } };

__attribute__((constructor)) static void shim_init(void)
{
    for (int i = 0; i < 16383 * 2 + 1; i++) ExpGolombBits[i] = (UINT8)orc_mvd_bits(i - 16383);
}

/* closed 1-D inverse transforms -> oracle */
#define IDCT_FWD(NAME, TYPE, LG) \
    void NAME(COEFF *in, intptr_t is, COEFF *out, intptr_t os, SINT32 line, SINT32 skip, SINT32 shift) \
    { orc_idct1d(TYPE, LG, in, is, out, os, line, skip, shift); }
IDCT_FWD(Xin26xIDct2P2, 0, 1) IDCT_FWD(Xin26xIDct2P4, 0, 2) IDCT_FWD(Xin26xIDct2P8, 0, 3)
IDCT_FWD(Xin26xIDct2P16, 0, 4) IDCT_FWD(Xin26xIDct2P32, 0, 5) IDCT_FWD(Xin26xIDct2P64, 0, 6)
IDCT_FWD(Xin26xIDct8P4, 1, 2) IDCT_FWD(Xin26xIDct8P8, 1, 3) IDCT_FWD(Xin26xIDct8P16, 1, 4) IDCT_FWD(Xin26xIDct8P32, 1, 5)
IDCT_FWD(Xin26xIDst7P4, 2, 2) IDCT_FWD(Xin26xIDst7P8, 2, 3) IDCT_FWD(Xin26xIDst7P16, 2, 4) IDCT_FWD(Xin26xIDst7P32, 2, 5)

/* closed 1-D forward transforms (reached through the function table) -> oracle */
#define FDCT_FWD(NAME, TYPE, LG) \
    static void NAME(COEFF *in, intptr_t is, COEFF *out, intptr_t os, SINT32 line, SINT32 shift) \
    { orc_fdct1d(TYPE, LG, in, is, out, os, line, shift); }
FDCT_FWD(shim_fdct2_2, 0, 1) FDCT_FWD(shim_fdct2_4, 0, 2) FDCT_FWD(shim_fdct2_8, 0, 3)
FDCT_FWD(shim_fdct2_16, 0, 4) FDCT_FWD(shim_fdct2_32, 0, 5) FDCT_FWD(shim_fdct2_64, 0, 6)
FDCT_FWD(shim_fdct8_4, 1, 2) FDCT_FWD(shim_fdct8_8, 1, 3) FDCT_FWD(shim_fdct8_16, 1, 4) FDCT_FWD(shim_fdct8_32, 1, 5)
FDCT_FWD(shim_fdst7_4, 2, 2) FDCT_FWD(shim_fdst7_8, 2, 3) FDCT_FWD(shim_fdst7_16, 2, 4) FDCT_FWD(shim_fdst7_32, 2, 5)

static void shim_fdct2_wxh(COEFF *in, intptr_t is, COEFF *out, intptr_t os, UINT32 w, UINT32 h, COEFF *tmp, SINT32 s1, SINT32 s2)
{ (void)tmp; orc_fdct2_wxh(in, is, out, os, w, h, s1, s2); }
static void shim_fskip(COEFF *in, intptr_t is, COEFF *out, intptr_t os, UINT32 w, UINT32 h, COEFF *tmp)
{ (void)tmp; orc_fskip_wxh(in, is, out, os, w, h); }
static void shim_sad(PIXEL *in, intptr_t is, PIXEL *ref, intptr_t rs, UINT32 w, UINT32 h, UINT32 *sad)
{ orc_sad(in, is, ref, rs, w, h, sad); }
static void shim_sub(PIXEL *in, intptr_t is, PIXEL *pr, intptr_t ps, COEFF *d, intptr_t ds, UINT32 w, UINT32 h)
{ orc_block_sub(in, is, pr, ps, d, ds, w, h); }
static void shim_add(COEFF *r, intptr_t rs, PIXEL *pr, intptr_t ps, PIXEL *o, intptr_t os, UINT32 w, UINT32 h)
{ orc_block_add(r, rs, pr, ps, o, os, w, h); }

/* open functions of the reference used to fill the table */
void Xin266InterpCopy(const PIXEL *, intptr_t, PIXEL *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266LumaInterpHor(const PIXEL *, intptr_t, PIXEL *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266LumaInterpVet(const PIXEL *, intptr_t, PIXEL *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266LumaInterpHorVet(const PIXEL *, intptr_t, PIXEL *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266ChromaInterpHor(const PIXEL *, intptr_t, PIXEL *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266ChromaInterpVet(const PIXEL *, intptr_t, PIXEL *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266ChromaInterpHorVet(const PIXEL *, intptr_t, PIXEL *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266InterpCopyU8S16(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266ChromaInterpHorU8S16(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266ChromaInterpVetU8S16(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266ChromaInterpHorVetU8S16(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266LumaInterpHorU8S16(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266LumaInterpVetU8S16(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266LumaInterpHorVetU8S16(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32, UINT32);
void Xin266BiliInterpCopy(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void Xin266BiliInterpHor(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void Xin266BiliInterpVet(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void Xin266BiliInterpHorVet(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void Xin266CopyAndPad(PIXEL *, intptr_t, PIXEL *, intptr_t, UINT32, UINT32);
void Xin26xComputeSadS16(SINT16 *, intptr_t, SINT16 *, intptr_t, UINT32, UINT32, UINT32, UINT32 *);
void Xin266CopyAndPadUv(PIXEL *, PIXEL *, intptr_t, PIXEL *, PIXEL *, intptr_t, UINT32, UINT32);
void Xin266InterpAvgS16U8(const SINT16 *, intptr_t, const SINT16 *, intptr_t, PIXEL *, intptr_t, UINT32, UINT32);
void Xin266InterpWeightS16U8(const SINT16 *, intptr_t, const SINT16 *, intptr_t, PIXEL *, intptr_t, UINT32, UINT32,
                             SINT32, SINT32);
void Xin266IDct2WxH(COEFF *, intptr_t, COEFF *, intptr_t, UINT32, UINT32, COEFF *, SINT32, SINT32);
void Xin266ISkipWxH(COEFF *, intptr_t, COEFF *, intptr_t, UINT32, UINT32);
void Xin266QuantInvQuant(COEFF *, COEFF *, COEFF *, intptr_t, UINT32, UINT32, UINT32, UINT32, SINT32, SINT32, SINT32,
                         SINT32, SINT32, SINT32, UINT64 *);
void Xin266PreRdoq(COEFF *, COEFF *, COEFF *, intptr_t, UINT32, UINT32, UINT32, UINT32, SINT32, xin_scan_pos *, UINT64 *);

void shim_fill_table(xin_func_struct *fs)
{
    static const XinFor1dDct f2[7] = { 0, shim_fdct2_2, shim_fdct2_4, shim_fdct2_8, shim_fdct2_16, shim_fdct2_32, shim_fdct2_64 };
    static const XinFor1dDct f8[7] = { 0, 0, shim_fdct8_4, shim_fdct8_8, shim_fdct8_16, shim_fdct8_32, 0 };
    static const XinFor1dDct f7[7] = { 0, 0, shim_fdst7_4, shim_fdst7_8, shim_fdst7_16, shim_fdst7_32, 0 };
    static const XinInv1dDct i2[7] = { 0, Xin26xIDct2P2, Xin26xIDct2P4, Xin26xIDct2P8, Xin26xIDct2P16, Xin26xIDct2P32, Xin26xIDct2P64 };
    static const XinInv1dDct i8[7] = { 0, 0, Xin26xIDct8P4, Xin26xIDct8P8, Xin26xIDct8P16, Xin26xIDct8P32, 0 };
    static const XinInv1dDct i7[7] = { 0, 0, Xin26xIDst7P4, Xin26xIDst7P8, Xin26xIDst7P16, Xin26xIDst7P32, 0 };
    memset(fs, 0, sizeof(*fs));
    for (int lg = 0; lg < XIN_BLOCK_NUM; lg++) {
        fs->pfXinComputeSad[lg] = shim_sad;
        fs->pfXinLumaInterp[0][0][lg] = Xin266InterpCopy;
        fs->pfXinLumaInterp[1][0][lg] = Xin266LumaInterpHor;
        fs->pfXinLumaInterp[0][1][lg] = Xin266LumaInterpVet;
        fs->pfXinLumaInterp[1][1][lg] = Xin266LumaInterpHorVet;
        /* chroma, S16 and bi-average entries as Xin266FuncInit sets them
         * (h266_encoder/source/h266_func_init.c:532-620) */
        fs->pfXinChromaInterp[0][0][lg] = Xin266InterpCopy;
        fs->pfXinChromaInterp[1][0][lg] = Xin266ChromaInterpHor;
        fs->pfXinChromaInterp[0][1][lg] = Xin266ChromaInterpVet;
        fs->pfXinChromaInterp[1][1][lg] = Xin266ChromaInterpHorVet;
        fs->pfXinChromaInterpS16[0][0][lg] = Xin266InterpCopyU8S16;
        fs->pfXinChromaInterpS16[1][0][lg] = Xin266ChromaInterpHorU8S16;
        fs->pfXinChromaInterpS16[0][1][lg] = Xin266ChromaInterpVetU8S16;
        fs->pfXinChromaInterpS16[1][1][lg] = Xin266ChromaInterpHorVetU8S16;
        fs->pfXinInterpAvg[lg] = Xin266InterpAvgS16U8;
        /* DMVR entries (h266_func_init.c:118-125,460-530,645-646) */
        fs->pfXinLumaInterpS16[0][0][lg] = Xin266InterpCopyU8S16;
        fs->pfXinLumaInterpS16[1][0][lg] = Xin266LumaInterpHorU8S16;
        fs->pfXinLumaInterpS16[0][1][lg] = Xin266LumaInterpVetU8S16;
        fs->pfXinLumaInterpS16[1][1][lg] = Xin266LumaInterpHorVetU8S16;
        fs->pfXinBiliInterp[0][0][lg] = Xin266BiliInterpCopy;
        fs->pfXinBiliInterp[1][0][lg] = Xin266BiliInterpHor;
        fs->pfXinBiliInterp[0][1][lg] = Xin266BiliInterpVet;
        fs->pfXinBiliInterp[1][1][lg] = Xin266BiliInterpHorVet;
        fs->pfXinComputeSadS16[lg] = Xin26xComputeSadS16;
        fs->pfXinInterpWeight[lg] = Xin266InterpWeightS16U8;
        fs->pfXinBlockSubForDct[lg] = shim_sub;
        fs->pfXinBlockAddForDct[lg] = shim_add;
        fs->pfXinQuantInvQuant[lg] = Xin266QuantInvQuant;
        fs->pfXinFor2dSkip[lg] = shim_fskip;
        fs->pfXinInv2dSkip[lg] = Xin266ISkipWxH;
        for (int lh = 0; lh < XIN_BLOCK_NUM; lh++) {
            fs->pfXinFor2dDct2[lg][lh] = shim_fdct2_wxh;
            fs->pfXinInv2dDct2[lg][lh] = Xin266IDct2WxH;
        }
        if (lg < 7) {
            fs->pfXinFor1dDct[XIN_DCT2][lg] = f2[lg]; fs->pfXinFor1dDct[XIN_DCT8][lg] = f8[lg]; fs->pfXinFor1dDct[XIN_DST7][lg] = f7[lg];
            fs->pfXinInv1dDct[XIN_DCT2][lg] = i2[lg]; fs->pfXinInv1dDct[XIN_DCT8][lg] = i8[lg]; fs->pfXinInv1dDct[XIN_DST7][lg] = i7[lg];
        }
    }
    fs->pfXinPreRdoq = Xin266PreRdoq;
    fs->pfXinCopyAndPad = Xin266CopyAndPad;
    fs->pfXinCopyAndPadUv = Xin266CopyAndPadUv;
}

/* 8-argument form declared at h266_encoder/include/h266_inter_prediction.h:43 */
void Xin266LumaInterpolation(xin_func_struct *fs, const PIXEL *src, intptr_t ss, PIXEL *dst, intptr_t ds,
                             SINT32 frac, UINT32 lgw, UINT32 h)
{
    SINT32 fx = frac & XIN_MV_FRAC_MASK, fy = (frac >> XIN_MV_FRAC_BITS) & XIN_MV_FRAC_MASK;
    fs->pfXinLumaInterp[!!fx][!!fy][lgw](src, ss, dst, ds, frac, 1u << lgw, h, 0);
}

/* closed DMVR helpers (h26x_core/include/h26x_compute_dist.h:942,
 * h26x_block_utility.h:23,335,343) -> oracle */
void Xin26xComputeSadS16(SINT16 *a, intptr_t as, SINT16 *b, intptr_t bs, UINT32 w, UINT32 h, UINT32 sub, UINT32 *sad)
{ orc_sad_s16(a, as, b, bs, w, h, sub, sad); }
void Xin26xBlockCopy(PIXEL *src, intptr_t ss, PIXEL *dst, intptr_t ds, UINT32 w, UINT32 h) { orc_block_copy(src, ss, dst, ds, w, h); }
void Xin26xBlockPad1(PIXEL *buf, intptr_t bs, UINT32 w, UINT32 h, UINT32 pw, UINT32 ph) { orc_block_pad(buf, bs, w, h, pw, ph); }
void Xin26xBlockPad2(PIXEL *buf, intptr_t bs, UINT32 w, UINT32 h, UINT32 pw, UINT32 ph) { orc_block_pad(buf, bs, w, h, pw, ph); }

/* affine MV rounding (h266_encoder/source/h266_get_neighbour_mv.c:1380), referenced by the
 * affine branch of h266_inter_prediction.c; no harness reaches that branch */
void Xin266RoundAffineMv(SINT32 *mvx, SINT32 *mvy, SINT32 shift) { (void)mvx; (void)mvy; (void)shift; }

/* LMCS chroma residual scaling: never enabled by the harnesses */
void Xin266FwdScaleSignal(COEFF *r, intptr_t s, UINT32 w, UINT32 h, SINT32 scale) { (void)r; (void)s; (void)w; (void)h; (void)scale; }
void Xin266InvScaleSignal(COEFF *r, intptr_t s, UINT32 w, UINT32 h, SINT32 scale) { (void)r; (void)s; (void)w; (void)h; (void)scale; }
