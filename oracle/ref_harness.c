/*
 * ref_harness.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Flat C entry points around the reference's open drivers, which take the
 * encoder's section / sequence / CU structures.  Each harness fills the few
 * fields the function reads (everything else zero) and calls it unmodified:
 *   Xin266FDctWxH       h266_encoder/source/h266_forward_trans.c:45
 *   Xin266IDctWxH       h266_encoder/source/h266_inverse_trans.c:117
 *   Xin266SubFDctWxH    h266_encoder/source/h266_sub_dct.c:47
 *   Xin266IDctAdd       h266_encoder/source/h266_idct_add.c:45
 *   Xin266FullSubPelMe  h266_encoder/source/h266_sub_pel_refine.c:81
 *   Xin266Transform     h266_encoder/source/h266_trans_quant.c:61
 * The quant parameter table of Xin266ConstructQuantParam (static in
 * h266_encoder_create.c:1677) is rebuilt here from the same formula.
 */
#include "xin_typedef.h"
#include "string.h"
#include "basic_macro.h"
#include "h266_constant.h"
#include "xin_video_common.h"
#include "h26x_definition.h"
#include "h266_definition.h"
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
#include "h266_motion_est.h"
#include "h266_forward_trans.h"
#include "h266_inverse_trans.h"
#include "h266_sub_dct.h"
#include "h266_idct_add.h"
#include "h266_trans_recon.h"
#include "h266_inter_pred_context.h"

void shim_fill_table(xin_func_struct *fs);
extern const UINT32 calcLog2[256];
void Xin266Transform(xin_sec_struct *secSet, xin_cu_struct *cu, xin_fast_md_buf *fastBuf, UINT32 mtsIdx, UINT32 planeIdx);

typedef struct harness {
    xin_sec_struct  sec;
    xin_seq_struct  seq;
    xin_pic_struct  pic;
    xin_func_struct fs;
    xin_me_struct   me;
    xin_ref_picture pw;
    COEFF           temp[4 * 128 * 128];
    xin_quant_param qp0[128], qp1[128];
} harness;

static harness *harness_new(int enable_mts)
{
    harness *h = (harness *)calloc(1, sizeof(harness));
    shim_fill_table(&h->fs);
    h->sec.seqSet = &h->seq;
    h->sec.picSet = &h->pic;
    h->sec.funcSet = &h->fs;
    h->sec.meSet = &h->me;
    h->sec.tempBuffer = (UINT8 *)h->temp;
    h->pic.pictureWrite = &h->pw;
    h->seq.config.internalBitDepth = XIN_INTERNAL_BIT_DEPTH;
    h->seq.config.enableMts = enable_mts;
    for (UINT32 qp = 0; qp < 128; qp++) {
        static const UINT32 qm[2][6] = { { 26214, 23302, 20560, 18396, 16384, 14564 }, { 18396, 16384, 14564, 13107, 11651, 10280 } };
        static const UINT32 iqm[2][6] = { { 40, 45, 51, 57, 64, 72 }, { 57, 64, 72, 80, 90, 102 } };
        UINT32 rem = qp % 6, per = qp / 6;
        h->qp0[qp].qMult = (SINT32)qm[0][rem]; h->qp0[qp].iqMult = (SINT32)(iqm[0][rem] << per);
        h->qp1[qp].qMult = (SINT32)qm[1][rem]; h->qp1[qp].iqMult = (SINT32)(iqm[1][rem] << per);
        h->qp0[qp].qShift = h->qp1[qp].qShift = (SINT32)(14 + (15 - XIN_INTERNAL_BIT_DEPTH) + per);
        h->qp0[qp].iqShift = h->qp1[qp].iqShift = 6 - (15 - XIN_INTERNAL_BIT_DEPTH);
    }
    h->seq.quantParam[0] = h->qp0;
    h->seq.quantParam[1] = h->qp1;
    return h;
}

void ref_fdct_wxh(COEFF *in, intptr_t is, COEFF *out, intptr_t os, UINT32 comp, UINT32 w, UINT32 h,
                  UINT32 mts, BOOL is_intra, BOOL enable_mts)
{
    harness *hs = harness_new(enable_mts);
    Xin266FDctWxH(&hs->sec, in, is, out, os, comp, w, h, mts, is_intra);
    free(hs);
}

void ref_idct_wxh(COEFF *in, intptr_t is, COEFF *out, intptr_t os, UINT32 w, UINT32 h,
                  BOOL is_intra, UINT32 comp, UINT32 mts, BOOL enable_mts)
{
    harness *hs = harness_new(enable_mts);
    Xin266IDctWxH(&hs->sec, in, is, out, os, w, h, is_intra, comp, mts);
    free(hs);
}

void ref_sub_fdct_wxh(PIXEL *in, intptr_t is, PIXEL *pred, intptr_t ps, COEFF *out, intptr_t os,
                      UINT32 comp, UINT32 mts, SINT32 w, SINT32 h, BOOL is_intra, BOOL enable_mts)
{
    harness *hs = harness_new(enable_mts);
    Xin266SubFDctWxH(&hs->sec, in, is, pred, ps, out, os, comp, mts, w, h, is_intra);
    free(hs);
}

void ref_idct_add(COEFF *in, intptr_t is, PIXEL *pred, intptr_t ps, PIXEL *out, intptr_t os,
                  BOOL is_intra, UINT32 comp, UINT32 mts, UINT32 w, UINT32 h, BOOL enable_mts)
{
    harness *hs = harness_new(enable_mts);
    Xin266IDctAdd(&hs->sec, in, is, pred, ps, out, os, is_intra, comp, mts, w, h);
    free(hs);
}

/* mv and cost in/out: io[0]=mvx, io[1]=mvy (quarter-pel), io[2]=cost */
void ref_full_subpel_me(PIXEL *in, intptr_t is, PIXEL *ref_at_pu, intptr_t rs, UINT32 w, UINT32 h,
                        SINT32 mvpx, SINT32 mvpy, UINT32 lambda,
                        SINT32 min_mvx, SINT32 min_mvy, SINT32 max_mvx, SINT32 max_mvy, SINT32 *io)
{
    harness *hs = harness_new(0);
    xin_me_struct *me = &hs->me;
    me->input = in; me->inputStride = is; me->ref = ref_at_pu; me->refStride = rs;
    me->width = w; me->height = h; me->sadLambda = lambda;
    me->predMv.mv.mvX = (SINT16)mvpx; me->predMv.mv.mvY = (SINT16)mvpy;
    me->bestMv.mv.mvX = (SINT16)io[0]; me->bestMv.mv.mvY = (SINT16)io[1]; me->bestCost = (UINT32)io[2];
    me->minMv.mv.mvX = (SINT16)min_mvx; me->minMv.mv.mvY = (SINT16)min_mvy;
    me->maxMv.mv.mvX = (SINT16)max_mvx; me->maxMv.mv.mvY = (SINT16)max_mvy;
    Xin266FullSubPelMe(&hs->sec, 0, 0);
    io[0] = me->bestMv.mv.mvX; io[1] = me->bestMv.mv.mvY; io[2] = (SINT32)me->bestCost;
    free(hs);
}

/* One CU with one TU of w x h (TU = CU) at the origin of the given planes.
 * Returns t, q, r with stride cs and the non-zero CG map. */
void ref_transform_tu(PIXEL *in, intptr_t is, PIXEL *pred, intptr_t ps, COEFF *t, COEFF *q, COEFF *r, intptr_t cs,
                      UINT32 w, UINT32 h, UINT32 plane, UINT32 mts, SINT32 qp, BOOL rdoq, UINT32 rdoq_thr,
                      BOOL intra_frame, BOOL is_intra, BOOL enable_mts, xin_scan_pos *scan_cg, UINT64 *nz)
{
    harness *hs = harness_new(enable_mts);
    xin_cu_struct cu; xin_tu_struct tu; xin_fast_md_buf fast; xin_full_md_buf full;
    UINT32 comp = plane != 0, lw = calcLog2[w], lh = calcLog2[h];
    memset(&cu, 0, sizeof cu); memset(&tu, 0, sizeof tu); memset(&fast, 0, sizeof fast); memset(&full, 0, sizeof full);
    hs->seq.config.enableRdoq = rdoq;
    hs->seq.config.rdoqThrVal = rdoq_thr;
    hs->pw.frameType = intra_frame ? XIN_I_FRAME : XIN_P_FRAME;
    hs->sec.qp = qp; hs->sec.uvQp = qp;
    hs->sec.inputYStride = is; hs->sec.inputUvStride = is;
    hs->sec.reshapeCu[plane] = in;
    cu.lgTuWidth[comp] = (UINT8)lw; cu.lgTuHeight[comp] = (UINT8)lh;
    cu.tu[0] = &tu;
    tu.lgWidth[comp] = (UINT8)lw; tu.lgHeight[comp] = (UINT8)lh;
    tu.lgCGWidth[comp] = 2; tu.lgCGHeight[comp] = 2;
    tu.scanOrderCG[comp] = scan_cg;
    fast.fullBuf = &full;
    fast.type = is_intra ? XIN_INTRA_MODE : 0;
    fast.predBuf[plane] = pred;
    fast.lumaStride = ps; fast.chromaStride = ps;
    full.coeffStride[comp] = cs;
    full.tuNum = 1;
    full.tCoefBuf[mts][plane] = t; full.qCoefBuf[mts][plane] = q; full.rCoefBuf[mts][plane] = r;
    Xin266Transform(&hs->sec, &cu, &fast, mts, plane);
    *nz = full.nzCGMapRs[mts][0][plane];
    free(hs);
}

/* ---- dependent quantisation --------------------------------------------
 * Xin266DepQuant (h266_encoder/source/h266_dep_quant.c:1789) on tables built
 * by the reference's own Xin266ContructScanOrder (h266_scan_order.c:83),
 * Xin266CreateDepQuantRom (h266_dep_quant.c:494) and Xin266CreateDepQuant
 * (:323).  For a Cr block the Cb rate tables are built first from the same
 * contexts: the reference reuses the tables of the previous call for Cr
 * (:296-311), and in the encoder that call is the Cb block of the same TU. */
#include "h266_dep_quant_struct.h"
#include "h266_dep_quant.h"
SINT32 Xin266ContructScanOrder(xin_seq_struct *seqSet);
void Xin266PreDepQuant(COEFF *, COEFF *, COEFF *, intptr_t, UINT32, UINT32, UINT32, UINT32, SINT32,
                       xin_scan_pos *, xin_scan_pos *, SINT32 *);

static xin_seq_struct *dq_seq;
static xin_sec_struct *dq_sec;
static xin_func_struct dq_fs;

static void dq_setup(void)
{
    if (dq_seq) return;
    dq_seq = (xin_seq_struct *)calloc(1, sizeof(xin_seq_struct));
    dq_sec = (xin_sec_struct *)calloc(1, sizeof(xin_sec_struct));
    dq_seq->config.enableDepQuant = 1;
    dq_seq->funcSet = &dq_fs;
    dq_fs.pfXinPreDepQuant = Xin266PreDepQuant;
    Xin266ContructScanOrder(dq_seq);
    Xin266CreateDepQuantRom(dq_seq);
    dq_sec->seqSet = dq_seq;
    Xin266CreateDepQuant(dq_sec);
}

void ref_dep_quant(COEFF *t, intptr_t stride, int w, int h, int qp, int comp,
                   xin_prob_model *ctx, int root_cbf, COEFF *q, COEFF *r, UINT64 *nz)
{
    static xin_full_md_buf full;
    static xin_fast_md_buf fast;
    xin_tu_struct tu;
    UINT32 lw = calcLog2[w], lh = calcLog2[h], ct = comp != 0;
    dq_setup();
    xin_dep_quant *dq = dq_sec->depQuant;
    memset(&tu, 0, sizeof tu);
    dq->context = ctx;
    full.tuNum = 1;
    fast.fullBuf = &full;
    fast.type = root_cbf ? 0 : XIN_INTRA_MODE;
    tu.scanOrderCG[ct] = dq_seq->scanOrderCG[lh][lw];
    tu.scanOrder[ct] = dq_seq->scanOrder[2][2];
    if (comp == 2)
        Xin266InitContext(dq, &fast, dq->tuParam[lw][lh][1], ctx, PLANE_CHROMA_U);
    Xin266DepQuant(dq, &fast, &tu, t, r, q, stride, (UINT32)qp, w, h, nz, (UINT32)comp);
}

/* the reference's trellis parameters for lg(w)+lg(h) = lgsum, QP qp (xin_dp_param) */
void ref_dq_param(int qp, int lgsum, xin_dp_param *out)
{
    dq_setup();
    *out = dq_seq->dpParam[lgsum][qp];
}

/* bilinear DMVR prediction (h266_core/source/h266_bilinear_filter.c:46-260) by variant,
 * the way pfXinBiliInterp[!!fx][!!fy] selects it (h266_encoder/source/h266_func_init.c:496-530) */
void Xin266BiliInterpCopy(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void Xin266BiliInterpHor(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void Xin266BiliInterpVet(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void Xin266BiliInterpHorVet(const PIXEL *, intptr_t, SINT16 *, intptr_t, SINT32, UINT32, UINT32);
void ref_bili_interp(int variant, const PIXEL *src, intptr_t ss, SINT16 *dst, intptr_t ds, SINT32 frac, UINT32 w, UINT32 h)
{
    switch (variant) {
    case 0: Xin266BiliInterpCopy(src, ss, dst, ds, frac, w, h); break;
    case 1: Xin266BiliInterpHor(src, ss, dst, ds, frac, w, h); break;
    case 2: Xin266BiliInterpVet(src, ss, dst, ds, frac, w, h); break;
    default: Xin266BiliInterpHorVet(src, ss, dst, ds, frac, w, h); break;
    }
}

/* ---- motion-compensation call sites ------------------------------------
 * Xin266LumaInterPred (h266_encoder/source/h266_inter_prediction.c:302) and
 * Xin266ChromaMotionComp (:612) called unmodified on a picture set whose
 * reference lists hold the given planes: the MV is clipped to the CU's
 * window, split into an integer offset and a phase, and dispatched through
 * the table (chroma: 1/32 phase of the luma 1/16 position).  ref_*: picture
 * origins (inside the padding), luma stride rs, chroma stride crs; mv in
 * 1/16 luma pel; ref_idx1 < 0 selects the uni-prediction branch. */
void Xin266LumaInterPred(xin_sec_struct *, xin_pu_struct *, PIXEL *, intptr_t, xin_mv32_u *, SINT32, SINT32, BOOL);
void Xin266ChromaMotionComp(xin_sec_struct *, SINT32, SINT32, PIXEL *, PIXEL *, intptr_t, xin_mv32_u *, SINT8 *, UINT8);

static harness *mc_harness(SINT32 cu_x, SINT32 cu_y, SINT32 min_mvx, SINT32 min_mvy, SINT32 max_mvx, SINT32 max_mvy,
                           xin_cu_struct *cu)
{
    harness *hs = harness_new(0);
    memset(cu, 0, sizeof *cu);
    cu->cuPelX = (UINT32)cu_x; cu->cuPelY = (UINT32)cu_y;
    hs->sec.cu = cu;
    hs->sec.minMv.mv.mvX = (SINT16)min_mvx; hs->sec.minMv.mv.mvY = (SINT16)min_mvy;
    hs->sec.maxMv.mv.mvX = (SINT16)max_mvx; hs->sec.maxMv.mv.mvY = (SINT16)max_mvy;
    return hs;
}

void ref_luma_inter_pred(PIXEL *ref_origin, intptr_t rs, PIXEL *pred, intptr_t ps, SINT32 mvx16, SINT32 mvy16,
                         SINT32 cu_x, SINT32 cu_y, SINT32 min_mvx, SINT32 min_mvy, SINT32 max_mvx, SINT32 max_mvy,
                         UINT32 w, UINT32 h, BOOL alt_hpel)
{
    xin_cu_struct cu; xin_pu_struct pu; xin_ref_picture rp; xin_mv32_u mv;
    harness *hs = mc_harness(cu_x, cu_y, min_mvx, min_mvy, max_mvx, max_mvy, &cu);
    memset(&pu, 0, sizeof pu); memset(&rp, 0, sizeof rp);
    pu.width = (UINT8)w; pu.height = (UINT8)h; pu.lgWidth = (UINT8)calcLog2[w]; pu.lgHeight = (UINT8)calcLog2[h];
    rp.refBuf[PLANE_LUMA] = ref_origin; rp.refStride[PLANE_LUMA] = rs;
    hs->pic.pictureRead[0][0] = &rp;
    mv.mv.mv32X = mvx16; mv.mv.mv32Y = mvy16;
    Xin266LumaInterPred(&hs->sec, &pu, pred, ps, &mv, 0, 0, alt_hpel);
    free(hs);
}

void ref_chroma_motion_comp(PIXEL *ref_u0, PIXEL *ref_v0, PIXEL *ref_u1, PIXEL *ref_v1, intptr_t crs,
                            PIXEL *pred_u, PIXEL *pred_v, intptr_t ps, const SINT32 *mv16, SINT32 ref_idx0,
                            SINT32 ref_idx1, UINT32 bcw_idx, SINT32 cu_x, SINT32 cu_y, SINT32 min_mvx, SINT32 min_mvy,
                            SINT32 max_mvx, SINT32 max_mvy, UINT32 w, UINT32 h)
{
    xin_cu_struct cu; xin_ref_picture rp0, rp1; xin_mv32_u mv[2]; SINT8 ri[2];
    harness *hs = mc_harness(cu_x, cu_y, min_mvx, min_mvy, max_mvx, max_mvy, &cu);
    memset(&rp0, 0, sizeof rp0); memset(&rp1, 0, sizeof rp1);
    rp0.refBuf[PLANE_CHROMA_U] = ref_u0; rp0.refBuf[PLANE_CHROMA_V] = ref_v0; rp0.refStride[PLANE_CHROMA] = crs;
    rp1.refBuf[PLANE_CHROMA_U] = ref_u1; rp1.refBuf[PLANE_CHROMA_V] = ref_v1; rp1.refStride[PLANE_CHROMA] = crs;
    hs->pic.pictureRead[XIN_LIST_0][0] = &rp0;
    hs->pic.pictureRead[XIN_LIST_1][0] = &rp1;
    mv[0].mv.mv32X = mv16[0]; mv[0].mv.mv32Y = mv16[1]; mv[1].mv.mv32X = mv16[2]; mv[1].mv.mv32Y = mv16[3];
    ri[0] = (SINT8)ref_idx0; ri[1] = (SINT8)ref_idx1;
    Xin266ChromaMotionComp(&hs->sec, (SINT32)w, (SINT32)h, pred_u, pred_v, ps, mv, ri, (UINT8)bcw_idx);
    free(hs);
}

/* Xin266LumaMotionComp (h266_encoder/source/h266_inter_prediction.c:433), called
 * unmodified with both lists set (its bi-prediction branch, default BCW weight) */
void Xin266LumaMotionComp(xin_sec_struct *, SINT32, SINT32, PIXEL *, intptr_t, xin_mv32_u *, SINT8 *, UINT8, UINT32);

void ref_luma_motion_comp(PIXEL *ref0, PIXEL *ref1, intptr_t rs, PIXEL *pred, intptr_t ps, const SINT32 *mv16,
                          SINT32 cu_x, SINT32 cu_y, SINT32 min_mvx, SINT32 min_mvy, SINT32 max_mvx, SINT32 max_mvy,
                          UINT32 w, UINT32 h)
{
    xin_cu_struct cu; xin_ref_picture rp0, rp1; xin_mv32_u mv[2]; SINT8 ri[2] = { 0, 0 };
    harness *hs = mc_harness(cu_x, cu_y, min_mvx, min_mvy, max_mvx, max_mvy, &cu);
    memset(&rp0, 0, sizeof rp0); memset(&rp1, 0, sizeof rp1);
    rp0.refBuf[PLANE_LUMA] = ref0; rp0.refStride[0] = rs;
    rp1.refBuf[PLANE_LUMA] = ref1; rp1.refStride[0] = rs;
    hs->pic.pictureRead[XIN_LIST_0][0] = &rp0;
    hs->pic.pictureRead[XIN_LIST_1][0] = &rp1;
    mv[0].mv.mv32X = mv16[0]; mv[0].mv.mv32Y = mv16[1]; mv[1].mv.mv32X = mv16[2]; mv[1].mv.mv32Y = mv16[3];
    Xin266LumaMotionComp(&hs->sec, (SINT32)w, (SINT32)h, pred, ps, mv, ri, XIN_BCW_DEFAULT, 0);
    free(hs);
}

/* ---- DMVR ----------------------------------------------------------------
 * Xin266LumaMotionCompDmvr (h266_encoder/source/h266_inter_prediction.c:1178),
 * which runs Xin266DeriveMvFromDmvr (:975), called unmodified on a picture set
 * whose lists hold ref0 / ref1 (picture origins, stride rs); writes the
 * sub-block refinements (x, y pairs, 1/16 pel) and the refined prediction. */
void Xin266LumaMotionCompDmvr(xin_sec_struct *, xin_pu_struct *, PIXEL *, intptr_t, xin_mv32_u *, SINT8 *, xin_mv_s *, BOOL);
void Xin266CopyAndPad(PIXEL *, intptr_t, PIXEL *, intptr_t, UINT32, UINT32);
void Xin266CopyAndPadUv(PIXEL *, PIXEL *, intptr_t, PIXEL *, PIXEL *, intptr_t, UINT32, UINT32);

void ref_dmvr_luma(PIXEL *ref0, PIXEL *ref1, intptr_t rs, SINT32 cu_x, SINT32 cu_y, SINT32 min_mvx, SINT32 min_mvy,
                   SINT32 max_mvx, SINT32 max_mvy, UINT32 w, UINT32 h, const SINT32 *mv16, BOOL alt_hpel, SINT16 *mvd,
                   PIXEL *pred, intptr_t ps)
{
    xin_cu_struct cu; xin_pu_struct pu; xin_ref_picture rp0, rp1; xin_mv32_u mv[2]; SINT8 ri[2] = { 0, 0 };
    xin_mv_s sub[64];
    harness *hs = mc_harness(cu_x, cu_y, min_mvx, min_mvy, max_mvx, max_mvy, &cu);
    /* the derivation's two bilinear buffers of BILI_BUF_STRIDE^2 samples */
    SINT16 *tmp = (SINT16 *)calloc(2 * BILI_BUF_STRIDE * BILI_BUF_STRIDE, sizeof(SINT16));
    hs->sec.tempBuffer = (UINT8 *)tmp;
    memset(&pu, 0, sizeof pu); memset(&rp0, 0, sizeof rp0); memset(&rp1, 0, sizeof rp1);
    pu.width = (UINT8)w; pu.height = (UINT8)h; pu.lgWidth = (UINT8)calcLog2[w]; pu.lgHeight = (UINT8)calcLog2[h];
    rp0.refBuf[PLANE_LUMA] = ref0; rp0.refStride[PLANE_LUMA] = rs;
    rp1.refBuf[PLANE_LUMA] = ref1; rp1.refStride[PLANE_LUMA] = rs;
    hs->pic.pictureRead[XIN_LIST_0][0] = &rp0;
    hs->pic.pictureRead[XIN_LIST_1][0] = &rp1;
    mv[0].mv.mv32X = mv16[0]; mv[0].mv.mv32Y = mv16[1]; mv[1].mv.mv32X = mv16[2]; mv[1].mv.mv32Y = mv16[3];
    Xin266LumaMotionCompDmvr(&hs->sec, &pu, pred, ps, mv, ri, sub, alt_hpel);
    UINT32 n = ((w + 15) / 16) * ((h + 15) / 16);
    for (UINT32 i = 0; i < n; i++) { mvd[2 * i] = sub[i].mvX; mvd[2 * i + 1] = sub[i].mvY; }
    free(tmp);
    free(hs);
}

void ref_copy_and_pad(PIXEL *ref, intptr_t rs, PIXEL *pad, intptr_t ps, UINT32 w, UINT32 h)
{
    Xin266CopyAndPad(ref, rs, pad, ps, w, h);
}

void ref_copy_and_pad_uv(PIXEL *ref_u, PIXEL *ref_v, intptr_t rs, PIXEL *pad_u, PIXEL *pad_v, intptr_t ps, UINT32 w, UINT32 h)
{
    Xin266CopyAndPadUv(ref_u, ref_v, rs, pad_u, pad_v, ps, w, h);
}

/* ---- fast sub-pel search by variance -----------------------------------
 * Xin266FastSubPelMeVar (h266_encoder/source/h266_sub_pel_refine.c:214) called
 * unmodified on an ME state whose interpolation buffers are laid out as
 * Xin266ConstructMe sets them (h266_encoder/source/h266_create_section.c:45-230,
 * a static function): four XIN_ME_BUF_STRIDE^2 planes, the half-pel pointers
 * and the quarter-pel pointer pairs.  The pairs are generated from
 * orc_qpel_pair; tests/test_oracle_vs_ref.py checks that rule against the
 * assignments in h266_create_section.c read as text.  Variance and the
 * half-pel planes go to the oracle (closed in the reference). */
static void shim_var(PIXEL *in, intptr_t is, PIXEL *p, intptr_t ps, UINT32 w, UINT32 h, UINT32 *v)
{ orc_var(in, is, p, ps, w, h, v); }
static void shim_avg_var(PIXEL *in, intptr_t is, PIXEL *a, PIXEL *b, intptr_t ps, UINT32 w, UINT32 h, UINT32 *v)
{ orc_avg_var(in, is, a, b, ps, w, h, v); }
static void shim_half_pel(PIXEL *ref, intptr_t rs, UINT32 w, UINT32 h, PIXEL *ip, PIXEL *hp, PIXEL *vp, PIXEL *hvp,
                          intptr_t stride, BOOL alt)
{ orc_interpo_half_pel(ref, rs, w, h, ip, hp, vp, hvp, stride, alt); }

/* pointer of half-grid point (px, py) in the planes (origins as Xin266ConstructMe) */
static PIXEL *fsme_grid(PIXEL *integ, PIXEL *hb, PIXEL *vb, PIXEL *hvb, int px, int py)
{
    const intptr_t S = XIN_ME_BUF_STRIDE;
    if (!(px & 1) && !(py & 1)) return integ + S + 1 + (py / 2) * S + px / 2;
    if (!(py & 1)) return hb + 2 * S + (py / 2) * S + (px + 1) / 2;
    if (!(px & 1)) return vb + 1 + ((py + 1) / 2) * S + px / 2;
    return hvb + ((py + 1) / 2) * S + (px + 1) / 2;
}


void ref_fast_subpel_me_var(PIXEL *in, intptr_t is, PIXEL *ref_at_pu, intptr_t rs, UINT32 w, UINT32 h, SINT32 mvpx,
                            SINT32 mvpy, UINT64 lambda, SINT32 imv, SINT32 min_mvx, SINT32 min_mvy, SINT32 max_mvx,
                            SINT32 max_mvy, SINT32 *io)
{
    static const int off[9][2] = { { -1, 0 }, { 1, 0 }, { 0, -1 }, { 0, 1 }, { -1, -1 }, { 1, -1 }, { -1, 1 }, { 1, 1 }, { 0, 0 } };
    xin_me_struct *me = (xin_me_struct *)calloc(1, sizeof(xin_me_struct));
    PIXEL *buf = (PIXEL *)calloc(4 * XIN_ME_BUF_STRIDE * XIN_ME_BUF_STRIDE, sizeof(PIXEL));
    PIXEL *integ = buf, *hb = buf + XIN_ME_BUF_STRIDE * XIN_ME_BUF_STRIDE;
    PIXEL *vb = hb + XIN_ME_BUF_STRIDE * XIN_ME_BUF_STRIDE, *hvb = vb + XIN_ME_BUF_STRIDE * XIN_ME_BUF_STRIDE;
    for (int lg = 0; lg < XIN_ME_SIZE_NUM; lg++) {
        me->funcSet.pfXinComputeVar[lg] = shim_var;
        me->funcSet.pfXinComputeAvgVar[lg] = shim_avg_var;
    }
    me->funcSet.pfXinInterpoHalfPel = shim_half_pel;
    me->interpBuf = buf; me->integPel = integ; me->halfPelH = hb; me->halfPelV = vb; me->halfPelHv = hvb;
    me->interpStride = XIN_ME_BUF_STRIDE;
    for (int p = 0; p < POS_NUM; p++) me->halfPel[p] = fsme_grid(integ, hb, vb, hvb, off[p][0], off[p][1]);
    for (int hpos = 0; hpos <= POS_NUM; hpos++)
        for (int q = 0; q < POS_NUM; q++) {
            int32_t pr[4];
            orc_qpel_pair(off[hpos][0], off[hpos][1], off[q][0], off[q][1], pr);
            me->qBufA[hpos][q] = fsme_grid(integ, hb, vb, hvb, pr[0], pr[1]);
            me->qBufB[hpos][q] = fsme_grid(integ, hb, vb, hvb, pr[2], pr[3]);
        }
    me->input = in; me->inputStride = is; me->ref = ref_at_pu; me->refStride = rs;
    me->width = w; me->height = h; me->sseLambda = lambda; me->iMvMode = imv;
    me->predMv.mv.mvX = (SINT16)mvpx; me->predMv.mv.mvY = (SINT16)mvpy;
    me->bestMv.mv.mvX = (SINT16)io[0]; me->bestMv.mv.mvY = (SINT16)io[1];
    me->bestPos = 77;
    me->minMv.mv.mvX = (SINT16)min_mvx; me->minMv.mv.mvY = (SINT16)min_mvy;
    me->maxMv.mv.mvX = (SINT16)max_mvx; me->maxMv.mv.mvY = (SINT16)max_mvy;
    Xin266FastSubPelMeVar(me, 0, 0);
    io[0] = me->bestMv.mv.mvX; io[1] = me->bestMv.mv.mvY; io[2] = (SINT32)me->bestPos;
    free(buf);
    free(me);
}
