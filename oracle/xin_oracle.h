/*
 * xin_oracle.h -- CPU oracle for the xin26x VVC encoder pixel hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * hot-path arithmetic, used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py as the checker.  Nothing in the
 * product (xin26x_gb300/, libxingpu.so) links, loads or calls it.
 *
 * Build: compiled twice, once per bit depth, like the reference's compile-time
 * switch ENABLE_10BIT_ENCODER (video_api/video_common/include/xin_typedef.h:72-96):
 *   -DORC_BITDEPTH=8  -> opix = uint8_t,  ocoef = int16_t  (liboracle8.so)
 *   -DORC_BITDEPTH=10 -> opix = uint16_t, ocoef = int32_t  (liboracle10.so)
 *
 * Parity status per function is stated in its comment:
 *   "pinned (open C)"  -- the reference implementation is open C; the oracle
 *                         restates it and tests/test_oracle_vs_ref.py checks it
 *                         against that C compiled in place (oracle/_ref) and
 *                         against the committed golden fixtures.
 *   "pinned (H.266)"   -- normative arithmetic of the H.266 standard.
 *   "unpinned"         -- the reference ships only a closed binary for it;
 *                         restated from the signature, the open call sites and
 *                         a published method that is named in the comment.
 */
#ifndef XIN_ORACLE_H
#define XIN_ORACLE_H

#include <stdint.h>

#ifndef ORC_BITDEPTH
#define ORC_BITDEPTH 8
#endif

#if ORC_BITDEPTH == 10
typedef uint16_t opix;
typedef int32_t  ocoef;
#else
typedef uint8_t  opix;
typedef int16_t  ocoef;
#endif

#define ORC_MAX_PIX ((1 << ORC_BITDEPTH) - 1)

#ifdef __cplusplus
extern "C" {
#endif

/* scan position triple, same layout as xin_scan_pos
 * (h266_encoder/include/h266_trans_unit_struct.h:23-28) */
typedef struct orc_scan_pos { uint32_t posX, posY, posIdx; } orc_scan_pos;

int  orc_bitdepth(void);

/* ---- distortion (closed in the reference: h26x_core/include/h26x_compute_dist.h) */
void orc_sad(const opix *in, intptr_t is, const opix *ref, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad);
void orc_sad_xn(const opix *in, intptr_t is, const opix *const *ref, int n, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad);
void orc_avg_sad(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad);
void orc_avg_sad_xn(const opix *in, intptr_t is, const opix *const *a, const opix *const *b, int n, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad);
void orc_satd(const opix *in, intptr_t is, const opix *ref, intptr_t rs, uint32_t w, uint32_t h, uint32_t *satd);
void orc_avg_satd(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *satd);
void orc_weight_sad(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, int32_t wa, int32_t wb, uint32_t *sad);
void orc_weight_satd(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, int32_t wa, int32_t wb, uint32_t *satd);
void orc_hada8x8(const opix *in, intptr_t is, uint32_t *satd);
void orc_var(const opix *in, intptr_t is, const opix *ref, intptr_t rs, uint32_t w, uint32_t h, uint32_t *var);
void orc_avg_var(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *var);

/* ---- interpolation (open in the reference: h266_core/source/h266_luma_mc.c, h266_chroma_mc.c) */
void orc_interp_copy(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_interp_copy_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_hor(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_vet(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_hv(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_hor_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_vet_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_hv_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_vet_s16_pix(const int16_t *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_luma_vet_s16_s16(const int16_t *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_hor(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_vet(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_hv(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_hor_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_vet_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_hv_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_vet_s16_pix(const int16_t *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_vet_s16_s16(const int16_t *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi);
void orc_interp_avg(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, opix *dst, intptr_t ds, uint32_t w, uint32_t h);
void orc_interp_weight(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, opix *dst, intptr_t ds, uint32_t w, uint32_t h, int32_t wa, int32_t wb);
/* bilinear DMVR prediction (h266_core/source/h266_bilinear_filter.c:46-260); pinned (open C) */
void orc_bili_interp(int variant, const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h);

/* call-site dispatch (h266_encoder/source/h266_inter_prediction.c) */
void orc_luma_interpolation(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t lgw, uint32_t h, uint32_t fi);
void orc_chroma_interpolation(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t lgw, uint32_t h);
void orc_luma_inter_pred(const opix *ref_origin, intptr_t rs, opix *pred, intptr_t ps, int32_t mvx16, int32_t mvy16,
                         int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                         uint32_t w, uint32_t h, uint32_t fi);
void orc_chroma_motion_comp(const opix *ref_origin, intptr_t rs, opix *pred, intptr_t ps, int32_t mvx16, int32_t mvy16,
                            int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                            uint32_t w, uint32_t h);
/* bi-prediction branches of Xin266LumaMotionComp / Xin266ChromaMotionComp: mv16 = L0 (x, y), L1 (x, y) in 1/16 pel */
void orc_luma_motion_comp_bi(const opix *ref0, const opix *ref1, intptr_t rs, opix *pred, intptr_t ps, const int32_t *mv16,
                             int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                             uint32_t w, uint32_t h);
void orc_chroma_motion_comp_bi(const opix *ref0, const opix *ref1, intptr_t rs, opix *pred, intptr_t ps, const int32_t *mv16,
                               int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                               uint32_t w, uint32_t h);
/* target of the bi refinement: clip(2 in - pred) */
void orc_bi_me_input(const opix *in, intptr_t is, const opix *pred, intptr_t ps, opix *out, intptr_t os, uint32_t w, uint32_t h);

/* ---- transforms (1-D closed, 2-D wrappers open) */
const int16_t *orc_tr_matrix(int type, int n);   /* [n][n] row = basis function k */
void orc_fdct1d(int type, int lg, const ocoef *in, intptr_t is, ocoef *out, intptr_t os, int32_t line, int32_t shift);
void orc_idct1d(int type, int lg, const ocoef *in, intptr_t is, ocoef *out, intptr_t os, int32_t line, int32_t skip_line, int32_t shift);
void orc_fdct2_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h, int32_t s1, int32_t s2);
void orc_idct2_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h, int32_t s1, int32_t s2);
void orc_fskip_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h);
void orc_iskip_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h);
void orc_fdct_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t comp, uint32_t w, uint32_t h,
                  uint32_t mts, int is_intra, int enable_mts);
void orc_idct_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h,
                  int is_intra, uint32_t comp, uint32_t mts, int enable_mts);
void orc_block_sub(const opix *in, intptr_t is, const opix *pred, intptr_t ps, ocoef *diff, intptr_t ds, uint32_t w, uint32_t h);
void orc_block_add(const ocoef *res, intptr_t rs, const opix *pred, intptr_t ps, opix *rec, intptr_t os, uint32_t w, uint32_t h);
void orc_sub_fdct_wxh(const opix *in, intptr_t is, const opix *pred, intptr_t ps, ocoef *out, intptr_t os,
                      uint32_t comp, uint32_t mts, int32_t w, int32_t h, int is_intra, int enable_mts);
void orc_idct_add(const ocoef *in, intptr_t is, const opix *pred, intptr_t ps, opix *out, intptr_t os,
                  int is_intra, uint32_t comp, uint32_t mts, uint32_t w, uint32_t h, int enable_mts);

/* ---- quant (open: h266_encoder/source/h266_quant_inv_quant.c, h266_trans_quant.c) */
void orc_quant_inv_quant(ocoef *q, const ocoef *t, ocoef *r, intptr_t stride, uint32_t w, uint32_t h,
                         uint32_t cgw, uint32_t cgh, int32_t qmult, int32_t qadd, int32_t qshift,
                         int32_t iqmult, int32_t iqadd, int32_t iqshift, uint64_t *nz);
void orc_pre_rdoq(const ocoef *t, ocoef *r, ocoef *q, intptr_t stride, uint32_t w, uint32_t h,
                  uint32_t cgw, uint32_t cgh, int32_t thr, const orc_scan_pos *scan_cg, uint64_t *nz);
typedef struct orc_qparams { int32_t qmult, qadd, qshift, iqmult, iqadd, iqshift; } orc_qparams;
void orc_quant_params(int32_t qp, uint32_t lgw, uint32_t lgh, uint32_t mts, int rdoq, int intra_frame, orc_qparams *p);
void orc_transform_tu(const opix *in, intptr_t is, const opix *pred, intptr_t ps,
                      ocoef *t, ocoef *q, ocoef *r, intptr_t cs, uint32_t w, uint32_t h, uint32_t comp,
                      uint32_t mts, int32_t qp, int rdoq, int intra_frame, int is_intra, int enable_mts, uint64_t *nz);

/* one residual block through forward transform (MTS type), zero-out, quant /
 * dequant (4x4 CGs) and inverse transform: the TU arithmetic of Xin266Transform
 * (h266_trans_quant.c:131-220) followed by Xin266IDctWxH, on a residual input */
void orc_tq_block(const ocoef *res, intptr_t rs, uint32_t w, uint32_t h, uint32_t comp, uint32_t mts, int32_t qp,
                  int rdoq, int intra_frame, int is_intra, int enable_mts,
                  ocoef *q, ocoef *r, ocoef *res_out, intptr_t os, uint64_t *nz);

/* ---- motion estimation */
uint32_t orc_mvd_bits(int32_t v);
void orc_exp_golomb_table(uint32_t *tab32767);
typedef struct orc_me_io {
    int32_t  best_mvx, best_mvy;      /* quarter-pel, in/out */
    uint32_t best_cost;               /* in/out */
    uint32_t best_sad;                /* out (integer search only) */
} orc_me_io;
void orc_mv_window(int32_t frame_w, int32_t frame_h, int32_t ctu, int32_t cu_x, int32_t cu_y, int32_t cu_w, int32_t cu_h,
                   int32_t *min_mvx, int32_t *min_mvy, int32_t *max_mvx, int32_t *max_mvy);
void orc_me_full(const opix *in, intptr_t is, const opix *ref_at_pu, intptr_t rs, uint32_t w, uint32_t h,
                 int32_t mvpx, int32_t mvpy, int32_t range, uint32_t lambda,
                 int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy, orc_me_io *io);
void orc_full_subpel_me(const opix *in, intptr_t is, const opix *ref_at_pu, intptr_t rs, uint32_t w, uint32_t h,
                        int32_t mvpx, int32_t mvpy, uint32_t lambda,
                        int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy, orc_me_io *io);

/* ---- hierarchical integer search (restated; the reference's is closed) */
void orc_downscale2x2(const opix *in, intptr_t is, int row_above, int row_below, opix *out, intptr_t os,
                      uint32_t ow, uint32_t oh);
void orc_hier_search(const opix *in, intptr_t is, const opix *ref, intptr_t rs, int32_t min_x, int32_t max_x,
                     int32_t min_y, int32_t max_y, uint32_t w, uint32_t h, int32_t *best_x, int32_t *best_y);
typedef struct orc_hier_in {
    const opix *in[3];  intptr_t in_stride[3];    /* current block at full, 1/2 and 1/4 resolution */
    const opix *ref[3]; intptr_t ref_stride[3];   /* reference at the block's position, same levels */
    const int32_t *cand; uint32_t ncand;           /* quarter-pel candidate MVs (x, y pairs) */
} orc_hier_in;
void orc_me_hier(const orc_hier_in *hi, uint32_t w, uint32_t h, int32_t mvpx, int32_t mvpy, int32_t range_x,
                 int32_t range_y, uint32_t lambda, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                 orc_me_io *io);

/* ---- fast sub-pel search by variance (a9) ------------------------------- */
void orc_half_grid_block(const opix *ref, intptr_t rs, int32_t px, int32_t py, uint32_t w, uint32_t h, uint32_t fi,
                         opix *out, intptr_t os);
void orc_qpel_pair(int32_t hx, int32_t hy, int32_t qx, int32_t qy, int32_t p[4]);
void orc_interpo_half_pel(const opix *ref, intptr_t rs, uint32_t w, uint32_t h, opix *integ, opix *hb, opix *vb, opix *hvb,
                          intptr_t stride, int alt);
/* io in: mvx, mvy (quarter-pel, integer positions); out: mvx, mvy, best_pos.
 * lambda: the ME state's sseLambda; imv: its iMvMode (0 or 3 = half-pel AMVR) */
void orc_fast_subpel_me_var(const opix *in, intptr_t is, const opix *ref_at_pu, intptr_t rs, uint32_t w, uint32_t h,
                            int32_t mvpx, int32_t mvpy, uint64_t lambda, int32_t imv, int32_t min_mvx, int32_t min_mvy,
                            int32_t max_mvx, int32_t max_mvy, int32_t *io);

/* ---- DMVR: the encoder's emulation of decoder-side MV refinement --------- */
void orc_sad_s16(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, uint32_t w, uint32_t h, uint32_t sub,
                 uint32_t *sad);
void orc_block_copy(const opix *src, intptr_t ss, opix *dst, intptr_t ds, uint32_t w, uint32_t h);
void orc_block_pad(opix *buf, intptr_t bs, uint32_t w, uint32_t h, uint32_t pw, uint32_t ph);
void orc_copy_and_pad(const opix *ref, intptr_t rs, opix *pad, intptr_t ps, uint32_t w, uint32_t h);
void orc_copy_and_pad_uv(const opix *ref_u, const opix *ref_v, intptr_t rs, opix *pad_u, opix *pad_v, intptr_t ps,
                         uint32_t w, uint32_t h);
/* one bi-predicted CU: ref0 / ref1 picture origins (stride rs), CU at (cu_x, cu_y),
 * window [min, max] (full-pel), mv16 = L0 x, y, L1 x, y (1/16 pel); writes the
 * per-16x16 sub-block L0 refinements mvd[2 * n] (1/16 pel; L1 gets the negation)
 * and the refined bi-prediction pred (w x h) */
void orc_dmvr_luma(const opix *ref0, const opix *ref1, intptr_t rs, int32_t cu_x, int32_t cu_y, int32_t min_mvx,
                   int32_t min_mvy, int32_t max_mvx, int32_t max_mvy, uint32_t w, uint32_t h, const int32_t mv16[4],
                   int alt_hpel, int16_t *mvd, opix *pred, intptr_t ps);

/* ---- frame hot path: one CU through ME + MC + TQ + recon (the batched GPU frame stage's checker) */
typedef struct orc_frame_desc {
    int32_t width, height, ctu;            /* luma size, CTU size (padding = ctu + 16) */
    const opix *in[3];  intptr_t in_stride[2];    /* current picture planes, [0]=Y stride, [1]=UV stride */
    const opix *ref[3]; intptr_t ref_stride[2];   /* padded reference planes, pointers at picture (0,0) */
    int32_t search_range;
    uint32_t sad_lambda;
    int32_t qp, uv_qp;
    int32_t intra_frame;                   /* 0 for P/B: qAdd = 85 << (qShift - 9) */
    int32_t search_mode;                   /* 0 exhaustive, 1 by resolution levels (orc_me_hier) */
    const opix *in_lo[2];  intptr_t in_lo_stride[2];    /* search_mode 1: luma at 1/2 and 1/4 resolution, */
    const opix *ref_lo[2]; intptr_t ref_lo_stride[2];   /* pointers at picture (0,0) */
    int32_t tu_mode;                       /* 0 DCT2 + quant; 1 the preset-4 TU: MTS candidates with
                                              dependent quantisation (see orc_cu_hotpath) */
    const struct orc_prob *ctx;            /* tu_mode 1: the CABAC context set (ORC_NUM_CTX records) */
    int32_t refs;                          /* 2: a second reference (list 1) and the bi search */
    const opix *ref1[3];                   /* list 1's padded planes (strides as ref) */
    const opix *ref1_lo[2];                /* search_mode 1: list 1's luma at 1/2 and 1/4 resolution */
} orc_frame_desc;
typedef struct orc_cu_out {
    int32_t mvx, mvy;                      /* quarter-pel */
    uint32_t cost;                         /* after sub-pel */
    uint32_t int_cost;                     /* after integer search */
    uint64_t nz[3];
    uint64_t ssd[3];                       /* recon vs input per plane */
    /* tu_mode 1 */
    uint32_t satd_cost;                    /* (SATD << 8) + MV bits * lambda of the final luma prediction */
    uint32_t ncand;                        /* luma transform candidates: 1 (64x64) or 5 */
    uint64_t nz_mts[5];                    /* luma per candidate: DCT2, then MTS index 2..5 */
    uint64_t ssd_mts[5];
    /* refs 2: list 1's uni search, the bi pair and the choice */
    int32_t mvx1, mvy1;
    uint32_t cost1, int_cost1;
    int32_t bmv[4];                        /* L0 (x, y), L1 (x, y), quarter-pel */
    uint32_t bi_cost;
    uint32_t inter_dir;                    /* 1 list 0, 2 list 1, 3 bi */
} orc_cu_out;
void orc_cu_hotpath(const orc_frame_desc *f, int32_t cu_x, int32_t cu_y, int32_t size,
                    ocoef *q[3], intptr_t q_stride[2], opix *rec[3], intptr_t rec_stride[2], orc_cu_out *out);

/* ---- dependent quantisation (oracle_dq.c; pinned (open C)) -------------- */
/* context-state record, the reference's xin_prob_model
 * (h266_encoder/include/h266_cabac_struct.h:225-229): 6 bytes */
typedef struct orc_prob { uint16_t state[2]; uint8_t rate; } orc_prob;
#define ORC_NUM_CTX 401                    /* XIN_NUM_OF_CTX */
/* trellis quantiser parameters, the fields of xin_dp_param
 * (h266_encoder/include/h266_seq_struct.h:118-134) that it uses */
typedef struct orc_dq_param {
    int32_t qShift, qAdd, qScale, maxQIdx, thresLast, iqShift, iqScale, distShift, distAdd;
    int64_t distStepAdd, distOrgFact;
} orc_dq_param;
void    orc_dq_frac_bits(int s, uint32_t out[2]);
int     orc_dq_last_group(int pos);
int32_t orc_dq_rice_bits(int k, int n);
void    orc_dq_params(int qp, int lgsum, orc_dq_param *p);
/* Xin266DepQuant (h266_encoder/source/h266_dep_quant.c:1789): t, q, r share
 * the stride; q and r are written over min(w,32) x min(h,32).  root_cbf: the
 * block is the luma of an inter CU with one TU (the last-position rate then
 * carries the root cbf flag). */
void orc_dep_quant(const ocoef *t, intptr_t stride, int w, int h, int qp, int comp,
                   const orc_prob *ctx, int root_cbf, ocoef *q, ocoef *r, uint64_t *nz);

#ifdef __cplusplus
}
#endif
#endif
