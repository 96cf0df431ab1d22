/*
 * oracle_dq.c -- CPU oracle for dependent quantisation.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates the reference's open trellis quantiser
 *   Xin266DepQuant          h266_encoder/source/h266_dep_quant.c:1789-1992
 * with its helpers (rate tables :116-321, scan/neighbour tables :494-772,
 * quantiser parameters :774-857, pre-quantisation :920-952, candidate costs
 * :954-1100, decision :1117-1222, state updates :1224-1599, last-position
 * search :1683-1770).  Parity: pinned (open C): tests/test_oracle_vs_ref.py runs
 * this against h266_dep_quant.c compiled in place, and tests/golden holds vectors
 * made by that build.
 *
 * Data flow (as in the reference): coefficients are visited in reverse diagonal
 * scan from the last position whose |t| exceeds the last-position threshold.
 * Four quantiser states each keep the best path ending in them; per position a
 * decision records, per target state, the level chosen and the state it came
 * from; a backward walk over the decisions yields the levels, and a forward
 * dequantisation with the state machine yields the reconstructed coefficients.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "xin_oracle.h"

/* context indices in the reference's context array
 * (h266_encoder/include/h266_cabac_struct.h:130-213) */
enum {
    DQC_ROOT_CBF = 76, DQC_CBF_Y = 77, DQC_CBF_U = 81, DQC_CBF_V = 83,
    DQC_SIGGRP_L = 86, DQC_SIGGRP_C = 88, DQC_SIG_L = 90, DQC_SIG_C = 126,
    DQC_PAR_L = 150, DQC_PAR_C = 171, DQC_GT2_L = 182, DQC_GT1_L = 214,
    DQC_LASTX_L = 246, DQC_LASTX_C = 266, DQC_LASTY_L = 269, DQC_LASTY_C = 289
};

#define DQ_COST_INF   ((int64_t)((((uint64_t)1 << 63) - 1) >> 1))   /* h266_dep_quant_struct.h:27 */
#define DQ_REG_BINS   28                                            /* bins per 16 coefficients */

/* ---- rate model ---------------------------------------------------------- */

/* estimated bits (1/32768 units) of a bin coded with the probability state
 * s = (p0 + p1) >> 8: the bin is 1 with probability (s + 0.5) / 256.  Equals
 * the table cabacbinFracBits (h266_encoder/source/h266_entropy_write.c:52). */
void orc_dq_frac_bits(int s, uint32_t out[2])
{
    double p1 = (s + 0.5) / 256.0;
    out[0] = (uint32_t)floor(-log2(1.0 - p1) * 32768.0 + 0.5);
    out[1] = (uint32_t)floor(-log2(p1) * 32768.0 + 0.5);
}

/* group index of a last-position coordinate (H.266 7.4.11.11 binarisation):
 * equals lastSigXYGroupIdx (h266_entropy_write.c:145) */
int orc_dq_last_group(int pos)
{
    if (pos < 4) return pos;
    int l = 31 - __builtin_clz((unsigned)pos);
    return 2 * l + ((pos >> (l - 1)) & 1);
}

/* bits (x 32768) of abs_remainder value n with Rice parameter k: unary prefix
 * (n >> k) + 1 and k suffix bits below 6 prefix ones, else 6 ones followed by an
 * Exp-Golomb code of order k + 1 of n - (6 << k).  Equals goRiceBits
 * (h266_dep_quant.c:81-87) for k 0..3, n 0..31. */
int32_t orc_dq_rice_bits(int k, int n)
{
    int p = n >> k;
    if (p < 6) return (p + 1 + k) << 15;
    unsigned m = (unsigned)(n - (6 << k));
    int e = 31 - __builtin_clz((m >> (k + 1)) + 1);
    return (6 + 2 * e + 1 + (k + 1)) << 15;
}

/* Rice parameter from the local sum of absolute levels (H.266 Table 128),
 * auiGoRiceParsCoeff (h266_dep_quant.c:89-92) */
static int dq_rice_par(int sum)
{
    return sum < 7 ? 0 : sum < 14 ? 1 : sum < 28 ? 2 : 3;
}

typedef struct dq_rates {
    uint32_t sbb[2][2];
    uint32_t sig[3][12][2];
    uint32_t gtx[21][6];
    int32_t  lastx[32], lasty[32];
} dq_rates;

static void dq_bits_of(const orc_prob *ctx, int i, uint32_t out[2])
{
    orc_dq_frac_bits((ctx[i].state[0] + ctx[i].state[1]) >> 8, out);
}

/* Xin266InitContext (h266_dep_quant.c:285-321) and the four table builders
 * above it.  Chroma reads its greater-than-1 / greater-than-2 rates from the
 * luma contexts, as the reference does (:172-173). */
static void dq_build_rates(dq_rates *rt, const orc_prob *ctx, int comp, int w, int h, int root_cbf)
{
    int ch = comp != 0;
    uint32_t b[2], par[2], g1[2], g2[2];
    for (int i = 0; i < 2; i++) {
        dq_bits_of(ctx, (ch ? DQC_SIGGRP_C : DQC_SIGGRP_L) + i, b);
        rt->sbb[i][0] = b[0]; rt->sbb[i][1] = b[1];
    }
    int nsig = ch ? 8 : 12;
    for (int set = 0; set < 3; set++)
        for (int i = 0; i < nsig; i++) {
            dq_bits_of(ctx, (ch ? DQC_SIG_C : DQC_SIG_L) + set * nsig + i, b);
            rt->sig[set][i][0] = b[0]; rt->sig[set][i][1] = b[1];
        }
    int ngtx = ch ? 11 : 21;
    for (int i = 0; i < ngtx; i++) {
        dq_bits_of(ctx, (ch ? DQC_PAR_C : DQC_PAR_L) + i, par);
        dq_bits_of(ctx, DQC_GT1_L + i, g1);
        dq_bits_of(ctx, DQC_GT2_L + i, g2);
        uint32_t p0 = 32768 + par[0], p1 = 32768 + par[1];
        rt->gtx[i][0] = 0;
        rt->gtx[i][1] = g1[0] + 32768;
        rt->gtx[i][2] = g1[1] + p0 + g2[0];
        rt->gtx[i][3] = g1[1] + p1 + g2[0];
        rt->gtx[i][4] = g1[1] + p0 + g2[1];
        rt->gtx[i][5] = g1[1] + p1 + g2[1];
    }
    /* the cbf rate difference rides on the last-y cost */
    int cbf_ctx = (comp == 0 && root_cbf) ? DQC_ROOT_CBF : comp == 0 ? DQC_CBF_Y : comp == 1 ? DQC_CBF_U : DQC_CBF_V;
    dq_bits_of(ctx, cbf_ctx, b);
    int32_t cbf_delta = (int32_t)(b[1] - b[0]);
    static const int prefix_ctx[8] = { 0, 0, 0, 3, 6, 10, 15, 21 };
    for (int xy = 0; xy < 2; xy++) {
        int size = xy ? h : w;
        int lg = 31 - __builtin_clz((unsigned)size);
        int shift = comp == 0 ? (lg + 1) >> 2 : ((1 << lg) >> 3 > 2 ? 2 : (1 << lg) >> 3);
        int base = comp == 0 ? prefix_ctx[lg] + (xy ? DQC_LASTY_L : DQC_LASTX_L) : (xy ? DQC_LASTY_C : DQC_LASTX_C);
        int n = size < 32 ? size : 32;
        int gmax = orc_dq_last_group(n - 1);
        uint32_t acc = 0, cbits[16];
        uint32_t off = xy ? (uint32_t)cbf_delta : 0;
        for (int g = 0; g <= gmax; g++) {
            uint32_t suffix = g > 3 ? (uint32_t)(((g - 2) >> 1) << 15) : 0;
            if (g == gmax) { cbits[g] = acc + suffix + off; break; }
            dq_bits_of(ctx, base + (g >> shift), b);
            cbits[g] = acc + b[0] + suffix + off;
            acc += b[1];
        }
        int32_t *dst = xy ? rt->lasty : rt->lastx;
        for (int p = 0; p < n; p++) dst[p] = (int32_t)cbits[orc_dq_last_group(p)];
    }
}

/* ---- quantiser parameters (h266_dep_quant.c:774-857, per lg(w)+lg(h), QP) -- */

void orc_dq_params(int qp, int lgsum, orc_dq_param *p)
{
    static const int32_t qm[2][6] = { { 26214, 23302, 20560, 18396, 16384, 14564 },
                                      { 18396, 16384, 14564, 13107, 11651, 10280 } };
    static const int32_t iqm[2][6] = { { 40, 45, 51, 57, 64, 72 }, { 57, 64, 72, 80, 90, 102 } };
    int adj = lgsum & 1;
    int per = (qp + 1) / 6, rem = (qp + 1) - 6 * per;
    int nom_ts = 15 - ORC_BITDEPTH - (lgsum >> 1);
    int ts = nom_ts - adj;
    double lambda = 0.57 * pow(2.0, (qp - 12) / 3.0);
    memset(p, 0, sizeof(*p));
    p->qShift = 13 + per + ts;
    p->qAdd = -((3 << p->qShift) >> 1);
    p->qScale = qm[adj][rem];
    p->maxQIdx = (1 << 15) - 4;
    p->iqShift = 7 - ts;
    p->iqScale = iqm[adj][rem] << per;
    p->thresLast = p->qShift ? 8 << (p->qShift - 1) : 4;
    int dshift = 15 - 2 * nom_ts + p->qShift + adj;
    double q2 = (double)(p->qScale * p->qScale);
    double f = dshift < 0 ? 1.0 / ((double)((int64_t)1 << -dshift) * q2 * lambda)
                          : (double)((int64_t)1 << dshift) / (q2 * lambda);
    int64_t pw = (int64_t)(f * q2) + 1;
    int df;
    if (pw == 0) df = -1;
    else {
        uint32_t v = (uint32_t)((pw - 1) & 0xFFFFFFFF);
        df = v ? 31 - __builtin_clz(v) : 0;
    }
    df += 1;
    p->distShift = 62 + p->qShift - 30 - df;
    p->distAdd = (int32_t)(((int64_t)1 << p->distShift) >> 1);
    int s2 = p->distShift + p->qShift;
    p->distStepAdd = s2 >= 64 ? (int64_t)(f * pow(2, s2) + .5) : (int64_t)(f * (double)((int64_t)1 << s2) + .5);
    p->distOrgFact = (int64_t)(f * (double)((int64_t)1 << (p->distShift + 1)) + .5);
}

/* ---- scan tables --------------------------------------------------------- */

/* up-right diagonal scan of a w x h grid (h266_encoder/source/h266_scan_order.c:44-81) */
static void dq_diag(int w, int h, int *xs, int *ys)
{
    int x = 0, y = 0;
    for (int i = 0; i < w * h; i++) {
        xs[i] = x; ys[i] = y;
        if (x == w - 1 || y == 0) {
            y += x + 1; x = 0;
            if (y >= h) { x += y - (h - 1); y = h - 1; }
        } else { x++; y--; }
    }
}

typedef struct dq_scan {
    int n, nsbb, wsbb, hsbb;
    int px[1024], py[1024];          /* scan index -> position in the (<=32x32) region */
    int sbb_raster[64];              /* scan sub-block index -> raster sub-block index */
    int sbb_x[64], sbb_y[64];
    int nin[1024], in_of[1024][5];   /* inside neighbours (scan index within the sub-block) */
    int nout[1024], out_of[1024][5]; /* outside neighbours (absolute scan index) */
} dq_scan;

static void dq_build_scan(dq_scan *s, int w, int h)
{
    int ew = w < 32 ? w : 32, eh = h < 32 ? h : 32;
    int cx[16], cy[16], gx[64], gy[64];
    s->wsbb = ew >> 2; s->hsbb = eh >> 2; s->nsbb = s->wsbb * s->hsbb; s->n = ew * eh;
    dq_diag(4, 4, cx, cy);
    dq_diag(s->wsbb, s->hsbb, gx, gy);
    int sid[32][32];                 /* scan index by position (on the stack: callers run on several threads) */
    for (int b = 0; b < s->nsbb; b++) {
        s->sbb_x[b] = gx[b]; s->sbb_y[b] = gy[b]; s->sbb_raster[b] = gy[b] * s->wsbb + gx[b];
        for (int i = 0; i < 16; i++) {
            int k = b * 16 + i;
            s->px[k] = gx[b] * 4 + cx[i]; s->py[k] = gy[b] * 4 + cy[i];
            sid[s->py[k]][s->px[k]] = k;
        }
    }
    static const int dx[5] = { 1, 2, 1, 0, 0 }, dy[5] = { 0, 0, 1, 1, 2 };
    for (int k = 0; k < s->n; k++) {
        int beg = k & ~15;
        int ins[5], outs[5], ni = 0, no = 0;
        for (int j = 0; j < 5; j++) {
            int x = s->px[k] + dx[j], y = s->py[k] + dy[j];
            if (x >= ew || y >= eh) continue;
            int q = sid[y][x];
            if (q < beg + 16) ins[ni++] = q - beg; else outs[no++] = q;
        }
        /* ascending order, as the reference sorts them (h266_dep_quant.c:648-666) */
        for (int a = 0; a < ni; a++) for (int c = a + 1; c < ni; c++) if (ins[c] < ins[a]) { int t = ins[a]; ins[a] = ins[c]; ins[c] = t; }
        for (int a = 0; a < no; a++) for (int c = a + 1; c < no; c++) if (outs[c] < outs[a]) { int t = outs[a]; outs[a] = outs[c]; outs[c] = t; }
        s->nin[k] = ni; s->nout[k] = no;
        for (int j = 0; j < ni; j++) s->in_of[k][j] = ins[j];
        for (int j = 0; j < no; j++) s->out_of[k][j] = outs[j];
    }
}

/* position type of a scan index (h266_dep_quant.c:437-446) */
enum { DQ_IN = 0, DQ_SBB_FIRST = 1, DQ_SBB_LAST = 2 };
static int dq_ptype(const dq_scan *s, int k)
{
    int in = k & 15;
    if (in == 15 && k > 16 && k < s->n - 1) return DQ_SBB_FIRST;
    if (in == 0 && k > 0 && k < s->n - 16) return DQ_SBB_LAST;
    return DQ_IN;
}

/* significance / gtx context offsets from the diagonal of a position (:466-476) */
static void dq_ctx_offsets(int luma, int x, int y, int *sig, int *gtx)
{
    int d = x + y;
    if (luma) { *sig = d < 2 ? 8 : d < 5 ? 4 : 0; *gtx = d < 1 ? 16 : d < 3 ? 11 : d < 10 ? 6 : 1; }
    else      { *sig = d < 2 ? 4 : 0;             *gtx = d < 1 ? 6 : 1; }
}

/* ---- trellis ------------------------------------------------------------- */

typedef struct dq_st {
    int64_t cost;
    uint8_t lv[16];          /* levels of the current sub-block along the path */
    uint8_t sum[16];         /* per position: sum of neighbour levels (clipped) */
    uint8_t tpl[16];         /* per position: (neighbour count << 5) | sum of min(4+(l&1), l) */
    int nsig, rem, ref;
    const uint32_t *sbb;     /* rates of the coded-sub-block flag 0 / 1 */
    uint32_t sig[2];
    const uint32_t *gtx;
    int rice, rzero, id;
} dq_st;

typedef struct dq_sbbctx { uint8_t flags[64]; uint8_t lv[1024]; } dq_sbbctx;
typedef struct dq_dec { int64_t cost[4]; int16_t lv[4]; int8_t from[4]; } dq_dec;
typedef struct dq_pq { int64_t dd; int lv; } dq_pq;

typedef struct dq_work {
    dq_rates rt;
    dq_scan  sc;
    orc_dq_param par;
    dq_st    a[4], b[4], c[4], start;       /* three rotating state sets */
    dq_st   *cur, *prv, *skp;
    dq_sbbctx ctxa[4], ctxb[4];
    dq_sbbctx *ccur, *cprv;
    dq_dec   dec[1024][2];
    int      luma, ew, eh;
} dq_work;

static void dq_state_init(dq_work *wk, dq_st *s, int id)
{
    memset(s, 0, sizeof(*s));
    s->cost = DQ_COST_INF; s->rem = 4; s->ref = -1; s->id = id;
    const uint32_t *sg = wk->rt.sig[id > 1 ? id - 1 : 0][0];
    s->sig[0] = sg[0]; s->sig[1] = sg[1];
    s->gtx = wk->rt.gtx[0];
    s->sbb = wk->rt.sbb[0];
}

static const uint32_t *dq_sig_set(dq_work *wk, int id, int ctx)
{
    return wk->rt.sig[id > 1 ? id - 1 : 0][ctx];
}

/* rate of coding |level| lv >= 1 in the regular-bin regime */
static int64_t dq_level_bits(const dq_st *s, const uint32_t *gtx, int rice, int lv)
{
    if (lv < 4) return gtx[lv];
    int v = (lv - 4) >> 1;
    return (int64_t)gtx[lv - 2 * v] + orc_dq_rice_bits(rice, v < 31 ? v : 31);
    (void)s;
}

static void dq_prequant(int a, const orc_dq_param *p, dq_pq pq[4])
{
    int64_t org = (int64_t)a * p->qScale;
    int64_t qi = (org + p->qAdd) >> p->qShift;
    int q = (int)(qi < 1 ? 1 : qi > p->maxQIdx ? p->maxQIdx : qi);
    int64_t base = (int64_t)((uint64_t)q * (uint64_t)p->distStepAdd - (uint64_t)org * (uint64_t)p->distOrgFact);
    for (int k = 0; k < 4; k++) {
        int64_t m = (int64_t)((uint64_t)(base + k * p->distStepAdd) * (uint64_t)(int64_t)(q + k));
        pq[(q + k) & 3].dd = (m + p->distAdd) >> p->distShift;
        pq[(q + k) & 3].lv = (q + k + 1) >> 1;
    }
}

/* candidates of one source state for its two target states (h266_dep_quant.c:954-1046) */
static void dq_candidates(dq_st *s, int pt, const dq_pq *pa, const dq_pq *pb, dq_dec *d, int ta, int tb)
{
    int64_t ca = s->cost + pa->dd, cb = s->cost + pb->dd, cz = s->cost;
    int zero_ok = 1;
    if (s->rem >= 4) {
        ca += dq_level_bits(s, s->gtx, s->rice, pa->lv);
        cb += dq_level_bits(s, s->gtx, s->rice, pb->lv);
        if (pt == DQ_IN) { ca += s->sig[1]; cb += s->sig[1]; cz += s->sig[0]; }
        else if (pt == DQ_SBB_FIRST) {
            ca += s->sbb[1] + s->sig[1]; cb += s->sbb[1] + s->sig[1]; cz += s->sbb[1] + s->sig[0];
        } else if (s->nsig) { ca += s->sig[1]; cb += s->sig[1]; cz += s->sig[0]; }
        else zero_ok = 0;          /* an all-zero sub-block is coded through the skip path */
    } else {
        ca += (1 << 15) + orc_dq_rice_bits(s->rice, pa->lv <= s->rzero ? pa->lv - 1 : (pa->lv < 31 ? pa->lv : 31));
        cb += (1 << 15) + orc_dq_rice_bits(s->rice, pb->lv <= s->rzero ? pb->lv - 1 : (pb->lv < 31 ? pb->lv : 31));
        cz += orc_dq_rice_bits(s->rice, s->rzero);
    }
    if (!zero_ok) cz = d->cost[ta];
    if (ca < cz && ca < d->cost[ta]) { d->cost[ta] = ca; d->lv[ta] = (int16_t)pa->lv; d->from[ta] = (int8_t)s->id; }
    else if (cz < d->cost[ta])       { d->cost[ta] = cz; d->lv[ta] = 0;               d->from[ta] = (int8_t)s->id; }
    if (cb < d->cost[tb])            { d->cost[tb] = cb; d->lv[tb] = (int16_t)pb->lv; d->from[tb] = (int8_t)s->id; }
}

static void dq_set_rice(dq_st *s, int in)
{
    if (s->rem >= 4) {
        int v = s->sum[in] - 20;
        s->rice = dq_rice_par(v < 0 ? 0 : v > 31 ? 31 : v);
    }
}

static void dq_decide(dq_work *wk, int k, int a, dq_dec *d)
{
    dq_pq pq[4];
    int pt = dq_ptype(&wk->sc, k), in = k & 15;
    for (int t = 0; t < 4; t++) { d->cost[t] = DQ_COST_INF >> 1; d->lv[t] = -1; d->from[t] = -2; }
    dq_prequant(a, &wk->par, pq);
    if (pq[0].lv >= 4 || pq[2].lv >= 4) { dq_set_rice(&wk->prv[0], in); dq_set_rice(&wk->prv[1], in); }
    if (pq[1].lv >= 4 || pq[3].lv >= 4) { dq_set_rice(&wk->prv[2], in); dq_set_rice(&wk->prv[3], in); }
    dq_candidates(&wk->prv[0], pt, &pq[0], &pq[2], d, 0, 2);
    dq_candidates(&wk->prv[1], pt, &pq[0], &pq[2], d, 2, 0);
    dq_candidates(&wk->prv[2], pt, &pq[3], &pq[1], d, 1, 3);
    dq_candidates(&wk->prv[3], pt, &pq[3], &pq[1], d, 3, 1);
    if (pt == DQ_SBB_LAST)
        for (int t = 0; t < 4; t++) {
            int64_t c = wk->skp[t].cost + wk->skp[t].sbb[0];
            if (c < d->cost[t]) { d->cost[t] = c; d->lv[t] = 0; d->from[t] = (int8_t)(4 | t); }
        }
    /* a path may also start here: last significant position = k */
    int last = wk->rt.lastx[wk->sc.px[k]] + wk->rt.lasty[wk->sc.py[k]];
    for (int t = 0; t < 4; t += 2) {
        int64_t c = pq[t].dd + last + dq_level_bits(&wk->start, wk->start.gtx, 0, pq[t].lv);
        if (c < d->cost[t]) { d->cost[t] = c; d->lv[t] = (int16_t)pq[t].lv; d->from[t] = -1; }
    }
}

/* next-position contexts of a state from its template (:1312-1320, :1509-1531) */
static void dq_next_ctx(dq_work *wk, dq_st *s, int k, int eos)
{
    int nin = (k - 1) & 15, so, go;
    dq_ctx_offsets(wk->luma, wk->sc.px[k - 1], wk->sc.py[k - 1], &so, &go);
    int sum = s->sum[nin], a1 = s->tpl[nin] & 31, cnt = s->tpl[nin] >> 5;
    if (s->rem >= 4) {
        int i1 = (a1 + 1) >> 1;
        const uint32_t *sg = dq_sig_set(wk, s->id, so + (i1 < 3 ? i1 : 3));
        s->sig[0] = sg[0]; s->sig[1] = sg[1];
        int g = a1 - cnt;
        s->gtx = wk->rt.gtx[go + (g < 4 ? g : 4)];
        if (!eos) {
            int v = sum - 20;
            s->rice = dq_rice_par(v < 0 ? 0 : v > 31 ? 31 : v);
        }
    } else {
        int v = sum < 31 ? sum : 31;
        s->rice = dq_rice_par(v);
        s->rzero = (s->id < 2 ? 1 : 2) << s->rice;
    }
}

/* within a sub-block (:1426-1536) */
static void dq_update_in(dq_work *wk, int k, const dq_dec *d)
{
    int in = k & 15;
    for (int t = 0; t < 4; t++) {
        dq_st *s = &wk->cur[t];
        int lv = d->lv[t];
        s->cost = d->cost[t];
        if (d->from[t] <= -2) continue;
        if (d->from[t] >= 0) {
            const dq_st *p = &wk->prv[d->from[t]];
            s->nsig = p->nsig + (lv != 0);
            s->ref = p->ref;
            s->sbb = p->sbb;
            s->rem = p->rem - 1;
            if (s->rem >= 4) s->rem -= lv < 2 ? lv : 3;
            memcpy(s->lv, p->lv, 16); memcpy(s->sum, p->sum, 16); memcpy(s->tpl, p->tpl, 16);
        } else {
            s->nsig = 1; s->ref = -1;
            s->rem = wk->ew * wk->eh * DQ_REG_BINS / 16 - (lv < 2 ? lv : 3);
            memset(s->lv, 0, 16); memset(s->sum, 0, 16); memset(s->tpl, 0, 16);
        }
        if (lv) {
            s->lv[in] = (uint8_t)(lv < 255 ? lv : 255);
            int m45 = lv < 4 + (lv & 1) ? lv : 4 + (lv & 1);
            /* every later position of this sub-block that has position k as a neighbour */
            int beg = k & ~15;
            for (int j = 0; j < 16; j++) {
                int m = beg + j;
                for (int u = 0; u < wk->sc.nin[m]; u++)
                    if (wk->sc.in_of[m][u] == in) {
                        int v = s->sum[j] + lv;
                        s->sum[j] = (uint8_t)(v < 255 ? v : 255);
                        s->tpl[j] = (uint8_t)(s->tpl[j] + 32 + m45);
                    }
            }
        }
        dq_next_ctx(wk, s, k, 0);
    }
}

/* at the first coefficient (in scan order) of a sub-block: close it, open the
 * next one (:1224-1424) */
static void dq_update_eos(dq_work *wk, int k, const dq_dec *d)
{
    int in = k & 15, b = k >> 4;
    int braster = wk->sc.sbb_raster[b];
    /* right / below neighbours of the sub-block opened next (scan index b - 1) */
    int nraster = wk->sc.sbb_raster[b - 1];
    int right = wk->sc.sbb_x[b - 1] < wk->sc.wsbb - 1 ? nraster + 1 : 0;
    int below = wk->sc.sbb_y[b - 1] < wk->sc.hsbb - 1 ? nraster + wk->sc.wsbb : 0;
    for (int t = 0; t < 4; t++) {
        dq_st *s = &wk->cur[t];
        int lv = d->lv[t];
        const dq_st *p = NULL;
        s->cost = d->cost[t];
        if (d->from[t] <= -2) continue;
        if (d->from[t] >= 4) {
            p = &wk->skp[d->from[t] - 4];
            s->nsig = 0; s->rem = p->rem;
            memset(s->lv, 0, 16);
        } else if (d->from[t] >= 0) {
            p = &wk->prv[d->from[t]];
            s->nsig = p->nsig + (lv != 0);
            s->rem = p->rem - 1;
            if (s->rem >= 4) s->rem -= lv < 2 ? lv : 3;
            memcpy(s->lv, p->lv, 16);
        } else {
            s->nsig = 1;
            s->rem = wk->ew * wk->eh * DQ_REG_BINS / 16;
            if (s->rem >= 4) s->rem -= lv < 2 ? lv : 3;
            memset(s->lv, 0, 16);
        }
        int cap = 254 + (lv & 1);
        s->lv[in] = (uint8_t)(lv < cap ? lv : cap);
        /* sub-block context of the new path: the predecessor's, plus this sub-block */
        dq_sbbctx *nc = &wk->ccur[t];
        if (p && p->ref >= 0) *nc = wk->cprv[p->ref];
        else memset(nc, 0, sizeof(*nc));
        nc->flags[braster] = s->nsig != 0;
        memcpy(nc->lv + k, s->lv, 16);
        int sig_nb = (right && nc->flags[right]) || (below && nc->flags[below]);
        s->rice = 0; s->ref = t; s->sbb = wk->rt.sbb[sig_nb]; s->nsig = 0;
        memset(s->lv, 0, 16); memset(s->sum, 0, 16); memset(s->tpl, 0, 16);
        if (sig_nb || (right && below && nc->flags[below + 1])) {
            int beg = k - 16;
            for (int j = 0; j < 16; j++) {
                int m = beg + j, sa = 0, a1 = 0, cnt = 0;
                for (int u = 0; u < wk->sc.nout[m]; u++) {
                    int v = nc->lv[wk->sc.out_of[m][u]];
                    sa += v; a1 += v < 4 + (v & 1) ? v : 4 + (v & 1); cnt += v != 0;
                }
                s->tpl[j] = (uint8_t)((cnt << 5) | a1);
                s->sum[j] = (uint8_t)(sa < 127 ? sa : 127);
            }
        }
        dq_next_ctx(wk, s, k, 1);
    }
}

void orc_dep_quant(const ocoef *t, intptr_t stride, int w, int h, int qp, int comp,
                   const orc_prob *ctx, int root_cbf, ocoef *q, ocoef *r, uint64_t *nz)
{
    dq_work *wk = (dq_work *)calloc(1, sizeof(dq_work));
    int lgw = 31 - __builtin_clz((unsigned)w), lgh = 31 - __builtin_clz((unsigned)h);
    wk->luma = comp == 0;
    wk->ew = w < 32 ? w : 32; wk->eh = h < 32 ? h : 32;
    dq_build_rates(&wk->rt, ctx, comp, w, h, root_cbf);
    dq_build_scan(&wk->sc, w, h);
    orc_dq_params(qp, lgw + lgh, &wk->par);
    const orc_dq_param *par = &wk->par;

    for (int y = 0; y < wk->eh; y++)
        for (int x = 0; x < wk->ew; x++) { q[y * stride + x] = 0; r[y * stride + x] = 0; }

    /* last position: the highest scan index whose |t| exceeds the threshold (:1683-1770) */
    int thr = par->thresLast / (par->qScale << 2), first = -1;
    for (int k = wk->sc.n - 1; k >= 0 && first < 0; k--) {
        int v = t[wk->sc.py[k] * stride + wk->sc.px[k]];
        if ((v < 0 ? -v : v) > thr) first = k;
    }
    *nz = 0;
    if (first < 0) { free(wk); return; }

    wk->cur = wk->a; wk->prv = wk->b; wk->skp = wk->c;
    wk->ccur = wk->ctxa; wk->cprv = wk->ctxb;
    for (int i = 0; i < 4; i++) { dq_state_init(wk, &wk->a[i], i); dq_state_init(wk, &wk->b[i], i); dq_state_init(wk, &wk->c[i], i); }
    dq_state_init(wk, &wk->start, 0);

    for (int k = first; k >= 0; k--) {
        int v = t[wk->sc.py[k] * stride + wk->sc.px[k]];
        dq_dec *d = &wk->dec[k][0];
        dq_st *tmp = wk->prv; wk->prv = wk->cur; wk->cur = tmp;
        dq_decide(wk, k, v < 0 ? -v : v, d);
        if (k == 0) continue;
        if ((k & 15) == 0) {
            dq_sbbctx *tc = wk->ccur; wk->ccur = wk->cprv; wk->cprv = tc;
            dq_update_eos(wk, k, d);
            wk->dec[k][1] = *d;
        } else dq_update_in(wk, k, d);
        if (dq_ptype(&wk->sc, k) == DQ_SBB_FIRST) { tmp = wk->prv; wk->prv = wk->skp; wk->skp = tmp; }
    }

    /* best final state, then walk the decisions back (:1919-1947) */
    int64_t best = 0;
    int st = -1;
    for (int i = 0; i < 4; i++) if (wk->dec[0][0].cost[i] < best) { best = wk->dec[0][0].cost[i]; st = i; }
    int k = 0;
    while (st >= 0) {
        const dq_dec *d;
        if (st >= 4 && (k & 15) != 0) {          /* inside a skipped sub-block */
            q[wk->sc.py[k] * stride + wk->sc.px[k]] = 0;
            k++;
            continue;
        }
        d = &wk->dec[k][st >> 2];
        int lv = d->lv[st & 3];
        int v = t[wk->sc.py[k] * stride + wk->sc.px[k]];
        q[wk->sc.py[k] * stride + wk->sc.px[k]] = (ocoef)(v < 0 ? -lv : lv);
        st = d->from[st & 3];
        k++;
    }

    /* dequantisation along the state machine, from the last coded position (:1949-1989) */
    int iqadd = 1 << (par->iqShift - 1), state = 0;
    uint64_t map = 0;
    for (int j = k - 1; j >= 0; j--) {
        int x = wk->sc.px[j], y = wk->sc.py[j];
        int lv = q[y * stride + x];
        if (lv) {
            int qi = 2 * lv + (lv > 0 ? -(state >> 1) : (state >> 1));
            int v = (qi * par->iqScale + iqadd) >> par->iqShift;
            r[y * stride + x] = (ocoef)(v < -32768 ? -32768 : v > 32767 ? 32767 : v);
            map |= (uint64_t)1 << wk->sc.sbb_raster[j >> 4];
        }
        state = (32040 >> ((state << 2) + ((lv & 1) << 1))) & 3;
    }
    *nz = map;
    free(wk);
}
