/*
 * xg_dq.cuh -- dependent quantisation (trellis-coded quantisation, H.266 8.7.3
 * with the encoder's rate-distortion trellis) for batches of transform blocks:
 * the reference's Xin266DepQuant (h266_encoder/source/h266_dep_quant.c:1789),
 * reached through xin_func_struct.pfXinDepQuant (h266_encoder/include/h266_func_struct.h:795,
 * called from h266_trans_quant.c:192).
 *
 * Work split.  A block is walked coefficient by coefficient in reverse scan
 * order; at each coefficient four quantiser states each keep the cheapest path
 * that ends in them.  The transitions of the reference (0->{0,2}, 1->{2,0},
 * 2->{1,3}, 3->{3,1}, plus "skip this sub-block" and "start here") give
 * targets 0 and 2 their candidates from states 0 and 1 only, and targets 1
 * and 3 from states 2 and 3 only.  So two lanes own a block: lane h holds
 * states 2h and 2h + 1, prices their three candidates each (level A, level B,
 * zero), decides targets h and h + 2 and builds their new states with no
 * exchange; at the end of the step the lanes swap one state each.  A warp
 * runs 16 blocks side by side.
 *
 * State layout.  The reference copies a 48-byte template (levels and
 * neighbour sums) and a per-path copy of every earlier sub-block's levels with
 * each transition.  Here a state carries the 16 levels of its current
 * sub-block (four words of bytes, clipped like the reference's bytes) and the
 * same levels capped at 4 or 5 by parity (the values the neighbour sums
 * take); the neighbour sums at a position are byte dot products of those words
 * with the position's inside-neighbour mask, plus the outside-neighbour
 * template built when the sub-block was entered.  Earlier sub-blocks are kept
 * once per (sub-block, state) in a 16-slot ring (the farthest right / below
 * neighbour of a 4x4 sub-block in a 32x32 diagonal scan is 15 sub-blocks
 * away); a path's sub-block context is a 64-bit significance map plus a 2-bit
 * state tag per ring slot.  The decisions (one byte per state) go to a
 * per-block scratch column in global memory; after the trellis one lane
 * walks them back and dequantises along the state machine.
 *
 * The blocks of a warp come from one length bucket, so every thread is at
 * the same position of its current sub-block at every step: the sub-block
 * boundary work never diverges within a warp.
 */
#ifndef XG_DQ_CUH
#define XG_DQ_CUH

#include <math.h>
#include <mutex>
#include <vector>

#define XG_DQ_THREADS  128                      /* trellis threads per CTA: 64 blocks, two lanes each */
#define XG_DQ_MAXN     1024                     /* coefficients of the 32x32 region */
#define XG_DQ_RSETS    16                       /* context sets whose rate tables are staged in shared memory */
#define XG_DQ_MAX_CTAS (152 * 2)                /* trellis CTAs of a run at most (GB300: 152 SMs): two per SM; a third
                                                   lengthens the longest trellises more than it adds */
#define XG_DQ_SLOT_BYTES (XG_DQ_MAXN * 4 + 64 * 16) /* per trellis lane pair: decisions and ring */
#define XG_DQ_INF      ((long long)((((unsigned long long)1 << 63) - 1) >> 1))
#define XG_DQ_REG_BINS 28

/* context indices of the reference's context array (h266_encoder/include/h266_cabac_struct.h:130-213) */
enum {
    XG_DQC_ROOT_CBF = 76, XG_DQC_CBF_Y = 77, XG_DQC_CBF_U = 81, XG_DQC_CBF_V = 83,
    XG_DQC_SIGGRP_L = 86, XG_DQC_SIGGRP_C = 88, XG_DQC_SIG_L = 90, XG_DQC_SIG_C = 126,
    XG_DQC_PAR_L = 150, XG_DQC_PAR_C = 171, XG_DQC_GT2_L = 182, XG_DQC_GT1_L = 214,
    XG_DQC_LASTX_L = 246, XG_DQC_LASTX_C = 266, XG_DQC_LASTY_L = 269, XG_DQC_LASTY_C = 289
};

struct XgDqParam {              /* per (lg w + lg h, QP): the fields of xin_dp_param that the trellis reads */
    int32_t qShift, qAdd, qScale, maxQIdx, thresLast, iqShift, iqScale, distShift, distAdd, pad;
    long long distStepAdd, distOrgFact;
};
struct XgDqRates {              /* per (context set, luma / chroma), 1/32768-bit units */
    uint32_t sbb[2][2];
    uint32_t sig[3][12][2];
    uint32_t gtx[21][6];
};

/* last-position rates per (context set, luma / chroma, x / y, log2 size - 2, position) */
#define XG_DQ_LAST_WORDS (2 * 2 * 5 * 32)

__constant__ uint32_t c_dq_frac[256][2];        /* bits of a bin at probability state (p0 + p1) >> 8 */
__constant__ int32_t  c_dq_shape_off[16];       /* start of each region shape in the scan tables */
__constant__ uint4    c_dq_inm[16];             /* byte masks of the inside neighbours of 4x4 scan position i */

/* the 4x4 up-right diagonal scan (h266_encoder/source/h266_scan_order.c:44-81):
 * column and row of scan index i, and the scan index of (x, y) */
__host__ __device__ constexpr int xg_dq_s4x(int i) { return (int)((0x3323213210210100ull >> (4 * i)) & 15); }
__host__ __device__ constexpr int xg_dq_s4y(int i) { return (int)((0x3231230123012010ull >> (4 * i)) & 15); }
__host__ __device__ constexpr int xg_dq_s4i(int x, int y)
{
    int r = -1;
    for (int i = 0; i < 16; i++)
        if (xg_dq_s4x(i) == x && xg_dq_s4y(i) == y) r = i;
    return r;
}
/* the neighbour template of a position: (x+1, y), (x+2, y), (x+1, y+1), (x, y+1), (x, y+2) */
__host__ __device__ constexpr int xg_dq_ndx(int u) { return u == 0 || u == 2 ? 1 : u == 1 ? 2 : 0; }
__host__ __device__ constexpr int xg_dq_ndy(int u) { return u < 2 ? 0 : u == 4 ? 2 : 1; }
/* scan index of raster position y * 4 + x in a 4x4 sub-block (the inverse of the above) */
__host__ __device__ constexpr int xg_dq_s4r(int p) { return (int)((0xFDA6EB73C8419520ull >> (4 * p)) & 15); }
/* scan index of position (x, y) of a square n x n region (n = 4 .. 32): the
 * sub-block's index in the diagonal order of the (n/4)^2 grid, then the 4x4 scan */
__host__ __device__ __forceinline__ int xg_dq_scan_sq(int x, int y, int n)
{
    const int g = n >> 2, gx = x >> 2, gy = y >> 2, d = gx + gy;
    const int before = d < g ? d * (d + 1) / 2 : g * g - (2 * g - 1 - d) * (2 * g - d) / 2;
    const int lo = d - (g - 1) > 0 ? d - (g - 1) : 0;
    return (before + gx - lo) * 16 + xg_dq_s4r((y & 3) * 4 + (x & 3));
}

struct XgDqTables {
    uint2 *d_step;              /* per shape, per scan index: position, type, sub-block, context offsets */
    uint32_t *d_sbn;            /* per shape, per sub-block: scan indices of its right, below and
                                   below-right neighbours (bytes 0..2, 255 = none) */
    XgDqParam *d_par;           /* [lg w + lg h - 4][QP 0..51] */
    bool ok;
};
static XgDqTables g_dq;
static std::once_flag g_dq_once;

/* ---------------------------------------------------------------- host tables */

/* up-right diagonal scan of a w x h grid (h266_encoder/source/h266_scan_order.c:44-81) */
static void xg_dq_diag(int w, int h, std::vector<int> &xs, std::vector<int> &ys)
{
    xs.resize(w * h); ys.resize(w * h);
    int x = 0, y = 0;
    for (int i = 0; i < w * h; i++) {
        xs[i] = x; ys[i] = y;
        if (x == w - 1 || y == 0) {
            y += x + 1; x = 0;
            if (y >= h) { x += y - (h - 1); y = h - 1; }
        } else { x++; y--; }
    }
}

/* trellis parameters of h266_dep_quant.c:774-857, same double arithmetic */
static void xg_dq_param(int qp, int lgsum, XgDqParam *p)
{
    static const int32_t qm[2][6] = { { 26214, 23302, 20560, 18396, 16384, 14564 },
                                      { 18396, 16384, 14564, 13107, 11651, 10280 } };
    static const int32_t iqm[2][6] = { { 40, 45, 51, 57, 64, 72 }, { 57, 64, 72, 80, 90, 102 } };
    int adj = lgsum & 1, per = (qp + 1) / 6, rem = (qp + 1) - 6 * per;
    int nom_ts = 15 - XG_BITDEPTH - (lgsum >> 1), ts = nom_ts - adj;
    double lambda = 0.57 * pow(2.0, (qp - 12) / 3.0);
    memset(p, 0, sizeof *p);
    p->qShift = 13 + per + ts;
    p->qAdd = -((3 << p->qShift) >> 1);
    p->qScale = qm[adj][rem];
    p->maxQIdx = (1 << 15) - 4;
    p->iqShift = 7 - ts;
    p->iqScale = iqm[adj][rem] << per;
    p->thresLast = p->qShift ? 8 << (p->qShift - 1) : 4;
    int dshift = 15 - 2 * nom_ts + p->qShift + adj;
    double q2 = (double)(p->qScale * p->qScale);
    double f = dshift < 0 ? 1.0 / ((double)((long long)1 << -dshift) * q2 * lambda) : (double)((long long)1 << dshift) / (q2 * lambda);
    long long pw = (long long)(f * q2) + 1;
    int df;
    if (pw == 0) df = -1;
    else { uint32_t v = (uint32_t)((pw - 1) & 0xFFFFFFFF); df = v ? 31 - __builtin_clz(v) : 0; }
    df += 1;
    p->distShift = 62 + p->qShift - 30 - df;
    p->distAdd = (int32_t)(((long long)1 << p->distShift) >> 1);
    int s2 = p->distShift + p->qShift;
    p->distStepAdd = s2 >= 64 ? (long long)(f * pow(2, s2) + .5) : (long long)(f * (double)((long long)1 << s2) + .5);
    p->distOrgFact = (long long)(f * (double)((long long)1 << (p->distShift + 1)) + .5);
}

static void xg_dq_init_tables(void)
{
    g_dq.ok = false;
    /* rate of a bin: -log2(p) * 32768 rounded, with p(1) = (s + 0.5) / 256 (equals the
     * reference's cabacbinFracBits, h266_encoder/source/h266_entropy_write.c:52) */
    uint32_t frac[256][2];
    for (int s = 0; s < 256; s++) {
        double p1 = (s + 0.5) / 256.0;
        frac[s][0] = (uint32_t)floor(-log2(1.0 - p1) * 32768.0 + 0.5);
        frac[s][1] = (uint32_t)floor(-log2(p1) * 32768.0 + 0.5);
    }
    std::vector<uint2> step;
    std::vector<uint32_t> sbn;
    int32_t off[16];
    for (int sh = 0; sh < 16; sh++) {
        int ew = 4 << (sh >> 2), eh = 4 << (sh & 3), n = ew * eh, ws = ew >> 2, hs = eh >> 2;
        off[sh] = (int32_t)step.size();
        std::vector<int> cx, cy, gx, gy;
        xg_dq_diag(4, 4, cx, cy);
        xg_dq_diag(ws, hs, gx, gy);
        for (int i = 0; i < 16; i++)
            if (cx[i] != xg_dq_s4x(i) || cy[i] != xg_dq_s4y(i) || xg_dq_s4r(cy[i] * 4 + cx[i]) != i)
                return;                                                      /* the device's 4x4 scan constants */
        std::vector<int> px(n), py(n), sbs(ws * hs);
        for (int b = 0; b < ws * hs; b++) {
            sbs[gy[b] * ws + gx[b]] = b;
            for (int i = 0; i < 16; i++) { px[b * 16 + i] = gx[b] * 4 + cx[i]; py[b * 16 + i] = gy[b] * 4 + cy[i]; }
        }
        if (ew == eh)                                                        /* the square regions' scan formula */
            for (int k = 0; k < n; k++)
                if (xg_dq_scan_sq(px[k], py[k], ew) != k) return;
        for (int k = 0; k < n; k++) {
            int in = k & 15;
            int ptype = (in == 15 && k > 16 && k < n - 1) ? 1 : (in == 0 && k > 0 && k < n - 16) ? 2 : 0;
            int braster = gy[k >> 4] * ws + gx[k >> 4];
            /* significance / gtx context offsets of the position's diagonal, luma and chroma
             * (h266_dep_quant.c:466-476): luma sig 0/4/8, gtx 1/6/11/16; chroma sig 0/4, gtx 1/6 */
            const int dg = px[k] + py[k];
            const uint32_t ls = dg < 2 ? 2 : dg < 5 ? 1 : 0, lg = dg < 1 ? 3 : dg < 3 ? 2 : dg < 10 ? 1 : 0;
            const uint32_t cs = dg < 2 ? 1 : 0, cg = dg < 1 ? 1 : 0;
            uint2 e;
            e.x = (uint32_t)px[k] | (uint32_t)py[k] << 5 | (uint32_t)ptype << 10 | (uint32_t)braster << 15 |
                  ls << 21 | lg << 23 | cs << 25 | cg << 26;
            e.y = 0;
            step.push_back(e);
        }
        for (int b = 0; b < ws * hs; b++) {
            uint32_t r = gx[b] + 1 < ws ? (uint32_t)sbs[gy[b] * ws + gx[b] + 1] : 255u;
            uint32_t d = gy[b] + 1 < hs ? (uint32_t)sbs[(gy[b] + 1) * ws + gx[b]] : 255u;
            uint32_t rd = r != 255u && d != 255u ? (uint32_t)sbs[(gy[b] + 1) * ws + gx[b] + 1] : 255u;
            sbn.push_back(r | d << 8 | rd << 16);
        }
    }
    uint4 inm[16];
    for (int i = 0; i < 16; i++) {
        uint32_t m[4] = { 0, 0, 0, 0 };
        for (int u = 0; u < 5; u++) {
            int x = xg_dq_s4x(i) + xg_dq_ndx(u), y = xg_dq_s4y(i) + xg_dq_ndy(u);
            if (x < 4 && y < 4) { int j = xg_dq_s4i(x, y); m[j >> 2] |= 255u << (8 * (j & 3)); }
        }
        inm[i] = make_uint4(m[0], m[1], m[2], m[3]);
    }
    std::vector<XgDqParam> par(9 * 52);
    for (int lg = 4; lg <= 12; lg++)
        for (int qp = 0; qp < 52; qp++) xg_dq_param(qp, lg, &par[(lg - 4) * 52 + qp]);
    if (xg_cuda_check(cudaMemcpyToSymbol(c_dq_frac, frac, sizeof frac), "dq tables") ||
        xg_cuda_check(cudaMemcpyToSymbol(c_dq_shape_off, off, sizeof off), "dq tables") ||
        xg_cuda_check(cudaMemcpyToSymbol(c_dq_inm, inm, sizeof inm), "dq tables") ||
        xg_cuda_check(cudaMalloc(&g_dq.d_step, step.size() * sizeof(uint2)), "dq tables") ||
        xg_cuda_check(cudaMalloc(&g_dq.d_sbn, sbn.size() * sizeof(uint32_t)), "dq tables") ||
        xg_cuda_check(cudaMalloc(&g_dq.d_par, par.size() * sizeof(XgDqParam)), "dq tables") ||
        xg_cuda_check(cudaMemcpy(g_dq.d_step, step.data(), step.size() * sizeof(uint2), cudaMemcpyHostToDevice), "dq tables") ||
        xg_cuda_check(cudaMemcpy(g_dq.d_sbn, sbn.data(), sbn.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "dq tables") ||
        xg_cuda_check(cudaMemcpy(g_dq.d_par, par.data(), par.size() * sizeof(XgDqParam), cudaMemcpyHostToDevice), "dq tables"))
        return;
    g_dq.ok = true;
}

static bool xg_dq_tables(void)
{
    std::call_once(g_dq_once, xg_dq_init_tables);
    if (!g_dq.ok) xg_set_error(XIN_GPU_ERR_CUDA, "dep_quant: table set-up failed");
    return g_dq.ok;
}

/* ------------------------------------------------------------ rate tables */

__device__ __forceinline__ const uint32_t *xg_dq_bits(const xin_gpu_prob *ctx, int i)
{
    return c_dq_frac[(ctx[i].state[0] + ctx[i].state[1]) >> 8];
}

/* Xin266SetSigSbbFracBits / SetSigFlagBits / SetGtxFlagBits (h266_dep_quant.c:116-206)
 * for every context set and both channel types; one CTA per set.  The chroma
 * greater-than-1 / greater-than-2 rates come from the luma contexts, as in the
 * reference (:172-173).  Also the rates of the last position
 * (Xin266SetLastCoeffOffset, :208-283) per channel type, coordinate and block
 * side, without the coded-block-flag term of the y table (added per block). */
__global__ void k_dq_rates(const xin_gpu_prob *__restrict__ sets, XgDqRates *__restrict__ out, uint32_t *__restrict__ lasts)
{
    const xin_gpu_prob *ctx = sets + (size_t)blockIdx.x * XIN_GPU_NUM_CTX;
    if (threadIdx.x < 20) {
        const int ch = threadIdx.x / 10, xy = (threadIdx.x / 5) & 1, lg = 2 + threadIdx.x % 5;
        const int luma = ch == 0, nn = min(1 << lg, 32);
        const int shift = luma ? (lg + 1) >> 2 : min((1 << lg) >> 3, 2);
        const int cbase = luma ? (lg == 2 ? 0 : lg == 3 ? 3 : lg == 4 ? 6 : lg == 5 ? 10 : 15) + (xy ? XG_DQC_LASTY_L : XG_DQC_LASTX_L)
                               : (xy ? XG_DQC_LASTY_C : XG_DQC_LASTX_C);
        const int gmax = nn - 1 < 4 ? nn - 1 : 2 * (31 - __clz(nn - 1)) + (((nn - 1) >> (30 - __clz(nn - 1))) & 1);
        uint32_t *row = lasts + (size_t)blockIdx.x * XG_DQ_LAST_WORDS + ((ch * 2 + xy) * 5 + lg - 2) * 32;
        uint32_t acc = 0, cbits = 0;
        int gdone = 0;
        /* groups in increasing order; positions map to non-decreasing groups, so one pass fills the table */
        for (int p = 0; p < 32; p++) {
            if (p < nn) {
                const int g = p < 4 ? p : 2 * (31 - __clz(p)) + ((p >> (30 - __clz(p))) & 1);
                while (gdone <= g) {
                    const uint32_t suf = gdone > 3 ? (uint32_t)(((gdone - 2) >> 1) << 15) : 0;
                    if (gdone == gmax) cbits = acc + suf;
                    else {
                        const uint32_t *b = xg_dq_bits(ctx, cbase + (gdone >> shift));
                        cbits = acc + b[0] + suf;
                        acc += b[1];
                    }
                    gdone++;
                }
            }
            row[p] = p < nn ? cbits : 0u;
        }
    }
    for (int ch = 0; ch < 2; ch++) {
        XgDqRates *rt = out + blockIdx.x * 2 + ch;
        int nsig = ch ? 8 : 12, ngtx = ch ? 11 : 21;
        for (int i = threadIdx.x; i < 2 + 3 * nsig + ngtx; i += blockDim.x) {
            if (i < 2) {
                const uint32_t *b = xg_dq_bits(ctx, (ch ? XG_DQC_SIGGRP_C : XG_DQC_SIGGRP_L) + i);
                rt->sbb[i][0] = b[0]; rt->sbb[i][1] = b[1];
            } else if (i < 2 + 3 * nsig) {
                int j = i - 2, set = j / nsig, c = j % nsig;
                const uint32_t *b = xg_dq_bits(ctx, (ch ? XG_DQC_SIG_C : XG_DQC_SIG_L) + j);
                rt->sig[set][c][0] = b[0]; rt->sig[set][c][1] = b[1];
            } else {
                int c = i - 2 - 3 * nsig;
                const uint32_t *pb = xg_dq_bits(ctx, (ch ? XG_DQC_PAR_C : XG_DQC_PAR_L) + c);
                const uint32_t *g1 = xg_dq_bits(ctx, XG_DQC_GT1_L + c);
                const uint32_t *g2 = xg_dq_bits(ctx, XG_DQC_GT2_L + c);
                uint32_t p0 = 32768 + pb[0], p1 = 32768 + pb[1];
                rt->gtx[c][0] = 0;
                rt->gtx[c][1] = g1[0] + 32768;
                rt->gtx[c][2] = g1[1] + p0 + g2[0];
                rt->gtx[c][3] = g1[1] + p1 + g2[0];
                rt->gtx[c][4] = g1[1] + p0 + g2[1];
                rt->gtx[c][5] = g1[1] + p1 + g2[1];
            }
        }
    }
}

/* ------------------------------------------------------------------ trellis */

#define XG_DQ_PAIRS (XG_DQ_THREADS / 2)          /* blocks per CTA: one lane pair per block */
#define XG_DQ_TPLS  (XG_DQ_PAIRS + 1)            /* template row pitch: the two lanes of a pair read
                                                   different rows, which then fall in different banks */
struct XgDqSmem {
    uint32_t tpl[4 * 16][XG_DQ_TPLS];      /* outside-neighbour template [state * 16 + position][pair] */
    unsigned long long cfl[4][XG_DQ_PAIRS];  /* per template owner: coded flags of the earlier sub-blocks */
    uint32_t cvr[4][XG_DQ_PAIRS];          /* per template owner: ring version (state) of each slot */
    int32_t  rice[4][32];                  /* abs_remainder bits, Rice parameter k, value n */
    XgDqRates rt[XG_DQ_RSETS][2];          /* rate tables of the first context sets */
};

/* a state's small fields in one word: remaining context-coded bins (16 bits,
 * signed), coded levels in the current sub-block, template owner + 1, coded
 * flag of the right / below sub-blocks */
__device__ __forceinline__ uint32_t xg_pk(int rem, int ns, int ref, int sgb)
{
    return (uint32_t)(rem & 0xFFFF) | (uint32_t)ns << 16 | (uint32_t)(ref + 1) << 21 | (uint32_t)sgb << 24;
}
__device__ __forceinline__ int xg_pk_rem(uint32_t p) { return (int)(int16_t)(p & 0xFFFFu); }
__device__ __forceinline__ int xg_pk_ns(uint32_t p) { return (int)((p >> 16) & 31u); }
__device__ __forceinline__ int xg_pk_ref(uint32_t p) { return (int)((p >> 21) & 7u) - 1; }
__device__ __forceinline__ int xg_pk_sgb(uint32_t p) { return (int)((p >> 24) & 1u); }

/* Rice parameter from a neighbour sum (H.266 Table 128) */
__device__ __forceinline__ int xg_dq_rpar(int v) { return v < 7 ? 0 : v < 14 ? 1 : v < 28 ? 2 : 3; }

/* byte i (a constant after unrolling) of 16 bytes */
__device__ __forceinline__ uint32_t xg_dq_byte16(const uint4 &w, int i)
{
    const uint32_t x = i < 4 ? w.x : i < 8 ? w.y : i < 12 ? w.z : w.w;
    return (x >> (8 * (i & 3))) & 255u;
}

/* a neighbour level's share of a template: sum | min(4 + parity, v) << 11 | (v != 0) << 16 */
__device__ __forceinline__ uint32_t xg_dq_tplc(uint32_t v)
{
    return v | min(4u + (v & 1u), v) << 11 | (uint32_t)(v != 0u) << 16;
}

/* Outside-neighbour templates of the 16 positions of a sub-block (the sums
 * Xin266UpdateStateEOS builds from earlier sub-blocks, h266_dep_quant.c:1386-1440):
 * from the levels of its right (R), below (B) and below-right (D, first byte)
 * neighbours, 16 bytes each in scan order and zero where the neighbour is
 * absent or not coded.  Entry: min(sum, 127) | sum of min(4 + parity, v) << 7
 * | count << 12. */
__device__ __forceinline__ void xg_dq_build_tpl(const uint4 R, const uint4 B, uint32_t D, uint32_t *dst)
{
    uint32_t cr[2][4], cb[4][2];
#pragma unroll
    for (int y = 0; y < 4; y++) {
        cr[0][y] = xg_dq_tplc(xg_dq_byte16(R, xg_dq_s4i(0, y)));
        cr[1][y] = xg_dq_tplc(xg_dq_byte16(R, xg_dq_s4i(1, y)));
    }
#pragma unroll
    for (int x = 0; x < 4; x++) {
        cb[x][0] = xg_dq_tplc(xg_dq_byte16(B, xg_dq_s4i(x, 0)));
        cb[x][1] = xg_dq_tplc(xg_dq_byte16(B, xg_dq_s4i(x, 1)));
    }
    const uint32_t cd = xg_dq_tplc(D & 255u);
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int x = xg_dq_s4x(j), y = xg_dq_s4y(j);
        uint32_t acc = 0;
#pragma unroll
        for (int u = 0; u < 5; u++) {
            const int nx = x + xg_dq_ndx(u), ny = y + xg_dq_ndy(u);
            if (nx < 4 && ny < 4) continue;
            acc += (nx >= 4 && ny >= 4) ? cd : nx >= 4 ? cr[nx - 4][ny] : cb[nx][ny - 4];
        }
        dst[j * XG_DQ_TPLS] = min(acc & 2047u, 127u) | ((acc >> 11) & 31u) << 7 | (acc >> 16) << 12;
    }
}

/* ---- pass 1: per block (one warp each) gather the low 32x32 in scan order into
 * tscan, find the last position (Xin266PreDepQuant, h266_dep_quant.c:1683-1770),
 * zero q and r, and count the block into its length bucket: 0 = nothing above
 * the threshold (q, r, nz are final), b = 1 + last position / 16 otherwise. */
__global__ void __launch_bounds__(256)
k_dq_prep(const xin_gpu_dq_block *__restrict__ jobs, int njobs, const uint32_t *__restrict__ soff,
          const xg_coef *__restrict__ tin, xg_coef *__restrict__ tscan, xg_coef *__restrict__ qout,
          xg_coef *__restrict__ rout, unsigned long long *__restrict__ nzout, const uint2 *__restrict__ step_tab, const XgDqParam *__restrict__ par_tab, int32_t *__restrict__ first_out,
          int *__restrict__ counts, int full)
{
    const int lane = threadIdx.x & 31;
    const int nw = gridDim.x * (blockDim.x >> 5);
    /* bucket counts of this CTA's blocks, added to the global ones once at the end
     * (one global atomic per bucket and CTA instead of one per block) */
    __shared__ int hist[66];
    for (int b = threadIdx.x; b < 66; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < njobs; i += nw) {
        const xin_gpu_dq_block jb = jobs[i];
        const int lgw = jb.log2_w, lgh = jb.log2_h, ew = min(1 << lgw, 32), eh = min(1 << lgh, 32), n = ew * eh;
        const uint2 *ST = step_tab + c_dq_shape_off[(min(lgw, 5) - 2) * 4 + (min(lgh, 5) - 2)];
        const XgDqParam *P = par_tab + (lgw + lgh - 4) * 52 + jb.qp;
        const int thr = P->thresLast / (P->qScale << 2);
        const xg_coef *T = tin + jb.offset;
        xg_coef *TS = tscan + soff[i];
        int best = -1;
        for (int k = lane; k < n; k += 32) {
            const uint32_t e = __ldg(&ST[k].x);
            const xg_coef v = T[((e >> 5) & 31) * jb.stride + (e & 31)];
            TS[k] = v;
            if ((v < 0 ? -v : v) > thr) best = k;
        }
        best = __reduce_max_sync(0xffffffffu, best);
        const int zlw = full ? lgw : min(lgw, 5), zh = full ? 1 << lgh : eh;
        xg_coef *QO = qout + jb.offset, *RO = rout + jb.offset;
        for (int e = lane; e < (zh << zlw); e += 32) {
            const int y = e >> zlw, x = e & ((1 << zlw) - 1);
            QO[y * jb.stride + x] = 0;
            RO[y * jb.stride + x] = 0;
        }
        if (lane == 0) {
            first_out[i] = best;
            atomicAdd(&hist[best < 0 ? 0 : (best >> 4) + 1], 1);
            if (best < 0) nzout[i] = 0;
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 66; b += blockDim.x)
        if (hist[b]) atomicAdd(&counts[b], hist[b]);
}

/* ---- pass 1 for blocks whose producer already wrote the scan-order copy, the
 * last positions and zeroed q / r (the preset-4 TU stage's forward transforms):
 * count the length buckets (per CTA, then one global atomic per bucket) */
__global__ void __launch_bounds__(256) k_dq_count(int njobs, const int32_t *__restrict__ first, int *__restrict__ counts)
{
    __shared__ int hist[66];
    for (int b = threadIdx.x; b < 66; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < njobs; i += gridDim.x * blockDim.x) {
        const int f = first[i];
        atomicAdd(&hist[f < 0 ? 0 : (f >> 4) + 1], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 66; b += blockDim.x)
        if (hist[b]) atomicAdd(&counts[b], hist[b]);
}

/* ---- pass 2: order the blocks longest first (bucket 65 .. 1), then the empty ones */
__global__ void k_dq_order(int njobs, const int32_t *__restrict__ first, const int *__restrict__ counts,
                           int *__restrict__ cursor, int32_t *__restrict__ order)
{
    __shared__ int off[66];
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = 65; b >= 1; b--) { off[b] = acc; acc += counts[b]; }
        off[0] = acc;
    }
    __syncthreads();
    /* whole warps walk the list (inactive lanes past the end), so that the lanes
     * of one bucket take their places with one atomic: the leader reserves them */
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); i0 < njobs; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + lane;
        const int b = i < njobs ? (first[i] < 0 ? 0 : (first[i] >> 4) + 1) : 66;
        const unsigned peers = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(peers) - 1, rank = __popc(peers & ((1u << lane) - 1));
        int base = 0;
        if (lane == leader && b < 66) base = atomicAdd(&cursor[b], __popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (b < 66) order[off[b] + base + rank] = i;
    }
}

/* ---- pass 3: the trellis.  Two lanes per block.  The transitions pair the
 * states: targets 0 and 2 have their candidates from states 0 and 1 only,
 * targets 1 and 3 from states 2 and 3 only.  So lane h of a pair holds states
 * 2h and 2h + 1, prices their candidates, decides targets h and h + 2 and
 * builds their new states without any exchange; at the end of the step the
 * lanes swap one state each (lane 0 gives target 2, lane 1 gives target 1), so
 * that lane h again holds states 2h and 2h + 1.  A warp takes the next 16
 * blocks of the ordered list: its blocks walk the same number of sub-blocks
 * and are at the same position of a sub-block at every step. */

/* one state's registers: cost, levels of its current sub-block (bytes) and the
 * same levels capped at 4 + parity, packed small fields */
struct XgDqState { long long cost; uint32_t pk, L[4], F[4]; };

/* The new state of target t (Xin266UpdateState / Xin266UpdateStateEOS,
 * h266_dep_quant.c:1224-1536) from this lane's states before the step:
 * df is the source state (2h + j from local state j), -1 "start", 4 + t
 * "skip", -2 none.  A target without a candidate (only the odd ones at the
 * last position) keeps a cost no later candidate can win with, so its other
 * fields do not matter.  srcref: the template owner whose sub-block context the
 * new path continues (for the sub-block boundary).  sp: the packed fields of
 * the target's "skip" record. */
__device__ __forceinline__ XgDqState xg_dq_next(const XgDqState (&S)[2], int h, int df, int lvv, long long dc,
                                                int in, int regbins, uint32_t sp, int &ns, int &srcref)
{
    XgDqState n;
    const bool l1 = df == 2 * h + 1, fresh = df == -1 || df >= 4;
    const uint32_t pp = l1 ? S[1].pk : S[0].pk;
    const int dec = lvv < 2 ? lvv : 3;
    int r = xg_pk_rem(pp) - 1;
    if (r >= 4) r -= dec;
    int nsg = xg_pk_ns(pp) + (lvv != 0), rf = xg_pk_ref(pp);
    {
        /* "start here" and "skip", by selects */
        int r0 = regbins;
        if (in != 0 || r0 >= 4) r0 -= dec;
        const bool st = df == -1, sk = df >= 4;
        r = st ? r0 : sk ? xg_pk_rem(sp) : r;
        nsg = st ? 1 : sk ? 0 : nsg;
        rf = st ? -1 : sk ? xg_pk_ref(sp) : rf;
    }
    ns = nsg; srcref = rf;
    n.cost = dc;
    n.pk = xg_pk(r, nsg, rf, xg_pk_sgb(pp));
#pragma unroll
    for (int i = 0; i < 4; i++) {
        n.L[i] = fresh ? 0u : l1 ? S[1].L[i] : S[0].L[i];
        n.F[i] = fresh ? 0u : l1 ? S[1].F[i] : S[0].F[i];
    }
    {
        /* the level at this position: clipped to a byte (at a sub-block's first
         * position keeping its parity), and capped at 4 + parity; word in >> 2 by
         * masks, not by index, so the words stay in registers.  Without a level
         * (zero, or no candidate) a zero goes to a byte that is zero already. */
        const int lvi = df > -2 ? max(lvv, 0) : 0;
        const uint32_t b = in ? (uint32_t)min(lvi, 255) : (uint32_t)min(lvi, 254 + (lvi & 1));
        const uint32_t fb = (uint32_t)min(4 + (lvi & 1), lvi);
        const int wi = in >> 2, sh = (in & 3) * 8;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t sel = 0u - (uint32_t)(i == wi), bm = (255u << sh) & sel;
            n.L[i] = (n.L[i] & ~bm) | ((b << sh) & sel);
            n.F[i] = (n.F[i] & ~bm) | ((fb << sh) & sel);
        }
    }
    return n;
}

__device__ __forceinline__ long long xg_dq_shfl64x(unsigned m, long long v)
{
    const int lo = __shfl_xor_sync(m, (int)(unsigned long long)v, 1);
    const int hi = __shfl_xor_sync(m, (int)((unsigned long long)v >> 32), 1);
    return (long long)(((unsigned long long)(unsigned)hi << 32) | (unsigned)lo);
}

template <bool SHR>
__device__ __forceinline__ void xg_dq_block(XgDqSmem &sm, int job, const xin_gpu_dq_block &jb, int first,
                                            const uint32_t *__restrict__ soff, const xg_coef *__restrict__ tscan,
                                            xg_coef *__restrict__ qout, xg_coef *__restrict__ rout,
                                            unsigned long long *__restrict__ nzout, const xin_gpu_prob *__restrict__ sets,
                                            int nsets, const XgDqRates *__restrict__ rates,
                                            const uint32_t *__restrict__ lasts, const uint2 *__restrict__ step_tab,
                                            const uint32_t *__restrict__ sbn_tab, const XgDqParam *__restrict__ par_tab,
                                            uint32_t *__restrict__ codes, uint4 *__restrict__ ring, size_t NP)
{
    const int lane = threadIdx.x & 31, h = lane & 1, pi = threadIdx.x >> 1;
    const unsigned pm = 3u << (lane & 30);
    const int lgw = jb.log2_w, lgh = jb.log2_h, w = 1 << lgw, h2 = 1 << lgh;
    const int ew = min(w, 32), eh = min(h2, 32);
    const int shape = (min(lgw, 5) - 2) * 4 + (min(lgh, 5) - 2);
    const uint2 *ST = step_tab + c_dq_shape_off[shape];
    const uint32_t *SBN = sbn_tab + (c_dq_shape_off[shape] >> 4);
    const XgDqParam P = par_tab[(lgw + lgh - 4) * 52 + jb.qp];
    const int luma = jb.comp == 0, ch = luma ? 0 : 1;
    /* the rate tables from shared memory when every set is staged there (the loads are
     * then shared-memory loads, not generic ones, on the step's dependent chain) */
    const XgDqRates *RT = SHR ? &sm.rt[jb.ctx_set][ch] : rates + jb.ctx_set * 2 + ch;
    const xin_gpu_prob *CX = sets + (size_t)jb.ctx_set * XIN_GPU_NUM_CTX;
    const uint32_t *LX = lasts + (size_t)jb.ctx_set * XG_DQ_LAST_WORDS + ((ch * 2 + 0) * 5 + lgw - 2) * 32;
    const uint32_t *LY = lasts + (size_t)jb.ctx_set * XG_DQ_LAST_WORDS + ((ch * 2 + 1) * 5 + lgh - 2) * 32;
    uint32_t cbfoff;
    {
        const int cc = (luma && jb.root_cbf) ? XG_DQC_ROOT_CBF : jb.comp == 0 ? XG_DQC_CBF_Y : jb.comp == 1 ? XG_DQC_CBF_U : XG_DQC_CBF_V;
        const uint32_t *cb = xg_dq_bits(CX, cc);
        cbfoff = cb[1] - cb[0];
    }
    const xg_coef *TS = tscan + soff[job];
    uint32_t *CD = codes + (size_t)blockIdx.x * XG_DQ_PAIRS + pi;          /* decisions of position k at CD[k * NP] */
    uint4 *RG = ring + (size_t)blockIdx.x * XG_DQ_PAIRS + pi;             /* ring row (slot, state) at RG[(slot * 4 + state) * NP] */
    uint32_t *TP = &sm.tpl[0][pi];                                         /* template (state, position) at TP[(state * 16 + position) * TPLS] */
    const int regbins = ew * eh * XG_DQ_REG_BINS / 16;
    /* this lane's quantisation index classes: candidate A and B of states 2h, 2h + 1
     * (lane 0 also prices "start" of targets 0 and 2 with classes 0 and 2) */
    const int cA = h ? 3 : 0, cB = h ? 1 : 2;
    const int tf = h, ts = h + 2;                 /* the targets this lane decides */

    XgDqState S[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        S[j].cost = XG_DQ_INF;
#pragma unroll
        for (int i = 0; i < 4; i++) { S[j].L[i] = 0; S[j].F[i] = 0; }
        S[j].pk = xg_pk(4, 0, -1, 0);
        const int s = 2 * h + j;
        sm.cfl[s][pi] = 0; sm.cvr[s][pi] = 0;
    }
    __syncwarp(pm);
    /* the "skip" records (state at the top of the current sub-block) of this lane's
     * targets tf and ts: cost and packed fields */
    long long skc[2] = { XG_DQ_INF, XG_DQ_INF };
    uint32_t skp[2] = { xg_pk(4, 0, -1, 0), xg_pk(4, 0, -1, 0) };

    const int top = first | 15;
    /* loads ahead of the steps that use them: coefficient and position entry one
     * and two steps ahead, the last-position rates of the next position */
    auto clampk = [first](int x) { return max(min(x, first), 0); };
    auto lastxy = [&](uint32_t e) {
        return (long long)(int32_t)__ldg(&LX[e & 31]) + (long long)(int32_t)(__ldg(&LY[(e >> 5) & 31]) + cbfoff);
    };
    xg_coef cv = TS[first];
    uint2 ce = __ldg(&ST[clampk(top)]), ce1 = __ldg(&ST[clampk(top - 1)]);
    long long clxy = lastxy(ce.x);
    for (int k = top; k >= 0; k--) {
        const int in = k & 15, sb = k >> 4;
        const xg_coef nv = TS[clampk(k - 1)];
        const uint2 ne2 = __ldg(&ST[clampk(k - 2)]);
        const long long nlxy = lastxy(ce1.x);
        if (k <= first) {
            const uint32_t ex = ce.x;
            const int av = cv < 0 ? -(int)cv : (int)cv;
            const int ptype = (ex >> 10) & 3;
            const int sigoff = 4 * (int)(luma ? (ex >> 21) & 3 : (ex >> 25) & 1);
            const int gtxoff = 1 + 5 * (int)(luma ? (ex >> 23) & 3 : (ex >> 26) & 1);

            /* pre-quantisation (Xin266PreQuantCoeff, h266_dep_quant.c:920-952): for this lane's
             * classes the level and its distortion change */
            const long long org = (long long)av * P.qScale;
            const long long qi = (org + P.qAdd) >> P.qShift;
            const int q = (int)(qi < 1 ? 1 : qi > P.maxQIdx ? P.maxQIdx : qi);
            const long long bse = (long long)((unsigned long long)q * (unsigned long long)P.distStepAdd -
                                              (unsigned long long)org * (unsigned long long)P.distOrgFact);
            long long dd[2];
            int lv[2], gi[2], ri[2];
#pragma unroll
            for (int c = 0; c < 2; c++) {
                const int kk = ((c ? cB : cA) - q) & 3;
                const long long m = (long long)((unsigned long long)(bse + kk * P.distStepAdd) * (unsigned long long)(long long)(q + kk));
                dd[c] = (m + P.distAdd) >> P.distShift;
                lv[c] = (q + kk + 1) >> 1;
                gi[c] = lv[c] < 4 ? lv[c] : 4 + (lv[c] & 1);            /* column of the gtx rate table */
                ri[c] = min(max((lv[c] - 4) >> 1, 0), 31);                /* Rice index of the remainder */
            }

            /* ---- candidates of this lane's states (Xin266CheckRdCosts, h266_dep_quant.c:954-1046) ---- */
            const uint4 m = c_dq_inm[in];
            long long caz[2], cb[2];
            int saz[2], laz[2];
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const uint32_t spk = S[j].pk;
                const int sref = xg_pk_ref(spk), srem = xg_pk_rem(spk);
                const uint32_t tv0 = TP[(max(sref, 0) * 16 + in) * XG_DQ_TPLS];  /* loaded either way: no branch */
                const uint32_t tv = sref >= 0 ? tv0 : 0u;
                uint32_t sum = tv & 127u, a1 = (tv >> 7) & 31u;
                const uint32_t f0 = S[j].F[0] & m.x, f1 = S[j].F[1] & m.y, f2 = S[j].F[2] & m.z, f3 = S[j].F[3] & m.w;
                sum = __dp4a(S[j].L[0] & m.x, 0x01010101u, sum);
                sum = __dp4a(S[j].L[1] & m.y, 0x01010101u, sum);
                sum = __dp4a(S[j].L[2] & m.z, 0x01010101u, sum);
                sum = __dp4a(S[j].L[3] & m.w, 0x01010101u, sum);
                a1 = __dp4a(f0, 0x01010101u, a1);
                a1 = __dp4a(f1, 0x01010101u, a1);
                a1 = __dp4a(f2, 0x01010101u, a1);
                a1 = __dp4a(f3, 0x01010101u, a1);
                /* capped levels are at most 5, so + 7 sets bit 3 of a byte exactly where it is non-zero */
                const uint32_t nzb = ((f0 + 0x07070707u) & 0x08080808u) | ((f1 + 0x07070707u) & 0x08080808u) >> 1 |
                                     ((f2 + 0x07070707u) & 0x08080808u) >> 2 | ((f3 + 0x07070707u) & 0x08080808u) >> 3;
                const uint32_t cnt = (tv >> 12) + (uint32_t)__popc(nzb);

                const bool rc = srem >= 4;                           /* context-coded bins left */
                const int rice = xg_dq_rpar(rc ? min(max((int)sum - 20, 0), 31) : min((int)sum, 31));
                const int rzero = (h ? 2 : 1) << rice;               /* read only without context-coded bins */
                const uint2 sg = *reinterpret_cast<const uint2 *>(&RT->sig[h ? 1 + j : 0][sigoff + min((int)(a1 + 1) >> 1, 3)][0]);
                const uint32_t *gx = RT->gtx[gtxoff + min((int)(a1 - cnt), 4)];
                const int lvA = lv[0], lvB = lv[1];
                const int xA = rc ? ri[0] : (lvA <= rzero ? lvA - 1 : min(lvA, 31));
                const int xB = rc ? ri[1] : (lvB <= rzero ? lvB - 1 : min(lvB, 31));
                const uint32_t rA = (uint32_t)sm.rice[rice][xA], rB = (uint32_t)sm.rice[rice][xB];
                /* significance and coded-sub-block rates, by selects (the two states'
                 * chains then interleave): at a sub-block's first position in scan
                 * order the sub-block flag, elsewhere the significance flag, except
                 * at a sub-block's last position with nothing coded yet, where the
                 * level cannot be zero */
                const uint32_t sb1 = RT->sbb[xg_pk_sgb(spk)][1];
                const bool p1 = ptype == 1, sig_on = p1 || ptype == 0 || xg_pk_ns(spk) != 0;
                const uint32_t addAB = (p1 ? sb1 : 0u) + (sig_on ? sg.y : 0u);
                const uint32_t addZ = (p1 ? sb1 : 0u) + (sig_on ? sg.x : 0u);
                const bool zok = !rc || sig_on;
                const uint32_t tA = rc ? gx[gi[0]] + (lvA >= 4 ? rA : 0u) + addAB : (1u << 15) + rA;
                const uint32_t tB = rc ? gx[gi[1]] + (lvB >= 4 ? rB : 0u) + addAB : (1u << 15) + rB;
                const uint32_t tZ = rc ? addZ : (uint32_t)sm.rice[rice][rzero];
                const long long ca = S[j].cost + dd[0] + (long long)tA;
                cb[j] = S[j].cost + dd[1] + (long long)tB;
                const long long cz = S[j].cost + (long long)tZ;
                if (!zok || ca < cz) { caz[j] = ca; saz[j] = cA; laz[j] = lvA; }
                else                 { caz[j] = cz; saz[j] = 4;  laz[j] = 0; }
            }

            /* ---- decisions of targets tf = h (A / zero of state 2h, then B of 2h + 1) and
             * ts = h + 2 (B of state 2h, then A / zero of 2h + 1), then "skip the
             * sub-block" and, for targets 0 and 2, "start here" ---- */
            long long dc[2];
            int dfrom[2], dlv[2];
            uint32_t code = 0;
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const int t = u ? ts : tf;
                long long c1 = u ? cb[0] : caz[0], c2 = u ? caz[1] : cb[1];
                const int e1 = u ? cB : saz[0], e2 = u ? saz[1] : cB;
                const int f1 = u ? 2 * h : 2 * h, f2 = 2 * h + 1;
                const int g1 = u ? lv[1] : laz[0], g2 = u ? laz[1] : lv[1];
                long long d = XG_DQ_INF >> 1;
                int dsel = 7, df = -2, dl = -1;
                if (c1 < d) { d = c1; dsel = e1; df = f1; dl = g1; }
                if (c2 < d) { d = c2; dsel = e2; df = f2; dl = g2; }
                {
                    /* skip the sub-block (only at a sub-block's first position in scan order) */
                    const long long c = skc[u] + (long long)RT->sbb[xg_pk_sgb(skp[u])][0];
                    const bool take = (ptype == 2) & (c < d);
                    d = take ? c : d; dsel = take ? 4 : dsel; df = take ? 4 + t : df; dl = take ? 0 : dl;
                }
                {
                    /* start here (the last position): targets 0 and 2 (lane 0), classes 0 and 2;
                     * priced on both lanes so that the warp does not branch */
                    const int c = u;
                    const long long cs = dd[c] + clxy + (long long)RT->gtx[0][gi[c]] + (lv[c] >= 4 ? sm.rice[0][ri[c]] : 0);
                    const bool take = (h == 0) & (cs < d);
                    d = take ? cs : d; dsel = take ? t : dsel; df = take ? -1 : df; dl = take ? lv[c] : dl;
                }
                dc[u] = d; dfrom[u] = df; dlv[u] = dl;
                code |= (uint32_t)((df + 2) | dsel << 4) << (8 * t);
            }
            code |= __shfl_xor_sync(pm, code, 1);
            if (h == 0) CD[(size_t)k * NP] = code;

            if (ptype == 1) {
                /* the records of targets h and h + 2 are states h and h + 2 before the
                 * step: lane 0 holds state 0 and gets state 2 (lane 1's first), lane 1
                 * holds state 3 and gets state 1 (lane 0's second) */
                const long long oc = xg_dq_shfl64x(pm, h ? S[0].cost : S[1].cost);
                const uint32_t op = __shfl_xor_sync(pm, h ? S[0].pk : S[1].pk, 1);
                skc[0] = h ? oc : S[0].cost; skp[0] = h ? op : S[0].pk;
                skc[1] = h ? S[1].cost : oc; skp[1] = h ? S[1].pk : op;
            }

            /* ---- new states of tf and ts, then the swap ---- */
            XgDqState N[2];
            int nns[2], srcref[2];
            if (k > 0) {
#pragma unroll
                for (int u = 0; u < 2; u++)
                    N[u] = xg_dq_next(S, h, dfrom[u], dlv[u], dc[u], in, regbins, skp[u], nns[u], srcref[u]);
                if (in == 0) {
                    /* first coefficient (in scan order) of sub-block sb: close it and open sb - 1.
                     * The sub-block context of a new path is its predecessor's (that of the owner
                     * of its template) plus this sub-block; its levels go to the ring. */
                    const int slot = sb & 15;
                    unsigned long long nfl[2];
                    uint32_t nvr[2];
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const int t = u ? ts : tf, cr = srcref[u];
                        const unsigned long long fl = cr >= 0 ? sm.cfl[cr][pi] : 0ull;
                        const uint32_t fv = cr >= 0 ? sm.cvr[cr][pi] : 0u;
                        nfl[u] = (fl & ~(1ull << sb)) | (unsigned long long)(nns[u] != 0) << sb;
                        nvr[u] = (fv & ~(3u << (2 * slot))) | (uint32_t)t << (2 * slot);
                        if (dfrom[u] > -2) RG[(size_t)(slot * 4 + t) * NP] = make_uint4(N[u].L[0], N[u].L[1], N[u].L[2], N[u].L[3]);
                    }
                    __syncwarp(pm);                  /* both lanes' ring rows written, old contexts read */
                    const uint32_t nb = __ldg(&SBN[sb - 1]);
                    const int nR = nb & 255, nB = (nb >> 8) & 255, nD = (nb >> 16) & 255;
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const int t = u ? ts : tf;
                        if (dfrom[u] > -2) {
                            const unsigned long long fl = nfl[u];
                            const bool sR = nR != 255 && ((fl >> nR) & 1), sB = nB != 255 && ((fl >> nB) & 1);
                            const bool sD = nD != 255 && ((fl >> nD) & 1);
                            const int nsb = sR || sB;
                            uint32_t *dst = TP + (size_t)t * 16 * XG_DQ_TPLS;
                            if (nsb || sD) {
                                const uint4 z = make_uint4(0, 0, 0, 0);
                                const uint4 vR = sR ? RG[(size_t)((nR & 15) * 4 + ((nvr[u] >> (2 * (nR & 15))) & 3)) * NP] : z;
                                const uint4 vB = sB ? RG[(size_t)((nB & 15) * 4 + ((nvr[u] >> (2 * (nB & 15))) & 3)) * NP] : z;
                                const uint4 vD = sD ? RG[(size_t)((nD & 15) * 4 + ((nvr[u] >> (2 * (nD & 15))) & 3)) * NP] : z;
                                xg_dq_build_tpl(vR, vB, vD.x, dst);
                            } else {
#pragma unroll
                                for (int j = 0; j < 16; j++) dst[j * XG_DQ_TPLS] = 0;
                            }
                            N[u].pk = xg_pk(xg_pk_rem(N[u].pk), 0, t, nsb);
                            sm.cfl[t][pi] = fl; sm.cvr[t][pi] = nvr[u];
#pragma unroll
                            for (int i = 0; i < 4; i++) { N[u].L[i] = 0; N[u].F[i] = 0; }
                        }
                    }
                    __syncwarp(pm);                  /* templates and contexts visible to both lanes */
                }
            } else {
#pragma unroll
                for (int u = 0; u < 2; u++) { N[u] = S[u]; N[u].cost = dc[u]; }
            }
            /* lane 0 keeps target 0 and gives target 2; lane 1 keeps target 3 and gives target 1 */
            {
                XgDqState got;
                got.cost = xg_dq_shfl64x(pm, h ? N[0].cost : N[1].cost);
                got.pk = __shfl_xor_sync(pm, h ? N[0].pk : N[1].pk, 1);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    got.L[i] = __shfl_xor_sync(pm, h ? N[0].L[i] : N[1].L[i], 1);
                    got.F[i] = __shfl_xor_sync(pm, h ? N[0].F[i] : N[1].F[i], 1);
                }
                /* by selects: the two lanes of a pair take different sides */
                S[0].cost = h ? got.cost : N[0].cost; S[1].cost = h ? N[1].cost : got.cost;
                S[0].pk = h ? got.pk : N[0].pk;       S[1].pk = h ? N[1].pk : got.pk;
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    S[0].L[i] = h ? got.L[i] : N[0].L[i]; S[1].L[i] = h ? N[1].L[i] : got.L[i];
                    S[0].F[i] = h ? got.F[i] : N[0].F[i]; S[1].F[i] = h ? N[1].F[i] : got.F[i];
                }
            }
        }
        cv = nv; ce = ce1; ce1 = ne2; clxy = nlxy;
    }

    /* ---- best final state, then walk the decisions from position 0 up
     * (h266_dep_quant.c:1919-1947), on lane 0.  The state a coefficient was
     * quantised in is the source state of its decision (0 for the last
     * position), so each level is dequantised as it is found (:1949-1989 walks
     * the same state machine forward from the last position). */
    const long long o0 = xg_dq_shfl64x(pm, S[0].cost), o1 = xg_dq_shfl64x(pm, S[1].cost);
    if (h) return;
    const long long fc[4] = { S[0].cost, S[1].cost, o0, o1 };
    long long best = 0;
    int st = -1;
#pragma unroll
    for (int s = 0; s < 4; s++)
        if (fc[s] < best) { best = fc[s]; st = s; }
    unsigned long long map = 0;
    const int iqadd = 1 << (P.iqShift - 1);
    xg_coef *QO = qout + jb.offset, *RO = rout + jb.offset;
    const int stride = jb.stride;
    uint32_t ncode = CD[0];
    xg_coef nval = TS[0];
    uint32_t nent = __ldg(&ST[0].x);
    for (int k = 0; st >= 0 && k <= first; k++) {
        const uint32_t c = ncode, ent = nent;
        const int v = nval;
        const int kn = min(k + 1, first);
        ncode = CD[(size_t)kn * NP]; nval = TS[kn]; nent = __ldg(&ST[kn].x);
        int lv = 0, ps = 0;
        if (!(st >= 4 && (k & 15))) {
            const uint32_t byte = (c >> (8 * (st & 3))) & 255u;
            const int sel = (int)(byte >> 4), from = (int)(byte & 15) - 2;
            const int av = v < 0 ? -v : v;
            const long long qi = ((long long)av * P.qScale + P.qAdd) >> P.qShift;
            const int q = (int)(qi < 1 ? 1 : qi > P.maxQIdx ? P.maxQIdx : qi);
            lv = sel >= 4 ? 0 : (q + ((sel - q) & 3) + 1) >> 1;
            ps = from >= 0 && from < 4 ? from : 0;
            st = from;
        }
        if (lv) {
            const int x = ent & 31, y = (ent >> 5) & 31;
            const int qv = v < 0 ? -lv : lv;
            const int qidx = 2 * qv + (qv > 0 ? -(ps >> 1) : (ps >> 1));
            const int rv = (qidx * P.iqScale + iqadd) >> P.iqShift;
            QO[y * stride + x] = (xg_coef)qv;
            RO[y * stride + x] = (xg_coef)(rv < -32768 ? -32768 : rv > 32767 ? 32767 : rv);
            map |= 1ull << ((ent >> 15) & 63);
        }
    }
    nzout[job] = map;
}

/* min blocks 3: three CTAs of 128 threads per SM */
__global__ void __launch_bounds__(XG_DQ_THREADS, 3)
k_dq(const xin_gpu_dq_block *__restrict__ jobs, int njobs, int *__restrict__ counter, const int *__restrict__ counts,
     const int32_t *__restrict__ order, const int32_t *__restrict__ firsts, const uint32_t *__restrict__ soff,
     const xg_coef *__restrict__ tscan, xg_coef *__restrict__ qout, xg_coef *__restrict__ rout,
     unsigned long long *__restrict__ nzout, const xin_gpu_prob *__restrict__ sets, int nsets,
     const XgDqRates *__restrict__ rates, const uint32_t *__restrict__ lasts, const uint2 *__restrict__ step_tab,
     const uint32_t *__restrict__ sbn_tab, const XgDqParam *__restrict__ par_tab, uint32_t *__restrict__ codes,
     uint4 *__restrict__ ring)
{
    extern __shared__ __align__(16) unsigned char xg_dq_raw[];
    XgDqSmem &sm = *reinterpret_cast<XgDqSmem *>(xg_dq_raw);
    const int lane = threadIdx.x & 31;
    const size_t NP = (size_t)gridDim.x * XG_DQ_PAIRS;
    const int ntr = njobs - counts[0];

    for (int i = threadIdx.x; i < 128; i += blockDim.x) {
        int k = i >> 5, n = i & 31, p = n >> k;
        int bits;
        if (p < 6) bits = p + 1 + k;
        else { unsigned mm = (unsigned)(n - (6 << k)); bits = 6 + 2 * (31 - __clz((int)((mm >> (k + 1)) + 1))) + 1 + (k + 1); }
        sm.rice[k][n] = bits << 15;
    }
    {
        const int nw = min(nsets, XG_DQ_RSETS) * 2 * (int)(sizeof(XgDqRates) / 4);
        const uint32_t *src = reinterpret_cast<const uint32_t *>(rates);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sm.rt[0][0]);
        for (int i = threadIdx.x; i < nw; i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();

    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(counter, 16);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= ntr) break;
        const int idx = base + (lane >> 1);
        if (idx < ntr) {
            const int job = order[idx];
            const xin_gpu_dq_block jb = jobs[job];
            if (nsets <= XG_DQ_RSETS)
                xg_dq_block<true>(sm, job, jb, firsts[job], soff, tscan, qout, rout, nzout, sets, nsets, rates, lasts,
                                  step_tab, sbn_tab, par_tab, codes, ring, NP);
            else
                xg_dq_block<false>(sm, job, jb, firsts[job], soff, tscan, qout, rout, nzout, sets, nsets, rates, lasts,
                                   step_tab, sbn_tab, par_tab, codes, ring, NP);
        }
        __syncwarp(0xffffffffu);
    }
}

/* ---------------------------------------------------------------- launches */

/* the trellis kernel's shared memory (above the 48 KB default) and the CTAs
 * that fit on the GPU at once; 0 if the attribute could not be set */
static int xg_dq_resident_ctas(void)
{
    static int ctas = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaFuncSetAttribute(k_dq, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(XgDqSmem)) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        cudaFuncSetAttribute(k_dq, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_dq, XG_DQ_THREADS, sizeof(XgDqSmem));
        ctas = sms * (per > 0 ? per : 1);
    });
    if (!ctas) xg_set_error(XIN_GPU_ERR_CUDA, "dep_quant: kernel set-up failed");
    return ctas;
}

/* Device work area of a run, in order: job counter, bucket counts and cursors
 * (1 KB); rates and last-position rates of nsets context sets; last positions
 * and order of njobs blocks; the scan-order copy of the blocks (nscan
 * coefficients); per trellis thread (nslots) its decision column and its ring
 * of earlier sub-blocks' levels. */
struct XgDqArea {
    int *counter, *counts, *cursor;
    XgDqRates *rates;
    uint32_t *lasts;
    int32_t *first, *order;
    xg_coef *tscan;
    uint32_t *codes;
    uint4 *ring;
};
static size_t xg_dq_area_bytes(int nsets, int njobs, size_t nscan, int nslots, XgDqArea *a, char *base)
{
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = (o + bytes + 255) & ~(size_t)255; return base ? base + at : nullptr; };
    char *hdr = take(1024);
    char *rt = take((size_t)nsets * 2 * sizeof(XgDqRates));
    char *la = take((size_t)nsets * XG_DQ_LAST_WORDS * 4);
    char *fi = take((size_t)njobs * 4);
    char *od = take((size_t)njobs * 4);
    char *ts = take(nscan * sizeof(xg_coef));
    char *cd = take((size_t)nslots * XG_DQ_MAXN * 4);
    char *rg = take((size_t)nslots * 64 * sizeof(uint4));
    static_assert(XG_DQ_SLOT_BYTES == XG_DQ_MAXN * 4 + 64 * sizeof(uint4), "trellis slot bytes");
    if (a && base) {
        a->counter = (int *)hdr; a->counts = (int *)hdr + 1; a->cursor = (int *)hdr + 80;
        a->rates = (XgDqRates *)rt; a->lasts = (uint32_t *)la; a->first = (int32_t *)fi; a->order = (int32_t *)od;
        a->tscan = (xg_coef *)ts; a->codes = (uint32_t *)cd; a->ring = (uint4 *)rg;
    }
    return o;
}

static int xg_dq_enqueue(const xin_gpu_dq_block *d_jobs, const uint32_t *d_soff, int njobs,
                         const xg_coef *t, xg_coef *q, xg_coef *r, unsigned long long *nz, const xin_gpu_prob *d_sets,
                         int nsets, const XgDqArea &A, int max_ctas, int full, cudaStream_t st, bool count = true)
{
    int ctas = (njobs + XG_DQ_PAIRS - 1) / XG_DQ_PAIRS;
    if (ctas > max_ctas) ctas = max_ctas;
    if (xg_cuda_check(cudaMemsetAsync(A.counter, 0, 1024, st), "dq counters")) return XIN_GPU_ERR_CUDA;
    k_dq_rates<<<nsets, 64, 0, st>>>(d_sets, A.rates, A.lasts);
    const int pw = 8, pblocks = std::min((njobs + pw - 1) / pw, 152 * 16);
    k_dq_prep<<<pblocks, pw * 32, 0, st>>>(d_jobs, njobs, d_soff, t, A.tscan, q, r, nz, g_dq.d_step, g_dq.d_par,
                                           A.first, A.counts, full);
    k_dq_order<<<std::min((njobs + 255) / 256, 152 * 4), 256, 0, st>>>(njobs, A.first, A.counts, A.cursor, A.order);
    k_dq<<<ctas, XG_DQ_THREADS, sizeof(XgDqSmem), st>>>(d_jobs, njobs, A.counter, A.counts, A.order, A.first, d_soff,
                                                        A.tscan, q, r, nz, d_sets, nsets, A.rates, A.lasts, g_dq.d_step,
                                                        g_dq.d_sbn, g_dq.d_par, A.codes, A.ring);
    if (count) xg_count_launch(4);
    return xg_cuda_check(cudaGetLastError(), "dep_quant launch");
}

/* the trellis for blocks already gathered (scan-order copy in A.tscan at d_soff,
 * last positions in A.first, q and r zeroed, nz of blocks without a trellis
 * written); the counters are cleared by the caller before the producer runs */
static int xg_dq_enqueue_gathered(const xin_gpu_dq_block *d_jobs, const uint32_t *d_soff, int njobs, xg_coef *q, xg_coef *r,
                                  unsigned long long *nz, const xin_gpu_prob *d_sets, int nsets, const XgDqArea &A,
                                  int max_ctas, cudaStream_t st)
{
    int ctas = (njobs + XG_DQ_PAIRS - 1) / XG_DQ_PAIRS;
    if (ctas > max_ctas) ctas = max_ctas;
    k_dq_rates<<<nsets, 64, 0, st>>>(d_sets, A.rates, A.lasts);
    k_dq_count<<<std::min((njobs + 255) / 256, 152 * 4), 256, 0, st>>>(njobs, A.first, A.counts);
    k_dq_order<<<std::min((njobs + 255) / 256, 152 * 4), 256, 0, st>>>(njobs, A.first, A.counts, A.cursor, A.order);
    k_dq<<<ctas, XG_DQ_THREADS, sizeof(XgDqSmem), st>>>(d_jobs, njobs, A.counter, A.counts, A.order, A.first, d_soff,
                                                        A.tscan, q, r, nz, d_sets, nsets, A.rates, A.lasts, g_dq.d_step,
                                                        g_dq.d_sbn, g_dq.d_par, A.codes, A.ring);
    return xg_cuda_check(cudaGetLastError(), "dep_quant launch");
}

static int xg_dq_validate(const xin_gpu_dq_block *b, int32_t n, size_t ncoeffs, int32_t nsets)
{
    for (int i = 0; i < n; i++) {
        const xin_gpu_dq_block &j = b[i];
        if (j.log2_w < 2 || j.log2_w > 6 || j.log2_h < 2 || j.log2_h > 6 || j.qp > 51 || j.comp > 2 ||
            j.ctx_set >= (uint32_t)nsets || j.stride < (1u << j.log2_w)) {
            xg_set_error(XIN_GPU_ERR_ARG, "dep_quant: block %d: sizes 4..64, QP 0..51, component 0..2, a context set "
                         "below %d and a stride of at least the width are required", i, nsets);
            return XIN_GPU_ERR_ARG;
        }
        size_t end = (size_t)j.offset + (size_t)((1u << j.log2_h) - 1) * j.stride + (1u << j.log2_w);
        if (end > ncoeffs) {
            xg_set_error(XIN_GPU_ERR_ARG, "dep_quant: block %d reaches past the %zu coefficients", i, ncoeffs);
            return XIN_GPU_ERR_ARG;
        }
    }
    return XIN_GPU_OK;
}

/* ------------------------------------------------------------------- plan */

struct xin_gpu_dq_plan {
    int device;
    int32_t nblocks, nsets, ctas;
    size_t ncoeffs, nscan;
    xin_gpu_dq_block *d_jobs;
    uint32_t *d_soff;               /* start of each block's scan-order copy */
    char *d_area;
    XgDqArea area;
};

extern "C" void xin_gpu_dq_plan_destroy(xin_gpu_dq_plan *p);

extern "C" int xin_gpu_dq_plan_create(const xin_gpu_dq_block *blocks, int32_t nblocks, size_t ncoeffs, int32_t nsets,
                                      xin_gpu_dq_plan **out)
{
    xin_gpu_clear_error();
    if (!blocks || nblocks <= 0 || nsets <= 0 || !out) {
        xg_set_error(XIN_GPU_ERR_ARG, "dq_plan_create: bad argument");
        return XIN_GPU_ERR_ARG;
    }
    *out = nullptr;
    if (!xg_thread() || !xg_dq_tables()) return xin_gpu_last_status();
    int st = xg_dq_validate(blocks, nblocks, ncoeffs, nsets);
    if (st) return st;
    std::vector<uint32_t> soff(nblocks);
    size_t nscan = 0;
    for (int i = 0; i < nblocks; i++) {
        soff[i] = (uint32_t)nscan;
        nscan += (size_t)std::min(1 << blocks[i].log2_w, 32) * std::min(1 << blocks[i].log2_h, 32);
    }
    xin_gpu_dq_plan *p = new xin_gpu_dq_plan();
    cudaGetDevice(&p->device);
    p->nblocks = nblocks; p->nsets = nsets; p->ncoeffs = ncoeffs; p->nscan = nscan;
    const int res = xg_dq_resident_ctas();
    if (!res) { delete p; return xin_gpu_last_status(); }
    p->ctas = std::min(std::min(res, XG_DQ_MAX_CTAS), (nblocks + XG_DQ_PAIRS - 1) / XG_DQ_PAIRS);
    const size_t bytes = xg_dq_area_bytes(nsets, nblocks, nscan, p->ctas * XG_DQ_PAIRS, nullptr, nullptr);
    if (nscan >= (1ull << 32) ||
        xg_cuda_check(cudaMalloc(&p->d_soff, (size_t)nblocks * 4), "dq plan") ||
        xg_cuda_check(cudaMemcpy(p->d_soff, soff.data(), (size_t)nblocks * 4, cudaMemcpyHostToDevice), "dq plan") ||
        xg_cuda_check(cudaMalloc(&p->d_jobs, (size_t)nblocks * sizeof(xin_gpu_dq_block)), "dq plan") ||
        xg_cuda_check(cudaMemcpy(p->d_jobs, blocks, (size_t)nblocks * sizeof(xin_gpu_dq_block), cudaMemcpyHostToDevice), "dq plan") ||
        xg_cuda_check(cudaMalloc(&p->d_area, bytes), "dq plan")) {
        if (nscan >= (1ull << 32)) xg_set_error(XIN_GPU_ERR_ARG, "dq_plan_create: too many coefficients");
        xin_gpu_dq_plan_destroy(p);
        return xin_gpu_last_status();
    }
    xg_dq_area_bytes(nsets, nblocks, nscan, p->ctas * XG_DQ_PAIRS, &p->area, p->d_area);
    *out = p;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_dq_plan_run(xin_gpu_dq_plan *p, const XG_COEFF *t, XG_COEFF *q, XG_COEFF *r, uint64_t *nz,
                                   const xin_gpu_prob *ctx_sets, void *stream)
{
    xin_gpu_clear_error();
    if (!p || !t || !q || !r || !nz || !ctx_sets) {
        xg_set_error(XIN_GPU_ERR_ARG, "dq_plan_run: bad argument");
        return XIN_GPU_ERR_ARG;
    }
    cudaGetLastError();
    return xg_dq_enqueue(p->d_jobs, p->d_soff, p->nblocks, (const xg_coef *)t, (xg_coef *)q, (xg_coef *)r,
                         (unsigned long long *)nz, ctx_sets, p->nsets, p->area, p->ctas, 1, (cudaStream_t)stream);
}

extern "C" void xin_gpu_dq_plan_destroy(xin_gpu_dq_plan *p)
{
    if (!p) return;
    cudaFree(p->d_jobs);
    cudaFree(p->d_soff);
    cudaFree(p->d_area);
    delete p;
}

extern "C" int xin_gpu_dep_quant_batch_device(const xin_gpu_dq_block *blocks, int32_t nblocks, const XG_COEFF *t, XG_COEFF *q,
                                              XG_COEFF *r, uint64_t *nz, size_t ncoeffs, const xin_gpu_prob *ctx_sets,
                                              int32_t nsets, void *stream)
{
    xin_gpu_dq_plan *p = nullptr;
    int st = xin_gpu_dq_plan_create(blocks, nblocks, ncoeffs, nsets, &p);
    if (st) return st;
    st = xin_gpu_dq_plan_run(p, t, q, r, nz, ctx_sets, stream);
    if (!st) st = xg_cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "dq sync");
    xin_gpu_dq_plan_destroy(p);
    return st;
}

extern "C" int xin_gpu_dep_quant_batch(const xin_gpu_dq_block *blocks, int32_t nblocks, const XG_COEFF *t, XG_COEFF *q,
                                       XG_COEFF *r, uint64_t *nz, size_t ncoeffs, const xin_gpu_prob *ctx_sets, int32_t nsets)
{
    xin_gpu_clear_error();
    if (!blocks || nblocks <= 0 || !t || !q || !r || !nz || !ctx_sets || nsets <= 0) {
        xg_set_error(XIN_GPU_ERR_ARG, "dep_quant_batch: bad argument");
        return XIN_GPU_ERR_ARG;
    }
    XgThread *th = xg_thread();
    if (!th) return xin_gpu_last_status();
    xin_gpu_dq_plan *p = nullptr;
    int st = xin_gpu_dq_plan_create(blocks, nblocks, ncoeffs, nsets, &p);
    if (st) return st;
    size_t bytes = ncoeffs * sizeof(xg_coef), cbytes = (size_t)nsets * XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob);
    xg_coef *d_t = nullptr, *d_q = nullptr, *d_r = nullptr;
    unsigned long long *d_nz = nullptr;
    xin_gpu_prob *d_c = nullptr;
    if (xg_cuda_check(cudaMalloc(&d_t, bytes), "dq alloc") || xg_cuda_check(cudaMalloc(&d_q, bytes), "dq alloc") ||
        xg_cuda_check(cudaMalloc(&d_r, bytes), "dq alloc") || xg_cuda_check(cudaMalloc(&d_nz, (size_t)nblocks * 8), "dq alloc") ||
        xg_cuda_check(cudaMalloc(&d_c, cbytes), "dq alloc"))
        st = XIN_GPU_ERR_CUDA;
    if (!st && (xg_cuda_check(cudaMemcpyAsync(d_t, t, bytes, cudaMemcpyHostToDevice, th->stream), "dq h2d") ||
                xg_cuda_check(cudaMemcpyAsync(d_c, ctx_sets, cbytes, cudaMemcpyHostToDevice, th->stream), "dq h2d") ||
                xg_cuda_check(cudaMemsetAsync(d_q, 0, bytes, th->stream), "dq clear") ||
                xg_cuda_check(cudaMemsetAsync(d_r, 0, bytes, th->stream), "dq clear")))
        st = XIN_GPU_ERR_CUDA;
    if (!st) st = xin_gpu_dq_plan_run(p, (const XG_COEFF *)d_t, (XG_COEFF *)d_q, (XG_COEFF *)d_r, (uint64_t *)d_nz, d_c, th->stream);
    if (!st && (xg_cuda_check(cudaMemcpyAsync(q, d_q, bytes, cudaMemcpyDeviceToHost, th->stream), "dq d2h") ||
                xg_cuda_check(cudaMemcpyAsync(r, d_r, bytes, cudaMemcpyDeviceToHost, th->stream), "dq d2h") ||
                xg_cuda_check(cudaMemcpyAsync(nz, d_nz, (size_t)nblocks * 8, cudaMemcpyDeviceToHost, th->stream), "dq d2h") ||
                xg_sync(th)))
        st = XIN_GPU_ERR_CUDA;
    cudaFree(d_t); cudaFree(d_q); cudaFree(d_r); cudaFree(d_nz); cudaFree(d_c);
    xin_gpu_dq_plan_destroy(p);
    return st;
}

/* ---------------------------------------------------- per-call drop-in form */

/* XinDepQuant (h266_encoder/include/h266_func_struct.h:664-676).  Reads the
 * context pointer of the reference's xin_dep_quant, the mode of its
 * xin_fast_md_buf and the TU count of the xin_full_md_buf behind it (offsets
 * in xingpu.h); the scan order is the standard one, so tu is not read.
 * Writes q and r over min(width,32) x min(height,32), as the reference does. */
extern "C" void XinGpuDepQuant(void *depQuant, void *fastBuf, void *tu, XG_COEFF *tCoeff, XG_COEFF *rCoeff, XG_COEFF *qCoeff,
                               intptr_t coeffStride, uint32_t qp, int32_t width, int32_t height, uint64_t *nzCGBitMapRs,
                               uint32_t compId)
{
    (void)tu;
    XgThread *th = xg_thread();
    if (!th) return;
    (void)cudaGetLastError();
    xin_gpu_clear_error();
    if (!depQuant || !fastBuf || !tCoeff || !rCoeff || !qCoeff || !nzCGBitMapRs || compId > 2 || qp > 51 ||
        width < 4 || width > 64 || height < 4 || height > 64 || (width & (width - 1)) || (height & (height - 1)) ||
        coeffStride < width) {
        xg_set_error(XIN_GPU_ERR_ARG, "XinGpuDepQuant: bad argument");
        return;
    }
    if (!xg_dq_tables() || !xg_dq_resident_ctas()) return;
    const xin_gpu_prob *ctx = *(const xin_gpu_prob *const *)((const char *)depQuant + XIN_GPU_DQ_CONTEXT_OFFSET);
    const void *full = *(const void *const *)((const char *)fastBuf + XIN_GPU_FASTBUF_FULLBUF_OFFSET);
    const uint32_t type = *(const uint32_t *)((const char *)fastBuf + XIN_GPU_FASTBUF_TYPE_OFFSET);
    if (!ctx || !full) { xg_set_error(XIN_GPU_ERR_ARG, "XinGpuDepQuant: no context or no full-RD buffer"); return; }
    const uint32_t tunum = *(const uint32_t *)((const char *)full + XIN_GPU_FULLBUF_TUNUM_OFFSET);
    const int ew = width < 32 ? width : 32, eh = height < 32 ? height : 32;
    xin_gpu_dq_block jb;
    jb.offset = 0; jb.stride = (uint16_t)ew;
    jb.log2_w = (uint8_t)(31 - __builtin_clz((unsigned)width)); jb.log2_h = (uint8_t)(31 - __builtin_clz((unsigned)height));
    jb.qp = (uint8_t)qp; jb.comp = (uint8_t)compId;
    jb.root_cbf = (uint8_t)(compId == 0 && type != XIN_GPU_INTRA_MODE && tunum == 1);
    jb.reserved = 0; jb.ctx_set = 0;
    const size_t cbytes = XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob);
    const xg_coef *dt = (const xg_coef *)xg_stage_in(th, tCoeff, coeffStride, ew, eh, sizeof(xg_coef));
    xg_coef *dq = (xg_coef *)xg_dalloc(th, (size_t)ew * eh * sizeof(xg_coef));
    xg_coef *dr = (xg_coef *)xg_dalloc(th, (size_t)ew * eh * sizeof(xg_coef));
    unsigned long long *dnz = (unsigned long long *)xg_dalloc(th, 8);
    xin_gpu_dq_block *dj = (xin_gpu_dq_block *)xg_stage_in(th, &jb, 1, 1, 1, sizeof jb);
    xin_gpu_prob *dc = (xin_gpu_prob *)xg_stage_in(th, ctx, (intptr_t)cbytes, cbytes, 1, 1);
    const uint32_t zero = 0;
    uint32_t *dso = (uint32_t *)xg_stage_in(th, &zero, 1, 1, 1, 4);
    const size_t abytes = xg_dq_area_bytes(1, 1, (size_t)ew * eh, XG_DQ_PAIRS, nullptr, nullptr);
    char *area = (char *)xg_dalloc(th, abytes);
    if (!dt || !dq || !dr || !dnz || !dj || !dc || !dso || !area) return;
    XgDqArea A;
    xg_dq_area_bytes(1, 1, (size_t)ew * eh, XG_DQ_PAIRS, &A, area);
    if (xg_dq_enqueue(dj, dso, 1, dt, dq, dr, dnz, dc, 1, A, 1, 0, th->stream)) return;
    if (xg_stage_out(th, qCoeff, coeffStride, dq, ew, eh, sizeof(xg_coef)) ||
        xg_stage_out(th, rCoeff, coeffStride, dr, ew, eh, sizeof(xg_coef)) ||
        xg_cuda_check(cudaMemcpyAsync(th->hbuf, dnz, 8, cudaMemcpyDeviceToHost, th->stream), "d2h") || xg_sync(th))
        return;
    *nzCGBitMapRs = *(uint64_t *)th->hbuf;
}

#endif
