/*
 * xg_dq.cuh -- dependent quantisation (trellis-coded quantisation, H.266 8.7.3
 * with the encoder's rate-distortion trellis) for batches of transform blocks:
 * the reference's Xin266DepQuant (h266_encoder/source/h266_dep_quant.c:1789),
 * reached through xin_func_struct.pfXinDepQuant (h266_encoder/include/h266_func_struct.h:795,
 * called from h266_trans_quant.c:192).
 *
 * Work split.  A block is walked coefficient by coefficient in reverse scan
 * order; at each coefficient four quantiser states each keep the cheapest path
 * that ends in them.  One quad of lanes owns one block, lane s owning state s,
 * so a warp runs eight blocks side by side.  Per coefficient every lane prices
 * the three candidates its state offers (level A, level B, zero), the quad
 * swaps them with two shuffle exchanges, and lane t keeps the cheapest path
 * into state t (the fixed transition pattern of the reference: 0->{0,2},
 * 1->{2,0}, 2->{1,3}, 3->{3,1}, plus "skip this sub-block" and "start here").
 *
 * State layout.  The reference copies a 48-byte template (levels and
 * neighbour sums) and a per-path copy of every earlier sub-block's levels with
 * each transition.  Here a state carries only the 16 levels of its current
 * sub-block (four registers, clipped like the reference's bytes) and their
 * parities; the neighbour sums at a position are recomputed from those levels
 * plus the outside-neighbour template that was built when the sub-block was
 * entered.  Earlier sub-blocks are kept once per (sub-block, state) in a
 * 16-slot ring in shared memory (the farthest right / below neighbour of a
 * 4x4 sub-block in a 32x32 diagonal scan is 15 sub-blocks away); a path's
 * sub-block context is a 64-bit significance map plus a 2-bit state tag per
 * ring slot.  The decisions (one byte per state) and the quantisation index of
 * each position go to a per-quad scratch area in global memory; after the
 * trellis, lane 0 of the quad walks them back and dequantises along the state
 * machine.
 *
 * The sub-block steps of all quads in a warp are phase aligned (each quad
 * starts at the top of the sub-block holding its last significant position),
 * so the sub-block boundary work never diverges within a warp.
 */
#ifndef XG_DQ_CUH
#define XG_DQ_CUH

#include <math.h>
#include <mutex>
#include <vector>

#define XG_DQ_QUADS    32                       /* blocks per CTA (4 warps x 8 quads) */
#define XG_DQ_THREADS  (XG_DQ_QUADS * 4)
#define XG_DQ_MAXN     1024                     /* coefficients of the 32x32 region */
#define XG_DQ_SCR_WORDS (XG_DQ_MAXN + XG_DQ_MAXN / 2)   /* per quad: decisions (u32) + indices (u16) */
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

__constant__ uint32_t c_dq_frac[256][2];        /* bits of a bin at probability state (p0 + p1) >> 8 */
__constant__ int32_t  c_dq_shape_off[16];       /* start of each region shape in the scan tables */

struct XgDqTables {
    uint2 *d_step;              /* per shape, per scan index: position, type, inside neighbours */
    uint4 *d_tpl;               /* per shape, per scan index: outside neighbours */
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
    std::vector<uint4> tpl;
    int32_t off[16];
    static const int dx[5] = { 1, 2, 1, 0, 0 }, dy[5] = { 0, 0, 1, 1, 2 };
    for (int sh = 0; sh < 16; sh++) {
        int ew = 4 << (sh >> 2), eh = 4 << (sh & 3), n = ew * eh, ws = ew >> 2, hs = eh >> 2;
        off[sh] = (int32_t)step.size();
        std::vector<int> cx, cy, gx, gy;
        xg_dq_diag(4, 4, cx, cy);
        xg_dq_diag(ws, hs, gx, gy);
        std::vector<int> px(n), py(n), sid(n);
        for (int b = 0; b < ws * hs; b++)
            for (int i = 0; i < 16; i++) {
                int k = b * 16 + i;
                px[k] = gx[b] * 4 + cx[i]; py[k] = gy[b] * 4 + cy[i];
                sid[py[k] * ew + px[k]] = k;
            }
        for (int k = 0; k < n; k++) {
            int beg = k & ~15, in = k & 15;
            int ins[5], outs[5], ni = 0, no = 0;
            for (int j = 0; j < 5; j++) {
                int x = px[k] + dx[j], y = py[k] + dy[j];
                if (x >= ew || y >= eh) continue;
                int q = sid[y * ew + x];
                if (q < beg + 16) ins[ni++] = q - beg; else outs[no++] = q;
            }
            int ptype = (in == 15 && k > 16 && k < n - 1) ? 1 : (in == 0 && k > 0 && k < n - 16) ? 2 : 0;
            int braster = gy[k >> 4] * ws + gx[k >> 4];
            /* significance / gtx context offsets of the position's diagonal, luma and chroma
             * (h266_dep_quant.c:466-476): luma sig 0/4/8, gtx 1/6/11/16; chroma sig 0/4, gtx 1/6 */
            const int dg = px[k] + py[k];
            const uint32_t ls = dg < 2 ? 2 : dg < 5 ? 1 : 0, lg = dg < 1 ? 3 : dg < 3 ? 2 : dg < 10 ? 1 : 0;
            const uint32_t cs = dg < 2 ? 1 : 0, cg = dg < 1 ? 1 : 0;
            uint2 e;
            e.x = (uint32_t)px[k] | (uint32_t)py[k] << 5 | (uint32_t)ptype << 10 | (uint32_t)ni << 12 | (uint32_t)braster << 15 |
                  ls << 21 | lg << 23 | cs << 25 | cg << 26;
            e.y = 0;
            for (int j = 0; j < ni; j++) e.y |= (uint32_t)ins[j] << (4 * j);
            step.push_back(e);
            uint32_t nb[5] = { 0, 0, 0, 0, 0 };
            for (int j = 0; j < no; j++) {
                int sb = outs[j] >> 4;
                nb[j] = (uint32_t)sb | (uint32_t)(outs[j] & 15) << 6 | (uint32_t)(gy[sb] * ws + gx[sb]) << 10;
            }
            tpl.push_back(make_uint4((uint32_t)no | nb[0] << 16, nb[1] | nb[2] << 16, nb[3] | nb[4] << 16, 0));
        }
    }
    std::vector<XgDqParam> par(9 * 52);
    for (int lg = 4; lg <= 12; lg++)
        for (int qp = 0; qp < 52; qp++) xg_dq_param(qp, lg, &par[(lg - 4) * 52 + qp]);
    if (xg_cuda_check(cudaMemcpyToSymbol(c_dq_frac, frac, sizeof frac), "dq tables") ||
        xg_cuda_check(cudaMemcpyToSymbol(c_dq_shape_off, off, sizeof off), "dq tables") ||
        xg_cuda_check(cudaMalloc(&g_dq.d_step, step.size() * sizeof(uint2)), "dq tables") ||
        xg_cuda_check(cudaMalloc(&g_dq.d_tpl, tpl.size() * sizeof(uint4)), "dq tables") ||
        xg_cuda_check(cudaMalloc(&g_dq.d_par, par.size() * sizeof(XgDqParam)), "dq tables") ||
        xg_cuda_check(cudaMemcpy(g_dq.d_step, step.data(), step.size() * sizeof(uint2), cudaMemcpyHostToDevice), "dq tables") ||
        xg_cuda_check(cudaMemcpy(g_dq.d_tpl, tpl.data(), tpl.size() * sizeof(uint4), cudaMemcpyHostToDevice), "dq tables") ||
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
 * reference (:172-173). */
__global__ void k_dq_rates(const xin_gpu_prob *__restrict__ sets, XgDqRates *__restrict__ out)
{
    const xin_gpu_prob *ctx = sets + (size_t)blockIdx.x * XIN_GPU_NUM_CTX;
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

/* 16-byte aligned: the ring is written with 16-byte stores */
struct __align__(16) XgDqQuad {
    uint16_t tpl[4][16];            /* outside-neighbour template per sub-block context */
    uint32_t ring[16][4][4];        /* levels of earlier sub-blocks: [slot][state][16 bytes] */
    int32_t  last[2][32];           /* rate of the last position, x and y */
    XgDqRates rt;                   /* the block's rate tables (its context set and channel) */
};
static_assert(sizeof(XgDqQuad) % 16 == 0 && offsetof(XgDqQuad, ring) % 16 == 0, "ring rows must stay 16-byte aligned");
struct XgDqSmem {
    XgDqQuad quad[XG_DQ_QUADS];
    int32_t  rice[4][32];           /* abs_remainder bits, Rice parameter k, value n */
};

__device__ __forceinline__ uint32_t xg_dq_byte(uint32_t l0, uint32_t l1, uint32_t l2, uint32_t l3, int j)
{
    uint32_t w = (j & 8) ? ((j & 4) ? l3 : l2) : ((j & 4) ? l1 : l0);
    return (w >> ((j & 3) * 8)) & 255u;
}

/* Rice parameter from a neighbour sum (H.266 Table 128) */
__device__ __forceinline__ int xg_dq_rpar(int v) { return v < 7 ? 0 : v < 14 ? 1 : v < 28 ? 2 : 3; }

__device__ __forceinline__ long long xg_dq_shfl64(unsigned m, long long v, int src)
{
    int lo = __shfl_sync(m, (int)(unsigned long long)v, src, 4);
    int hi = __shfl_sync(m, (int)((unsigned long long)v >> 32), src, 4);
    return (long long)(((unsigned long long)(unsigned)hi << 32) | (unsigned)lo);
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

/* ---- pass 3: the trellis.  One CTA = 4 warps x 8 quads; each warp takes the
 * next 8 blocks of the ordered list (so its quads walk the same number of
 * sub-blocks). */
/* min blocks 1: the compiler keeps more of the step in registers (137 here),
 * which shortens the serial step; the trellis is bound by that latency, not by
 * the number of resident warps */
__global__ void __launch_bounds__(XG_DQ_THREADS, 1)
k_dq(const xin_gpu_dq_block *__restrict__ jobs, int njobs, int *__restrict__ counter, const int *__restrict__ counts,
     const int32_t *__restrict__ order, const int32_t *__restrict__ firsts, const uint32_t *__restrict__ soff,
     const xg_coef *__restrict__ tscan, xg_coef *__restrict__ qout, xg_coef *__restrict__ rout,
     unsigned long long *__restrict__ nzout, const xin_gpu_prob *__restrict__ sets,
     const XgDqRates *__restrict__ rates, const uint2 *__restrict__ step_tab, const uint4 *__restrict__ tpl_tab,
     const XgDqParam *__restrict__ par_tab, uint32_t *__restrict__ scratch)
{
    extern __shared__ __align__(16) unsigned char xg_dq_raw[];
    XgDqSmem &sm = *reinterpret_cast<XgDqSmem *>(xg_dq_raw);
    const int lane = threadIdx.x & 31, qd = lane >> 2, s = lane & 3;
    const unsigned qmask = 0xFu << (qd * 4);
    XgDqQuad &Q = sm.quad[threadIdx.x >> 2];
    uint32_t *codes = scratch + (size_t)(blockIdx.x * XG_DQ_QUADS + (threadIdx.x >> 2)) * XG_DQ_MAXN;
    const int ntr = njobs - counts[0];

    for (int i = threadIdx.x; i < 128; i += blockDim.x) {
        int k = i >> 5, n = i & 31, p = n >> k;
        int bits;
        if (p < 6) bits = p + 1 + k;
        else { unsigned m = (unsigned)(n - (6 << k)); bits = 6 + 2 * (31 - __clz((int)((m >> (k + 1)) + 1))) + 1 + (k + 1); }
        sm.rice[k][n] = bits << 15;
    }
    __syncthreads();

    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(counter, 8);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= ntr) break;
        const bool has = base + qd < ntr;
        const int job = has ? order[base + qd] : 0;

        /* ---- block set-up (every lane of the quad holds the same values) ---- */
        const xin_gpu_dq_block jb = jobs[job];
        const int first = has ? firsts[job] : -1;
        const int lgw = jb.log2_w, lgh = jb.log2_h, w = 1 << lgw, h = 1 << lgh;
        const int ew = min(w, 32), eh = min(h, 32), ws = ew >> 2, hs = eh >> 2;
        const int shape = (min(lgw, 5) - 2) * 4 + (min(lgh, 5) - 2);
        const uint2 *ST = step_tab + c_dq_shape_off[shape];
        const uint4 *TT = tpl_tab + c_dq_shape_off[shape];
        const XgDqParam P = par_tab[(lgw + lgh - 4) * 52 + jb.qp];
        const int luma = jb.comp == 0;
        const XgDqRates *RT = rates + jb.ctx_set * 2 + (luma ? 0 : 1);
        const xin_gpu_prob *CX = sets + (size_t)jb.ctx_set * XIN_GPU_NUM_CTX;
        const int stride = jb.stride;
        const xg_coef *TS = tscan + soff[job];
        xg_coef *QO = qout + jb.offset, *RO = rout + jb.offset;

        /* last-position rates (Xin266SetLastCoeffOffset, h266_dep_quant.c:208-283): lane 0 x, lane 1 y */
        if (has && s < 2) {
            const int xy = s, size = xy ? h : w, lg = xy ? lgh : lgw, nn = min(size, 32);
            const int shift = luma ? (lg + 1) >> 2 : min((1 << lg) >> 3, 2);
            const int cbase = luma ? (lg == 2 ? 0 : lg == 3 ? 3 : lg == 4 ? 6 : lg == 5 ? 10 : 15) + (xy ? XG_DQC_LASTY_L : XG_DQC_LASTX_L)
                                   : (xy ? XG_DQC_LASTY_C : XG_DQC_LASTX_C);
            uint32_t off = 0;
            if (xy) {
                int cc = (luma && jb.root_cbf) ? XG_DQC_ROOT_CBF : jb.comp == 0 ? XG_DQC_CBF_Y : jb.comp == 1 ? XG_DQC_CBF_U : XG_DQC_CBF_V;
                const uint32_t *cb = xg_dq_bits(CX, cc);
                off = cb[1] - cb[0];
            }
            const int gmax = nn - 1 < 4 ? nn - 1 : 2 * (31 - __clz(nn - 1)) + (((nn - 1) >> (30 - __clz(nn - 1))) & 1);
            uint32_t acc = 0, cbits = 0;
            int gdone = 0;
            /* groups in increasing order; positions map to non-decreasing groups, so one pass fills the table */
            for (int p = 0; p < nn; p++) {
                const int g = p < 4 ? p : 2 * (31 - __clz(p)) + ((p >> (30 - __clz(p))) & 1);
                while (gdone <= g) {
                    const uint32_t suf = gdone > 3 ? (uint32_t)(((gdone - 2) >> 1) << 15) : 0;
                    if (gdone == gmax) cbits = acc + suf + off;
                    else {
                        const uint32_t *b = xg_dq_bits(CX, cbase + (gdone >> shift));
                        cbits = acc + b[0] + suf + off;
                        acc += b[1];
                    }
                    gdone++;
                }
                Q.last[xy][p] = (int32_t)cbits;
            }
        }
        if (has) {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(RT);
            uint32_t *dst = reinterpret_cast<uint32_t *>(&Q.rt);
            for (int i = s; i < (int)(sizeof(XgDqRates) / 4); i += 4) dst[i] = __ldg(src + i);
        }
        __syncwarp(0xffffffffu);

        /* ---- trellis state of lane s (state s) ---- */
        long long cost = XG_DQ_INF;
        uint32_t l0 = 0, l1 = 0, l2 = 0, l3 = 0, par16 = 0;
        int rem = 4, nsig = 0, ref = -1, signb = 0;
        unsigned long long cflags = 0;
        uint32_t cvers = 0;
        long long skcost = XG_DQ_INF;
        int skrem = 4, skref = -1, sksignb = 0;
        const int regbins = ew * eh * XG_DQ_REG_BINS / 16;
        const int top = first | 15;
        int nsteps = first >= 0 ? top + 1 : 0;
        nsteps = __reduce_max_sync(0xffffffffu, nsteps);
        const uint32_t *sigset = &Q.rt.sig[s > 1 ? s - 1 : 0][0][0];
        const int src1 = s == 1 ? 2 : s == 2 ? 1 : s;      /* first exchange reads candidate A/Z */
        const int src2 = src1 ^ 1;                         /* second exchange reads candidate B */
        /* coefficients of the current / next sub-block: lane s holds scan positions 4s..4s+3 */
        xg_coef c0 = 0, c1 = 0, c2 = 0, c3 = 0, n0 = 0, n1 = 0, n2 = 0, n3 = 0;
        uint4 ea = make_uint4(0, 0, 0, 0), eb = make_uint4(0, 0, 0, 0);
        auto load_sb = [&](int sb, xg_coef &a0, xg_coef &a1, xg_coef &a2, xg_coef &a3) {
            const xg_coef *src = TS + sb * 16 + 4 * s;
#if XG_BITDEPTH == 8
            const uint2 raw = *reinterpret_cast<const uint2 *>(src);
            a0 = (xg_coef)(raw.x & 0xFFFF); a1 = (xg_coef)(raw.x >> 16); a2 = (xg_coef)(raw.y & 0xFFFF); a3 = (xg_coef)(raw.y >> 16);
#else
            const int4 raw = *reinterpret_cast<const int4 *>(src);
            a0 = raw.x; a1 = raw.y; a2 = raw.z; a3 = raw.w;
#endif
        };

        for (int stp = 0; stp < nsteps; stp++) {
            const int k = top - stp;
            if (k < 0 || k > first) continue;                      /* uniform within the quad */
            const int in = k & 15, sb = k >> 4;
            if (k == first || in == 15) {
                if (k == first) load_sb(sb, c0, c1, c2, c3);
                else { c0 = n0; c1 = n1; c2 = n2; c3 = n3; }
                if (sb > 0) load_sb(sb - 1, n0, n1, n2, n3);
                const uint4 *e4 = reinterpret_cast<const uint4 *>(ST + sb * 16 + 4 * s);
                ea = __ldg(e4); eb = __ldg(e4 + 1);
            }
            const int sub = in & 3, srcl = in >> 2;
            const xg_coef mine = sub == 0 ? c0 : sub == 1 ? c1 : sub == 2 ? c2 : c3;
            const uint32_t mex = sub == 0 ? ea.x : sub == 1 ? ea.z : sub == 2 ? eb.x : eb.z;
            const uint32_t mey = sub == 0 ? ea.y : sub == 1 ? ea.w : sub == 2 ? eb.y : eb.w;
            int av = __shfl_sync(qmask, (int)mine, srcl, 4);
            uint2 se;
            se.x = __shfl_sync(qmask, mex, srcl, 4);
            se.y = __shfl_sync(qmask, mey, srcl, 4);
            av = av < 0 ? -av : av;
            const int px = se.x & 31, py = (se.x >> 5) & 31, ptype = (se.x >> 10) & 3, nin = (se.x >> 12) & 7;

            /* context of this state at position k */
            uint32_t tv = ref >= 0 ? Q.tpl[ref][in] : 0u;
            int sum = tv & 127, a1 = (tv >> 7) & 31, cnt = tv >> 12;
            if (l0 | l1 | l2 | l3) {
#pragma unroll
                for (int u = 0; u < 5; u++) {
                    if (u < nin) {
                        int j = (se.y >> (4 * u)) & 15;
                        int l = (int)xg_dq_byte(l0, l1, l2, l3, j);
                        if (l) { sum += l; cnt++; a1 += min(4 + (int)((par16 >> j) & 1), l); }
                    }
                }
                sum = min(sum, 255);
            }
            const int sigoff = 4 * (int)(luma ? (se.x >> 21) & 3 : (se.x >> 25) & 1);
            const int gtxoff = 1 + 5 * (int)(luma ? (se.x >> 23) & 3 : (se.x >> 26) & 1);
            uint32_t sig0 = 0, sig1 = 0;
            const uint32_t *gtx = Q.rt.gtx[0];
            int rice, rzero = 0;
            if (rem >= 4) {
                const uint32_t *sg = sigset + 2 * (sigoff + min((a1 + 1) >> 1, 3));
                sig0 = sg[0]; sig1 = sg[1];
                gtx = Q.rt.gtx[gtxoff + min(a1 - cnt, 4)];
                rice = xg_dq_rpar(min(max(sum - 20, 0), 31));
            } else {
                rice = xg_dq_rpar(min(sum, 31));
                rzero = (s < 2 ? 1 : 2) << rice;
            }

            /* pre-quantisation (Xin266PreQuantCoeff, h266_dep_quant.c:920-952) */
            const long long org = (long long)av * P.qScale;
            long long qi = (org + P.qAdd) >> P.qShift;
            const int q = (int)(qi < 1 ? 1 : qi > P.maxQIdx ? P.maxQIdx : qi);
            const long long bse = (long long)((unsigned long long)q * (unsigned long long)P.distStepAdd -
                                              (unsigned long long)org * (unsigned long long)P.distOrgFact);
            auto ddof = [&](int i) -> long long {
                int kk = (i - q) & 3;
                long long m = (long long)((unsigned long long)(bse + kk * P.distStepAdd) * (unsigned long long)(long long)(q + kk));
                return (m + P.distAdd) >> P.distShift;
            };
            auto lvof = [&](int i) -> int { return (q + ((i - q) & 3) + 1) >> 1; };
            /* lane s prices quantisation index class s; lanes 0 / 1 take classes 0 and 2,
             * lanes 2 / 3 classes 3 and 1 (A and B), even lanes also their own for "start" */
            const int iA = s < 2 ? 0 : 3, iB = s < 2 ? 2 : 1;
            const int lvA = lvof(iA), lvB = lvof(iB);
            const long long ddS = ddof(s);
            const long long ddA = xg_dq_shfl64(qmask, ddS, iA), ddB = xg_dq_shfl64(qmask, ddS, iB);

            /* candidates of this state (Xin266CheckRdCosts, h266_dep_quant.c:954-1046) */
            long long ca = cost + ddA, cb = cost + ddB, cz = cost;
            bool zero_ok = true;
            if (rem >= 4) {
                ca += gtx[lvA < 4 ? lvA : 4 + (lvA & 1)] + (lvA >= 4 ? sm.rice[rice][min((lvA - 4) >> 1, 31)] : 0);
                cb += gtx[lvB < 4 ? lvB : 4 + (lvB & 1)] + (lvB >= 4 ? sm.rice[rice][min((lvB - 4) >> 1, 31)] : 0);
                if (ptype == 1) {
                    const uint32_t sb1 = Q.rt.sbb[signb][1];
                    ca += sb1 + sig1; cb += sb1 + sig1; cz += sb1 + sig0;
                } else if (ptype == 0 || nsig) {
                    ca += sig1; cb += sig1; cz += sig0;
                } else zero_ok = false;
            } else {
                ca += (1 << 15) + sm.rice[rice][lvA <= rzero ? lvA - 1 : min(lvA, 31)];
                cb += (1 << 15) + sm.rice[rice][lvB <= rzero ? lvB - 1 : min(lvB, 31)];
                cz += sm.rice[rice][rzero];
            }
            long long caz;
            int saz;
            if (!zero_ok || ca < cz) { caz = ca; saz = iA; } else { caz = cz; saz = 4; }

            /* exchange: first every lane publishes A/Z, then B */
            const long long r1 = xg_dq_shfl64(qmask, caz, src1), r2 = xg_dq_shfl64(qmask, cb, src2);
            const int sels = __shfl_sync(qmask, saz | iB << 4, src1, 4);
            const int sels2 = __shfl_sync(qmask, saz | iB << 4, src2, 4);
            long long cc1, cc2;
            int s1, s2, f1, f2;
            if (s < 2) { cc1 = r1; s1 = sels & 15; f1 = src1; cc2 = r2; s2 = sels2 >> 4; f2 = src2; }
            else       { cc1 = r2; s1 = sels2 >> 4; f1 = src2; cc2 = r1; s2 = sels & 15; f2 = src1; }

            /* decision for target state s */
            long long dc = XG_DQ_INF >> 1;
            int dsel = 7, dfrom = -2;
            if (cc1 < dc) { dc = cc1; dsel = s1; dfrom = f1; }
            if (cc2 < dc) { dc = cc2; dsel = s2; dfrom = f2; }
            if (ptype == 2) {
                long long c = skcost + Q.rt.sbb[sksignb][0];
                if (c < dc) { dc = c; dsel = 4; dfrom = 4 + s; }
            }
            if ((s & 1) == 0) {
                const int lvs = lvof(s);
                long long c = ddS + Q.last[0][px] + Q.last[1][py] + Q.rt.gtx[0][lvs < 4 ? lvs : 4 + (lvs & 1)] +
                              (lvs >= 4 ? sm.rice[0][min((lvs - 4) >> 1, 31)] : 0);
                if (c < dc) { dc = c; dsel = s; dfrom = -1; }
            }
            const int dlv = dsel == 4 ? 0 : dsel == 7 ? -1 : lvof(dsel);
            uint32_t code = (uint32_t)((dfrom + 2) | dsel << 4) << (8 * s);
            code |= __shfl_xor_sync(qmask, code, 1, 4);
            code |= __shfl_xor_sync(qmask, code, 2, 4);
            if (s == 0) codes[k] = code;

            if (ptype == 1) { skcost = cost; skrem = rem; skref = ref; sksignb = signb; }

            /* state update (Xin266UpdateState / Xin266UpdateStateEOS, h266_dep_quant.c:1224-1536) */
            const int psrc = dfrom >= 4 ? dfrom - 4 : dfrom >= 0 ? dfrom : s;
            const uint32_t pk = (uint32_t)(rem & 0xFFFF) | (uint32_t)nsig << 16 | (uint32_t)(ref + 1) << 22 | (uint32_t)signb << 25;
            const uint32_t spk = (uint32_t)(skrem & 0xFFFF) | (uint32_t)(skref + 1) << 16;
            const uint32_t p0 = __shfl_sync(qmask, l0, psrc, 4), p1 = __shfl_sync(qmask, l1, psrc, 4);
            const uint32_t p2 = __shfl_sync(qmask, l2, psrc, 4), p3 = __shfl_sync(qmask, l3, psrc, 4);
            const uint32_t ppar = __shfl_sync(qmask, par16, psrc, 4);
            const uint32_t ppk = __shfl_sync(qmask, pk, psrc, 4), pspk = __shfl_sync(qmask, spk, psrc, 4);
            cost = dc;
            if (k == 0) continue;
            const int p_rem = (int)(int16_t)(ppk & 0xFFFF), p_nsig = (ppk >> 16) & 31, p_ref = (int)((ppk >> 22) & 7) - 1;
            const int p_signb = (ppk >> 25) & 1;
            const int lv = dlv;
            if (in != 0) {
                if (dfrom >= 0) {
                    nsig = p_nsig + (lv != 0); ref = p_ref; signb = p_signb;
                    rem = p_rem - 1;
                    if (rem >= 4) rem -= lv < 2 ? lv : 3;
                    l0 = p0; l1 = p1; l2 = p2; l3 = p3; par16 = ppar;
                } else if (dfrom == -1) {
                    nsig = 1; ref = -1;
                    rem = regbins - (lv < 2 ? lv : 3);
                    l0 = l1 = l2 = l3 = 0; par16 = 0;
                }
                if (dfrom > -2 && lv) {
                    const uint32_t b = (uint32_t)min(lv, 255), sh = (in & 3) * 8, m = ~(255u << sh);
                    const int wi = in >> 2;
                    if (wi == 0) l0 = (l0 & m) | b << sh; else if (wi == 1) l1 = (l1 & m) | b << sh;
                    else if (wi == 2) l2 = (l2 & m) | b << sh; else l3 = (l3 & m) | b << sh;
                    par16 = (par16 & ~(1u << in)) | (uint32_t)(lv & 1) << in;
                }
            } else {
                /* first coefficient (in scan order) of sub-block sb: close it and open sb - 1 */
                const int slot = sb & 15;
                int srcref = -1;
                if (dfrom >= 4) {
                    nsig = 0; rem = (int)(int16_t)(pspk & 0xFFFF); srcref = (int)((pspk >> 16) & 7) - 1;
                    l0 = l1 = l2 = l3 = 0; par16 = 0;
                } else if (dfrom >= 0) {
                    nsig = p_nsig + (lv != 0);
                    rem = p_rem - 1;
                    if (rem >= 4) rem -= lv < 2 ? lv : 3;
                    l0 = p0; l1 = p1; l2 = p2; l3 = p3; par16 = ppar; srcref = p_ref;
                } else if (dfrom == -1) {
                    nsig = 1; rem = regbins;
                    if (rem >= 4) rem -= lv < 2 ? lv : 3;
                    l0 = l1 = l2 = l3 = 0; par16 = 0;
                }
                const bool upd = dfrom > -2;
                if (upd) {
                    const uint32_t cap = 254u + (uint32_t)(lv & 1);
                    l0 = (l0 & ~255u) | min((uint32_t)lv, cap);
                }
                /* sub-block context of the new path: the predecessor's plus this sub-block */
                const int cr = srcref >= 0 ? srcref : s;
                const uint32_t fl = __shfl_sync(qmask, (uint32_t)cflags, cr, 4);
                const uint32_t fh = __shfl_sync(qmask, (uint32_t)(cflags >> 32), cr, 4);
                const uint32_t fv = __shfl_sync(qmask, cvers, cr, 4);
                const int braster = (se.x >> 15) & 63;
                unsigned long long nfl = srcref >= 0 ? ((unsigned long long)fh << 32 | fl) : 0ull;
                uint32_t nvr = srcref >= 0 ? fv : 0u;
                nfl = (nfl & ~(1ull << braster)) | (unsigned long long)(nsig != 0) << braster;
                nvr = (nvr & ~(3u << (2 * slot))) | (uint32_t)s << (2 * slot);
                if (upd) *reinterpret_cast<uint4 *>(&Q.ring[slot][s][0]) = make_uint4(l0, l1, l2, l3);
                /* neighbours of sub-block sb - 1 */
                const uint32_t nx = __ldg(&ST[k - 1].x);
                const int r1 = (nx >> 15) & 63, x1 = r1 % ws, y1 = r1 / ws;
                const int right = x1 < ws - 1 ? r1 + 1 : 0, below = y1 < hs - 1 ? r1 + ws : 0;
                const int nsb = (right && ((nfl >> right) & 1)) || (below && ((nfl >> below) & 1));
                const bool need = nsb || (right && below && ((nfl >> (below + 1)) & 1));
                __syncwarp(qmask);
                if (upd) {
#pragma unroll 4
                    for (int j = 0; j < 16; j++) {
                        uint32_t t16 = 0;
                        if (need) {
                            const uint4 te = __ldg(&TT[k - 16 + j]);
                            const int no = te.x & 7;
                            int sa = 0, s1v = 0, cn = 0;
                            const uint32_t nbs[5] = { te.x >> 16, te.y & 0xFFFF, te.y >> 16, te.z & 0xFFFF, te.z >> 16 };
#pragma unroll
                            for (int u = 0; u < 5; u++) {
                                if (u < no) {
                                    const uint32_t nb = nbs[u];
                                    const int sbn = nb & 63, inner = (nb >> 6) & 15, rs = (nb >> 10) & 63, sl = sbn & 15;
                                    int v = 0;
                                    if ((nfl >> rs) & 1) {
                                        const int ver = (nvr >> (2 * sl)) & 3;
                                        v = reinterpret_cast<const uint8_t *>(&Q.ring[sl][ver][0])[inner];
                                    }
                                    sa += v; s1v += min(4 + (v & 1), v); cn += v != 0;
                                }
                            }
                            t16 = (uint32_t)min(sa, 127) | (uint32_t)s1v << 7 | (uint32_t)cn << 12;
                        }
                        Q.tpl[s][j] = (uint16_t)t16;
                    }
                    nsig = 0; l0 = l1 = l2 = l3 = 0; par16 = 0; ref = s; signb = nsb;
                    cflags = nfl; cvers = nvr;
                }
                __syncwarp(qmask);
            }
        }
        __syncwarp(qmask);

        /* ---- best final state, then walk the decisions from position 0 up
         * (h266_dep_quant.c:1919-1947).  The state a coefficient was quantised
         * in is the source state of its decision (0 for the last position), so
         * each level is dequantised as it is found (:1949-1989 walks the same
         * state machine forward from the last position). */
        const long long f0 = xg_dq_shfl64(qmask, cost, 0), f1v = xg_dq_shfl64(qmask, cost, 1);
        const long long f2v = xg_dq_shfl64(qmask, cost, 2), f3v = xg_dq_shfl64(qmask, cost, 3);
        if (has) {
            unsigned long long map = 0;
            long long best = 0;
            int st = -1;
            if (f0 < best) { best = f0; st = 0; }
            if (f1v < best) { best = f1v; st = 1; }
            if (f2v < best) { best = f2v; st = 2; }
            if (f3v < best) { best = f3v; st = 3; }
            const int iqadd = 1 << (P.iqShift - 1);
            uint32_t ncode = codes[s];
            int nval = TS[s];
            uint32_t nent = __ldg(&ST[s].x);
            for (int k0 = 0; st >= 0 && k0 <= first; k0 += 4) {
                const uint32_t mcode = ncode, ment = nent;
                const int mval = nval;
                if (k0 + 4 + s <= first) { ncode = codes[k0 + 4 + s]; nval = TS[k0 + 4 + s]; nent = __ldg(&ST[k0 + 4 + s].x); }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const uint32_t c = __shfl_sync(qmask, mcode, j, 4);
                    const int v = __shfl_sync(qmask, mval, j, 4);
                    const int k = k0 + j;
                    if (st >= 0 && k <= first) {
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
                        if (lv && s == j) {
                            const int x = ment & 31, y = (ment >> 5) & 31;
                            const int qv = v < 0 ? -lv : lv;
                            const int qidx = 2 * qv + (qv > 0 ? -(ps >> 1) : (ps >> 1));
                            const int rv = (qidx * P.iqScale + iqadd) >> P.iqShift;
                            QO[y * stride + x] = (xg_coef)qv;
                            RO[y * stride + x] = (xg_coef)(rv < -32768 ? -32768 : rv > 32767 ? 32767 : rv);
                            map |= 1ull << ((ment >> 15) & 63);
                        }
                    }
                }
            }
            map |= __shfl_xor_sync(qmask, map, 1, 4);
            map |= __shfl_xor_sync(qmask, map, 2, 4);
            if (s == 0) nzout[job] = map;
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
 * (256 B); rates of nsets context sets; last positions and order of njobs
 * blocks; the scan-order copy of the blocks (nscan coefficients); nquads
 * quads' decision areas. */
struct XgDqArea {
    int *counter, *counts, *cursor;
    XgDqRates *rates;
    int32_t *first, *order;
    xg_coef *tscan;
    uint32_t *codes;
};
static size_t xg_dq_area_bytes(int nsets, int njobs, size_t nscan, int nquads, XgDqArea *a, char *base)
{
    size_t o = 0;
    auto take = [&](size_t bytes) { size_t at = o; o = (o + bytes + 255) & ~(size_t)255; return base ? base + at : nullptr; };
    char *hdr = take(1024);
    char *rt = take((size_t)nsets * 2 * sizeof(XgDqRates));
    char *fi = take((size_t)njobs * 4);
    char *od = take((size_t)njobs * 4);
    char *ts = take(nscan * sizeof(xg_coef));
    char *cd = take((size_t)nquads * XG_DQ_MAXN * 4);
    if (a && base) {
        a->counter = (int *)hdr; a->counts = (int *)hdr + 1; a->cursor = (int *)hdr + 80;
        a->rates = (XgDqRates *)rt; a->first = (int32_t *)fi; a->order = (int32_t *)od;
        a->tscan = (xg_coef *)ts; a->codes = (uint32_t *)cd;
    }
    return o;
}

static int xg_dq_enqueue(const xin_gpu_dq_block *d_jobs, const uint32_t *d_soff, int njobs,
                         const xg_coef *t, xg_coef *q, xg_coef *r, unsigned long long *nz, const xin_gpu_prob *d_sets,
                         int nsets, const XgDqArea &A, int max_ctas, int full, cudaStream_t st, bool count = true)
{
    int ctas = (njobs + XG_DQ_QUADS - 1) / XG_DQ_QUADS;
    if (ctas > max_ctas) ctas = max_ctas;
    if (xg_cuda_check(cudaMemsetAsync(A.counter, 0, 1024, st), "dq counters")) return XIN_GPU_ERR_CUDA;
    k_dq_rates<<<nsets, 64, 0, st>>>(d_sets, A.rates);
    const int pw = 8, pblocks = std::min((njobs + pw - 1) / pw, 152 * 16);
    k_dq_prep<<<pblocks, pw * 32, 0, st>>>(d_jobs, njobs, d_soff, t, A.tscan, q, r, nz, g_dq.d_step, g_dq.d_par,
                                           A.first, A.counts, full);
    k_dq_order<<<std::min((njobs + 255) / 256, 152 * 4), 256, 0, st>>>(njobs, A.first, A.counts, A.cursor, A.order);
    k_dq<<<ctas, XG_DQ_THREADS, sizeof(XgDqSmem), st>>>(d_jobs, njobs, A.counter, A.counts, A.order, A.first, d_soff,
                                                        A.tscan, q, r, nz, d_sets, A.rates, g_dq.d_step, g_dq.d_tpl,
                                                        g_dq.d_par, A.codes);
    if (count) xg_count_launch(4);
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
    p->ctas = std::min(res, (nblocks + XG_DQ_QUADS - 1) / XG_DQ_QUADS);
    const size_t bytes = xg_dq_area_bytes(nsets, nblocks, nscan, p->ctas * XG_DQ_QUADS, nullptr, nullptr);
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
    xg_dq_area_bytes(nsets, nblocks, nscan, p->ctas * XG_DQ_QUADS, &p->area, p->d_area);
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
    const size_t abytes = xg_dq_area_bytes(1, 1, (size_t)ew * eh, XG_DQ_QUADS, nullptr, nullptr);
    char *area = (char *)xg_dalloc(th, abytes);
    if (!dt || !dq || !dr || !dnz || !dj || !dc || !dso || !area) return;
    XgDqArea A;
    xg_dq_area_bytes(1, 1, (size_t)ew * eh, XG_DQ_QUADS, &A, area);
    if (xg_dq_enqueue(dj, dso, 1, dt, dq, dr, dnz, dc, 1, A, 1, 0, th->stream)) return;
    if (xg_stage_out(th, qCoeff, coeffStride, dq, ew, eh, sizeof(xg_coef)) ||
        xg_stage_out(th, rCoeff, coeffStride, dr, ew, eh, sizeof(xg_coef)) ||
        xg_cuda_check(cudaMemcpyAsync(th->hbuf, dnz, 8, cudaMemcpyDeviceToHost, th->stream), "d2h") || xg_sync(th))
        return;
    *nzCGBitMapRs = *(uint64_t *)th->hbuf;
}

#endif
