/*
 * xg_tu.cuh -- the preset-4 TU stage of the frame form (stream tu_mode 1).
 *
 * Preset 4 codes a CU's residual with explicit MTS and dependent quantisation
 * (app/common/source/xin_encoder_option.c:196-197): the mode decision tries
 * each transform candidate through the dependent-quantisation branch of
 * Xin266Transform (h266_encoder/source/h266_trans_quant.c:61-245) and
 * reconstructs it with Xin266IDctAdd (h266_idct_add.c:45), then picks by its
 * CABAC rate estimate on the host.  The frame form computes every candidate for
 * every CU, TU = CU: luma DCT2 and, for CUs up to 32, the MTS pairs 2..5;
 * chroma DCT2.  Per picture, after the CU tails have written the prediction
 * residual planes:
 *
 *   k_tu_fwd     forward transforms of every (CU, plane, candidate) block, written
 *                in the trellis's scan order, with the trellis's set-up (last
 *                position above the threshold, q and r cleared)
 *   (DQ)         the dependent-quantisation trellis over all blocks (xg_dq.cuh),
 *                QPs from the picture, rates from the stream's context set
 *   k_tu_inv     inverse transforms, reconstruction (prediction = input -
 *                residual), SSD per block; the DCT2 candidate's levels and
 *                reconstruction go to the picture's output planes
 *   k_tu_satd    8x8 Hadamard SATD of the luma residual per CU
 *   k_tu_collect the per-CU records
 *
 * The transforms follow the CUDA-core batch engine (xg_tq_batch.cuh): groups
 * of G threads per block, operands in shared memory, the forward pass keeping
 * the low 32 frequencies (the trellis reads no others).
 */

struct XgTuState {
    int nc[4];                         /* luma candidates per level (1 at 64, else 5) */
    int16_t *resid;                    /* residual planes: per level Y, U, V (picture layout) */
    size_t res_off[4][3];
    xg_coef *Q, *R;                    /* candidate coefficient planes: levels, dequantised */
    size_t ncoef;
    size_t cand_off[4][3][5];
    unsigned long long *nz, *ssd;      /* per trellis block */
    uint32_t *satd;                    /* per CU (all levels) */
    int blk[4][3];                     /* first trellis block of (level, plane) */
    int nblocks;
    xin_gpu_dq_plan *plan;
    xin_gpu_prob *ctx;                 /* the context set (device) */
};

/* one level's view for the kernels */
struct XgTuLevel {
    const int16_t *resid[3];
    const xg_pix *org[3];
    int opitch[3];
    xg_coef *Q[3], *R[3];              /* candidate 0's plane of each plane; candidate c at + c * cstride */
    size_t cstride;                    /* elements between a luma candidate's planes */
    unsigned long long *nz, *ssd;      /* trellis blocks of plane 0 of this level */
    /* the trellis plan's set-up, written by the forward transforms: blocks are
     * numbered from blk0 (this level's first) */
    xg_coef *tscan;                    /* scan-order copies */
    const uint32_t *soff;              /* start of each block's copy */
    int32_t *first;                    /* last position above the threshold (-1: none) */
    const XgDqParam *par;              /* trellis parameters [lg w + lg h - 4][QP] */
    const XgPicParams *pp;             /* the picture's trellis QPs */
    int blk0;
    int blk[3];                        /* first block of each plane, relative to the level's first */
    xg_coef *qout[3];                  /* the picture's output planes of this level */
    xg_pix *recout[3];
    int W, S, cus_x, ncu, nc;
    const xin_gpu_cu_bi *bi;           /* refs 2: this level's bi records (the coded prediction) */
};

/* A transform matrix of N points (rows k < K = min(N, 32)) into a packed int8
 * operand of xg_mm_dp2 (|entries| <= 90): FWD, M(k, x) = T(k, x) (rows k, l = x),
 * the layout of the forward passes; otherwise M(x, k) = T(k, x) (rows x, l = k),
 * the layout of the inverse passes */
template <int N, bool FWD>
__device__ __forceinline__ void xg_tu_load_mat(uint32_t *dst, const int16_t *m, int tid, int nthreads)
{
    constexpr int K = N > 32 ? 32 : N;
    int8_t *d = reinterpret_cast<int8_t *>(dst);
    for (int i = tid; i < K * N; i += nthreads) {
        const int k = i / N, x = i % N;
        if (FWD) d[(((x >> 2) * K + k) << 2) | (x & 3)] = (int8_t)m[i];
        else d[(((k >> 2) * N + x) << 2) | (k & 3)] = (int8_t)m[i];
    }
}

/* one block's work area: a = the first pass's int16-pair operand, b = the second's */
template <int N>
struct XgTuWork {
    static constexpr int K = N > 32 ? 32 : N;
    alignas(16) int16_t a[N * N];
    alignas(16) int16_t b[N * K];
};

/* position and transform pair of CU cu, candidate c (DCT2, then MTS 2..5), plane pl */
struct XgTuJobPos { int px, py, pw, hor, ver; };
__device__ __forceinline__ XgTuJobPos xg_tu_job(const XgTuLevel &L, int pl, int cu, int c, int n)
{
    XgTuJobPos o;
    o.px = (cu % L.cus_x) * n;
    o.py = (cu / L.cus_x) * n;
    o.pw = pl ? L.W >> 1 : L.W;
    const int mts = c ? c + 1 : 0;
    o.hor = c_mts_tx[mts][0];
    o.ver = c_mts_tx[mts][1];
    return o;
}

/* Forward transforms of N x N blocks: CTA = CPB groups of NT threads, one CU each,
 * all of candidate blockIdx.y (the CTA loads its two matrices once).  Rows then
 * columns as dp2a products on the tails' packed operands; the low K x K
 * frequencies go to the candidate's coefficient plane. */
template <int N, int NT, int CPB>
__global__ void __launch_bounds__(NT * CPB) k_tu_fwd(XgTuLevel L, int pl)
{
    constexpr int K = N > 32 ? 32 : N, LG = N == 64 ? 6 : N == 32 ? 5 : N == 16 ? 4 : N == 8 ? 3 : 2;
    __shared__ alignas(16) uint32_t mh[K * N / 4], mv[K * N / 4];
    __shared__ XgTuWork<N> work[CPB];
    const int g = threadIdx.x / NT, tid = threadIdx.x % NT, c = blockIdx.y;
    const XgTuJobPos a0 = xg_tu_job(L, pl, 0, c, N);
    xg_tu_load_mat<N, true>(mh, xg_mat(a0.hor, LG), threadIdx.x, NT * CPB);
    xg_tu_load_mat<N, true>(mv, xg_mat(a0.ver, LG), threadIdx.x, NT * CPB);
    __syncthreads();
    const int cu = blockIdx.x * CPB + g;
    if (cu >= L.ncu) return;               /* no CTA-wide barrier follows */
    const XgTuJobPos a = xg_tu_job(L, pl, cu, c, N);
    XgTuWork<N> &w = work[g];
    const int16_t *src = L.resid[pl] + (size_t)a.py * a.pw + a.px;
    for (int o = tid; o < N * N; o += NT) { const int y = o >> LG, x = o & (N - 1); w.a[xg_d2<N>(y, x)] = src[(size_t)y * a.pw + x]; }
    xg_gsync<NT, CPB>(g);
    const int s1 = LG + XG_BITDEPTH + 6 - 15, s2 = LG + 6;
    /* rows: t1(y, k) = sum_x r(y, x) Th(k, x) */
    xg_mm_dp2<N, K, N, NT>(tid, reinterpret_cast<const uint32_t *>(w.a), mh, [&](int y, int k, int acc) {
        w.b[xg_d2<K>(k, y)] = (int16_t)xg_clip16(xg_rshift_rnd(acc, s1));
    });
    xg_gsync<NT, CPB>(g);
    /* the trellis's set-up (Xin266PreDepQuant, h266_dep_quant.c:1683-1770, as
     * k_dq_prep): the coefficients in scan order, the last one above the
     * threshold, q and r of the block cleared */
    const int b = L.blk[pl] + cu * (pl ? 1 : L.nc) + c;          /* block, from the level's first */
    const XgDqParam *P = L.par + (2 * LG - 4) * 52 + L.pp->dq_qp[pl ? 1 : 0];
    const int thr = P->thresLast / (P->qScale << 2);
    xg_coef *TS = L.tscan + L.soff[L.blk0 + b];
    int best = -1;
    /* columns: t(kv, kh) = sum_y t1(y, kh) Tv(kv, y), to scan position (kh, kv) */
    xg_mm_dp2<K, K, N, NT, true>(tid, reinterpret_cast<const uint32_t *>(w.b), mv, [&](int kh, int kv, int acc) {
        const int v = xg_clip16(xg_rshift_rnd(acc, s2)), k = xg_dq_scan_sq(kh, kv, K);
        TS[k] = (xg_coef)v;
        if ((v < 0 ? -v : v) > thr) best = max(best, k);
    });
    {
        xg_coef *QO = L.Q[pl] + (size_t)c * L.cstride + (size_t)a.py * a.pw + a.px;
        xg_coef *RO = L.R[pl] + (size_t)c * L.cstride + (size_t)a.py * a.pw + a.px;
        for (int o = tid; o < N * N; o += NT) {
            const int y = o >> LG, x = o & (N - 1);
            QO[(size_t)y * a.pw + x] = 0;
            RO[(size_t)y * a.pw + x] = 0;
        }
    }
    best = __reduce_max_sync(0xffffffffu, best);
    if (NT > 32) {
        __shared__ int gbest[CPB];
        if (tid == 0) gbest[g] = -1;
        xg_gsync<NT, CPB>(g);
        if ((tid & 31) == 0) atomicMax(&gbest[g], best);
        xg_gsync<NT, CPB>(g);
        best = gbest[g];
    }
    if (tid == 0) {
        L.first[L.blk0 + b] = best;
        if (best < 0) L.nz[b] = 0;
    }
}

/* Inverse transforms (Xin266IDctWxH, h266_inverse_trans.c:117-229: columns, then
 * rows; a skipped column line contributes zero, so its coefficients are loaded
 * as zeros), reconstruction from prediction = input - residual, SSD per block;
 * the DCT2 candidate's levels and reconstruction go to the picture's planes. */
template <int N, int NT, int CPB>
__global__ void __launch_bounds__(NT * CPB) k_tu_inv(XgTuLevel L, int pl)
{
    constexpr int K = N > 32 ? 32 : N, LG = N == 64 ? 6 : N == 32 ? 5 : N == 16 ? 4 : N == 8 ? 3 : 2;
    __shared__ alignas(16) uint32_t mv[K * N / 4], mh[K * N / 4];
    __shared__ XgTuWork<N> work[CPB];
    __shared__ unsigned long long ssd_g[CPB];
    const int g = threadIdx.x / NT, tid = threadIdx.x % NT, c = blockIdx.y;
    const XgTuJobPos a0 = xg_tu_job(L, pl, 0, c, N);
    xg_tu_load_mat<N, false>(mv, xg_mat(a0.ver, LG), threadIdx.x, NT * CPB);
    xg_tu_load_mat<N, false>(mh, xg_mat(a0.hor, LG), threadIdx.x, NT * CPB);
    if (threadIdx.x < CPB) ssd_g[threadIdx.x] = 0;
    __syncthreads();
    const int cu = blockIdx.x * CPB + g;
    if (cu >= L.ncu) return;
    const XgTuJobPos a = xg_tu_job(L, pl, cu, c, N);
    XgTuWork<N> &w = work[g];
    const size_t off = (size_t)a.py * a.pw + a.px;
    const int sline = (a.hor != 0 && N == 32) ? 16 : (N > 32 ? N - 32 : 0), jmax = N - sline;
    const xg_coef *rin = L.R[pl] + (size_t)c * L.cstride + off;
    for (int o = tid; o < K * K; o += NT) {
        const int kv = o / K, kh = o - kv * K;
        w.a[xg_d2<K>(kh, kv)] = kh < jmax ? (int16_t)rin[(size_t)kv * a.pw + kh] : (int16_t)0;
    }
    if (c == 0) {
        const xg_coef *qin = L.Q[pl] + off;
        for (int o = tid; o < N * N; o += NT) {
            const int y = o >> LG, x = o & (N - 1);
            L.qout[pl][off + (size_t)y * a.pw + x] = qin[(size_t)y * a.pw + x];
        }
    }
    xg_gsync<NT, CPB>(g);
    /* columns: t2(kh, y) = sum_kv c(kv, kh) Tv(kv, y) */
    xg_mm_dp2<K, N, K, NT>(tid, reinterpret_cast<const uint32_t *>(w.a), mv, [&](int kh, int y, int acc) {
        w.b[xg_d2<N>(y, kh)] = (int16_t)xg_clip16(xg_rshift_rnd(acc, 7));
    });
    xg_gsync<NT, CPB>(g);
    const int s2 = 6 + 15 - 1 - XG_BITDEPTH;
    const int16_t *res = L.resid[pl] + off;
    const xg_pix *org = L.org[pl] + (size_t)a.py * L.opitch[pl] + a.px;
    xg_pix *rec = L.recout[pl] + off;
    unsigned part = 0;
    /* rows: r'(y, x) = sum_kh t2(kh, y) Th(kh, x) */
    xg_mm_dp2<N, N, K, NT>(tid, reinterpret_cast<const uint32_t *>(w.b), mh, [&](int y, int x, int acc) {
        const int o = (int)org[(size_t)y * L.opitch[pl] + x];
        const int v = xg_clip_pix(o - (int)res[(size_t)y * a.pw + x] + xg_clip16(xg_rshift_rnd(acc, s2)));
        if (c == 0) rec[(size_t)y * a.pw + x] = (xg_pix)v;
        part += (unsigned)((o - v) * (o - v));
    });
    /* a thread holds at most ceil(N * N / NT) squared differences below 2^(2 bitdepth):
     * 32 lanes' sum fits 32 bits */
    static_assert((unsigned long long)((N * N + NT - 1) / NT) * 32 * ((1ull << XG_BITDEPTH) - 1) * ((1ull << XG_BITDEPTH) - 1) <
                      (1ull << 32), "warp SSD sum fits 32 bits");
    const unsigned wsum = __reduce_add_sync(0xffffffffu, part);
    if ((tid & 31) == 0) atomicAdd(&ssd_g[g], (unsigned long long)wsum);
    xg_gsync<NT, CPB>(g);
    if (tid == 0) L.ssd[L.blk[pl] + cu * (pl ? 1 : L.nc) + c] = ssd_g[g];
}

/* 8x8 Hadamard SATD (HM normalisation, as XinGpuComputeSatd) of the luma
 * residual, added per CU */
__global__ void k_tu_satd(XgTuLevel L, uint32_t *satd)
{
    const int tiles_row = L.cus_x * (L.S >> 3), per_cu = (L.S >> 3) * (L.S >> 3);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.ncu * per_cu) return;
    const int tx = i % tiles_row, ty = i / tiles_row;
    const int16_t *r = L.resid[0] + (size_t)(ty * 8) * L.W + tx * 8;
    int d[64];
#pragma unroll
    for (int y = 0; y < 8; y++)
#pragma unroll
        for (int x = 0; x < 8; x++) d[y * 8 + x] = r[(size_t)y * L.W + x];
    const int cu = (ty / (L.S >> 3)) * L.cus_x + tx / (L.S >> 3);
    atomicAdd(&satd[cu], (uint32_t)((xg_had8(d) + 2) >> 2));
}

__global__ void k_tu_collect(XgTuLevel L, const uint32_t *satd, xin_gpu_cu_result *res, xin_gpu_cu_mts *mts, const XgPicParams *pp)
{
    const int cu = blockIdx.x * blockDim.x + threadIdx.x;
    if (cu >= L.ncu) return;
    xin_gpu_cu_result &o = res[cu];
    xin_gpu_cu_mts &m = mts[cu];
    for (int pl = 0; pl < 3; pl++) {
        const int b = L.blk[pl] + cu * (pl ? 1 : L.nc);
        o.nz[pl] = L.nz[b];
        o.ssd[pl] = L.ssd[b];
    }
    /* the coded prediction's MV bits: list 0's MV, list 1's, or both of the pair */
    unsigned bits = xg_mvd_bits(o.mvx) + xg_mvd_bits(o.mvy);
    if (L.bi) {
        const xin_gpu_cu_bi &b = L.bi[cu];
        if (b.inter_dir == 2) bits = xg_mvd_bits(b.mvx1) + xg_mvd_bits(b.mvy1);
        if (b.inter_dir == 3) bits = xg_mvd_bits(b.bmv[0]) + xg_mvd_bits(b.bmv[1]) + xg_mvd_bits(b.bmv[2]) + xg_mvd_bits(b.bmv[3]);
    }
    m.satd_cost = (satd[cu] << XG_COST_FRACTION) + bits * pp->lambda;
    m.ncand = (uint32_t)L.nc;
    for (int c = 0; c < 5; c++) {
        m.nz[c] = c < L.nc ? L.nz[cu * L.nc + c] : 0ull;
        m.ssd[c] = c < L.nc ? L.ssd[cu * L.nc + c] : 0ull;
    }
}

/* QPs of the trellis blocks from the picture (luma blocks first per level) */
__global__ void k_tu_setqp(xin_gpu_dq_block *jobs, int n, const XgPicParams *pp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) jobs[i].qp = (uint8_t)pp->dq_qp[jobs[i].comp ? 1 : 0];
}

/* ------------------------------------------------------------------ host */

static int16_t *xg_tu_resid(XgTuState *u, int level, int plane) { return u->resid + u->res_off[level][plane]; }

/* device bytes of the TU stage for cfg (beside the stream's own) */
static uint64_t xg_tu_bytes(const xin_gpu_stream_cfg *c)
{
    uint64_t lq = (uint64_t)c->width * c->height, lc = lq / 4, coef = 0, res = 0, blocks = 0, cus = 0;
    for (int L = 0; L < 4; L++) {
        const int sz = XG_LEVEL_SIZE[L];
        if (!(c->level_mask & (uint32_t)sz)) continue;
        const uint64_t n = (uint64_t)(c->width / sz) * (c->height / sz);
        const int nc = sz == 64 ? 1 : 5;
        coef += nc * lq + 2 * lc;
        res += lq + 2 * lc;
        blocks += n * (nc + 2);
        cus += n;
    }
    const uint64_t slots = std::min<uint64_t>((uint64_t)XG_DQ_MAX_CTAS, (blocks + XG_DQ_PAIRS - 1) / XG_DQ_PAIRS) * XG_DQ_PAIRS;
    return 2 * coef * sizeof(xg_coef) + res * 2 + blocks * (16 + 16 + sizeof(xin_gpu_dq_block)) + cus * 4 +
           XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob) + coef * 2 /* the trellis plan's scan-order copies */ +
           slots * XG_DQ_SLOT_BYTES /* its decision columns and rings */;
}

static void xg_tu_free(XgTuState *u)
{
    if (!u) return;
    cudaFree(u->resid); cudaFree(u->Q); cudaFree(u->R);
    cudaFree(u->nz); cudaFree(u->ssd); cudaFree(u->satd); cudaFree(u->ctx);
    if (u->plan) xin_gpu_dq_plan_destroy(u->plan);
    delete u;
}

/* a neutral context set: every probability at one half, the middle window rate */
static void xg_tu_default_contexts(std::vector<xin_gpu_prob> &v)
{
    v.assign(XIN_GPU_NUM_CTX, xin_gpu_prob());
    for (auto &p : v) { p.state[0] = (uint16_t)(512 << 5); p.state[1] = (uint16_t)(8192 << 1); p.rate = 0x55; }
}

/* the TU state of picture set `set` (each set has its own, so that the TU
 * stages of two pictures in flight can overlap) */
static int xg_tu_open(xin_gpu_stream *s, int set)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    XgTuState *u = new (std::nothrow) XgTuState();
    if (!u) { xg_set_error(XIN_GPU_ERR_NOMEM, "stream_open: host allocation"); return XIN_GPU_ERR_NOMEM; }
    const size_t lq = (size_t)c.width * c.height, lc = lq / 4;
    size_t coef = 0, res = 0;
    int nblk = 0, ncu = 0;
    std::vector<xin_gpu_dq_block> blocks;
    for (int L = 0; L < 4; L++) {
        if (!s->lev_on[L]) continue;
        const int sz = XG_LEVEL_SIZE[L], n = s->lev_cx[L] * s->lev_cy[L];
        u->nc[L] = sz == 64 ? 1 : 5;
        for (int p = 0; p < 3; p++) {
            u->res_off[L][p] = res;
            res += p ? lc : lq;
            for (int cd = 0; cd < (p ? 1 : u->nc[L]); cd++) { u->cand_off[L][p][cd] = coef; coef += p ? lc : lq; }
        }
        const int lgs = sz == 64 ? 6 : sz == 32 ? 5 : sz == 16 ? 4 : 3;
        for (int p = 0; p < 3; p++) {
            u->blk[L][p] = nblk;
            const int bs = p ? sz / 2 : sz, pw = p ? c.width / 2 : c.width, nc = p ? 1 : u->nc[L];
            for (int j = 0; j < n; j++)
                for (int cd = 0; cd < nc; cd++) {
                    xin_gpu_dq_block b;
                    memset(&b, 0, sizeof b);
                    b.offset = (uint32_t)(u->cand_off[L][p][cd] + (size_t)((j / s->lev_cx[L]) * bs) * pw + (j % s->lev_cx[L]) * bs);
                    b.stride = (uint16_t)pw;
                    b.log2_w = b.log2_h = (uint8_t)(p ? lgs - 1 : lgs);
                    b.qp = 30;                       /* replaced per picture (k_tu_setqp) */
                    b.comp = (uint8_t)p;
                    b.root_cbf = p == 0;             /* an inter CU coded as one TU */
                    b.ctx_set = 0;
                    blocks.push_back(b);
                    nblk++;
                }
        }
        ncu += n;
    }
    u->ncoef = coef;
    u->nblocks = nblk;
    if (coef >= (1ull << 32) || c.width > 65535) {
        xg_set_error(XIN_GPU_ERR_ARG, "stream_open: picture too large for the preset-4 TU stage");
        xg_tu_free(u);
        return XIN_GPU_ERR_ARG;
    }
    cudaError_t e = cudaMalloc(&u->resid, res * 2);
    if (e == cudaSuccess) e = cudaMalloc(&u->Q, coef * sizeof(xg_coef));
    if (e == cudaSuccess) e = cudaMalloc(&u->R, coef * sizeof(xg_coef));
    if (e == cudaSuccess) e = cudaMalloc(&u->nz, (size_t)nblk * 8);
    if (e == cudaSuccess) e = cudaMalloc(&u->ssd, (size_t)nblk * 8);
    if (e == cudaSuccess) e = cudaMalloc(&u->satd, (size_t)(ncu ? ncu : 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&u->ctx, XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob));
    if (e == cudaSuccess) {
        std::vector<xin_gpu_prob> ctx;
        xg_tu_default_contexts(ctx);
        e = cudaMemcpy(u->ctx, ctx.data(), XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        const int st = e == cudaErrorMemoryAllocation ? XIN_GPU_ERR_NOMEM : XIN_GPU_ERR_CUDA;
        xg_set_error(st, "stream_open (TU stage): %s", cudaGetErrorString(e));
        cudaGetLastError();
        xg_tu_free(u);
        return st;
    }
    int st = xin_gpu_dq_plan_create(blocks.data(), nblk, coef, 1, &u->plan);
    if (st) { xg_tu_free(u); return st; }
    s->tu[set] = u;
    return XIN_GPU_OK;
}

template <int N, int NT, int CPB>
static void xg_tu_launch_n(const XgTuLevel &lv, int pl, bool fwd, cudaStream_t st)
{
    const dim3 grid((lv.ncu + CPB - 1) / CPB, pl ? 1 : lv.nc);
    if (fwd) k_tu_fwd<N, NT, CPB><<<grid, NT * CPB, 0, st>>>(lv, pl);
    else k_tu_inv<N, NT, CPB><<<grid, NT * CPB, 0, st>>>(lv, pl);
}

/* block size N of plane pl: a 128-thread CTA per block from 32 up, a warp per
 * block and four blocks a CTA below (the shapes of the CU tails) */
static void xg_tu_launch(const XgTuLevel &lv, int pl, bool fwd, cudaStream_t st)
{
    switch (pl ? lv.S >> 1 : lv.S) {
    case 64: xg_tu_launch_n<64, 128, 1>(lv, pl, fwd, st); break;
    case 32: xg_tu_launch_n<32, 128, 1>(lv, pl, fwd, st); break;
    case 16: xg_tu_launch_n<16, 32, 4>(lv, pl, fwd, st); break;
    case 8: xg_tu_launch_n<8, 32, 4>(lv, pl, fwd, st); break;
    default: xg_tu_launch_n<4, 32, 4>(lv, pl, fwd, st); break;
    }
}

/* the TU stage of the picture in slot cur (picture set t), on st; returns launches */
static int xg_tu_enqueue(xin_gpu_stream *s, int set, int cur, xin_gpu_stream::Set &t, cudaStream_t st)
{
    XgTuState *u = s->tu[set];
    const xin_gpu_stream_cfg &c = s->cfg;
    const size_t lq = (size_t)c.width * c.height, lc = lq / 4;
    int nl = 0;
    XgTuLevel lv[4];
    int li = 0;
    /* the levels' transforms are independent: level i after the first runs on
     * auxiliary stream i - 1 (fork here, join before the trellis and again at
     * the end) */
    cudaStream_t ls[4];
    int nls = 0;
    /* the trellis's bucket counters, before the forward transforms write its set-up */
    cudaMemsetAsync(u->plan->area.counter, 0, 1024, st);
    cudaEventRecord(s->ev_fork, st);
    for (int L = 0; L < 4; L++) {
        if (!s->lev_on[L]) continue;
        ls[L] = nls == 0 ? st : s->aux[nls - 1];
        if (nls > 0) cudaStreamWaitEvent(ls[L], s->ev_fork, 0);
        nls++;
    }
    auto join = [&]() {
        for (int i = 0; i + 1 < nls; i++) {
            cudaEventRecord(s->ev_join[i], s->aux[i]);
            cudaStreamWaitEvent(st, s->ev_join[i], 0);
        }
    };
    for (int L = 0; L < 4; L++) {
        if (!s->lev_on[L]) continue;
        XgTuLevel &v = lv[L];
        memset(&v, 0, sizeof v);
        for (int p = 0; p < 3; p++) {
            v.resid[p] = u->resid + u->res_off[L][p];
            v.org[p] = s->slot[cur][p].data;
            v.opitch[p] = s->slot[cur][p].pitch;
            v.Q[p] = u->Q + u->cand_off[L][p][0];
            v.R[p] = u->R + u->cand_off[L][p][0];
            v.blk[p] = u->blk[L][p] - u->blk[L][0];
            v.qout[p] = t.dq[p] + (p ? lc : lq) * li;
            v.recout[p] = t.drec[p] + (p ? lc : lq) * li;
        }
        v.cstride = lq;
        v.tscan = u->plan->area.tscan; v.soff = u->plan->d_soff; v.first = u->plan->area.first;
        v.par = g_dq.d_par; v.pp = t.dpp; v.blk0 = u->blk[L][0];
        v.nz = u->nz + u->blk[L][0];
        v.ssd = u->ssd + u->blk[L][0];
        v.W = c.width; v.S = XG_LEVEL_SIZE[L]; v.cus_x = s->lev_cx[L]; v.ncu = s->lev_cx[L] * s->lev_cy[L]; v.nc = u->nc[L];
        v.bi = t.dbi ? t.dbi + s->lev_first[L] : nullptr;
        li++;
        if (v.ncu == 0) continue;
        for (int p = 0; p < 3; p++) { xg_tu_launch(v, p, true, ls[L]); nl++; }
    }
    join();
    k_tu_setqp<<<(u->nblocks + 255) / 256, 256, 0, st>>>(u->plan->d_jobs, u->nblocks, t.dpp);
    nl++;
    xg_dq_enqueue_gathered(u->plan->d_jobs, u->plan->d_soff, u->plan->nblocks, u->Q, u->R, u->nz, u->ctx, 1, u->plan->area,
                           u->plan->ctas, st);
    nl += 4;
    cudaMemsetAsync(u->satd, 0, sizeof(uint32_t) * (s->ncus > 0 ? s->ncus : 1), st);
    cudaEventRecord(s->ev_fork, st);
    for (int L = 0; L < 4; L++)
        if (s->lev_on[L] && ls[L] != st) cudaStreamWaitEvent(ls[L], s->ev_fork, 0);
    for (int L = 0; L < 4; L++) {
        if (!s->lev_on[L]) continue;
        XgTuLevel &v = lv[L];
        if (v.ncu == 0) continue;
        for (int p = 0; p < 3; p++) { xg_tu_launch(v, p, false, ls[L]); nl++; }
        const int tiles = v.ncu * (v.S >> 3) * (v.S >> 3);
        k_tu_satd<<<(tiles + 255) / 256, 256, 0, ls[L]>>>(v, u->satd + s->lev_first[L]);
        k_tu_collect<<<(v.ncu + 127) / 128, 128, 0, ls[L]>>>(v, u->satd + s->lev_first[L], t.dres + s->lev_first[L],
                                                             t.dmts + s->lev_first[L], t.dpp);
        nl += 2;
    }
    join();
    return nl;
}

extern "C" int xin_gpu_stream_set_contexts(xin_gpu_stream *s, const xin_gpu_prob *ctx)
{
    xin_gpu_clear_error();
    if (!s || !ctx) { xg_set_error(XIN_GPU_ERR_ARG, "stream_set_contexts: null argument"); return XIN_GPU_ERR_ARG; }
    if (!s->tu[0]) { xg_set_error(XIN_GPU_ERR_STATE, "stream_set_contexts: the stream has no preset-4 TU stage (tu_mode 0)"); return XIN_GPU_ERR_STATE; }
    if (s->nsub != s->ndone) { xg_set_error(XIN_GPU_ERR_STATE, "stream_set_contexts: pictures in flight"); return XIN_GPU_ERR_STATE; }
    for (int i = 0; i < 2; i++)
        if (xg_cuda_check(cudaMemcpy(s->tu[i]->ctx, ctx, XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob), cudaMemcpyHostToDevice),
                          "stream_set_contexts"))
            return XIN_GPU_ERR_CUDA;
    return XIN_GPU_OK;
}
