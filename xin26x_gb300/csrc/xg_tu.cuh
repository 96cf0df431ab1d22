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
 *   k_tu_fwd     forward transforms of every (CU, plane, candidate) block
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
    xg_coef *T, *Q, *R;                /* candidate coefficient planes */
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
    xg_coef *T[3], *Q[3], *R[3];       /* candidate 0's plane of each plane; candidate c at + c * cstride */
    size_t cstride;                    /* elements between a luma candidate's planes */
    unsigned long long *nz, *ssd;      /* trellis blocks of plane 0 of this level */
    int blk[3];                        /* first block of each plane, relative to the level's first */
    xg_coef *qout[3];                  /* the picture's output planes of this level */
    xg_pix *recout[3];
    int W, S, cus_x, ncu, nc;
};

template <int G>
__device__ __forceinline__ void xg_tu_sync(int gid)
{
    if (G == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(G) : "memory");
}

/* position and transform pair of job j of plane pl */
struct XgTuJobPos { int px, py, pw, n, lg, c, hor, ver; };
__device__ __forceinline__ XgTuJobPos xg_tu_job(const XgTuLevel &L, int pl, int j)
{
    XgTuJobPos o;
    const int nc = pl ? 1 : L.nc, cu = j / nc;
    o.c = j - cu * nc;
    o.n = pl ? L.S >> 1 : L.S;
    o.lg = 31 - __clz(o.n);
    o.px = (cu % L.cus_x) * o.n;
    o.py = (cu / L.cus_x) * o.n;
    o.pw = pl ? L.W >> 1 : L.W;
    const int mts = o.c ? o.c + 1 : 0;     /* candidates: DCT2, then MTS 2..5 */
    o.hor = c_mts_tx[mts][0];
    o.ver = c_mts_tx[mts][1];
    return o;
}

template <int G>
__global__ void __launch_bounds__(256) k_tu_fwd(XgTuLevel L, int pl)
{
    extern __shared__ uint32_t tsw[];
    constexpr int NG = 256 / G;
    const int gid = threadIdx.x / G, t = threadIdx.x % G;
    const int n = pl ? L.S >> 1 : L.S, k = n > 32 ? 32 : n;
    int16_t *resT = (int16_t *)tsw + gid * (n * n + n * k), *t1T = resT + n * n;
    const int njobs = L.ncu * (pl ? 1 : L.nc);
    for (int j = blockIdx.x * NG + gid; j < njobs; j += gridDim.x * NG) {
        const XgTuJobPos a = xg_tu_job(L, pl, j);
        const int16_t *src = L.resid[pl] + (size_t)a.py * a.pw + a.px;
        for (int o = t; o < n * n; o += G) { const int y = o >> a.lg, x = o & (n - 1); resT[x * n + y] = src[(size_t)y * a.pw + x]; }
        xg_tu_sync<G>(gid);
        const int16_t *mh = xg_mat(a.hor, a.lg), *mv = xg_mat(a.ver, a.lg);
        const int s1 = a.lg + XG_BITDEPTH + 6 - 15, s2 = a.lg + 6;
        /* rows: t1T[i * k + f] = sum_x mh[f][x] res[i][x], f < k */
        xg_mm_rt<G>(t, k, n, n, mh, n, 1, resT, 1, n, [&](int f, int i, int acc) {
            t1T[i * k + f] = (int16_t)xg_clip16(xg_rshift_rnd(acc, s1));
        });
        xg_tu_sync<G>(gid);
        xg_coef *dst = L.T[pl] + (size_t)a.c * L.cstride + (size_t)a.py * a.pw + a.px;
        /* columns: T[fv][fh] = sum_i mv[fv][i] t1T[i * k + fh] */
        xg_mm_rt<G>(t, k, k, n, mv, n, 1, t1T, 1, k, [&](int fv, int fh, int acc) {
            dst[(size_t)fv * a.pw + fh] = (xg_coef)xg_clip16(xg_rshift_rnd(acc, s2));
        });
        xg_tu_sync<G>(gid);
    }
}

template <int G>
__global__ void __launch_bounds__(256) k_tu_inv(XgTuLevel L, int pl)
{
    extern __shared__ uint32_t tsw[];
    constexpr int NG = 256 / G;
    const int gid = threadIdx.x / G, t = threadIdx.x % G;
    const int n = pl ? L.S >> 1 : L.S, k = n > 32 ? 32 : n;
    int16_t *rr = (int16_t *)tsw + gid * (k * k + k * n), *t2 = rr + k * k;
    __shared__ unsigned long long ssd_g[NG];
    const int njobs = L.ncu * (pl ? 1 : L.nc);
    for (int j = blockIdx.x * NG + gid; j < njobs; j += gridDim.x * NG) {
        const XgTuJobPos a = xg_tu_job(L, pl, j);
        const size_t off = (size_t)a.py * a.pw + a.px;
        const xg_coef *rin = L.R[pl] + (size_t)a.c * L.cstride + off;
        for (int o = t; o < k * k; o += G) { const int y = o / k, x = o - y * k; rr[o] = (int16_t)rin[(size_t)y * a.pw + x]; }
        if (t == 0) ssd_g[gid] = 0;
        if (a.c == 0) {   /* the DCT2 candidate's levels to the picture's output plane */
            const xg_coef *qin = L.Q[pl] + off;
            for (int o = t; o < n * n; o += G) {
                const int y = o >> a.lg, x = o & (n - 1);
                L.qout[pl][off + (size_t)y * a.pw + x] = qin[(size_t)y * a.pw + x];
            }
        }
        xg_tu_sync<G>(gid);
        /* Xin266IDctWxH (h266_inverse_trans.c:117-229): columns j < jmax, then rows */
        const int16_t *mh = xg_mat(a.hor, a.lg), *mv = xg_mat(a.ver, a.lg);
        const int sline = (a.hor != 0 && n == 32) ? 16 : (n > 32 ? n - 32 : 0), jmax = n - sline;
        const int s2 = 6 + 15 - 1 - XG_BITDEPTH;
        xg_mm_rt<G>(t, jmax, n, k, rr, 1, k, mv, 1, n, [&](int jc, int y, int acc) {
            t2[jc * n + y] = (int16_t)xg_clip16(xg_rshift_rnd(acc, 7));
        });
        xg_tu_sync<G>(gid);
        const int16_t *res = L.resid[pl] + off;
        const xg_pix *org = L.org[pl] + (size_t)a.py * L.opitch[pl] + a.px;
        xg_pix *rec = L.recout[pl] + off;
        unsigned long long part = 0;
        xg_mm_rt<G>(t, n, n, jmax, t2, 1, n, mh, 1, n, [&](int y, int x, int acc) {
            const int o = (int)org[(size_t)y * L.opitch[pl] + x];
            const int pred = o - (int)res[(size_t)y * a.pw + x];
            const int v = xg_clip_pix(pred + xg_clip16(xg_rshift_rnd(acc, s2)));
            if (a.c == 0) rec[(size_t)y * a.pw + x] = (xg_pix)v;
            part += (unsigned long long)((o - v) * (o - v));
        });
        atomicAdd(&ssd_g[gid], part);
        xg_tu_sync<G>(gid);
        if (t == 0) L.ssd[L.blk[pl] + j] = ssd_g[gid];
    }
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
    m.satd_cost = (satd[cu] << XG_COST_FRACTION) + (xg_mvd_bits(o.mvx) + xg_mvd_bits(o.mvy)) * pp->lambda;
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

static int xg_tu_group(int n) { return n >= 64 ? 256 : n >= 32 ? 128 : n >= 16 ? 64 : 32; }

static size_t xg_tu_smem_fwd(int n, int G) { const int k = n > 32 ? 32 : n; return (size_t)(256 / G) * (n * n + n * k) * 2; }
static size_t xg_tu_smem_inv(int n, int G) { const int k = n > 32 ? 32 : n; return (size_t)(256 / G) * (k * k + k * n) * 2; }

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
    return 3 * coef * sizeof(xg_coef) + res * 2 + blocks * (16 + 16 + sizeof(xin_gpu_dq_block)) + cus * 4 +
           XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob) + coef * 2 /* the trellis plan's scan-order copies */;
}

static void xg_tu_free(XgTuState *u)
{
    if (!u) return;
    cudaFree(u->resid); cudaFree(u->T); cudaFree(u->Q); cudaFree(u->R);
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

static int xg_tu_open(xin_gpu_stream *s)
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
    if (e == cudaSuccess) e = cudaMalloc(&u->T, coef * sizeof(xg_coef));
    if (e == cudaSuccess) e = cudaMalloc(&u->Q, coef * sizeof(xg_coef));
    if (e == cudaSuccess) e = cudaMalloc(&u->R, coef * sizeof(xg_coef));
    if (e == cudaSuccess) e = cudaMalloc(&u->nz, (size_t)nblk * 8);
    if (e == cudaSuccess) e = cudaMalloc(&u->ssd, (size_t)nblk * 8);
    if (e == cudaSuccess) e = cudaMalloc(&u->satd, (size_t)(ncu ? ncu : 1) * 4);
    if (e == cudaSuccess) e = cudaMalloc(&u->ctx, XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob));
    if (e == cudaSuccess) e = cudaMemset(u->T, 0, coef * sizeof(xg_coef));
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
    /* the kernels' shared-memory limits, once for the largest layout */
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        const int lim = (int)xg_tu_smem_fwd(64, 256);
        attr_err = cudaFuncSetAttribute(k_tu_fwd<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (attr_err == cudaSuccess) attr_err = cudaFuncSetAttribute(k_tu_inv<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    });
    if (xg_cuda_check(attr_err, "TU stage smem attribute")) { xg_tu_free(u); return XIN_GPU_ERR_CUDA; }
    s->tu = u;
    return XIN_GPU_OK;
}

template <int G>
static void xg_tu_launch_pair(const XgTuLevel &lv, int pl, int n, bool fwd, cudaStream_t st)
{
    const int jobs = lv.ncu * (pl ? 1 : lv.nc), ng = 256 / G;
    const int grid = std::max(1, std::min((jobs + ng - 1) / ng, 152 * 8));
    if (fwd) k_tu_fwd<G><<<grid, 256, xg_tu_smem_fwd(n, G), st>>>(lv, pl);
    else k_tu_inv<G><<<grid, 256, xg_tu_smem_inv(n, G), st>>>(lv, pl);
}

static void xg_tu_launch(const XgTuLevel &lv, int pl, bool fwd, cudaStream_t st)
{
    const int n = pl ? lv.S >> 1 : lv.S;
    switch (xg_tu_group(n)) {
    case 256: xg_tu_launch_pair<256>(lv, pl, n, fwd, st); break;
    case 128: xg_tu_launch_pair<128>(lv, pl, n, fwd, st); break;
    case 64: xg_tu_launch_pair<64>(lv, pl, n, fwd, st); break;
    default: xg_tu_launch_pair<32>(lv, pl, n, fwd, st); break;
    }
}

/* the TU stage of the picture in slot cur (picture set t), on st; returns launches */
static int xg_tu_enqueue(xin_gpu_stream *s, int cur, xin_gpu_stream::Set &t, cudaStream_t st)
{
    XgTuState *u = s->tu;
    const xin_gpu_stream_cfg &c = s->cfg;
    const size_t lq = (size_t)c.width * c.height, lc = lq / 4;
    int nl = 0;
    XgTuLevel lv[4];
    int li = 0;
    for (int L = 0; L < 4; L++) {
        if (!s->lev_on[L]) continue;
        XgTuLevel &v = lv[L];
        memset(&v, 0, sizeof v);
        for (int p = 0; p < 3; p++) {
            v.resid[p] = u->resid + u->res_off[L][p];
            v.org[p] = s->slot[cur][p].data;
            v.opitch[p] = s->slot[cur][p].pitch;
            v.T[p] = u->T + u->cand_off[L][p][0];
            v.Q[p] = u->Q + u->cand_off[L][p][0];
            v.R[p] = u->R + u->cand_off[L][p][0];
            v.blk[p] = u->blk[L][p] - u->blk[L][0];
            v.qout[p] = t.dq[p] + (p ? lc : lq) * li;
            v.recout[p] = t.drec[p] + (p ? lc : lq) * li;
        }
        v.cstride = lq;
        v.nz = u->nz + u->blk[L][0];
        v.ssd = u->ssd + u->blk[L][0];
        v.W = c.width; v.S = XG_LEVEL_SIZE[L]; v.cus_x = s->lev_cx[L]; v.ncu = s->lev_cx[L] * s->lev_cy[L]; v.nc = u->nc[L];
        li++;
        if (v.ncu == 0) continue;
        for (int p = 0; p < 3; p++) { xg_tu_launch(v, p, true, st); nl++; }
    }
    k_tu_setqp<<<(u->nblocks + 255) / 256, 256, 0, st>>>(u->plan->d_jobs, u->nblocks, t.dpp);
    nl++;
    xg_dq_enqueue(u->plan->d_jobs, u->plan->d_soff, u->plan->nblocks, u->T, u->Q, u->R, u->nz, u->ctx, 1, u->plan->area,
                  u->plan->ctas, 1, st, false);
    nl += 4;
    cudaMemsetAsync(u->satd, 0, sizeof(uint32_t) * (s->ncus > 0 ? s->ncus : 1), st);
    for (int L = 0; L < 4; L++) {
        if (!s->lev_on[L]) continue;
        XgTuLevel &v = lv[L];
        if (v.ncu == 0) continue;
        for (int p = 0; p < 3; p++) { xg_tu_launch(v, p, false, st); nl++; }
        const int tiles = v.ncu * (v.S >> 3) * (v.S >> 3);
        k_tu_satd<<<(tiles + 255) / 256, 256, 0, st>>>(v, u->satd + s->lev_first[L]);
        k_tu_collect<<<(v.ncu + 127) / 128, 128, 0, st>>>(v, u->satd + s->lev_first[L], t.dres + s->lev_first[L],
                                                          t.dmts + s->lev_first[L], t.dpp);
        nl += 2;
    }
    return nl;
}

extern "C" int xin_gpu_stream_set_contexts(xin_gpu_stream *s, const xin_gpu_prob *ctx)
{
    xin_gpu_clear_error();
    if (!s || !ctx) { xg_set_error(XIN_GPU_ERR_ARG, "stream_set_contexts: null argument"); return XIN_GPU_ERR_ARG; }
    if (!s->tu) { xg_set_error(XIN_GPU_ERR_STATE, "stream_set_contexts: the stream has no preset-4 TU stage (tu_mode 0)"); return XIN_GPU_ERR_STATE; }
    if (s->nsub != s->ndone) { xg_set_error(XIN_GPU_ERR_STATE, "stream_set_contexts: pictures in flight"); return XIN_GPU_ERR_STATE; }
    return xg_cuda_check(cudaMemcpy(s->tu->ctx, ctx, XIN_GPU_NUM_CTX * sizeof(xin_gpu_prob), cudaMemcpyHostToDevice),
                         "stream_set_contexts");
}
