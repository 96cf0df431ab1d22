/*
 * xg_tq_batch.cuh -- batched transform / quant / inverse transform over many
 * residual blocks of mixed sizes and transform types (xin_gpu_tq_batch).
 *
 * Per block it computes what one TU of Xin266Transform
 * (h266_encoder/source/h266_trans_quant.c:61-245, no dependent quantisation,
 * no pre-RDOQ) followed by Xin266IDctWxH (h266_encoder/source/h266_inverse_trans.c:117)
 * computes on a residual: forward DCT2 / DST7 / DCT8 / transform skip with the
 * implicit-MTS rule (h266_forward_trans.c:75-86), zero-out beyond 32,
 * quant / dequant with 4x4 coding groups (h266_quant_inv_quant.c:27-139), and
 * the inverse transform with its skip-line rule.
 *
 * Blocks are grouped by size class on the host.  One launch per class runs a
 * grid of 256-thread CTAs split into groups of G threads (G = 32, 64, 128 or
 * 256); each group takes blocks of the class in turn and synchronises with a
 * named barrier.  G per class is the tile an autotuner picks by timing the
 * candidates on the class's blocks (xin_gpu_tq_batch with tile < 0), or a
 * fixed value.
 */
#include <algorithm>
#include <mutex>
#include <vector>

struct XgTqJob {              /* device copy of xin_gpu_tq_block */
    uint32_t off;
    uint8_t lw, lh, mts, flags;
    int32_t qp;
};

__constant__ int16_t c_qmult[2][6] = { { 26214, 23302, 20560, 18396, 16384, 14564 }, { 18396, 16384, 14564, 13107, 11651, 10280 } };
__constant__ int16_t c_iqmult[2][6] = { { 40, 45, 51, 57, 64, 72 }, { 57, 64, 72, 80, 90, 102 } };
/* MTS index -> (horizontal, vertical) transform, 4 = skip (h26x_core/include/h26x_trans_context.h:42-51) */
__constant__ int8_t c_mts_tx[6][2] = { { 0, 0 }, { 4, 4 }, { 2, 2 }, { 1, 2 }, { 2, 1 }, { 1, 1 } };

template <int G>
__device__ __forceinline__ void xg_group_sync(int gid)
{
    if (G == 32) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(G) : "memory");
}

/* runtime-size C(i, j) = sum_l A(i, l) B(j, l) for the G threads of a group */
template <int G, typename TA, typename TB, typename F>
__device__ __forceinline__ void xg_mm_rt(int t, int nI, int nJ, int nL, const TA *A, int asi, int asl, const TB *B, int bsj, int bsl, F epi)
{
    for (int o = t; o < nI * nJ; o += G) {
        int i = o / nJ, j = o - i * nJ;
        const TA *pa = A + i * asi;
        const TB *pb = B + j * bsj;
        int acc = 0;
#pragma unroll 4
        for (int l = 0; l < nL; l++) acc += (int)pa[l * asl] * (int)pb[l * bsl];
        epi(i, j, acc);
    }
}

/* shared-memory layout of one group, for blocks up to w x h (k = min(32, .)) */
__host__ __device__ inline int xg_tq_group_words(int w, int h)
{
    int kw = w > 32 ? 32 : w, kh = h > 32 ? 32 : h;
    /* int16: resT[w*h], t1T[h*kw], rr[kh*kw], t2[kw*h]; int32: qs[kh*kw] */
    int n16 = w * h + h * kw + kh * kw + kw * h;
    return (n16 + 1) / 2 + kh * kw + 4;   /* + the 8-byte non-zero map, aligned */
}

template <int G>
__global__ void __launch_bounds__(256) k_tq_batch(const XgTqJob *jobs, const uint32_t *list, int n, int w, int h,
                                                  const xg_coef *res, xg_coef *q, xg_coef *r, xg_coef *rout,
                                                  unsigned long long *nzout)
{
    extern __shared__ uint32_t smw[];
    constexpr int NG = 256 / G;
    const int gid = threadIdx.x / G, t = threadIdx.x % G;
    const int kw = w > 32 ? 32 : w, kh = h > 32 ? 32 : h;
    uint32_t *base = smw + gid * xg_tq_group_words(w, h);
    int16_t *resT = (int16_t *)base, *t1T = resT + w * h, *rr = t1T + h * kw, *t2 = rr + kh * kw;
    int32_t *qs = (int32_t *)(base + (w * h + h * kw + kh * kw + kw * h + 1) / 2);
    unsigned long long *nzs = (unsigned long long *)(qs + kh * kw + (((uintptr_t)(qs + kh * kw) & 7) ? 1 : 0));
    const int lw = 31 - __clz(w), lh = 31 - __clz(h);

    for (int bi = blockIdx.x * NG + gid; bi < n; bi += gridDim.x * NG) {
        const XgTqJob jb = jobs[list[bi]];
        const xg_coef *src = res + jb.off;
        int hor = c_mts_tx[jb.mts][0], ver = c_mts_tx[jb.mts][1];
        if ((jb.flags & 1) && !(jb.flags & 2) && (jb.flags & 16) && jb.mts == 0) {   /* implicit MTS */
            if (w >= 4 && w <= 16) hor = 2;
            if (h >= 4 && h <= 16) ver = 2;
        }
        /* quant parameters (Xin266ConstructQuantParam + Xin266Transform) */
        const int skip = hor == 4;
        const int adj = ((lw + lh) & 1) && !skip, lgs = (lw + lh) >> 1;
        const int qp = jb.qp + (XG_BITDEPTH == 10 ? 12 : 0), per = qp / 6, rem = qp % 6;
        const int qmult = c_qmult[adj][rem], iqmult = c_iqmult[adj][rem] << per;
        const int qshift = 14 + (15 - XG_BITDEPTH) + per - lgs - adj, iqshift = 6 - (15 - XG_BITDEPTH) + lgs + adj;
        const int qadd = ((jb.flags & 4) && !skip) ? (1 << (qshift - 1)) : (((jb.flags & 8) ? 171 : 85) << (qshift - 9));
        const int iqadd = !skip ? (1 << (iqshift - 1)) : (1 << ((iqshift - lgs) + (15 - XG_BITDEPTH) - 1));
        if (t == 0) *nzs = 0;
        /* residual, transposed: resT[x * h + y] */
        for (int o = t; o < w * h; o += G) { int y = o / w, x = o - y * w; resT[x * h + y] = (int16_t)src[o]; }
        xg_group_sync<G>(gid);
        if (!skip) {
            const int16_t *mh = xg_mat(hor, lw), *mv = xg_mat(ver, lh);
            const int s1 = lw + XG_BITDEPTH + 6 - 15, s2 = lh + 6;
            /* forward rows: t1T[i * kw + k] = sum_j mh[k][j] res[i][j] */
            xg_mm_rt<G>(t, kw, h, w, mh, w, 1, resT, 1, h, [&](int k, int i, int acc) {
                t1T[i * kw + k] = (int16_t)xg_clip16(xg_rshift_rnd(acc, s1));
            });
            xg_group_sync<G>(gid);
            /* forward columns + quant: (kv, kh) */
            xg_mm_rt<G>(t, kh, kw, h, mv, h, 1, t1T, 1, kw, [&](int kv, int kh2, int acc) {
                int tv = xg_clip16(xg_rshift_rnd(acc, s2)), a = abs(tv);
                int qv = (int)(((long long)a * qmult + qadd) >> qshift);
                qv = xg_clip16(tv < 0 ? -qv : qv);
                qs[kv * kw + kh2] = qv;
                rr[kv * kw + kh2] = (int16_t)xg_clip16((int)(((long long)qv * iqmult + iqadd) >> iqshift));
                if (qv) atomicOr(nzs, 1ull << ((kv >> 2) * (kw >> 2) + (kh2 >> 2)));
            });
        } else {
            /* transform skip: r << (15 - bd - (lw+lh)/2) (Xin26xFSkipWxH restated) */
            const int sh = 15 - XG_BITDEPTH - lgs;
            for (int o = t; o < kh * kw; o += G) {
                int kv = o / kw, kh2 = o - kv * kw;
                int v = resT[kh2 * h + kv];
                int tv = xg_clip16(sh >= 0 ? v * (1 << sh) : xg_rshift_rnd(v, -sh)), a = abs(tv);
                int qv = (int)(((long long)a * qmult + qadd) >> qshift);
                qv = xg_clip16(tv < 0 ? -qv : qv);
                qs[o] = qv;
                rr[o] = (int16_t)xg_clip16((int)(((long long)qv * iqmult + iqadd) >> iqshift));
                if (qv) atomicOr(nzs, 1ull << ((kv >> 2) * (kw >> 2) + (kh2 >> 2)));
            }
        }
        xg_group_sync<G>(gid);
        for (int o = t; o < w * h; o += G) {
            int y = o / w, x = o - y * w;
            bool in = y < kh && x < kw;
            q[jb.off + o] = in ? (xg_coef)qs[y * kw + x] : (xg_coef)0;
            r[jb.off + o] = in ? (xg_coef)rr[y * kw + x] : (xg_coef)0;
        }
        if (t == 0) nzout[list[bi]] = *nzs;
        if (!skip) {
            const int16_t *mh = xg_mat(hor, lw), *mv = xg_mat(ver, lh);
            const int sline = (hor != 0 && w == 32) ? 16 : (w > 32 ? w - 32 : 0), jmax = w - sline;
            const int s2 = 6 + 15 - 1 - XG_BITDEPTH;
            /* inverse columns j < jmax: t2[j * h + y] = sum_{k < kh} mv[k][y] r[k][j] */
            xg_mm_rt<G>(t, jmax, h, kh, rr, 1, kw, mv, 1, h, [&](int j, int y, int acc) {
                t2[j * h + y] = (int16_t)xg_clip16(xg_rshift_rnd(acc, 7));
            });
            xg_group_sync<G>(gid);
            /* inverse rows: out[y][x] = sum_{j < jmax} mh[j][x] t2[j * h + y] */
            xg_mm_rt<G>(t, h, w, jmax, t2, 1, h, mh, 1, w, [&](int y, int x, int acc) {
                rout[jb.off + y * w + x] = (xg_coef)xg_clip16(xg_rshift_rnd(acc, s2));
            });
        } else {
            const int sh = 15 - 8 - lgs;   /* Xin266ISkipWxH (h266_inverse_trans.c:91-115) */
            for (int o = t; o < w * h; o += G) {
                int y = o / w, x = o - y * w;
                int v = (y < kh && x < kw) ? rr[y * kw + x] : 0;
                rout[jb.off + o] = (xg_coef)(int16_t)(v >> sh);
            }
        }
        xg_group_sync<G>(gid);
    }
}

#include "xg_tq_tc.cuh"

/* ------------------------------------------------------------------ host */
struct XgTqTuner {
    std::mutex mu;
    int g[7][7];      /* tuned group size per (lw, lh), 0 = not tuned */
};
static XgTqTuner g_tq_tuner;

static int xg_tq_fixed_group(int w, int h) { return w * h >= 1024 ? 256 : (w * h >= 256 ? 128 : 64); }

static cudaError_t xg_tq_launch_class(int G, int nblk, int w, int h, const XgTqJob *jobs, const uint32_t *list,
                                      const xg_coef *res, xg_coef *q, xg_coef *r, xg_coef *rout, unsigned long long *nz,
                                      cudaStream_t st)
{
    int ng = 256 / G;
    size_t smem = (size_t)ng * xg_tq_group_words(w, h) * 4;
    int sms = 152;
    int grid = std::min((nblk + ng - 1) / ng, sms * 8);
    if (grid < 1) grid = 1;
    /* per-kernel limit set once to the largest group layout (200 KB), never
     * lowered, so that concurrent callers with other block sizes cannot race */
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        const int lim = 200 * 1024;
        attr_err = cudaFuncSetAttribute(k_tq_batch<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (attr_err == cudaSuccess) attr_err = cudaFuncSetAttribute(k_tq_batch<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (attr_err == cudaSuccess) attr_err = cudaFuncSetAttribute(k_tq_batch<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (attr_err == cudaSuccess) attr_err = cudaFuncSetAttribute(k_tq_batch<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
    });
    if (attr_err != cudaSuccess) return attr_err;
    switch (G) {
    case 32: k_tq_batch<32><<<grid, 256, smem, st>>>(jobs, list, nblk, w, h, res, q, r, rout, nz); break;
    case 64: k_tq_batch<64><<<grid, 256, smem, st>>>(jobs, list, nblk, w, h, res, q, r, rout, nz); break;
    case 128: k_tq_batch<128><<<grid, 256, smem, st>>>(jobs, list, nblk, w, h, res, q, r, rout, nz); break;
    default: k_tq_batch<256><<<grid, 256, smem, st>>>(jobs, list, nblk, w, h, res, q, r, rout, nz); break;
    }
    xg_count_launch(1);
    return cudaGetLastError();
}

/* group size of one class: fixed, explicit, or autotuned (times every candidate
 * on this class's blocks with the caller's arrays, then caches the winner) */
static int xg_tq_pick(int c, int cls_first, int cls_n, const XgTqJob *d_jobs, const uint32_t *d_list, const xg_coef *res,
                      xg_coef *q, xg_coef *r, xg_coef *rout, unsigned long long *nz, int32_t tile, cudaStream_t st, int *G)
{
    int lw = c / 7, lh = c % 7, w = 1 << lw, h = 1 << lh;
    if (tile > 0) *G = tile;
    else if (tile == 0 || tile == XIN_GPU_TQ_TENSOR) *G = xg_tq_fixed_group(w, h);
    else {
        std::lock_guard<std::mutex> lock(g_tq_tuner.mu);
        *G = g_tq_tuner.g[lw][lh];
        if (!*G) {
            cudaEvent_t a, b;
            if (xg_cuda_check(cudaEventCreate(&a), "tq autotune") || xg_cuda_check(cudaEventCreate(&b), "tq autotune"))
                return XIN_GPU_ERR_CUDA;
            float best = 1e30f;
            int bestG = xg_tq_fixed_group(w, h);
            for (int cand : { 32, 64, 128, 256 }) {
                if ((size_t)(256 / cand) * xg_tq_group_words(w, h) * 4 > 200 * 1024) continue;
                for (int rep = 0; rep < 3; rep++) {
                    cudaEventRecord(a, st);
                    cudaError_t e = xg_tq_launch_class(cand, cls_n, w, h, d_jobs, d_list + cls_first, res, q, r, rout, nz, st);
                    cudaEventRecord(b, st);
                    if (e == cudaSuccess) e = cudaEventSynchronize(b);
                    if (e != cudaSuccess) { cudaEventDestroy(a); cudaEventDestroy(b); return xg_cuda_check(e, "tq autotune"); }
                    float ms = 0;
                    cudaEventElapsedTime(&ms, a, b);
                    if (rep && ms < best) { best = ms; bestG = cand; }
                }
            }
            cudaEventDestroy(a); cudaEventDestroy(b);
            g_tq_tuner.g[lw][lh] = *G = bestG;
        }
    }
    if ((size_t)(256 / *G) * xg_tq_group_words(w, h) * 4 > 200 * 1024) *G = 256;
    return XIN_GPU_OK;
}

/* a validated, sorted block list resident on the device */
struct xin_gpu_tq_plan {
    int device;
    int32_t nblocks;
    size_t ncoeffs;
    int32_t tile;               /* as requested */
    XgTqJob *d_jobs;
    uint32_t *d_list;           /* blocks on the CUDA cores, by size class */
    int first[50], cnt[50];
    int G[49];                  /* resolved group size per class, 0 = not resolved yet */
    /* tensor-core form (tile == XIN_GPU_TQ_TENSOR): transform blocks in tiles of one
     * size and transform pair; transform-skip blocks stay on the CUDA cores */
    XgTcTile *d_tiles;
    uint32_t *d_tlist;
    int ntiles;
    int *d_err;                 /* [0] set by a tensor-core wait that timed out; [1] the tile queue's counter */
    long long wait_tries;       /* polls of one tensor-core wait before it gives up */
};

/* MTS index -> (horizontal, vertical) transform of the host (4 = skip) */
static const int8_t h_mts_tx[6][2] = { { 0, 0 }, { 4, 4 }, { 2, 2 }, { 1, 2 }, { 2, 1 }, { 1, 1 } };

/* tiles of the tensor-core form: transform blocks grouped by (size, hor, ver),
 * each tile up to 128 / max(h, min(w, 32)) blocks of one group */
static void xg_tq_tiles(const xin_gpu_tq_block *blocks, int32_t n, std::vector<XgTcTile> &tiles, std::vector<uint32_t> &tlist,
                        std::vector<uint32_t> &skip)
{
    std::vector<std::pair<uint32_t, uint32_t>> keyed;     /* (group key, block) */
    for (int i = 0; i < n; i++) {
        const xin_gpu_tq_block &b = blocks[i];
        int hor = h_mts_tx[b.mts][0], ver = h_mts_tx[b.mts][1];
        /* transform skip, and blocks whose offset does not allow the tensor kernel's
         * 8-sample vector loads, stay on the CUDA cores */
        if (hor == 4 || (b.offset & 7)) { skip.push_back((uint32_t)i); continue; }
        if ((b.flags & 1) && !(b.flags & 2) && (b.flags & 16) && b.mts == 0) {   /* implicit MTS */
            if (b.log2w <= 4) hor = 2;
            if (b.log2h <= 4) ver = 2;
        }
        keyed.push_back({ (uint32_t)((b.log2w * 7 + b.log2h) * 9 + hor * 3 + ver), (uint32_t)i });
    }
    /* largest blocks first: the longest tiles start earliest */
    std::stable_sort(keyed.begin(), keyed.end(), [](const std::pair<uint32_t, uint32_t> &a, const std::pair<uint32_t, uint32_t> &b) {
        return a.first > b.first;
    });
    tlist.resize(keyed.size());
    for (size_t i = 0; i < keyed.size();) {
        size_t j = i;
        while (j < keyed.size() && keyed[j].first == keyed[i].first) j++;
        const uint32_t key = keyed[i].first, cls = key / 9;
        const int lw = cls / 7, lh = cls % 7, w = 1 << lw, h = 1 << lh, kw = w > 32 ? 32 : w;
        const int per = 128 / (h > kw ? h : kw);
        for (size_t k = i; k < j; k += per) {
            XgTcTile t;
            memset(&t, 0, sizeof t);
            t.first = (uint32_t)k;
            t.count = (uint8_t)std::min<size_t>(per, j - k);
            t.lw = (uint8_t)lw; t.lh = (uint8_t)lh; t.hor = (uint8_t)((key % 9) / 3); t.ver = (uint8_t)(key % 3);
            tiles.push_back(t);
        }
        for (size_t k = i; k < j; k++) tlist[k] = keyed[k].second;
        i = j;
    }
}

/* enqueue every class on st; resolves group sizes on first use */
static int xg_tq_plan_enqueue(xin_gpu_tq_plan *p, const xg_coef *res, xg_coef *q, xg_coef *r, xg_coef *rout,
                              unsigned long long *nz, cudaStream_t st)
{
    if (p->ntiles && (((uintptr_t)res | (uintptr_t)q | (uintptr_t)r | (uintptr_t)rout) & 15)) {
        xg_set_error(XIN_GPU_ERR_ARG, "tq_plan_run: the tensor-core form needs 16-byte aligned arrays");
        return XIN_GPU_ERR_ARG;
    }
    if (p->ntiles) {
        /* persistent CTAs: as many as fit at once (shared memory keeps it to at most
         * four per SM, within the SM's 512 TMEM columns) */
        static std::once_flag attr_once;
        static cudaError_t attr_err = cudaSuccess;
        static int resident = 0;
        std::call_once(attr_once, [] {
            attr_err = cudaFuncSetAttribute(k_tq_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, XG_TC_SMEM);
            int dev = 0, sms = 0, smem_sm = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
            const int per_sm = smem_sm / (XG_TC_SMEM + 1024);     /* the runtime keeps 1 KB per CTA */
            resident = std::max(1, std::min(per_sm, 4)) * sms;
        });
        if (xg_cuda_check(attr_err, "tq tensor smem attribute")) return XIN_GPU_ERR_CUDA;
        const int grid = std::min(p->ntiles, resident);
        if (xg_cuda_check(cudaMemsetAsync(p->d_err + 1, 0, sizeof(int), st), "tq tile queue")) return XIN_GPU_ERR_CUDA;
        k_tq_tc<<<grid, XG_TC_THREADS, XG_TC_SMEM, st>>>(p->d_tiles, p->ntiles, p->d_jobs, p->d_tlist, res, q, r, rout, nz, p->d_err,
                                                           p->d_err + 1, p->wait_tries);
        xg_count_launch(1);
        if (xg_cuda_check(cudaGetLastError(), "tq tensor launch")) return XIN_GPU_ERR_CUDA;
    }
    for (int c = 0; c < 49; c++) {
        if (!p->cnt[c]) continue;
        if (!p->G[c]) {
            int s = xg_tq_pick(c, p->first[c], p->cnt[c], p->d_jobs, p->d_list, res, q, r, rout, nz, p->tile, st, &p->G[c]);
            if (s) return s;
        }
        cudaError_t e = xg_tq_launch_class(p->G[c], p->cnt[c], 1 << (c / 7), 1 << (c % 7), p->d_jobs, p->d_list + p->first[c],
                                           res, q, r, rout, nz, st);
        if (e != cudaSuccess) return xg_cuda_check(e, "tq launch");
    }
    return XIN_GPU_OK;
}

static int xg_tq_validate(const xin_gpu_tq_block *blocks, int32_t n, size_t ncoeffs, std::vector<XgTqJob> &jobs,
                          std::vector<uint32_t> &list, int first[50], int cnt[50])
{
    jobs.resize(n);
    for (int c = 0; c < 50; c++) { first[c] = 0; cnt[c] = 0; }
    for (int i = 0; i < n; i++) {
        const xin_gpu_tq_block &b = blocks[i];
        if (b.log2w < 2 || b.log2w > 6 || b.log2h < 2 || b.log2h > 6 || b.mts > 5 || b.qp < 0 || b.qp > 63 ||
            (b.mts >= 1 && (b.log2w > 5 || b.log2h > 5)) ||   /* skip and MTS pairs stop at 32 */
            (size_t)b.offset + ((size_t)1 << (b.log2w + b.log2h)) > ncoeffs) {
            xg_set_error(XIN_GPU_ERR_ARG, "tq_batch: block %d invalid (size, MTS type, QP or offset beyond %zu coefficients)", i, ncoeffs);
            return XIN_GPU_ERR_ARG;
        }
        jobs[i] = { b.offset, b.log2w, b.log2h, b.mts, b.flags, b.qp };
        cnt[b.log2w * 7 + b.log2h]++;
    }
    for (int c = 1; c < 50; c++) first[c] = first[c - 1] + cnt[c - 1];
    int pos[50];
    for (int c = 0; c < 50; c++) pos[c] = first[c];
    list.resize(n);
    for (int i = 0; i < n; i++) list[pos[blocks[i].log2w * 7 + blocks[i].log2h]++] = (uint32_t)i;
    return XIN_GPU_OK;
}

extern "C" void xin_gpu_tq_plan_destroy(xin_gpu_tq_plan *p)
{
    if (!p) return;
    cudaFree(p->d_jobs);
    cudaFree(p->d_list);
    cudaFree(p->d_tiles);
    cudaFree(p->d_tlist);
    cudaFree(p->d_err);
    delete p;
}

/* XIN_GPU_ERR_TIMEOUT if a tensor-core wait of an earlier run gave up (synchronises) */
static int xg_tq_plan_status(xin_gpu_tq_plan *p)
{
    if (!p->d_err) return XIN_GPU_OK;
    int e = 0;
    if (xg_cuda_check(cudaMemcpy(&e, p->d_err, sizeof e, cudaMemcpyDeviceToHost), "tq status")) return XIN_GPU_ERR_CUDA;
    if (e) {
        /* reported once: later runs start with a clear flag */
        if (xg_cuda_check(cudaMemset(p->d_err, 0, sizeof(int)), "tq status")) return XIN_GPU_ERR_CUDA;
        xg_set_error(XIN_GPU_ERR_TIMEOUT, "tq_batch: a tensor-core wait timed out");
        return XIN_GPU_ERR_TIMEOUT;
    }
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_tq_plan_create(const xin_gpu_tq_block *blocks, int32_t nblocks, size_t ncoeffs, int32_t tile,
                                      xin_gpu_tq_plan **out)
{
    xin_gpu_clear_error();
    if (!blocks || nblocks <= 0 || !out ||
        (tile != XIN_GPU_TQ_TENSOR && tile != -1 && tile != 0 && tile != 32 && tile != 64 && tile != 128 && tile != 256)) {
        xg_set_error(XIN_GPU_ERR_ARG, "tq_plan_create: bad argument (tile must be -2, -1, 0, 32, 64, 128 or 256)");
        return XIN_GPU_ERR_ARG;
    }
    *out = nullptr;
    if (!xg_thread()) return xin_gpu_last_status();
    std::vector<XgTqJob> jobs;
    std::vector<uint32_t> list;
    xin_gpu_tq_plan *p = new xin_gpu_tq_plan();
    int st = xg_tq_validate(blocks, nblocks, ncoeffs, jobs, list, p->first, p->cnt);
    if (st) { delete p; return st; }
    cudaGetDevice(&p->device);
    p->nblocks = nblocks;
    p->ncoeffs = ncoeffs;
    p->tile = tile;
    p->wait_tries = XG_TC_WAIT_TRIES;
    std::vector<XgTcTile> tiles;
    std::vector<uint32_t> tlist;
    if (tile == XIN_GPU_TQ_TENSOR) {
        /* transform blocks go to the tensor cores; the CUDA-core classes keep the skip blocks */
        std::vector<uint32_t> skip;
        xg_tq_tiles(blocks, nblocks, tiles, tlist, skip);
        for (int c = 0; c < 50; c++) { p->first[c] = 0; p->cnt[c] = 0; }
        for (uint32_t i : skip) p->cnt[blocks[i].log2w * 7 + blocks[i].log2h]++;
        for (int c = 1; c < 50; c++) p->first[c] = p->first[c - 1] + p->cnt[c - 1];
        int pos[50];
        for (int c = 0; c < 50; c++) pos[c] = p->first[c];
        list.assign(skip.size() ? skip.size() : 1, 0);
        for (uint32_t i : skip) list[pos[blocks[i].log2w * 7 + blocks[i].log2h]++] = i;
        p->ntiles = (int)tiles.size();
    }
    if (xg_cuda_check(cudaMalloc(&p->d_jobs, jobs.size() * sizeof(XgTqJob)), "tq plan") ||
        xg_cuda_check(cudaMalloc(&p->d_list, list.size() * 4), "tq plan") ||
        xg_cuda_check(cudaMemcpy(p->d_jobs, jobs.data(), jobs.size() * sizeof(XgTqJob), cudaMemcpyHostToDevice), "tq plan") ||
        xg_cuda_check(cudaMemcpy(p->d_list, list.data(), list.size() * 4, cudaMemcpyHostToDevice), "tq plan")) {
        xin_gpu_tq_plan_destroy(p);
        return XIN_GPU_ERR_CUDA;
    }
    if (p->ntiles &&
        (xg_cuda_check(cudaMalloc(&p->d_tiles, tiles.size() * sizeof(XgTcTile)), "tq plan") ||
         xg_cuda_check(cudaMalloc(&p->d_tlist, tlist.size() * 4), "tq plan") ||
         xg_cuda_check(cudaMalloc(&p->d_err, 2 * sizeof(int)), "tq plan") ||
         xg_cuda_check(cudaMemset(p->d_err, 0, 2 * sizeof(int)), "tq plan") ||
         xg_cuda_check(cudaMemcpy(p->d_tiles, tiles.data(), tiles.size() * sizeof(XgTcTile), cudaMemcpyHostToDevice), "tq plan") ||
         xg_cuda_check(cudaMemcpy(p->d_tlist, tlist.data(), tlist.size() * 4, cudaMemcpyHostToDevice), "tq plan"))) {
        xin_gpu_tq_plan_destroy(p);
        return XIN_GPU_ERR_CUDA;
    }
    *out = p;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_tq_plan_run(xin_gpu_tq_plan *p, const XG_COEFF *resid, XG_COEFF *q, XG_COEFF *r, XG_COEFF *resid_out,
                                   uint64_t *nz, void *stream)
{
    xin_gpu_clear_error();
    if (!p || !resid || !q || !r || !resid_out || !nz) {
        xg_set_error(XIN_GPU_ERR_ARG, "tq_plan_run: bad argument");
        return XIN_GPU_ERR_ARG;
    }
    cudaGetLastError();
    return xg_tq_plan_enqueue(p, (const xg_coef *)resid, (xg_coef *)q, (xg_coef *)r, (xg_coef *)resid_out,
                              (unsigned long long *)nz, (cudaStream_t)stream);
}

extern "C" int xin_gpu_tq_plan_tiles(const xin_gpu_tq_plan *p, int32_t *tiles)
{
    if (!p || !tiles) { xg_set_error(XIN_GPU_ERR_ARG, "tq_plan_tiles: bad argument"); return XIN_GPU_ERR_ARG; }
    for (int c = 0; c < 49; c++) tiles[c] = p->G[c];
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_tq_plan_status(xin_gpu_tq_plan *p)
{
    xin_gpu_clear_error();
    if (!p) { xg_set_error(XIN_GPU_ERR_ARG, "tq_plan_status: null plan"); return XIN_GPU_ERR_ARG; }
    return xg_tq_plan_status(p);
}

extern "C" int xin_gpu_tq_plan_set_wait_tries(xin_gpu_tq_plan *p, int64_t tries)
{
    xin_gpu_clear_error();
    if (!p || tries < 0) { xg_set_error(XIN_GPU_ERR_ARG, "tq_plan_set_wait_tries: bad argument"); return XIN_GPU_ERR_ARG; }
    p->wait_tries = tries ? (long long)tries : 0;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_tq_batch_device(const xin_gpu_tq_block *blocks, int32_t nblocks, const XG_COEFF *resid, XG_COEFF *q,
                                       XG_COEFF *r, XG_COEFF *resid_out, uint64_t *nz, size_t ncoeffs, int32_t tile,
                                       void *stream, int32_t *tiles_used)
{
    xin_gpu_tq_plan *p = nullptr;
    int st = xin_gpu_tq_plan_create(blocks, nblocks, ncoeffs, tile, &p);
    if (st) return st;
    st = xin_gpu_tq_plan_run(p, resid, q, r, resid_out, nz, stream);
    if (!st) st = xg_cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "tq sync");
    if (!st) st = xg_tq_plan_status(p);
    if (!st && tiles_used) xin_gpu_tq_plan_tiles(p, tiles_used);
    xin_gpu_tq_plan_destroy(p);
    return st;
}

extern "C" int xin_gpu_tq_batch(const xin_gpu_tq_block *blocks, int32_t nblocks, const XG_COEFF *resid, XG_COEFF *q, XG_COEFF *r,
                                XG_COEFF *resid_out, uint64_t *nz, size_t ncoeffs, int32_t tile)
{
    xin_gpu_clear_error();
    if (!blocks || nblocks <= 0 || !resid || !q || !r || !resid_out || !nz) {
        xg_set_error(XIN_GPU_ERR_ARG, "tq_batch: bad argument");
        return XIN_GPU_ERR_ARG;
    }
    if (tile > 0 && tile != 32 && tile != 64 && tile != 128 && tile != 256) {
        xg_set_error(XIN_GPU_ERR_ARG, "tq_batch: tile must be -2 (tensor cores), -1 (autotune), 0 (fixed), 32, 64, 128 or 256");
        return XIN_GPU_ERR_ARG;
    }
    XgThread *t = xg_thread();
    if (!t) return xin_gpu_last_status();
    xin_gpu_tq_plan *p = nullptr;
    int st = xin_gpu_tq_plan_create(blocks, nblocks, ncoeffs, tile, &p);
    if (st) return st;
    size_t bytes = ncoeffs * sizeof(xg_coef);
    xg_coef *d_res = (xg_coef *)xg_dalloc(t, bytes), *d_q = (xg_coef *)xg_dalloc(t, bytes), *d_r = (xg_coef *)xg_dalloc(t, bytes),
            *d_o = (xg_coef *)xg_dalloc(t, bytes);
    unsigned long long *d_nz = (unsigned long long *)xg_dalloc(t, (size_t)nblocks * 8);
    if (!d_res || !d_q || !d_r || !d_o || !d_nz) { xin_gpu_tq_plan_destroy(p); return xin_gpu_last_status(); }
    st = xg_cuda_check(cudaMemcpyAsync(d_res, resid, bytes, cudaMemcpyHostToDevice, t->stream), "tq h2d");
    /* samples that no block covers come back as zeros, not as staging leftovers */
    if (!st) st = xg_cuda_check(cudaMemsetAsync(d_q, 0, bytes, t->stream), "tq clear") ||
                  xg_cuda_check(cudaMemsetAsync(d_r, 0, bytes, t->stream), "tq clear") ||
                  xg_cuda_check(cudaMemsetAsync(d_o, 0, bytes, t->stream), "tq clear") ? XIN_GPU_ERR_CUDA : XIN_GPU_OK;
    if (!st) st = xin_gpu_tq_plan_run(p, (const XG_COEFF *)d_res, (XG_COEFF *)d_q, (XG_COEFF *)d_r, (XG_COEFF *)d_o,
                                      (uint64_t *)d_nz, t->stream);
    if (!st)
        st = xg_cuda_check(cudaMemcpyAsync(q, d_q, bytes, cudaMemcpyDeviceToHost, t->stream), "tq d2h") ||
             xg_cuda_check(cudaMemcpyAsync(r, d_r, bytes, cudaMemcpyDeviceToHost, t->stream), "tq d2h") ||
             xg_cuda_check(cudaMemcpyAsync(resid_out, d_o, bytes, cudaMemcpyDeviceToHost, t->stream), "tq d2h") ||
             xg_cuda_check(cudaMemcpyAsync(nz, d_nz, (size_t)nblocks * 8, cudaMemcpyDeviceToHost, t->stream), "tq d2h")
                 ? XIN_GPU_ERR_CUDA : XIN_GPU_OK;
    if (!st) st = xg_cuda_check(cudaStreamSynchronize(t->stream), "tq sync");
    if (!st) st = xg_tq_plan_status(p);
    xin_gpu_tq_plan_destroy(p);
    return st;
}
