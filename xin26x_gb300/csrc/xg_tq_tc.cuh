/*
 * xg_tq_tc.cuh -- the batched transform / quant of xg_tq_batch.cuh on the
 * tensor cores (tcgen05, accumulators in tensor memory).
 *
 * Every transform pass is a product of 16-bit integer samples with the
 * transform matrix (entries of magnitude <= 90).  The tensor cores compute it
 * exactly in f16 x f16 -> f32: a sample x (int16) is split into x = 256 hi + lo
 * with lo in [0, 255] and hi in [-128, 127], both exact in f16; each half's
 * product sum is an integer below 2^24 in magnitude (64 x 255 x 90), exact in
 * f32; hi * 256 + lo in int32 is then the integer sum the reference computes.
 *
 * A CTA (128 threads, one TMEM lane per thread) takes a tile of up to
 * 128 / max(h, min(w, 32)) blocks that share size and transform types and runs
 * the four passes in order, each as M = 128 rows x N x K MMAs (K-major
 * operands in shared memory, no swizzle) for the high and the low halves:
 *   F1  rows (b, i)  K = j  N = k  : t1 = clip16(rnd(sum, s1))            (Xin26xFDct*)
 *   F2  rows (b, k)  K = i  N = kv : coefficient, quant / dequant  (A MN-major) (Xin266QuantInvQuant)
 *   I1  rows (b, j)  K = kv N = y  : t2 = clip16(rnd(sum, 7))              (Xin26xIDct*, columns)
 *   I2  rows (b, y)  K = j  N = x  : out = clip16(rnd(sum, 20 - bd)) (A MN-major) (rows, skip-line rule)
 * The epilogue of a pass (tcgen05.ld, one row per thread) writes the next
 * pass's A operand in shared memory.  A pass has one CTA barrier (before its
 * MMA); every thread then waits for the commit itself, so the epilogue needs no
 * second one.  Work that does not depend on the pass (the next tile's job
 * records, the zero tails of 64-wide blocks, the non-zero maps) runs while its
 * MMA is in flight.  Transform-skip blocks stay on the CUDA cores
 * (xg_tq_batch.cuh).
 */

#include <cuda_fp16.h>

#define XG_TC_THREADS 128
#define XG_TC_KMAX 64                     /* K and N of any pass are at most 64 */
#define XG_TC_A_BYTES (128 * XG_TC_KMAX * 2)
#define XG_TC_B_BYTES (32 * XG_TC_KMAX * 2)    /* one pass's B: at most 32 x 64 or 64 x 32 */
/* dynamic shared memory: A hi, A lo, the four passes' B (kept while the tile
 * group does not change), then small state (the mbarrier, the TMEM address, job
 * records and non-zero maps of two tiles); 50 KB lets four CTAs share an SM,
 * and no more (4 x 128 TMEM columns = the SM's 512) */
#define XG_TC_SMEM (50 * 1024)
#define XG_TC_TMEM_COLS 128               /* hi accumulator at column 0, lo at 64 */

struct XgTcTile {
    uint32_t first;                       /* index into the sorted block list */
    uint8_t count, lw, lh, hor, ver;      /* blocks; log2 sizes; transform types (0 DCT2, 1 DCT8, 2 DST7) */
    uint8_t pad[3];
};

/* byte offset of element (row, k) in a K-major, no-swizzle operand with kp
 * (a multiple of 16) columns: 8-row x 16-byte core matrices, K-direction stride
 * 128 B, row-group stride kp * 16 B */
__device__ __forceinline__ int xg_tc_off(int row, int k, int kp) { return ((row >> 3) * (kp >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2; }

__device__ __forceinline__ uint64_t xg_tc_desc(uint32_t saddr, int kp)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(128 >> 4) << 16;                       /* K-direction core-matrix stride */
    d |= (uint64_t)(((kp >> 3) * 128) >> 4) << 32;         /* 8-row-group stride */
    d |= (uint64_t)1 << 46;                                /* descriptor version */
    return d;
}

/* byte offset of element (m, k) in an MN-major, no-swizzle A operand (128 rows):
 * core matrices of 8 K-rows x 8 M-elements (16 bytes), M-direction stride 128 B
 * (the descriptor's SBO), K-direction stride 2048 B (its LBO) */
__device__ __forceinline__ int xg_tc_mn_off(int m, int k) { return (m >> 3) * 128 + (k >> 3) * 2048 + (k & 7) * 16 + (m & 7) * 2; }

__device__ __forceinline__ uint64_t xg_tc_desc_mn(uint32_t saddr)
{
    uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
    d |= (uint64_t)(2048 >> 4) << 16;                      /* K-direction core-matrix stride */
    d |= (uint64_t)(128 >> 4) << 32;                       /* M-direction core-matrix stride */
    d |= (uint64_t)1 << 46;                                /* descriptor version */
    return d;
}

/* Conversions without the conversion unit.  In: two int16 values (the halves
 * of w) as exact f16 pairs hi = x >> 8 in [-128, 127] and lo = x & 255: the
 * bytes are or-ed under the exponent of 1024 (where the f16 step is 1), and
 * 1024 (+ 128 for the sign-flipped high byte) is taken off by one half2
 * subtraction, exact for integers below 2048.  Out: an accumulator (an integer
 * below 2^22 in magnitude) plus 1.5 * 2^23 has the integer in its low mantissa
 * bits. */
__device__ __forceinline__ void xg_tc_split2(uint32_t w, uint32_t &hi, uint32_t &lo)
{
    const uint32_t l = (w & 0x00FF00FFu) | 0x64006400u;                  /* 1024 + lo */
    const uint32_t h = ((w >> 8) & 0x00FF00FFu) ^ 0x64806480u;            /* 1152 + hi */
    const __half2 lh = __hsub2(*(const __half2 *)&l, __halves2half2(__ushort_as_half(0x6400), __ushort_as_half(0x6400)));
    const __half2 hh = __hsub2(*(const __half2 *)&h, __halves2half2(__ushort_as_half(0x6480), __ushort_as_half(0x6480)));
    lo = *(const uint32_t *)&lh;
    hi = *(const uint32_t *)&hh;
}

/* 256 * hi + lo from the raw f32 accumulators of the two halves */
__device__ __forceinline__ int xg_tc_comb(uint32_t h, uint32_t l)
{
    const uint32_t bh = __float_as_uint(__uint_as_float(h) + 12582912.0f), bl = __float_as_uint(__uint_as_float(l) + 12582912.0f);
    return (int)(bh * 256u + bl - 257u * 0x4B400000u);
}

/* D[hi|lo] (128 x np) = A[hi|lo] (128 x kp) . B (np x kp)^T, issued by one thread;
 * A K-major, or MN-major when a_mn (instruction-descriptor bit 15) */
__device__ __forceinline__ void xg_tc_mma(uint32_t tmem, uint32_t ahi, uint32_t alo, uint32_t b, int kp, int np, uint32_t mbar,
                                          bool a_mn)
{
    const uint32_t idesc = (1u << 4) | (a_mn ? 1u << 15 : 0u) | ((uint32_t)(np >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    for (int h = 0; h < 2; h++) {
        const uint32_t a = h ? alo : ahi;
        for (int kk = 0; kk < kp / 16; kk++) {
            const uint64_t ad = a_mn ? xg_tc_desc_mn(a + kk * 4096) : xg_tc_desc(a + kk * 256, kp);
            const uint64_t bd = xg_tc_desc(b + kk * 256, kp);
            const uint32_t en = kk > 0;
            asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                         ::"r"(tmem + (h ? 64u : 0u)), "l"(ad), "l"(bd), "r"(idesc), "r"(en) : "memory");
        }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

/* default bound of a wait for an MMA commit: about a second */
#define XG_TC_WAIT_TRIES (1LL << 26)

/* bounded wait for the commit of phase `phase`; false after `tries` polls */
__device__ __forceinline__ bool xg_tc_wait(uint32_t mbar, uint32_t phase, long long tries)
{
    uint32_t done = 0;
    for (long long it = 0; it < tries && !done; it++)
        asm volatile("{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}"
                     : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
    return done != 0;
}

/* columns [c0, c0 + 8) of this thread's TMEM lane, hi and lo combined */
__device__ __forceinline__ void xg_tc_row8(uint32_t tmem, int warp, int c0, int out[8])
{
    uint32_t h[8], l[8];
    const uint32_t a = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(h[0]), "=r"(h[1]), "=r"(h[2]), "=r"(h[3]), "=r"(h[4]), "=r"(h[5]), "=r"(h[6]), "=r"(h[7]) : "r"(a));
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(l[0]), "=r"(l[1]), "=r"(l[2]), "=r"(l[3]), "=r"(l[4]), "=r"(l[5]), "=r"(l[6]), "=r"(l[7]) : "r"(a + 64));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 8; j++) out[j] = xg_tc_comb(h[j], l[j]);
}

/* columns [c0, c0 + 16) of this thread's TMEM lane, hi and lo combined: both
 * loads in flight before one wait */
__device__ __forceinline__ void xg_tc_row16(uint32_t tmem, int warp, int c0, int out[16])
{
    uint32_t h[16], l[16];
    const uint32_t a = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(h[0]), "=r"(h[1]), "=r"(h[2]), "=r"(h[3]), "=r"(h[4]), "=r"(h[5]), "=r"(h[6]), "=r"(h[7]),
                   "=r"(h[8]), "=r"(h[9]), "=r"(h[10]), "=r"(h[11]), "=r"(h[12]), "=r"(h[13]), "=r"(h[14]), "=r"(h[15])
                 : "r"(a));
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(l[0]), "=r"(l[1]), "=r"(l[2]), "=r"(l[3]), "=r"(l[4]), "=r"(l[5]), "=r"(l[6]), "=r"(l[7]),
                   "=r"(l[8]), "=r"(l[9]), "=r"(l[10]), "=r"(l[11]), "=r"(l[12]), "=r"(l[13]), "=r"(l[14]), "=r"(l[15])
                 : "r"(a + 64));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) out[j] = xg_tc_comb(h[j], l[j]);
}

/* eight int16 values as the f16 halves of one 16-byte core-matrix row each */
__device__ __forceinline__ void xg_tc_put8(uint8_t *ahi, uint8_t *alo, int off, const int x[8])
{
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int p = 0; p < 4; p++) xg_tc_split2(__byte_perm(x[2 * p], x[2 * p + 1], 0x5410), hw[p], lw[p]);
    *(uint4 *)(ahi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *(uint4 *)(alo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
}

/* four int16 values as f16 halves, 8 bytes each */
__device__ __forceinline__ void xg_tc_put4(uint8_t *ahi, uint8_t *alo, int off, const int x[4])
{
    uint32_t hw[2], lw[2];
#pragma unroll
    for (int p = 0; p < 2; p++) xg_tc_split2(__byte_perm(x[2 * p], x[2 * p + 1], 0x5410), hw[p], lw[p]);
    *(uint2 *)(ahi + off) = make_uint2(hw[0], hw[1]);
    *(uint2 *)(alo + off) = make_uint2(lw[0], lw[1]);
}

__global__ void __launch_bounds__(XG_TC_THREADS) k_tq_tc(const XgTcTile *tiles, int ntiles, const XgTqJob *jobs,
                                                        const uint32_t *list, const xg_coef *res, xg_coef *q, xg_coef *r,
                                                        xg_coef *rout, unsigned long long *nzout, int *err,
                                                        int *next_tile, long long wait_tries)
{
    extern __shared__ __align__(1024) uint8_t smc[];
    uint8_t *ahi = smc, *alo = smc + XG_TC_A_BYTES, *bm = smc + 2 * XG_TC_A_BYTES;   /* bm: [4][XG_TC_B_BYTES] */
    uint64_t *mbar = (uint64_t *)(bm + 4 * XG_TC_B_BYTES);
    uint32_t *tslot = (uint32_t *)(mbar + 1);
    unsigned long long *snz = (unsigned long long *)(mbar + 2);         /* [2][32] per-block non-zero maps, by tile parity */
    XgTqJob *sjob = (XgTqJob *)(snz + 64);                              /* [2][32] job records, by tile parity */
    int *snext = (int *)(sjob + 64);                                    /* [2] the tile after this one, by parity */
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t s_ahi = (uint32_t)__cvta_generic_to_shared(ahi), s_alo = (uint32_t)__cvta_generic_to_shared(alo);
    const uint32_t s_b = (uint32_t)__cvta_generic_to_shared(bm), s_mbar = (uint32_t)__cvta_generic_to_shared(mbar);
    static_assert(2 * XG_TC_A_BYTES + 4 * XG_TC_B_BYTES + 16 + 64 * 8 + 64 * sizeof(XgTqJob) + 8 <= XG_TC_SMEM, "shared layout");
    /* tiles from a queue: CTA i starts with tile i, then takes tile gridDim.x + (the
     * counter's next value).  The tiles come largest first, so taking the next one
     * whenever a CTA is free balances them (a static split gave the CTAs with the
     * 64 x 64 tiles several times the average work) */
    const int t0 = blockIdx.x;
    /* the A operands once: padding lanes that a pass does not write then hold finite
     * values (zeros, or an earlier pass's), which meet zero B entries or land in
     * accumulator rows no epilogue reads */
    for (int e = tid; e < 2 * XG_TC_A_BYTES / 16; e += XG_TC_THREADS) ((uint4 *)smc)[e] = make_uint4(0, 0, 0, 0);
    if (t0 < ntiles && tid < tiles[t0].count) { sjob[tid] = jobs[list[tiles[t0].first + tid]]; snz[tid] = 0; }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"((uint32_t)__cvta_generic_to_shared(tslot)), "r"(XG_TC_TMEM_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared.b64 [%0], %1;" ::"r"(s_mbar), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tslot;
    uint32_t phase = 0;
    bool tout = false;                    /* this warp's last wait gave up (the same in every lane) */

    /* the one barrier of a pass: every thread's operand writes visible to the MMA
     * issuer and the previous accumulator reads finished; false (for the whole CTA)
     * when a warp's wait gave up */
    auto sync_pass = [&]() -> bool {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        const int bad = __syncthreads_or(tout);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        return !bad;
    };
    auto issue = [&](int bi, int kp, int np, bool a_mn) {
        if (tid == 0) xg_tc_mma(tmem, s_ahi, s_alo, s_b + bi * XG_TC_B_BYTES, kp, np, s_mbar, a_mn);
    };
    /* each thread's own bounded wait for the commit: after it the thread may read the
     * accumulator and overwrite the operands; a warp with a lane that gave up skips
     * its epilogue and the next barrier ends the CTA's loop */
    auto wait_pass = [&]() {
        const bool done = xg_tc_wait(s_mbar, phase, wait_tries);
        phase ^= 1;
        tout = !__all_sync(0xffffffffu, done);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    };
    /* B number bi (np x kp) from an int16 matrix: B[n][k] = m[n * ms_n + k * ms_k] for n < nv, k < kv, else 0 */
    auto load_b = [&](int bi, const int16_t *m, int ms_n, int ms_k, int nv, int kv, int np, int kp) {
        uint8_t *bb = bm + bi * XG_TC_B_BYTES;
        const int lkp = 31 - __clz(kp);                                   /* kp: 16, 32 or 64 */
        for (int e0 = tid; e0 < np * kp; e0 += 8 * XG_TC_THREADS) {
            int16_t v[8];                 /* eight independent loads in flight, then the stores */
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * XG_TC_THREADS, n = e >> lkp, k = e & (kp - 1);
                v[u] = (e < np * kp && n < nv && k < kv) ? m[n * ms_n + k * ms_k] : (int16_t)0;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int e = e0 + u * XG_TC_THREADS;
                if (e < np * kp) *(__half *)(bb + xg_tc_off(e >> lkp, e & (kp - 1), kp)) = __int2half_rn(v[u]);
            }
        }
    };

    int cached = -1;                      /* group (sizes and transform pair) whose B are loaded */
    for (int ti = t0, cur = 0; ti < ntiles; cur ^= 1) {
        const XgTcTile tl = tiles[ti];
        const int T = tl.count, lw = tl.lw, lh = tl.lh, w = 1 << lw, h = 1 << lh;
        const int kw = w > 32 ? 32 : w, kh = h > 32 ? 32 : h;
        const int sline = (tl.hor != 0 && w == 32) ? 16 : (w > 32 ? w - 32 : 0), jmax = w - sline;
        const int16_t *mh = xg_mat(tl.hor, lw), *mv = xg_mat(tl.ver, lh);
        const XgTqJob *tj = sjob + cur * 32;
        unsigned long long *tnz = snz + cur * 32;
        const int p16 = 16;
        auto rnd16 = [&](int v) { return (v + p16 - 1) & ~(p16 - 1); };
        const int group = ((lw * 7 + lh) * 3 + tl.hor) * 3 + tl.ver;

        /* the next tile, read by all after the barrier below (this slot's readers, two
         * tiles back, have passed the previous tile's barriers) */
        if (tid == 0) snext[cur] = (int)gridDim.x + atomicAdd(next_tile, 1);
        /* ---- F1: A[(b, i)][j] = residual; B[k][j] = mh[k][j] (every thread has seen the
         * previous tile's last MMA complete: operands and B are free) */
        const int kp1 = rnd16(w), np1 = rnd16(kw);
        if (!tout) {
            if (group != cached) {
                load_b(0, mh, w, 1, kw, w, rnd16(kw), rnd16(w));         /* F1: B[k][j] = mh[k][j] */
                load_b(1, mv, h, 1, kh, h, rnd16(kh), rnd16(h));         /* F2: B[kv][i] = mv[kv][i] */
                load_b(2, mv, 1, h, h, kh, rnd16(h), rnd16(kh));         /* I1: B[y][kv] = mv[kv][y] */
                load_b(3, mh, 1, w, w, jmax, rnd16(w), rnd16(jmax));     /* I2: B[x][j] = mh[j][x] */
                cached = group;
            }
            /* eight consecutive samples per load (16-byte aligned: the plan keeps block
             * offsets at multiples of 8), four chunks in flight per thread */
            const int nchunk = (T * h * w) >> 3, lbs = lw + lh;
            for (int c0 = tid; c0 < nchunk; c0 += 4 * XG_TC_THREADS) {
                xg_coef v[4][8];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int c = c0 + u * XG_TC_THREADS;
                    if (c < nchunk) {
                        const int e = c << 3, b = e >> lbs, o = e & ((1 << lbs) - 1);
                        const uint4 *src = (const uint4 *)(res + tj[b].off + o);
                        *(uint4 *)v[u] = src[0];
                        if (sizeof(xg_coef) == 4) *(uint4 *)(v[u] + 4) = src[1];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int c = c0 + u * XG_TC_THREADS;
                    if (c >= nchunk) continue;
                    const int e = c << 3, b = e >> lbs, o = e & ((1 << lbs) - 1);
                    int x8[8];
#pragma unroll
                    for (int x = 0; x < 8; x++) x8[x] = (int16_t)v[u][x];
                    if (w >= 8) {         /* one core-matrix row: columns j .. j + 7 of row i */
                        xg_tc_put8(ahi, alo, xg_tc_off(b * h + (o >> lw), o & (w - 1), kp1), x8);
                    } else {              /* w = 4: two rows of four (o is a multiple of 8) */
                        xg_tc_put4(ahi, alo, xg_tc_off(b * h + (o >> 2), 0, kp1), x8);
                        xg_tc_put4(ahi, alo, xg_tc_off(b * h + (o >> 2) + 1, 0, kp1), x8 + 4);
                    }
                }
            }
        }
        if (!sync_pass()) break;
        issue(0, kp1, np1, false);
        /* the next tile's job records, while the MMA runs: this buffer's last readers
         * (the previous tile) finished before the barrier above */
        const int nxt = snext[cur];
        if (nxt < ntiles) {
            const XgTcTile tn = tiles[nxt];
            if (tid < tn.count) { sjob[(cur ^ 1) * 32 + tid] = jobs[list[tn.first + tid]]; snz[(cur ^ 1) * 32 + tid] = 0; }
        }
        wait_pass();
        /* ---- F1 epilogue -> F2 operand A[(b, k)][i] = t1, MN-major: a thread's values for
         * consecutive k are consecutive rows */
        const int kp2 = rnd16(h), np2 = rnd16(kh);
        if (!tout) {
            const int m = tid, b = m >> lh, i = m & (h - 1);
            const bool valid = m < T * h;
            const int s1 = lw + XG_BITDEPTH + 6 - 15;
            for (int c = 0; c < rnd16(kw); c += 16) {
                int v[16];
                xg_tc_row16(tmem, warp, c, v);
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] = xg_clip16(xg_rshift_rnd(v[j], s1));
                if (valid) {
                    if (kw >= 8) {
                        xg_tc_put8(ahi, alo, xg_tc_mn_off(b * kw + c, i), v);
                        if (c + 8 < kw) xg_tc_put8(ahi, alo, xg_tc_mn_off(b * kw + c + 8, i), v + 8);
                    } else {
                        xg_tc_put4(ahi, alo, xg_tc_mn_off(b * kw, i), v);
                    }
                }
            }
        }
        if (!sync_pass()) break;
        issue(1, kp2, np2, true);
        wait_pass();
        /* ---- F2 epilogue: quant / dequant, q and r out; -> I1 operand A[(b, j)][kv] = r (the same rows) */
        const int kp3 = rnd16(kh), np3 = rnd16(h);
        if (!tout) {
            const int lkw = lw > 5 ? 5 : lw;
            const int m = tid, b = m >> lkw, k = m & (kw - 1);     /* row (b, k): coefficients C[kv][k] */
            const bool valid = m < T * kw;
            const XgTqJob jb = tj[valid ? b : 0];
            const int s2 = lh + 6;
            /* quant parameters (Xin266ConstructQuantParam + Xin266Transform), as in k_tq_batch */
            const int adj = ((lw + lh) & 1), lgs = (lw + lh) >> 1;
            const int qp = jb.qp + (XG_BITDEPTH == 10 ? 12 : 0), per = qp / 6, rem = qp % 6;
            const int qmult = c_qmult[adj][rem], iqmult = c_iqmult[adj][rem] << per;
            const int qshift = 14 + (15 - XG_BITDEPTH) + per - lgs - adj, iqshift = 6 - (15 - XG_BITDEPTH) + lgs + adj;
            const int qadd = (jb.flags & 4) ? (1 << (qshift - 1)) : (((jb.flags & 8) ? 171 : 85) << (qshift - 9));
            const int iqadd = 1 << (iqshift - 1);
            unsigned long long nzb = 0;
            for (int c = 0; c < rnd16(kh); c += 16) {
                int v[16], rr[16];
                xg_tc_row16(tmem, warp, c, v);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int kv = c + j;
                    rr[j] = 0;                /* beyond kh: the I1 operand's zero padding */
                    if (!valid || kv >= kh) continue;
                    const int tv = xg_clip16(xg_rshift_rnd(v[j], s2)), a = abs(tv);
                    /* a * qmult + qadd < 2^15 * 26214 + 2^28 < 2^31: exact in 32 bits */
                    int qv = (int)(((uint32_t)a * (uint32_t)qmult + (uint32_t)qadd) >> qshift);
                    qv = xg_clip16(tv < 0 ? -qv : qv);
                    const int rv = xg_clip16((int)(((long long)qv * iqmult + iqadd) >> iqshift));
                    q[jb.off + kv * w + k] = (xg_coef)qv;
                    r[jb.off + kv * w + k] = (xg_coef)rv;
                    if (qv) nzb |= 1ull << ((kv >> 2) * (kw >> 2) + (k >> 2));
                    rr[j] = rv;
                }
                if (valid && k < jmax) {      /* row m of the I1 operand, columns c .. c + 15 */
                    xg_tc_put8(ahi, alo, xg_tc_off(m, c, kp3), rr);
                    xg_tc_put8(ahi, alo, xg_tc_off(m, c + 8, kp3), rr + 8);
                }
            }
            if (nzb) atomicOr(&tnz[b], nzb);
        }
        if (!sync_pass()) break;
        issue(2, kp3, np3, false);
        /* while the MMA runs: zeros of q / r beyond the kept 32 x 32 (64-wide or -high
         * blocks; a 16-byte chunk lies wholly inside or outside it) and the maps, whose
         * bits were all set before the barrier above */
        if (w > 32 || h > 32) {
            constexpr int E = 16 / (int)sizeof(xg_coef);
            const int nch = (w * h) / E;
            for (int bb = 0; bb < T; bb++) {
                const uint32_t off = tj[bb].off;
                for (int c = tid; c < nch; c += XG_TC_THREADS) {
                    const int o = c * E, y = o >> lw, x = o & (w - 1);
                    if (y >= kh || x >= kw) {
                        *(uint4 *)(q + off + o) = make_uint4(0, 0, 0, 0);
                        *(uint4 *)(r + off + o) = make_uint4(0, 0, 0, 0);
                    }
                }
            }
        }
        if (tid < T) nzout[list[tl.first + tid]] = tnz[tid];
        wait_pass();
        /* ---- I1 epilogue -> I2 operand A[(b, y)][j] = t2, MN-major (consecutive y, consecutive rows) */
        const int kp4 = rnd16(jmax), np4 = rnd16(w);
        if (!tout) {
            const int lkw = lw > 5 ? 5 : lw;
            const int m = tid, b = m >> lkw, j = m & (kw - 1);
            const bool valid = m < T * kw && j < jmax;
            for (int c = 0; c < rnd16(h); c += 16) {
                int v[16];
                xg_tc_row16(tmem, warp, c, v);
#pragma unroll
                for (int jj = 0; jj < 16; jj++) v[jj] = xg_clip16(xg_rshift_rnd(v[jj], 7));
                if (valid) {
                    if (h >= 8) {
                        xg_tc_put8(ahi, alo, xg_tc_mn_off(b * h + c, j), v);
                        if (c + 8 < h) xg_tc_put8(ahi, alo, xg_tc_mn_off(b * h + c + 8, j), v + 8);
                    } else {
                        xg_tc_put4(ahi, alo, xg_tc_mn_off(b * h, j), v);
                    }
                }
            }
        }
        if (!sync_pass()) break;
        issue(3, kp4, np4, true);
        wait_pass();
        /* ---- I2 epilogue: the reconstructed residual */
        if (!tout) {
            const int m = tid, b = m >> lh, y = m & (h - 1);
            const bool valid = m < T * h;
            const int s2 = 6 + 15 - 1 - XG_BITDEPTH;
            const int off = valid ? tj[b].off + y * w : 0;
            for (int c = 0; c < rnd16(w); c += 16) {
                int v[16];
                xg_tc_row16(tmem, warp, c, v);
                if (valid && w >= 4) {        /* four samples per store (the row starts 16-byte aligned) */
#pragma unroll
                    for (int x = 0; x < 16; x += 4)
                        if (c + x < w) {
                            xg_coef o4[4];
#pragma unroll
                            for (int u = 0; u < 4; u++) o4[u] = (xg_coef)xg_clip16(xg_rshift_rnd(v[x + u], s2));
                            if (sizeof(xg_coef) == 4) *(uint4 *)(rout + off + c + x) = *(const uint4 *)o4;
                            else *(uint2 *)(rout + off + c + x) = *(const uint2 *)o4;
                        }
                }
            }
        }
        ti = nxt;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    const bool ok = !__syncthreads_or(tout);
    if (!ok && tid == 0) {
        atomicExch(err, 1);
        /* the MMA whose wait gave up may still be writing the accumulators: wait for
         * its commit (again bounded) before the tensor memory is released */
        xg_tc_wait(s_mbar, phase ^ 1, XG_TC_WAIT_TRIES);
    }
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(XG_TC_TMEM_COLS) : "memory");
}
