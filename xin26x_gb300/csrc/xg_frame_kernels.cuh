/*
 * xg_frame_kernels.cuh -- kernels of the batched frame form.
 *
 *   k_pad            edge replication of a picture into its padded slot
 *                    (the layout of Xin266ConstructRefPicBuf / Xin26xExtendPicture,
 *                    h266_encoder/source/h266_encoder_create.c:1065-1077, with a
 *                    wider margin on the GPU)
 *   k_qpel_planes    the 15 fractional quarter-pel luma planes of a reference
 *                    picture, each sample computed exactly like
 *                    Xin266LumaInterpolation computes it for a block
 *   k_me_tiles       exhaustive integer search of every CU of every quadtree
 *                    level of a 64x64 tile, 8x8 SADs shared by all levels
 *   k_cu_tail<S>     per CU: Xin266FullSubPelMe on the quarter-pel planes, luma
 *                    and chroma motion compensation, residual, DCT2, quant /
 *                    dequant, inverse DCT2, reconstruction, SSD
 */
#include "xg_device.cuh"

/* ------------------------------------------------------------------ layout */
struct XgPlane {            /* padded plane: data points at picture (0, 0) */
    xg_pix *data;
    int pitch;              /* elements */
    int w, h, pad;          /* picture size and margin on each side */
};

/* ------------------------------------------------------------------ k_pad */
__global__ void k_pad(XgPlane p)
{
    int pw = p.w + 2 * p.pad, ph = p.h + 2 * p.pad;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pw * ph; i += gridDim.x * blockDim.x) {
        int x = i % pw - p.pad, y = i / pw - p.pad;
        if (x >= 0 && x < p.w && y >= 0 && y < p.h) continue;
        int sx = min(max(x, 0), p.w - 1), sy = min(max(y, 0), p.h - 1);
        p.data[(intptr_t)y * p.pitch + x] = p.data[(intptr_t)sy * p.pitch + sx];
    }
}

/* -------------------------------------------------------------- qpel planes
 * plane index q = (fy / 4) * 4 + fx / 4 for phases fx, fy in {0, 4, 8, 12};
 * q = 0 is the integer plane itself and is not written.  Samples are produced
 * for the padded area shrunk by the filter reach (3 before, 4 after). */
struct XgQpel { xg_pix *plane[16]; int pitch, w, h, pad; };

__global__ void k_qpel_planes(XgPlane ref, XgQpel qp)
{
    int q = blockIdx.z + 1;
    int fx = (q & 3) * 4, fy = (q >> 2) * 4;
    int x = blockIdx.x * blockDim.x + threadIdx.x - (qp.pad - 4);
    int y = blockIdx.y * blockDim.y + threadIdx.y - (qp.pad - 4);
    if (x >= qp.w + qp.pad - 4 || y >= qp.h + qp.pad - 4) return;
    const xg_pix *p = ref.data + (intptr_t)y * ref.pitch + x;
    const int8_t *th = c_luma_taps[0][fx], *tv = c_luma_taps[0][fy];
    int v;
    if (fx && !fy) v = xg_if_pix<8>(p, 1, th);
    else if (!fx && fy) v = xg_if_pix<8>(p, ref.pitch, tv);
    else v = xg_if_hv<8, false>(p, ref.pitch, th, tv);
    qp.plane[q][(intptr_t)y * qp.pitch + x] = (xg_pix)v;
}

/* -------------------------------------------------------------- k_me_tiles
 * Grid: (tiles_x, tiles_y, bands).  A CTA takes one 64x64 tile and one band of
 * candidate rows; warp w owns the 16x16 sub-block (w & 3, w >> 2), lane l the
 * l-th candidate of each group of 32 consecutive candidates (raster order of
 * the band).  The reference band sits in shared memory as one 32-bit word per
 * pixel position, word (r, x) holding pixels x .. x+3 of band row r, so the
 * four pixels at any candidate offset are one aligned word; the row pitch is
 * congruent to the candidate-row length modulo 32, so the 32 consecutive
 * candidates of a warp read 32 consecutive banks.  |a - b| of four pixels and
 * their sum is one vabsdiff4 with add-reduction.
 * Per candidate a warp has the SADs of its four 8x8 blocks and of its 16x16
 * block in registers (running minimum per lane); the 16x16 SADs of 128
 * candidates at a time go to shared memory, from which the 32x32 and 64x64
 * SADs are summed.  Every CU keeps (cost, raster index) as one 64-bit key; the
 * unsigned minimum over lanes, warps and CTAs (atomicMin) selects the smallest
 * cost and, among equal costs, the first candidate in raster order -- the
 * strict '<' raster search.  Costs: (SAD << 8) + (bits(4dx) + bits(4dy)) * lambda
 * (predictor 0).  8-bit pixels only (10-bit uses k_me_tiles_generic). */
#define XG_ME_TILE 64
#define XG_ME_THREADS 512
#define XG_ME_GROUP 128                 /* candidates per shared-memory phase */

/* per-picture values, read from device memory so one captured graph serves
 * every picture of a stream */
struct XgQuant { int qmult, qadd, qshift, iqmult, iqadd, iqshift; };
struct XgPicParams {
    uint32_t lambda;
    uint32_t reserved;
    XgQuant quant[4][3];                /* [level 64,32,16,8][plane] */
    const xg_pix *src[3];               /* device-resident source planes (device_io streams) */
    long long src_stride[3];
};

/* copy a device-resident picture into the padded slot (device_io streams) */
__global__ void k_copy_in(XgPlane y, XgPlane u, XgPlane v, const XgPicParams *pp)
{
    const int ny = y.w * y.h, nc = u.w * u.h;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ny + 2 * nc; i += gridDim.x * blockDim.x) {
        if (i < ny) {
            y.data[(intptr_t)(i / y.w) * y.pitch + i % y.w] = pp->src[0][(intptr_t)(i / y.w) * pp->src_stride[0] + i % y.w];
        } else {
            int k = i - ny, pl = k < nc ? 1 : 2;
            k -= (pl - 1) * nc;
            XgPlane &d = pl == 1 ? u : v;
            d.data[(intptr_t)(k / d.w) * d.pitch + k % d.w] = pp->src[pl][(intptr_t)(k / d.w) * pp->src_stride[pl] + k % d.w];
        }
    }
}

/* packed 8-bit SAD throughput probe: vabsdiff4 + dp4a on register data */
__global__ void k_sad_peak(const uint32_t *in, uint32_t *out, int iters)
{
    uint32_t a[8], b[8];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = 0; i < 8; i++) { a[i] = in[(t + i) & 1023]; b[i] = in[(t * 7 + i * 13) & 1023]; }
    uint32_t acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i += 4) {
            acc0 = __dp4a(__vabsdiffu4(a[i], b[i]), 0x01010101u, acc0);
            acc1 = __dp4a(__vabsdiffu4(a[i + 1], b[i + 1]), 0x01010101u, acc1);
            acc2 = __dp4a(__vabsdiffu4(a[i + 2], b[i + 2]), 0x01010101u, acc2);
            acc3 = __dp4a(__vabsdiffu4(a[i + 3], b[i + 3]), 0x01010101u, acc3);
        }
#pragma unroll
        for (int i = 0; i < 8; i++) { uint32_t tmp = a[i]; a[i] = b[(i + 1) & 7] ^ (uint32_t)it; b[(i + 1) & 7] = tmp; }
    }
    out[t] = acc0 + acc1 + acc2 + acc3;
}

struct XgMeParams {
    XgPlane cur, ref;
    int W, H, ctu, R;
    int band_rows;                      /* candidate rows per band */
    int row_words;                      /* words per band row (pitch of the word array) */
    unsigned long long *keys[4];        /* level 0..3 = 64, 32, 16, 8 (NULL = level off) */
    int cus_x[4];                       /* CUs per row of each level */
};

/* window of one CU (h266_encoder/source/h266_enc_init.c:1462-1465) intersected with [-R, R] */
__device__ __forceinline__ void xg_cu_window(const XgMeParams &p, int cx, int cy, int s, int &x0, int &x1, int &y0, int &y1)
{
    x0 = max(-p.R, (int)(int16_t)(-cx - p.ctu - 8));
    y0 = max(-p.R, (int)(int16_t)(-cy - p.ctu - 8));
    x1 = min(p.R, (int)(int16_t)(p.W + (p.ctu - s + 8) - cx));
    y1 = min(p.R, (int)(int16_t)(p.H + (p.ctu - s + 8) - cy));
}

/* acc + sum over the four bytes of |a - b|: one vabsdiff4 with add-reduction */
__device__ __forceinline__ uint32_t xg_sad4(uint32_t a, uint32_t b, uint32_t acc)
{
    uint32_t d;
    asm("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(acc));
    return d;
}

#if XG_BITDEPTH == 8
__global__ void __launch_bounds__(XG_ME_THREADS, 1) k_me_tiles(XgMeParams p, const XgPicParams *pp)
{
    extern __shared__ uint32_t sm[];
    const int tx0 = blockIdx.x * XG_ME_TILE, ty0 = blockIdx.y * XG_ME_TILE;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nx = 2 * p.R + 1;
    const int dyb0 = -p.R + (int)blockIdx.z * p.band_rows;
    const int ndy = min(p.band_rows, p.R - dyb0 + 1);
    const int ncand = nx * ndy;
    const int rows = XG_ME_TILE + ndy - 1;

    const int relw = nx + 60;                                /* word positions read per band row */
    uint32_t *refw = sm;                                     /* [rows][row_words] */
    uint32_t *mvcx = sm + (XG_ME_TILE + p.band_rows - 1) * p.row_words;   /* [nx] */
    uint32_t *mvcy = mvcx + nx;                              /* [band_rows] */
    uint32_t *s16 = mvcy + p.band_rows;                      /* [16][XG_ME_GROUP] */

    /* ---- stage the reference band: pixels (X0 + x .. X0 + x + 3, Y0 + r) -> refw[r * row_words + x] */
    const int X0 = tx0 - p.R, Y0 = ty0 + dyb0;
    for (int i = threadIdx.x; i < rows * relw; i += blockDim.x) {
        int r = i / relw, x = i - r * relw;
        const xg_pix *src = p.ref.data + (intptr_t)(Y0 + r) * p.ref.pitch + X0 + x;
        refw[r * p.row_words + x] = (uint32_t)src[0] | ((uint32_t)src[1] << 8) | ((uint32_t)src[2] << 16) | ((uint32_t)src[3] << 24);
    }
    const uint32_t lambda = pp->lambda;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) mvcx[i] = xg_mvd_bits(4 * (i - p.R)) * lambda;
    for (int i = threadIdx.x; i < ndy; i += blockDim.x) mvcy[i] = xg_mvd_bits(4 * (dyb0 + i)) * lambda;

    /* ---- this warp's 16x16 block of the current picture in registers */
    const int bx = (warp & 3) * 16, by = (warp >> 2) * 16;
    uint32_t cur[16][4];
#pragma unroll
    for (int r = 0; r < 16; r++)
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const xg_pix *c = p.cur.data + (intptr_t)(ty0 + by + r) * p.cur.pitch + tx0 + bx + 4 * k;
            cur[r][k] = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16) | ((uint32_t)c[3] << 24);
        }

    /* ---- per-lane running bests of the four 8x8 CUs and the 16x16 CU */
    int win[5][4];
    bool live[5];
    uint32_t best[5], bidx[5];
#pragma unroll
    for (int c = 0; c < 5; c++) {
        int s = c < 4 ? 8 : 16;
        int cx = tx0 + bx + (c < 4 ? (c & 1) * 8 : 0), cy = ty0 + by + (c < 4 ? (c >> 1) * 8 : 0);
        live[c] = p.keys[c < 4 ? 3 : 2] && cx + s <= p.W && cy + s <= p.H;
        xg_cu_window(p, cx, cy, s, win[c][0], win[c][1], win[c][2], win[c][3]);
        best[c] = 0xFFFFFFFFu; bidx[c] = 0xFFFFFFFFu;
    }
    /* 32x32 and 64x64 bookkeeping: thread t < 512 handles (cu32 = t >> 7, slot t & 127); t < 128 also the 64x64 */
    const int c32 = threadIdx.x >> 7, slot = threadIdx.x & 127;
    const int c32x = tx0 + (c32 & 1) * 32, c32y = ty0 + (c32 >> 1) * 32;
    const bool live32 = p.keys[1] && c32x + 32 <= p.W && c32y + 32 <= p.H;
    const bool live64 = threadIdx.x < 128 && p.keys[0] && tx0 + 64 <= p.W && ty0 + 64 <= p.H;
    int w32[4], w64[4];
    xg_cu_window(p, c32x, c32y, 32, w32[0], w32[1], w32[2], w32[3]);
    xg_cu_window(p, tx0, ty0, 64, w64[0], w64[1], w64[2], w64[3]);
    uint32_t best32 = 0xFFFFFFFFu, bidx32 = 0xFFFFFFFFu, best64 = 0xFFFFFFFFu, bidx64 = 0xFFFFFFFFu;
    __syncthreads();

    const int ngroups = (ncand + XG_ME_GROUP - 1) / XG_ME_GROUP;
    for (int g = 0; g < ngroups; g++) {
#pragma unroll 1
        for (int ch = 0; ch < XG_ME_GROUP / 32; ch++) {
            int ci = g * XG_ME_GROUP + ch * 32 + lane;
            bool valid = ci < ncand;
            int cc = valid ? ci : ncand - 1;
            int row = cc / nx, col = cc - row * nx;        /* dy = dyb0 + row, dx = col - R */
            const uint32_t *base = refw + (by + row) * p.row_words + bx + col;   /* block origin at this candidate */
            uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const uint32_t *q = base + r * p.row_words;
                a0 = xg_sad4(cur[r][0], q[0], a0); a0 = xg_sad4(cur[r][1], q[4], a0);
                a1 = xg_sad4(cur[r][2], q[8], a1); a1 = xg_sad4(cur[r][3], q[12], a1);
            }
#pragma unroll
            for (int r = 8; r < 16; r++) {
                const uint32_t *q = base + r * p.row_words;
                a2 = xg_sad4(cur[r][0], q[0], a2); a2 = xg_sad4(cur[r][1], q[4], a2);
                a3 = xg_sad4(cur[r][2], q[8], a3); a3 = xg_sad4(cur[r][3], q[12], a3);
            }
            uint32_t sum16 = a0 + a1 + a2 + a3;
            uint32_t mvc = mvcx[col] + mvcy[row];
            int dx = col - p.R, dy = dyb0 + row;
            uint32_t gidx = (uint32_t)((dy + p.R) * nx + col);
            uint32_t sads[5] = { a0, a1, a2, a3, sum16 };
#pragma unroll
            for (int c = 0; c < 5; c++) {
                uint32_t cost = (sads[c] << XG_COST_FRACTION) + mvc;
                bool ok = valid && live[c] && dx >= win[c][0] && dx <= win[c][1] && dy >= win[c][2] && dy <= win[c][3];
                if (ok && cost < best[c]) { best[c] = cost; bidx[c] = gidx; }
            }
            s16[warp * XG_ME_GROUP + ch * 32 + lane] = sum16;
        }
        __syncthreads();
        {
            int ci = g * XG_ME_GROUP + slot;
            if (ci < ncand) {
                int row = ci / nx, col = ci - row * nx;
                int dx = col - p.R, dy = dyb0 + row;
                uint32_t mvc = mvcx[col] + mvcy[row];
                uint32_t gidx = (uint32_t)((dy + p.R) * nx + col);
                /* warps of the 32x32 quadrant c32: (2*(c32&1) + {0,1}) + 4*(2*(c32>>1) + {0,1}) */
                int w0 = (c32 & 1) * 2 + (c32 >> 1) * 8;
                uint32_t s32 = s16[w0 * XG_ME_GROUP + slot] + s16[(w0 + 1) * XG_ME_GROUP + slot] +
                               s16[(w0 + 4) * XG_ME_GROUP + slot] + s16[(w0 + 5) * XG_ME_GROUP + slot];
                uint32_t cost = (s32 << XG_COST_FRACTION) + mvc;
                if (live32 && dx >= w32[0] && dx <= w32[1] && dy >= w32[2] && dy <= w32[3] && cost < best32) { best32 = cost; bidx32 = gidx; }
                if (live64) {
                    uint32_t s64 = 0;
#pragma unroll
                    for (int w = 0; w < 16; w++) s64 += s16[w * XG_ME_GROUP + slot];
                    uint32_t c64 = (s64 << XG_COST_FRACTION) + mvc;
                    if (dx >= w64[0] && dx <= w64[1] && dy >= w64[2] && dy <= w64[3] && c64 < best64) { best64 = c64; bidx64 = gidx; }
                }
            }
        }
        __syncthreads();
    }

    /* ---- publish: warp minimum of packed keys, then one atomicMin per CU and CTA */
#pragma unroll
    for (int c = 0; c < 5; c++) {
        unsigned long long k = ((unsigned long long)best[c] << 32) | bidx[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) { unsigned long long v = __shfl_xor_sync(0xffffffffu, k, o); k = v < k ? v : k; }
        if (lane == 0 && live[c] && k != ~0ull) {
            int s = c < 4 ? 8 : 16, L = c < 4 ? 3 : 2;
            int cx = tx0 + bx + (c < 4 ? (c & 1) * 8 : 0), cy = ty0 + by + (c < 4 ? (c >> 1) * 8 : 0);
            atomicMin(p.keys[L] + (cy / s) * p.cus_x[L] + cx / s, k);
        }
    }
    {
        unsigned long long k = ((unsigned long long)best32 << 32) | bidx32;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) { unsigned long long v = __shfl_xor_sync(0xffffffffu, k, o); k = v < k ? v : k; }
        if (lane == 0 && live32 && k != ~0ull) atomicMin(p.keys[1] + (c32y / 32) * p.cus_x[1] + c32x / 32, k);
        k = ((unsigned long long)best64 << 32) | bidx64;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) { unsigned long long v = __shfl_xor_sync(0xffffffffu, k, o); k = v < k ? v : k; }
        if (lane == 0 && live64 && k != ~0ull) atomicMin(p.keys[0] + (ty0 / 64) * p.cus_x[0] + tx0 / 64, k);
    }
}
#endif

/* generic (any bit depth) integer search: one CTA per (CU, candidate row band);
 * used for 10-bit pictures and as a cross-check of k_me_tiles */
__global__ void k_me_generic(XgMeParams p, const XgPicParams *pp, int level, int size, int cus_x)
{
    __shared__ unsigned long long red[32];
    int cu = blockIdx.x;
    int cx = (cu % cus_x) * size, cy = (cu / cus_x) * size;
    int x0, x1, y0, y1;
    xg_cu_window(p, cx, cy, size, x0, x1, y0, y1);
    int nx = 2 * p.R + 1;
    unsigned long long k = ~0ull;
    int dy = y0 + (int)blockIdx.y;
    for (; dy <= y1; dy += gridDim.y) {
        for (int dx = x0 + (int)threadIdx.x; dx <= x1; dx += blockDim.x) {
            uint32_t sad = 0;
            for (int y = 0; y < size; y++) {
                const xg_pix *a = p.cur.data + (intptr_t)(cy + y) * p.cur.pitch + cx;
                const xg_pix *b = p.ref.data + (intptr_t)(cy + y + dy) * p.ref.pitch + cx + dx;
                for (int x = 0; x < size; x++) sad += (uint32_t)abs((int)a[x] - (int)b[x]);
            }
            uint32_t cost = (sad << XG_COST_FRACTION) + (xg_mvd_bits(4 * dx) + xg_mvd_bits(4 * dy)) * pp->lambda;
            unsigned long long kk = ((unsigned long long)cost << 32) | (uint32_t)((dy + p.R) * nx + dx + p.R);
            k = kk < k ? kk : k;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { unsigned long long v = __shfl_xor_sync(0xffffffffu, k, o); k = v < k ? v : k; }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) k = red[i] < k ? red[i] : k;
        if (k != ~0ull) atomicMin(p.keys[level] + cu, k);
    }
}

/* -------------------------------------------------------------- k_cu_tail */

struct XgTailParams {
    XgPlane cur[3], ref[3];
    XgQpel qpel;
    int W, H, ctu, R;
    const unsigned long long *keys;   /* this level */
    int cus_x, first_cu, size, level;
    xg_coef *q[3];                    /* this level's coefficient planes (picture layout) */
    xg_pix *rec[3];                   /* this level's reconstructed planes */
    xin_gpu_cu_result *res;           /* all CUs */
};

/* forward 2-D DCT2 of an n x n residual in shared memory, keeping the outputs
 * below 32 in each direction (the rest is zeroed out downstream), then quant /
 * dequant with 4x4 coding groups over the low min(n, 32) square */
template <int N, int NT>
__device__ void xg_tq_block(const int *res, int *coef, int *rr, const XgQuant &qz, int s1, int s2, unsigned long long *nz,
                            xg_coef *qout, int qpitch, int16_t *tmp)
{
    constexpr int LG = N == 4 ? 2 : N == 8 ? 3 : N == 16 ? 4 : N == 32 ? 5 : 6;
    constexpr int K = N > 32 ? 32 : N;
    const int16_t *m = xg_mat(0, LG);
    /* pass 1 (rows): tmp[k * N + i] = row i, frequency k */
    for (int o = threadIdx.x; o < K * N; o += NT) {
        int k = o / N, i = o % N;
        int s = 0;
#pragma unroll 8
        for (int j = 0; j < N; j++) s += (int)m[k * N + j] * res[i * N + j];
        tmp[k * N + i] = (int16_t)xg_clip16(xg_rshift_rnd(s, s1));
    }
    __syncthreads();
    /* pass 2 (columns): coef[kv * K + kh] */
    for (int o = threadIdx.x; o < K * K; o += NT) {
        int kv = o / K, kh = o % K;
        int s = 0;
#pragma unroll 8
        for (int i = 0; i < N; i++) s += (int)m[kv * N + i] * (int)tmp[kh * N + i];
        int t = xg_clip16(xg_rshift_rnd(s, s2));
        int a = abs(t);
        int qv = (int)(((long long)a * qz.qmult + qz.qadd) >> qz.qshift);
        qv = xg_clip16(t < 0 ? -qv : qv);
        int rv = xg_clip16((int)(((long long)qv * qz.iqmult + qz.iqadd) >> qz.iqshift));
        coef[o] = qv;
        rr[o] = rv;
        if (qv) atomicOr(nz, 1ull << ((kv >> 2) * (K >> 2) + (kh >> 2)));
    }
    __syncthreads();
    for (int o = threadIdx.x; o < N * N; o += NT) {
        int y = o / N, x = o % N;
        qout[(intptr_t)y * qpitch + x] = (xg_coef)((y < K && x < K) ? coef[y * K + x] : 0);
    }
}

/* inverse 2-D DCT2 of the dequantised K x K low part (zero elsewhere), columns
 * first with lines >= 32 skipped (Xin266IDct2WxH), then rows; adds the
 * prediction, clips, writes the reconstruction and accumulates the SSD */
template <int N, int NT>
__device__ void xg_itq_block(const int *rr, const xg_pix *pred, const xg_pix *org, int opitch, xg_pix *rec, int rpitch,
                             int16_t *tmp, unsigned long long *ssd)
{
    constexpr int LG = N == 4 ? 2 : N == 8 ? 3 : N == 16 ? 4 : N == 32 ? 5 : 6;
    constexpr int K = N > 32 ? 32 : N;
    const int16_t *m = xg_mat(0, LG);
    const int s2 = 6 + 15 - 1 - XG_BITDEPTH;
    /* pass 1: column j < K (lines j >= 32 are zero): tmp[j * N + x] */
    for (int o = threadIdx.x; o < K * N; o += NT) {
        int j = o / N, x = o % N;
        int s = 0;
#pragma unroll 8
        for (int k = 0; k < K; k++) s += (int)m[k * N + x] * rr[k * K + j];
        tmp[j * N + x] = (int16_t)xg_clip16(xg_rshift_rnd(s, 7));
    }
    __syncthreads();
    unsigned long long acc = 0;
    for (int o = threadIdx.x; o < N * N; o += NT) {
        int y = o / N, x = o % N;
        int s = 0;
#pragma unroll 8
        for (int j = 0; j < K; j++) s += (int)m[j * N + x] * (int)tmp[j * N + y];
        int resid = xg_clip16(xg_rshift_rnd(s, s2));
        int v = xg_clip_pix((int)pred[o] + resid);
        rec[(intptr_t)y * rpitch + x] = (xg_pix)v;
        int d = (int)org[(intptr_t)y * opitch + x] - v;
        acc += (unsigned long long)(d * d);
    }
    atomicAdd(ssd, acc);
    __syncthreads();
}

/* one CTA per CU of size S (luma S x S, chroma S/2 x S/2), NT threads */
template <int S, int NT>
__global__ void __launch_bounds__(NT) k_cu_tail(XgTailParams p, const XgPicParams *pp)
{
    constexpr int C = S / 2;
    __shared__ int res[S * S];
    __shared__ int coef[(S > 32 ? 32 : S) * (S > 32 ? 32 : S)];
    __shared__ int rr[(S > 32 ? 32 : S) * (S > 32 ? 32 : S)];
    __shared__ int16_t tmp[S * S];
    __shared__ xg_pix pred[S * S];
    __shared__ uint32_t part[8][NT / 32];
    __shared__ int bmv[3];
    __shared__ unsigned long long nz[3], ssd[3];

    const int cu = blockIdx.x;
    const int cx = (cu % p.cus_x) * S, cy = (cu / p.cus_x) * S;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long key = p.keys[cu];
    const int nx = 2 * p.R + 1;
    const int gidx = (int)(uint32_t)key;
    const int imx = gidx % nx - p.R, imy = gidx / nx - p.R;
    if (threadIdx.x < 3) { nz[threadIdx.x] = 0; ssd[threadIdx.x] = 0; }
    if (threadIdx.x == 0) { bmv[0] = 4 * imx; bmv[1] = 4 * imy; bmv[2] = (int)(uint32_t)(key >> 32); }

    /* window (h266_enc_init.c:1462) */
    const int mnx = (int16_t)(-cx - p.ctu - 8), mny = (int16_t)(-cy - p.ctu - 8);
    const int mxx = (int16_t)(p.W + (p.ctu - S + 8) - cx), mxy = (int16_t)(p.H + (p.ctu - S + 8) - cy);
    __syncthreads();

    /* ---- Xin266FullSubPelMe on the quarter-pel planes (h266_sub_pel_refine.c:81-212) */
    const int offx[8] = { -1, 1, 0, 0, -1, 1, -1, 1 }, offy[8] = { 0, 0, -1, 1, -1, -1, 1, 1 };
    const xg_pix *org = p.cur[0].data + (intptr_t)cy * p.cur[0].pitch + cx;
    /* the search runs only when the integer start lies in the window (h266_sub_pel_refine.c:117-120) */
    const bool start_in = (bmv[0] >> 2) >= mnx && (bmv[1] >> 2) >= mny && (bmv[0] >> 2) <= mxx && (bmv[1] >> 2) <= mxy;
    for (int step = 2; step >= 1 && start_in; step--) {
        const int bx0 = bmv[0], by0 = bmv[1];
        uint32_t acc[8];
#pragma unroll
        for (int c = 0; c < 8; c++) acc[c] = 0;
        for (int i = threadIdx.x; i < S * S; i += NT) {
            int x = i % S, y = i / S;
            int o = org[(intptr_t)y * p.cur[0].pitch + x];
#pragma unroll
            for (int c = 0; c < 8; c++) {
                int tx = bx0 + offx[c] * step, ty = by0 + offy[c] * step;
                const xg_pix *pl = (tx & 3) | (ty & 3) ? p.qpel.plane[(ty & 3) * 4 + (tx & 3)] : p.ref[0].data;
                int v = pl[(intptr_t)(cy + y + (ty >> 2)) * p.qpel.pitch + cx + x + (tx >> 2)];
                acc[c] += (uint32_t)abs(o - v);
            }
        }
#pragma unroll
        for (int c = 0; c < 8; c++) {
            uint32_t s = acc[c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) part[c][warp] = s;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t bc = (uint32_t)bmv[2];
            int bx = bx0, by = by0;
            for (int c = 0; c < 8; c++) {
                uint32_t s = 0;
                for (int w = 0; w < NT / 32; w++) s += part[c][w];
                int tx = bx0 + offx[c] * step, ty = by0 + offy[c] * step;
                uint32_t cost = (s << XG_COST_FRACTION) + (xg_mvd_bits(tx) + xg_mvd_bits(ty)) * pp->lambda;
                if (cost < bc) { bc = cost; bx = tx; by = ty; }
            }
            bmv[0] = bx; bmv[1] = by; bmv[2] = (int)bc;
        }
        __syncthreads();
    }
    const int mvx = bmv[0], mvy = bmv[1];

    /* ---- luma MC (Xin266LumaInterPred: clamp to the window in 1/16 pel) */
    {
        int m16x = min(max(mvx * 4, mnx * 16), mxx * 16), m16y = min(max(mvy * 4, mny * 16), mxy * 16);
        int ox = cx * 16 + m16x, oy = cy * 16 + m16y;
        int q = ((oy & 15) >> 2) * 4 + ((ox & 15) >> 2);
        const xg_pix *pl = q ? p.qpel.plane[q] : p.ref[0].data;
        for (int i = threadIdx.x; i < S * S; i += NT) {
            int x = i % S, y = i / S;
            pred[i] = pl[(intptr_t)((oy >> 4) + y) * p.qpel.pitch + (ox >> 4) + x];
        }
    }
    __syncthreads();

    /* ---- luma TQ + reconstruction */
    const int lgS = S == 8 ? 3 : S == 16 ? 4 : S == 32 ? 5 : 6;
    for (int i = threadIdx.x; i < S * S; i += NT) res[i] = (int)org[(intptr_t)(i / S) * p.cur[0].pitch + i % S] - (int)pred[i];
    __syncthreads();
    xg_tq_block<S, NT>(res, coef, rr, pp->quant[p.level][0], lgS + XG_BITDEPTH + 6 - 15, lgS + 6, &nz[0],
                       p.q[0] + (intptr_t)cy * p.W + cx, p.W, tmp);
    xg_itq_block<S, NT>(rr, pred, org, p.cur[0].pitch, p.rec[0] + (intptr_t)cy * p.W + cx, p.W, tmp, &ssd[0]);

    /* ---- chroma: uni branch of Xin266ChromaMotionComp (1/32 phase, mask 31), TQ, reconstruction */
    {
        const int lgC = lgS - 1;
        int m16x = min(max(mvx * 4, mnx * 16), mxx * 16), m16y = min(max(mvy * 4, mny * 16), mxy * 16);
        int ox = cx * 16 + m16x, oy = cy * 16 + m16y;
        int fx = ox & 31, fy = oy & 31;
        const int8_t *th = c_chroma_taps[fx], *tv = c_chroma_taps[fy];
        const int W2 = p.W >> 1;
        for (int pl = 1; pl <= 2; pl++) {
            const XgPlane &rp = p.ref[pl];
            const xg_pix *src = rp.data + (intptr_t)(oy >> 5) * rp.pitch + (ox >> 5);
            for (int i = threadIdx.x; i < C * C; i += NT) {
                int x = i % C, y = i / C;
                const xg_pix *s = src + (intptr_t)y * rp.pitch + x;
                int v;
                if (!fx && !fy) v = s[0];
                else if (fx && !fy) v = xg_if_pix<4>(s, 1, th);
                else if (!fx && fy) v = xg_if_pix<4>(s, rp.pitch, tv);
                else v = xg_if_hv<4, false>(s, rp.pitch, th, tv);
                pred[i] = (xg_pix)v;
            }
            __syncthreads();
            const xg_pix *corg = p.cur[pl].data + (intptr_t)(cy >> 1) * p.cur[pl].pitch + (cx >> 1);
            for (int i = threadIdx.x; i < C * C; i += NT) res[i] = (int)corg[(intptr_t)(i / C) * p.cur[pl].pitch + i % C] - (int)pred[i];
            __syncthreads();
            xg_tq_block<C, NT>(res, coef, rr, pp->quant[p.level][pl], lgC + XG_BITDEPTH + 6 - 15, lgC + 6, &nz[pl],
                               p.q[pl] + (intptr_t)(cy >> 1) * W2 + (cx >> 1), W2, tmp);
            xg_itq_block<C, NT>(rr, pred, corg, p.cur[pl].pitch, p.rec[pl] + (intptr_t)(cy >> 1) * W2 + (cx >> 1), W2, tmp,
                                &ssd[pl]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        xin_gpu_cu_result *o = p.res + p.first_cu + cu;
        o->mvx = mvx; o->mvy = mvy; o->cost = (uint32_t)bmv[2]; o->int_cost = (uint32_t)(key >> 32);
        for (int i = 0; i < 3; i++) { o->nz[i] = nz[i]; o->ssd[i] = ssd[i]; }
    }
}
