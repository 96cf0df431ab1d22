/*
 * xg_frame_kernels.cuh -- kernels of the batched frame form.
 *
 *   k_fill_slot      a picture into its padded slot: copy-in (and 8-bit samples
 *                    << 2) with edge replication (the layout of
 *                    Xin266ConstructRefPicBuf / Xin26xExtendPicture,
 *                    h266_encoder/source/h266_encoder_create.c:1065-1077, with a
 *                    wider margin on the GPU), all planes in one launch
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
#include "xg_tma.cuh"

/* ------------------------------------------------------------------ layout */
struct XgPlane {            /* padded plane: data points at picture (0, 0) */
    xg_pix *data;
    int pitch;              /* elements */
    int w, h, pad;          /* picture size and margin on each side */
};

/* -------------------------------------------------------------- qpel planes
 * plane index q = (fy / 4) * 4 + fx / 4 for phases fx, fy in {0, 4, 8, 12};
 * q = 0 is the integer plane itself and is not written.  Samples are produced
 * for the padded area shrunk by the filter reach (3 before, 4 after). */
struct XgQpel { xg_pix *plane[16]; int pitch, w, h, pad; };

/* The three quarter-pel phases (4, 8, 12 of 16) of the luma 8-tap filter, tap k
 * of phase f = 0, 1, 2 (the 1/4 and 1/2 rows of the reference's luma filter
 * table, the 3/4 row mirrored): compile-time constants, so that every multiply
 * of the plane kernel takes an immediate; stream_open checks them against the
 * table the library builds. */
__host__ __device__ constexpr int xg_qp_tap(int f, int k)
{
    return f == 0 ? (k == 0 ? -1 : k == 1 ? 4 : k == 2 ? -10 : k == 3 ? 58 : k == 4 ? 17 : k == 5 ? -5 : k == 6 ? 1 : 0)
         : f == 1 ? ((k == 0 || k == 7) ? -1 : (k == 1 || k == 6) ? 4 : (k == 2 || k == 5) ? -11 : 40)
                  : xg_qp_tap(0, 7 - k);
}

/* A CTA covers a 64 x 32 block of positions for all 15 planes.  The reference
 * tile with the filter reach is staged in shared memory.  Pass 1, one position
 * (row, column) per thread step: its eight horizontal samples give the three
 * horizontal phases at once -- the first-stage values of every staged row, kept
 * in shared memory, and for the output rows the pixels of the three fy = 0
 * planes.  Pass 2, a column and a strip of XG_QP_STRIP output rows per thread:
 * a sliding window of STRIP + 7 values of each vertical source (the integer
 * samples, the three first-stage phases) gives the 12 planes with fy != 0, one
 * 8-tap sum per sample. */
/* device status bits of a picture */
#define XG_STATUS_TMA_WAIT 1                    /* a TMA load did not complete within its wait bound */

#define XG_QP_TW 64
#define XG_QP_TH 32
#define XG_QP_STRIP 8
/* staged tile row: the TW + 7 samples a tile needs start one sample into a
 * 16-byte-aligned TMA box (padded-plane column 1 + TW bx) */
#define XG_QP_BW ((XG_QP_TW + 8 + 16 / (int)sizeof(xg_pix) - 1) / (16 / (int)sizeof(xg_pix)) * (16 / (int)sizeof(xg_pix)))
static_assert(XG_QP_TW * (XG_QP_TH / XG_QP_STRIP) == 256, "pass 2 gives every thread of the CTA one column strip");
__device__ __forceinline__ void xg_qpel_planes_body(const CUtensorMap *tm, const XgPlane &ref, const XgQpel &qp,
                                                    int *status, long long wait_tries)
{
    constexpr int TW = XG_QP_TW, TH = XG_QP_TH, HR = TH + 7, ST = XG_QP_STRIP;
    __shared__ __align__(128) xg_pix tbox[HR][XG_QP_BW];
    __shared__ int16_t hs[3][HR][TW];
    __shared__ unsigned long long tbar;
    __shared__ int tok;
    const int lo = -(qp.pad - 4);                            /* first output position (x and y) */
    const int xe = qp.w + qp.pad - 4, ye = qp.h + qp.pad - 4; /* one past the last */
    const int x0 = lo + (int)blockIdx.x * TW, y0 = lo + (int)blockIdx.y * TH;
    const intptr_t pitch = qp.pitch;
    /* rows y0-3 .. y0+TH+3 and columns x0-3 .. x0+TW+4 of the padded plane by TMA
     * (zeros outside it): the box starts one column earlier, at padded column TW bx */
    if (threadIdx.x == 0) {
        if (!tm) {
            tok = 2;        /* no map (one not on a 64-byte boundary): plain loads */
        } else {
            xg_mbar_init(&tbar, 1);
            xg_mbar_expect_tx(&tbar, (uint32_t)sizeof tbox);
            xg_tma_load_2d(&tbox[0][0], tm, (int)blockIdx.x * TW, (int)blockIdx.y * TH + 1, &tbar);
            tok = xg_mbar_wait(&tbar, 0, wait_tries) ? 1 : 0;
            if (!tok) {
                /* report; once the copy has landed, stage the tile with plain loads */
                atomicOr(status, XG_STATUS_TMA_WAIT);
                tok = xg_mbar_wait(&tbar, 0, XG_TMA_WAIT_TRIES) ? 2 : 0;
            }
        }
    }
    __syncthreads();
    if (!tok) return;
    if (tok == 2) {
        for (int i = threadIdx.x; i < HR * (TW + 7); i += blockDim.x) {
            const int r = i / (TW + 7), c = i - r * (TW + 7), gy = y0 - 3 + r, gx = x0 - 3 + c;
            const bool in = gy >= -ref.pad && gy < ref.h + ref.pad && gx >= -ref.pad && gx < ref.w + ref.pad;
            tbox[r][c + 1] = in ? ref.data[(intptr_t)gy * ref.pitch + gx] : (xg_pix)0;
        }
        __syncthreads();
    }
    auto tile = [&](int r, int c) -> int { return tbox[r][c + 1]; };
    constexpr int sh1 = XG_IF_SHIFT - XG_IF_HEAD;
    for (int i = threadIdx.x; i < HR * TW; i += blockDim.x) {
        const int r = i / TW, c = i % TW;
        int a[8];
#pragma unroll
        for (int k = 0; k < 8; k++) a[k] = tile(r, c + k);
        int sum[3];
#pragma unroll
        for (int f = 0; f < 3; f++) {
            sum[f] = 0;
#pragma unroll
            for (int k = 0; k < 8; k++) sum[f] += a[k] * xg_qp_tap(f, k);
            hs[f][r][c] = (int16_t)((sum[f] - (XG_IF_OFF14 << sh1)) >> sh1);
        }
        const int oy = r - 3, gx = x0 + c, gy = y0 + oy;
        if (oy >= 0 && oy < TH && gx < xe && gy < ye) {
#pragma unroll
            for (int f = 0; f < 3; f++)
                qp.plane[1 + f][(intptr_t)gy * pitch + gx] = (xg_pix)xg_clip_pix((sum[f] + (1 << (XG_IF_SHIFT - 1))) >> XG_IF_SHIFT);
        }
    }
    __syncthreads();
    const int c = threadIdx.x % TW, oy0 = (threadIdx.x / TW) * ST, gx = x0 + c;
    if (gx >= xe) return;
    const int nrow = min(ST, ye - (y0 + oy0));               /* output rows of this strip inside the area */
#pragma unroll
    for (int src = 0; src < 4; src++) {                      /* 0: integer samples, 1..3: first-stage phase src - 1 */
        int w[ST + 7];
#pragma unroll
        for (int k = 0; k < ST + 7; k++) w[k] = src == 0 ? tile(oy0 + k, c + 3) : (int)hs[src - 1][oy0 + k][c];
#pragma unroll
        for (int j = 0; j < ST; j++) {
            if (j >= nrow) break;
            const intptr_t off = (intptr_t)(y0 + oy0 + j) * pitch + gx;
#pragma unroll
            for (int f = 0; f < 3; f++) {
                int v = 0;
#pragma unroll
                for (int k = 0; k < 8; k++) v += w[j + k] * xg_qp_tap(f, k);
                v = src == 0 ? xg_clip_pix((v + (1 << (XG_IF_SHIFT - 1))) >> XG_IF_SHIFT) : xg_s16_to_pix(v);
                qp.plane[(f + 1) * 4 + src][off] = (xg_pix)v;
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_qpel_planes(const __grid_constant__ CUtensorMap tm, const __grid_constant__ XgPlane ref,
                                                      const __grid_constant__ XgQpel qp, int *status, long long wait_tries)
{
    xg_qpel_planes_body(&tm, ref, qp, status, wait_tries);
}

/* Pictures of several streams of one shape in one launch (cross-stream
 * batches): grid z is the picture. */
#define XG_BATCH_MAX 8
struct XgQpelBatch {
    CUtensorMap tm[XG_BATCH_MAX];
    XgPlane ref[XG_BATCH_MAX];
    XgQpel qp[XG_BATCH_MAX];
    int *status[XG_BATCH_MAX];
    long long wait_tries;
};
static_assert(alignof(XgQpelBatch) % 64 == 0 && offsetof(XgQpelBatch, tm) == 0 && sizeof(CUtensorMap) % 64 == 0,
              "each picture's TMA map on a 64-byte boundary of the parameter");
__global__ void __launch_bounds__(256) k_qpel_planes_batch(const __grid_constant__ XgQpelBatch b)
{
    const int i = blockIdx.z;
    const CUtensorMap *tm = &b.tm[i];
    xg_qpel_planes_body(((uintptr_t)tm & 63) ? nullptr : tm, b.ref[i], b.qp[i], b.status[i], b.wait_tries);
}


/* -------------------------------------------------------------- k_me_tiles
 * Grid: (tiles_x, tiles_y, bands).  A CTA takes one 64x64 tile and one band of
 * candidate rows; warp w owns the 16x16 sub-block (w & 3, w >> 2).  A pass of a
 * warp covers 32 candidate columns x XG_ME_D consecutive candidate rows: lane l
 * takes one column and the XG_ME_D rows, so every reference word it loads
 * serves XG_ME_D current rows.  The reference band sits in shared memory as one 32-bit word per
 * pixel position, word (r, x) holding pixels x .. x+3 of band row r, so the
 * four pixels at any candidate offset are one aligned word; the row pitch is
 * congruent to the candidate-row length modulo 32, so the 32 consecutive
 * candidates of a warp read 32 consecutive banks.  |a - b| of four pixels and
 * their sum is one vabsdiff4 with add-reduction.
 * Per candidate a warp has the SADs of its four 8x8 blocks and of its 16x16
 * block in registers (running minimum per lane).  After each pass the four
 * warps of a 32x32 quadrant swap their 16x16 SADs through shared memory under a
 * 128-thread named barrier, each warp taking XG_ME_D / 4 of the candidate rows
 * for the 32x32 CU; the 32x32 SADs go to a ring from which the first
 * XG_ME_SLOTS threads (one candidate slot each) sum the 64x64 SADs every
 * p.agg_passes passes.  A candidate's 32-bit key is SAD * key_mul plus two
 * motion-cost table entries, one multiply-add.
 * Every CU keeps (cost, raster index) as one 64-bit key; the
 * unsigned minimum over lanes, warps and CTAs (atomicMin) selects the smallest
 * cost and, among equal costs, the first candidate in raster order -- the
 * strict '<' raster search.  Costs: (SAD << 8) + (bits(4dx) + bits(4dy)) * lambda
 * (predictor 0).
 * 10-bit pictures: a word holds two 16-bit pixels (word (r, x) = pixels x, x+1);
 * per pixel pair |a - b| + 1024 per lane comes from one packed add-then-max on
 * biased lanes and accumulates lane-wise (32 pairs per 8x8 quadrant fit 16 bits),
 * the bias removed at the end; the current 64x64 tile sits in shared memory
 * (read as broadcasts; each warp keeps a window of the XG_ME_D current rows a
 * reference row meets, with their negations).  Samples must be below 1024. */
#define XG_ME_TILE 64
#define XG_ME_THREADS 512

/* per-picture values, read from device memory so one captured graph serves
 * every picture of a stream */
struct XgQuant { int qmult, qadd, qshift, iqmult, iqadd, iqshift; };
struct XgPicParams {
    uint32_t lambda;
    int32_t status;                     /* written by the kernels: XG_STATUS_* bits (0 = fine) */
    XgQuant quant[5][3];                /* [level 64, 32, 16, 8, 128][plane] */
    const xg_pix *src[3];               /* device-resident source planes (device_io streams) */
    long long src_stride[3];
    int32_t dq_qp[2];                   /* preset-4 TU stage: luma / chroma QP the trellis gets */
};

/* Sources of k_fill_slot: where a picture's samples come from */
enum XgFillMode {
    XG_FILL_IN_PLACE = 0,   /* the slot's interior already holds the picture (host upload): margins only */
    XG_FILL_STAGED8 = 1,    /* 8-bit samples in the per-set device staging, rows of the plane width, << 2 */
    XG_FILL_DEV8 = 2,       /* 8-bit samples at the caller's device planes (picture parameters), << 2 */
    XG_FILL_DEVPIX = 3      /* samples of the library's depth at the caller's device planes */
};

/* Every position of the three padded planes of a slot: the source sample at the
 * position clamped to the picture (edge replication, the layout of
 * Xin266ConstructRefPicBuf / Xin26xExtendPicture), in one launch.  Grid
 * (column groups, padded rows, plane); a thread writes 8 consecutive samples of
 * one row with one 16-byte (8-byte) store: the margins are multiples of 16
 * samples and the slot's data and pitch multiples of 32 / 128, so a group starts
 * on a 16-byte boundary. */
__device__ __forceinline__ void xg_fill_slot_body(const XgPlane &y, const XgPlane &u, const XgPlane &v, const XgPicParams *pp,
                                                  const uint8_t *s0, const uint8_t *s1, const uint8_t *s2, int mode, int pl)
{
    XgPlane d = y;
    if (pl == 1) d = u;
    else if (pl == 2) d = v;
    const int yy = (int)blockIdx.y - d.pad, x0 = -d.pad + 8 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (yy >= d.h + d.pad || x0 >= d.w + d.pad) return;
    const int sy = min(max(yy, 0), d.h - 1);
    const bool inner_row = yy >= 0 && yy < d.h;
    if (mode == XG_FILL_IN_PLACE && inner_row && x0 >= 0 && x0 + 8 <= d.w) return;   /* interior already there */
    xg_pix vals[8];
    if (mode == XG_FILL_IN_PLACE || mode == XG_FILL_DEVPIX) {
        const xg_pix *row = mode == XG_FILL_IN_PLACE ? d.data + (intptr_t)sy * d.pitch : pp->src[pl] + (intptr_t)sy * pp->src_stride[pl];
#pragma unroll
        for (int j = 0; j < 8; j++) vals[j] = row[min(max(x0 + j, 0), d.w - 1)];
    } else {
        const uint8_t *row = mode == XG_FILL_STAGED8 ? (pl == 0 ? s0 : pl == 1 ? s1 : s2) + (intptr_t)sy * d.w
                                                     : reinterpret_cast<const uint8_t *>(pp->src[pl]) + (intptr_t)sy * pp->src_stride[pl];
#pragma unroll
        for (int j = 0; j < 8; j++) vals[j] = (xg_pix)((unsigned)row[min(max(x0 + j, 0), d.w - 1)] << (XG_BITDEPTH - 8));
    }
    xg_pix *o = d.data + (intptr_t)yy * d.pitch + x0;
    if (x0 + 8 <= d.w + d.pad) {
        if constexpr (sizeof(xg_pix) == 2) {
            uint4 w;
            w.x = vals[0] | ((uint32_t)vals[1] << 16); w.y = vals[2] | ((uint32_t)vals[3] << 16);
            w.z = vals[4] | ((uint32_t)vals[5] << 16); w.w = vals[6] | ((uint32_t)vals[7] << 16);
            *reinterpret_cast<uint4 *>(o) = w;
        } else {
            uint2 w;
            w.x = vals[0] | ((uint32_t)vals[1] << 8) | ((uint32_t)vals[2] << 16) | ((uint32_t)vals[3] << 24);
            w.y = vals[4] | ((uint32_t)vals[5] << 8) | ((uint32_t)vals[6] << 16) | ((uint32_t)vals[7] << 24);
            *reinterpret_cast<uint2 *>(o) = w;
        }
    } else {
        for (int j = 0; j < 8 && x0 + j < d.w + d.pad; j++) o[j] = vals[j];
    }
}

__global__ void __launch_bounds__(128) k_fill_slot(const __grid_constant__ XgPlane y, const __grid_constant__ XgPlane u,
                                                   const __grid_constant__ XgPlane v, const XgPicParams *pp, const uint8_t *s0,
                                                   const uint8_t *s1, const uint8_t *s2, int mode)
{
    xg_fill_slot_body(y, u, v, pp, s0, s1, s2, mode, blockIdx.z);
}

/* cross-stream batch: grid z = 3 x picture + plane; one fill mode for all */
struct XgFillBatch {
    XgPlane pl[XG_BATCH_MAX][3];
    const XgPicParams *pp[XG_BATCH_MAX];
    const uint8_t *s8[XG_BATCH_MAX][3];
    int mode;
};
__global__ void __launch_bounds__(128) k_fill_slot_batch(const __grid_constant__ XgFillBatch b)
{
    const int i = blockIdx.z / 3, pl = blockIdx.z % 3;
    xg_fill_slot_body(b.pl[i][0], b.pl[i][1], b.pl[i][2], b.pp[i], b.s8[i][0], b.s8[i][1], b.s8[i][2], b.mode, pl);
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

/* the one-instruction form the search kernel uses: vabsdiff4 with
 * add-reduction into the accumulator; 64 per loop trip (8 accumulators x 8
 * operands) so that loop overhead does not bound the rate */
__global__ void k_sad_peak_add(const uint32_t *in, uint32_t *out, int iters)
{
    uint32_t a[8], b[8];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = 0; i < 8; i++) { a[i] = in[(t + i) & 1023]; b[i] = in[(t * 7 + i * 13) & 1023]; }
    uint32_t acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++) {
                uint32_t d;
                asm volatile("vabsdiff4.u32.u32.u32.add %0, %1, %2, %3;" : "=r"(d) : "r"(a[i]), "r"(b[j]), "r"(acc[j]));
                acc[j] = d;
            }
        a[0] ^= (uint32_t)it;
    }
    uint32_t s = 0;
    for (int i = 0; i < 8; i++) s += acc[i];
    out[t] = s;
}

/* 10-bit form: the biased packed add-then-max per pixel pair plus a lane-wise
 * accumulate, what the 10-bit search kernel issues; 64 pairs per loop trip, the
 * reference words changed every trip (lanes stay below 1024) */
__global__ void k_sad_peak10(const uint32_t *in, uint32_t *out, int iters)
{
    uint32_t a[8], an[8], b[8], bn[8];
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int i = 0; i < 8; i++) {
        a[i] = in[(t + i) & 1023] & 0x03ff03ffu;
        b[i] = in[(t * 7 + i * 13) & 1023] & 0x03ff03ffu;
        an[i] = 0x04000400u - a[i];
        bn[i] = 0x04000400u - b[i];
    }
    uint32_t acc[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j += 2)
                acc[j] += __viaddmax_u16x2(a[i], bn[j], b[j] + an[i]) + __viaddmax_u16x2(a[i], bn[j + 1], b[j + 1] + an[i]);
#pragma unroll
        for (int j = 0; j < 8; j++) { b[j] ^= (uint32_t)it & 0x00ff00ffu; bn[j] = 0x04000400u - b[j]; }
    }
    uint32_t s = 0;
    for (int i = 0; i < 8; i++) s += acc[i];
    out[t] = s;
}

struct XgMeParams {
    XgPlane cur, ref;
    int W, H, ctu, R;
    int band_rows;                      /* candidate rows per band */
    int band_rows_alloc;                /* staged band rows: 64 + band_rows rounded up to XG_ME_D, minus 1 */
    int row_words;                      /* words per band row (pitch of the word array) */
    int agg_passes;                     /* passes buffered for the 32x32 / 64x64 sums, 1..XG_ME_NB_MAX */
    uint32_t key_mul;                   /* 1 << (XG_COST_FRACTION + key bits of the candidate row + sample shift) */
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

/* |a - b| + 1024 in each 16-bit lane of two 10-bit pixel pairs, given the
 * negations an = 1024 - a and bn = 1024 - b (lane-wise, no borrow since lanes are
 * below 1024): max(a + bn, b + an), one packed add-then-max (__viaddmax_u16x2).
 * Lanes stay below 2048, so 32 of them accumulate in a 16-bit lane exactly. */
__device__ __forceinline__ uint32_t xg_absdiff2_biased(uint32_t a, uint32_t an, uint32_t b, uint32_t bn)
{
    return __viaddmax_u16x2(a, bn, b + an);
}
#define XG_NEG2(x) (0x04000400u - (x))

/* Search geometry by the sample depth the search runs at (sbd): 8 = four
 * pixels a word, 10 = two.  The 10-bit library also runs the 8-bit form on
 * pictures that arrive as 8-bit samples (input_bitdepth 8): it packs the
 * 10-bit samples >> 2 and scales every SAD by 4, which is the 10-bit SAD of
 * samples that are multiples of 4.
 * Word positions per staged band row: the last word a warp reads starts at
 * 48 + (2R) + 12 (sbd 8) or 48 + (2R) + 14 (sbd 10). */
__host__ __device__ constexpr int xg_me_relw(int sbd, int nx) { return nx + (sbd == 8 ? 60 : 62); }
/* the current 64x64 tile in shared memory */
__host__ __device__ constexpr int xg_me_cur_words(int sbd) { return sbd == 8 ? 64 * 16 : 64 * 32; }
/* candidate rows per lane and pass, and the key bits that hold the row: sbd 8
 * 8 rows (the register window of current rows is 4 words a row), sbd 10 4 (8
 * words a row plus their negations) */
__host__ __device__ constexpr int xg_me_d(int sbd) { return sbd == 8 ? 8 : 4; }
__host__ __device__ constexpr int xg_me_db(int sbd) { return sbd == 8 ? 3 : 2; }
/* a compile-time flag as a value, for lambdas instantiated per flag */
template <bool B> struct xg_bool_c { static constexpr bool value = B; };
/* keys at or above this are not candidates (padding rows, windows) */
#define XG_ME_KEY_INVALID 0xC0000000u
#define XG_ME_SMEM_MAX (216 * 1024)       /* dynamic shared memory of k_me_tiles, under the 227 KB a CTA may have */
#define XG_ME_NB_MAX 8                    /* passes buffered between 64x64 updates (at most) */
/* 16x16 SADs [2][16][slots] (double-buffered per pass) + 32x32 SADs [2][nb][4][slots], slots = 32 x rows */
__host__ __device__ constexpr int xg_me_agg_words(int sbd, int nb) { return (2 * 16 + 2 * nb * 4) * 32 * xg_me_d(sbd); }
static_assert(xg_me_d(8) % 4 == 0 && (1 << xg_me_db(8)) == xg_me_d(8) && xg_me_d(10) % 4 == 0 && (1 << xg_me_db(10)) == xg_me_d(10),
              "the 32x32 exchange gives each of a quadrant's four warps rows / 4 candidate rows");
template <int SBD>
__global__ void __launch_bounds__(XG_ME_THREADS, 1) k_me_tiles(XgMeParams p, const XgPicParams *pp)
{
    const int band = blockIdx.z;
#include "xg_me_tiles_body.inc"
}

/* cross-stream batch: grid z = bands x picture + band (one band geometry for
 * all); the body is included again, as for k_cu_tail_batch */
struct XgMeBatch {
    XgMeParams p[XG_BATCH_MAX];
    const XgPicParams *pp[XG_BATCH_MAX];
    int bands;
};
template <int SBD>
__global__ void __launch_bounds__(XG_ME_THREADS, 1) k_me_tiles_batch(const __grid_constant__ XgMeBatch b)
{
    const int item = blockIdx.z / b.bands, band = blockIdx.z - item * b.bands;
    const XgMeParams &p = b.p[item];
    const XgPicParams *pp = b.pp[item];
#include "xg_me_tiles_body.inc"
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
    int16_t *resid[3];                /* set (the preset-4 TU stage follows): write the residual
                                         planes (picture layout) instead of transforming */
    /* refs 2: list 1 (its planes, quarter-pel planes and integer search) and the
     * bi records (all CUs) */
    XgPlane ref1[3];
    XgQpel qpel1;
    const unsigned long long *keys1;
    xin_gpu_cu_bi *bi;
};

/* synchronisation of the NT threads that work on one CU (group g of a CTA
 * holding CPB groups): the whole CTA, a named barrier, or the warp */
template <int NT, int CPB>
__device__ __forceinline__ void xg_gsync(int g)
{
    if (NT == 32) __syncwarp();
    else if (CPB == 1) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(NT) : "memory");
}

/* Output tiles of a thread in a NI x NJ product computed by NT threads: TI x TJ
 * outputs, consecutive threads consecutive j tiles. */
__host__ __device__ constexpr int xg_tile_j(int ni, int nj, int nt) { return (ni * nj >= 8 * nt && nj >= 64) ? 4 : ((ni * nj >= 2 * nt && nj >= 32) ? 2 : 1); }
__host__ __device__ constexpr int xg_tile_i(int ni, int nj, int nt)
{
    return (ni * nj / (nt * xg_tile_j(ni, nj, nt)) >= 4) ? 4 : ((ni * nj / (nt * xg_tile_j(ni, nj, nt)) >= 2) ? 2 : 1);
}

/* TN consecutive 32-bit words of shared memory as one vector load */
template <int TN>
__device__ __forceinline__ void xg_ldw(const uint32_t *p, uint32_t *v)
{
    if constexpr (TN == 8) { xg_ldw<4>(p, v); xg_ldw<4>(p + 4, v + 4); }
    else if constexpr (TN == 4) { const uint4 q = *reinterpret_cast<const uint4 *>(p); v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w; }
    else if constexpr (TN == 2) { const uint2 q = *reinterpret_cast<const uint2 *>(p); v[0] = q.x; v[1] = q.y; }
    else v[0] = p[0];
}

/* C(i, j) = sum_l D(i, l) * M(j, l), D int16 and M int8, exact in 32 bits, by the
 * NT threads of a group (tid = rank in the group); epi(i, j, acc) consumes every
 * output.  Tiles: TI x TJ outputs a thread, consecutive threads consecutive j
 * tiles; with IFAST one i row and up to 8 j a thread, consecutive threads
 * consecutive i (for an epilogue that stores along i).  Operands are interleaved in 32-bit words so that one vector load gives
 * a thread the words of its TI rows (TJ rows) at an l step, the loads of a warp
 * are broadcasts or consecutive words, and one dp2a multiplies two int16 samples
 * by two int8 coefficients:
 *   D2[(l / 2) * NI + i] = D(i, l), D(i, l + 1)  (int16 pairs)
 *   M4[(l / 4) * NJ + j] = M(j, l .. l + 3)      (int8 quads).  NL % 4 == 0. */
__host__ __device__ constexpr int xg_tile_jq(int ni, int nj, int nt)
{
    return ni * nj / nt >= 8 ? (nj >= 8 ? 8 : nj) : ni * nj / nt >= 4 ? 4 : ni * nj / nt >= 2 ? 2 : 1;
}
template <int NI, int NJ, int NL, int NT, bool IFAST = false, typename F>
__device__ __forceinline__ void xg_mm_dp2(int tid, const uint32_t *D2, const uint32_t *M4, F epi)
{
    constexpr int TJ = IFAST ? xg_tile_jq(NI, NJ, NT) : xg_tile_j(NI, NJ, NT), TI = IFAST ? 1 : xg_tile_i(NI, NJ, NT);
    constexpr int tj = NJ / TJ, ti = NI / TI, tiles = ti * tj;
    static_assert(NL % 4 == 0 && NI % TI == 0 && NJ % TJ == 0, "dp2a tiles");
    for (int t = tid; t < tiles; t += NT) {
        const int i0 = (IFAST ? t % ti : t / tj) * TI, j0 = (IFAST ? t / ti : t % tj) * TJ;
        int acc[TI][TJ];
#pragma unroll
        for (int a = 0; a < TI; a++)
#pragma unroll
            for (int b = 0; b < TJ; b++) acc[a][b] = 0;
#pragma unroll 4
        for (int l4 = 0; l4 < NL / 4; l4++) {
            uint32_t dlo[TI], dhi[TI], m[TJ];
            xg_ldw<TI>(D2 + (2 * l4) * NI + i0, dlo);
            xg_ldw<TI>(D2 + (2 * l4 + 1) * NI + i0, dhi);
            xg_ldw<TJ>(M4 + l4 * NJ + j0, m);
#pragma unroll
            for (int a = 0; a < TI; a++)
#pragma unroll
                for (int b = 0; b < TJ; b++) {
                    acc[a][b] = __dp2a_lo((int)dlo[a], (int)m[b], acc[a][b]);
                    acc[a][b] = __dp2a_hi((int)dhi[a], (int)m[b], acc[a][b]);
                }
        }
#pragma unroll
        for (int a = 0; a < TI; a++)
#pragma unroll
            for (int b = 0; b < TJ; b++) epi(i0 + a, j0 + b, acc[a][b]);
    }
}

/* element index of X(i, l) in the int16 pair layout of a D operand with NI rows */
template <int NI>
__device__ __forceinline__ int xg_d2(int i, int l) { return (((l >> 1) * NI + i) << 1) | (l & 1); }

/* Shared-memory work area of one N x N transform block (K = min(N, 32) kept
 * frequencies), every operand in the layout of the pass that reads it:
 *   res  residual r(y, x)           D of the forward row pass     (rows y, l = x)
 *   t1   row pass t1(y, k)          D of the forward column pass  (rows k, l = y)
 *   rr   dequantised c(kv, kh)      D of the inverse column pass  (rows kh, l = kv)
 *   t2   column pass t2(kh, y)      D of the inverse row pass     (rows y, l = kh)
 *   mf   DCT2 rows k < K, M(k, x) = T(k, x)   (rows k, l = x or y)
 *   mi   the transpose, M(x, k) = T(k, x)      (rows x, l = k) */
template <int N>
struct XgTqSmem {
    static constexpr int K = N > 32 ? 32 : N;
    alignas(16) uint32_t mf[K * N / 4];
    alignas(16) uint32_t mi[K * N / 4];
    alignas(16) int16_t res[N * N];
    alignas(16) int16_t t1[N * K];
    alignas(16) int16_t rr[K * K];
    alignas(16) int16_t t2[K * N];
};

/* the DCT2 matrix T(k, x) (rows k < K of the N-point transform, from the library's
 * table) into both packed layouts of a work area */
template <int N, int NT>
__device__ __forceinline__ void xg_tq_load_mat(XgTqSmem<N> &sm, const int16_t *m, int tid)
{
    constexpr int K = XgTqSmem<N>::K;
    int8_t *mf = reinterpret_cast<int8_t *>(sm.mf), *mi = reinterpret_cast<int8_t *>(sm.mi);
    for (int i = tid; i < K * N; i += NT) {
        const int k = i / N, x = i % N;
        const int8_t v = (int8_t)m[i];               /* |T(k, x)| <= 90 */
        mf[(((x >> 2) * K + k) << 2) | (x & 3)] = v;
        mi[(((k >> 2) * N + x) << 2) | (k & 3)] = v;
    }
}

/* forward DCT2 (rows, then columns), keeping frequencies below 32 (the rest is
 * zeroed out), quant / dequant over the low min(N, 32) square with 4x4 coding
 * groups (Xin266QuantInvQuant, h266_quant_inv_quant.c:27-139), coefficient plane
 * written with zeros beyond 32 */
template <int N, int NT, int CPB>
__device__ void xg_tq(XgTqSmem<N> &sm, const XgQuant &qz, int s1, int s2, unsigned long long *nz, xg_coef *qout, int qpitch,
                      int tid, int g)
{
    constexpr int K = XgTqSmem<N>::K;
    unsigned long long mask = 0;     /* this thread's nonzero 4x4 groups */
    /* rows: t1(y, k) = sum_x r(y, x) T(k, x) */
    xg_mm_dp2<N, K, N, NT>(tid, reinterpret_cast<const uint32_t *>(sm.res), sm.mf, [&](int y, int k, int acc) {
        sm.t1[xg_d2<K>(k, y)] = (int16_t)xg_clip16(xg_rshift_rnd(acc, s1));
    });
    xg_gsync<NT, CPB>(g);
    /* columns: c(kv, kh) = sum_y t1(y, kh) T(kv, y), then quant / dequant */
    xg_mm_dp2<K, K, N, NT, true>(tid, reinterpret_cast<const uint32_t *>(sm.t1), sm.mf, [&](int kh, int kv, int acc) {
        int t = xg_clip16(xg_rshift_rnd(acc, s2));
        int a = abs(t);
        int qv = (int)(((long long)a * qz.qmult + qz.qadd) >> qz.qshift);
        qv = xg_clip16(t < 0 ? -qv : qv);
        qout[(intptr_t)kv * qpitch + kh] = (xg_coef)qv;
        sm.rr[xg_d2<K>(kh, kv)] = (int16_t)xg_clip16((int)(((long long)qv * qz.iqmult + qz.iqadd) >> qz.iqshift));
        if (qv) mask |= 1ull << ((kv >> 2) * (K >> 2) + (kh >> 2));
    });
    /* one shared-memory OR per warp instead of one per nonzero coefficient */
    const unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)mask), hi = __reduce_or_sync(0xffffffffu, (unsigned)(mask >> 32));
    if ((tid & 31) == 0 && (lo | hi)) atomicOr(nz, ((unsigned long long)hi << 32) | lo);
    if (N > K)      /* the zeroed-out high frequencies */
        for (int o = tid; o < N * N; o += NT) {
            int y = o / N, x = o % N;
            if (y >= K || x >= K) qout[(intptr_t)y * qpitch + x] = (xg_coef)0;
        }
    xg_gsync<NT, CPB>(g);
}

/* inverse DCT2 of the dequantised low K x K part (zero elsewhere): columns
 * first, lines >= 32 skipped (Xin266IDct2WxH), then rows; adds the prediction,
 * clips, writes the reconstruction and accumulates the SSD */
template <int N, int NT, int CPB>
__device__ void xg_itq(XgTqSmem<N> &sm, const xg_pix *pred, int ppitch, const xg_pix *org, int opitch, xg_pix *rec, int rpitch,
                       unsigned long long *ssd, int tid, int g)
{
    constexpr int K = XgTqSmem<N>::K;
    const int s2 = 6 + 15 - 1 - XG_BITDEPTH;
    /* columns: t2(kh, y) = sum_kv c(kv, kh) T(kv, y) */
    xg_mm_dp2<K, N, K, NT>(tid, reinterpret_cast<const uint32_t *>(sm.rr), sm.mi, [&](int kh, int y, int acc) {
        sm.t2[xg_d2<N>(y, kh)] = (int16_t)xg_clip16(xg_rshift_rnd(acc, 7));
    });
    xg_gsync<NT, CPB>(g);
    unsigned long long part = 0;
    /* rows: r'(y, x) = sum_kh t2(kh, y) T(kh, x) */
    xg_mm_dp2<N, N, K, NT>(tid, reinterpret_cast<const uint32_t *>(sm.t2), sm.mi, [&](int y, int x, int acc) {
        int v = xg_clip_pix((int)pred[y * ppitch + x] + xg_clip16(xg_rshift_rnd(acc, s2)));
        rec[(intptr_t)y * rpitch + x] = (xg_pix)v;
        int d = (int)org[(intptr_t)y * opitch + x] - v;
        part += (unsigned long long)(d * d);
    });
    /* warp sum in 32 bits: a thread holds at most ceil(N * N / NT) squared
     * differences, each at most (2^bitdepth - 1)^2, so 32 threads' sum stays below 2^32 */
    static_assert((unsigned long long)((N * N + NT - 1) / NT) * 32 * ((1ull << XG_BITDEPTH) - 1) * ((1ull << XG_BITDEPTH) - 1) <
                      (1ull << 32), "warp SSD sum fits 32 bits");
    const unsigned wsum = __reduce_add_sync(0xffffffffu, (unsigned)part);
    if ((tid & 31) == 0) atomicAdd(ssd, (unsigned long long)wsum);
    xg_gsync<NT, CPB>(g);
}

/* transform sizes of a CU of size S: TU = CU up to 64; a 128 x 128 CU is coded as
 * four 64 x 64 luma and four 32 x 32 chroma TUs per plane (the largest transform) */
__host__ __device__ constexpr int xg_tu_luma(int s) { return s > 64 ? 64 : s; }
__host__ __device__ constexpr int xg_tu_chroma(int s) { return s > 64 ? 32 : s / 2; }

/* the shared state of one CU */
template <int S, int NT>
struct XgTailSmem {
    XgTqSmem<xg_tu_luma(S)> tl;
    XgTqSmem<xg_tu_chroma(S)> tc;
    xg_pix pred[S * S];
    uint32_t part[9][NT / 32];
    unsigned long long nz[3], ssd[3];
};
/* refs 2: each list's luma prediction and the bi search's target */
template <int S>
struct XgTailBiSmem {
    alignas(16) xg_pix bp[2][S * S];
    alignas(16) xg_pix tgt[S * S];
    alignas(16) int16_t hv[2][(S + 7) * S];    /* the coded bi prediction: each list's horizontal-pass rows */
};

/* CPB CUs of size S (luma S x S, chroma S/2 x S/2) per CTA, NT threads per CU
 * (NT = 32: one warp per CU, warp-synchronous) */
/* CTAs per SM the register allocation must allow: 64 x 64 CUs are held to five by
 * shared memory anyway, the other sizes keep eight 128-thread CTAs (64 registers).
 * The bi search's kernels: 64 x 64 two, 32 x 32 four, and the warp-per-CU sizes
 * eight (64 registers with a few spilled: 3.42-3.46 ms against 3.51-3.54 ms per
 * 1080p preset-4 picture at four, 3.46-3.50 at six) */
__host__ __device__ constexpr int xg_tail_min_ctas(int s, bool bi = false, int threads = 128)
{
    /* plain tails up to 32: 1024 threads an SM, so 64 registers a thread at any CTA size */
    return bi ? (s == 64 ? 2 : s == 32 ? 4 : 8) : s == 128 ? 2 : s == 64 ? 5 : 1024 / threads;
}
/* shared memory (dynamic) of a launch */
template <int S, int NT, int CPB, bool BI = false>
__host__ __device__ constexpr size_t xg_tail_smem()
{
    return (sizeof(XgTailSmem<S, NT>) + (BI ? sizeof(XgTailBiSmem<S>) : 0)) * CPB;
}

/* the sum of every thread's v over the NT threads of group g (all threads get it) */
template <int NT, int CPB>
__device__ __forceinline__ uint32_t xg_group_sum(uint32_t v, uint32_t *part, int g, int tid)
{
    v = __reduce_add_sync(0xffffffffu, v);
    if (NT == 32) return v;
    if ((tid & 31) == 0) part[tid >> 5] = v;
    xg_gsync<NT, CPB>(g);
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < NT / 32; w++) t += part[w];
    xg_gsync<NT, CPB>(g);
    return t;
}

/* Xin266FullSubPelMe on the quarter-pel planes (h266_sub_pel_refine.c:81-212) by
 * the NT threads of group g: org (pitch op) against the planes of qp from
 * (bx, by) (quarter-pel) with cost bc: two steps of eight neighbours in the
 * reference's fixed order, strict '<'.  The caller checks that the integer
 * start lies in the window (:117-120). */
template <int S, int NT, int CPB>
__device__ void xg_subpel(const xg_pix *org, intptr_t op, const XgQpel &qp, int cx, int cy, uint32_t lambda,
                          uint32_t (*part)[NT / 32], int g, int tid, int &bx, int &by, uint32_t &bc)
{
    /* candidate c of a step: (offx(c), offy(c)) * step, the fixed order of the
     * reference's eight neighbours; offsets + 1 packed two bits per candidate */
    auto offx = [](int c) { return (int)((0x8858u >> (2 * c)) & 3u) - 1; };   /* -1, 1, 0, 0, -1, 1, -1, 1 */
    auto offy = [](int c) { return (int)((0xA085u >> (2 * c)) & 3u) - 1; };   /*  0, 0, -1, 1, -1, -1, 1, 1 */
    const int lane = tid & 31, warp = tid >> 5;
    const intptr_t qpitch = qp.pitch;
    for (int step = 2; step >= 1; step--) {
        const int bx0 = bx, by0 = by;
        const xg_pix *cb[8];                              /* candidate blocks (top-left sample) */
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int tx = bx0 + offx(c) * step, ty = by0 + offy(c) * step;
            cb[c] = qp.plane[(ty & 3) * 4 + (tx & 3)] + (intptr_t)(cy + (ty >> 2)) * qpitch + cx + (tx >> 2);
        }
        uint32_t acc[8];
#pragma unroll
        for (int c = 0; c < 8; c++) acc[c] = 0;
        /* two pixels' 18 loads in flight a trip (deeper unrolling spills at 32 and 64) */
#pragma unroll 2
        for (int i = tid; i < S * S; i += NT) {
            const int x = i % S, y = i / S;
            const unsigned o = org[(intptr_t)y * op + x];
            const intptr_t off = (intptr_t)y * qpitch + x;
#pragma unroll
            for (int c = 0; c < 8; c++) acc[c] = __usad(o, (unsigned)cb[c][off], acc[c]);
        }
        /* butterfly over the warp that also transposes: lane l ends with the warp's
         * sum of candidate l >> 2 (9 shuffles for the eight sums) */
        uint32_t r4[4], r2[2];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const bool hi = lane & 16;
            r4[j] = (hi ? acc[4 + j] : acc[j]) + __shfl_xor_sync(0xffffffffu, hi ? acc[j] : acc[4 + j], 16);
        }
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const bool hi = lane & 8;
            r2[j] = (hi ? r4[2 + j] : r4[j]) + __shfl_xor_sync(0xffffffffu, hi ? r4[j] : r4[2 + j], 8);
        }
        uint32_t sad;
        {
            const bool hi = lane & 4;
            sad = (hi ? r2[1] : r2[0]) + __shfl_xor_sync(0xffffffffu, hi ? r2[0] : r2[1], 4);
        }
        sad += __shfl_xor_sync(0xffffffffu, sad, 2);
        sad += __shfl_xor_sync(0xffffffffu, sad, 1);
        const int c = lane >> 2;
        if (NT > 32) {                                   /* the group's warps: sums through shared memory */
            if ((lane & 3) == 0) part[c][warp] = sad;
            xg_gsync<NT, CPB>(g);
            uint32_t t = 0;
#pragma unroll
            for (int w = 0; w < NT / 32; w++) t += part[c][w];
            sad = t;
            xg_gsync<NT, CPB>(g);
        }
        /* strict '<' in the fixed candidate order (h266_sub_pel_refine.c:146-160):
         * the earliest candidate of the smallest cost, taken if below the best so far */
        const int tx = bx0 + offx(c) * step, ty = by0 + offy(c) * step;
        uint32_t cost = (sad << XG_COST_FRACTION) + (xg_mvd_bits(tx) + xg_mvd_bits(ty)) * lambda;
        int cc = c;
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
            const uint32_t oc = __shfl_xor_sync(0xffffffffu, cost, o);
            const int oi = __shfl_xor_sync(0xffffffffu, cc, o);
            if (oc < cost || (oc == cost && oi < cc)) { cost = oc; cc = oi; }
        }
        if (cost < bc) { bc = cost; bx = bx0 + offx(cc) * step; by = by0 + offy(cc) * step; }
    }
}

/* luma uni prediction of Xin266LumaInterPred (h266_inter_prediction.c:302-351):
 * the quarter-pel MV clamped to the window in 1/16 pel, read from the
 * quarter-pel plane of its phase (plane 0 is the reference itself) */
template <int S, int NT>
__device__ __forceinline__ void xg_luma_uni(const XgQpel &qp, int cx, int cy, int mvx, int mvy, int mnx, int mny, int mxx,
                                            int mxy, xg_pix *dst, int tid)
{
    const int m16x = min(max(mvx * 4, mnx * 16), mxx * 16), m16y = min(max(mvy * 4, mny * 16), mxy * 16);
    const int ox = cx * 16 + m16x, oy = cy * 16 + m16y;
    const xg_pix *pl = qp.plane[((oy & 15) >> 2) * 4 + ((ox & 15) >> 2)];
    for (int i = tid; i < S * S; i += NT) {
        const int x = i % S, y = i / S;
        dst[i] = pl[(intptr_t)((oy >> 4) + y) * qp.pitch + (ox >> 4) + x];
    }
}

/* the 14-bit intermediate of sample (x, y) of a block at 1/16-pel luma position
 * (ox, oy) in plane rp: pfXinLumaInterpS16 by phase (copy, H, V, HV; default
 * filter), and the same for chroma at 1/32 pel (pfXinChromaInterpS16) */
__device__ __forceinline__ int xg_luma_s16(const XgPlane &rp, int ox, int oy, int x, int y)
{
    const int fx = ox & 15, fy = oy & 15;
    const xg_pix *sp = rp.data + (intptr_t)((oy >> 4) + y) * rp.pitch + (ox >> 4) + x;
    if (!fx && !fy) return ((int)sp[0] << XG_IF_HEAD) - XG_IF_OFF14;
    const int8_t *th = c_luma_taps[0][fx], *tv = c_luma_taps[0][fy];
    if (!fy) return xg_if_to_s16<8>(sp, 1, th);
    if (!fx) return xg_if_to_s16<8>(sp, rp.pitch, tv);
    return xg_if_hv<8, true>(sp, rp.pitch, th, tv);
}
__device__ __forceinline__ int xg_chroma_s16(const XgPlane &rp, int ox, int oy, int x, int y)
{
    const int fx = ox & 31, fy = oy & 31;
    const xg_pix *sp = rp.data + (intptr_t)((oy >> 5) + y) * rp.pitch + (ox >> 5) + x;
    if (!fx && !fy) return ((int)sp[0] << XG_IF_HEAD) - XG_IF_OFF14;
    const int8_t *th = c_chroma_taps[fx], *tv = c_chroma_taps[fy];
    if (!fy) return xg_if_to_s16<4>(sp, 1, th);
    if (!fx) return xg_if_to_s16<4>(sp, rp.pitch, tv);
    return xg_if_hv<4, true>(sp, rp.pitch, th, tv);
}
/* Xin266InterpAvgS16U8 (h266_luma_mc.c:561): clip((a + b + 2^head + 2 * 8192) >> (head + 1)) */
__device__ __forceinline__ xg_pix xg_bi_avg(int a, int b)
{
    return (xg_pix)xg_clip_pix((a + b + (1 << XG_IF_HEAD) + 2 * XG_IF_OFF14) >> (XG_IF_HEAD + 1));
}

/* The bi search's integer step: the reference runs the closed Xin26xMotionEstBbdgs
 * with searchWidth = searchHeight = 4 around the list's uni MV
 * (h266_analyze_inter_cu.c:607-608,665-677); here every integer MV of the +-4
 * square around (ccx, ccy) inside the window, raster order, strict '<' from
 * UINT32_MAX, cost (SAD << 8) + bits(mv) * lambda with predictor 0, on the target
 * t (pitch S) against the list's luma plane rp.  A candidate row is one pass:
 * nine SADs a thread, summed over the group.  Leaves (bx, by, bc) = (0, 0,
 * UINT32_MAX) when no candidate lies in the window. */
template <int S, int NT, int CPB>
__device__ void xg_bi_square(const xg_pix *t, const XgPlane &rp, int cx, int cy, int ccx, int ccy, int mnx, int mny, int mxx,
                             int mxy, uint32_t lambda, uint32_t (*part)[NT / 32], int g, int tid, int &bx, int &by, uint32_t &bc)
{
    const int lane = tid & 31, warp = tid >> 5;
    bx = 0; by = 0; bc = 0xFFFFFFFFu;
    if constexpr (NT == 32 && S == 8) {
        /* 8 x 8 CUs: a lane takes whole candidates (c = lane, lane + 32, lane + 64),
         * then one warp minimum of (cost, raster index) -- the first of the lowest
         * cost, as the strict '<' in raster order keeps */
        unsigned long long best = ~0ull;
        for (int c = lane; c < 81; c += 32) {
            const int mx = ccx + c % 9 - 4, my = ccy + c / 9 - 4;
            if (mx < mnx || mx > mxx || my < mny || my > mxy) continue;
            const xg_pix *r = rp.data + (intptr_t)(cy + my) * rp.pitch + cx + mx;
            uint32_t sad = 0;
#pragma unroll 4
            for (int i = 0; i < S * S; i++) sad = __usad((unsigned)t[i], (unsigned)r[(intptr_t)(i / S) * rp.pitch + i % S], sad);
            const uint32_t cost = (sad << XG_COST_FRACTION) + (xg_mvd_bits(4 * mx) + xg_mvd_bits(4 * my)) * lambda;
            const unsigned long long k = ((unsigned long long)cost << 32) | (unsigned)c;
            best = k < best ? k : best;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ok = __shfl_xor_sync(0xffffffffu, best, o);
            best = ok < best ? ok : best;
        }
        if (best != ~0ull) {
            const int c = (int)(uint32_t)best;
            bc = (uint32_t)(best >> 32); bx = 4 * (ccx + c % 9 - 4); by = 4 * (ccy + c / 9 - 4);
        }
        return;
    }
    for (int dy = -4; dy <= 4; dy++) {
        const int my = ccy + dy;
        if (my < mny || my > mxy) continue;               /* uniform over the group */
        uint32_t acc[9];
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] = 0;
        /* the nine candidates of the row: columns ccx - 4 .. ccx + 4 (within the
         * reference's padding also where they leave the window) */
        const xg_pix *row = rp.data + (intptr_t)(cy + my) * rp.pitch + cx + ccx - 4;
        if constexpr (S >= 32) {
            /* a thread takes runs of eight target samples: sixteen reference samples,
             * loaded once, give all nine candidates' differences */
            for (int c = tid; c < S * S / 8; c += NT) {
                const int y = c / (S / 8), x0 = (c % (S / 8)) * 8;
                const xg_pix *r = row + (intptr_t)y * rp.pitch + x0;
                unsigned rv[16], tv[8];
#pragma unroll
                for (int j = 0; j < 16; j++) rv[j] = r[j];
#pragma unroll
                for (int j = 0; j < 8; j++) tv[j] = t[y * S + x0 + j];
#pragma unroll
                for (int k = 0; k < 9; k++)
#pragma unroll
                    for (int j = 0; j < 8; j++) acc[k] = __usad(tv[j], rv[j + k], acc[k]);
            }
        } else {
            for (int i = tid; i < S * S; i += NT) {
                const int x = i % S, y = i / S;
                const unsigned o = t[y * S + x];
                const xg_pix *r = row + (intptr_t)y * rp.pitch + x;
#pragma unroll
                for (int k = 0; k < 9; k++) acc[k] = __usad(o, (unsigned)r[k], acc[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < 9; k++) acc[k] = __reduce_add_sync(0xffffffffu, acc[k]);
        if (NT > 32) {
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < 9; k++) part[k][warp] = acc[k];
            xg_gsync<NT, CPB>(g);
#pragma unroll
            for (int k = 0; k < 9; k++) {
                uint32_t s = 0;
#pragma unroll
                for (int w = 0; w < NT / 32; w++) s += part[k][w];
                acc[k] = s;
            }
            xg_gsync<NT, CPB>(g);
        }
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int mx = ccx + k - 4;
            if (mx < mnx || mx > mxx) continue;
            const uint32_t c = (acc[k] << XG_COST_FRACTION) + (xg_mvd_bits(4 * mx) + xg_mvd_bits(4 * my)) * lambda;
            if (c < bc) { bc = c; bx = 4 * mx; by = 4 * my; }
        }
    }
}

/* SAD of org against the average of the two luma predictions (pfXinComputeAvgDist:
 * |o - ((a + b + 1) >> 1)|), summed over the group */
template <int S, int NT, int CPB>
__device__ __forceinline__ uint32_t xg_avg_sad(const xg_pix *org, intptr_t op, const xg_pix *a, const xg_pix *b,
                                               uint32_t (*part)[NT / 32], int g, int tid)
{
    uint32_t s = 0;
    for (int i = tid; i < S * S; i += NT) {
        const int x = i % S, y = i / S;
        s = __usad((unsigned)org[(intptr_t)y * op + x], ((unsigned)a[i] + (unsigned)b[i] + 1u) >> 1, s);
    }
    return xg_group_sum<NT, CPB>(s, part[0], g, tid);
}

/* SATD of org against a (or against the average of a and b, pfXinComputeAvgSatd):
 * sum over the 8 x 8 blocks of (Hadamard sum + 2) >> 2, summed over the group.
 * A warp takes a block at a time: lane l holds elements 2l and 2l + 1 (row-major),
 * and the 8 x 8 Hadamard is the 64-point Walsh-Hadamard transform of the block,
 * one butterfly stage per element-index bit (bit 0 inside the lane, bits 1..5
 * across lanes by shuffles); the sum of absolute values does not depend on the
 * order of the stages. */
template <int S, int NT, int CPB>
__device__ uint32_t xg_satd_blocks(const xg_pix *org, intptr_t op, const xg_pix *a, const xg_pix *b, uint32_t (*part)[NT / 32],
                                   int g, int tid)
{
    constexpr int NB = (S / 8) * (S / 8), NW = NT / 32;
    const int lane = tid & 31, warp = tid >> 5, y = lane >> 2, x = (lane & 3) * 2;
    uint32_t s = 0;
    for (int k = warp; k < NB; k += NW) {
        const int bx = (k % (S / 8)) * 8, by = (k / (S / 8)) * 8;
        const int i = (by + y) * S + bx + x;
        const xg_pix *o = org + (intptr_t)(by + y) * op + bx + x;
        int v0 = (int)o[0] - (b ? ((int)a[i] + (int)b[i] + 1) >> 1 : (int)a[i]);
        int v1 = (int)o[1] - (b ? ((int)a[i + 1] + (int)b[i + 1] + 1) >> 1 : (int)a[i + 1]);
        const int s0 = v0 + v1;
        v1 = v0 - v1;
        v0 = s0;
#pragma unroll
        for (int bit = 0; bit < 5; bit++) {
            const int p0 = __shfl_xor_sync(0xffffffffu, v0, 1 << bit), p1 = __shfl_xor_sync(0xffffffffu, v1, 1 << bit);
            const bool hi = (lane >> bit) & 1;
            v0 = hi ? p0 - v0 : v0 + p0;
            v1 = hi ? p1 - v1 : v1 + p1;
        }
        const uint32_t sum = __reduce_add_sync(0xffffffffu, (uint32_t)(abs(v0) + abs(v1)));
        s += (sum + 2) >> 2;
    }
    /* every lane of a warp holds the warp's total: one lane adds it */
    return xg_group_sum<NT, CPB>(lane == 0 ? s : 0u, part[0], g, tid);
}

template <int S, int NT, int CPB, bool BI>
__global__ void __launch_bounds__(NT * CPB, xg_tail_min_ctas(S, BI, NT * CPB)) k_cu_tail(XgTailParams p, const XgPicParams *pp, int ncu)
{
#include "xg_cu_tail_body.inc"
}

/* cross-stream batch (one list): grid y is the picture, every picture has ncu CUs
 * at this level.  The body is the single-picture kernel's, included again rather
 * than shared through a device function, so that the single-picture kernels keep
 * their register allocation. */
struct XgTailBatch {
    XgTailParams p[XG_BATCH_MAX];
    const XgPicParams *pp[XG_BATCH_MAX];
};
/* kernel parameters may take 32,764 bytes */
static_assert(sizeof(XgTailBatch) + sizeof(int) <= 32764 && sizeof(XgMeBatch) <= 32764 && sizeof(XgQpelBatch) <= 32764 &&
              sizeof(XgFillBatch) <= 32764, "batch parameters within the kernel parameter limit");
template <int S, int NT, int CPB>
__global__ void __launch_bounds__(NT * CPB, xg_tail_min_ctas(S, false, NT * CPB)) k_cu_tail_batch(const __grid_constant__ XgTailBatch b, int ncu)
{
    constexpr bool BI = false;
    const XgTailParams &p = b.p[blockIdx.y];
    const XgPicParams *pp = b.pp[blockIdx.y];
#include "xg_cu_tail_body.inc"
}
