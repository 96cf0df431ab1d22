/*
 * xg_me_percall.cuh -- per-call motion-estimation drivers operating on the
 * reference's ME state (xin_me_struct, mirrored in include/xingpu_me.h).
 *
 * XinGpuMotionEstFull  exhaustive integer search (stands in for the closed
 *                      Xin26xMotionEstFull, h26x_core/include/h26x_motion_est.h:23)
 * XinGpuFullSubPelMe   the half- then quarter-pel search of Xin266FullSubPelMe
 *                      (h266_encoder/source/h266_sub_pel_refine.c:81-212)
 */
#include "xg_device.cuh"
#include "../../include/xingpu_me.h"

/* packed search key: cost in the high word, 1 + raster index in the low word,
 * so an unsigned 64-bit minimum gives the smallest cost and, among equal
 * costs, the first candidate in raster order; key (start_cost << 32) | 0 is the
 * incoming best, which a candidate must beat strictly. */
__host__ __device__ __forceinline__ unsigned long long xg_key(uint32_t cost, uint32_t idx1) { return ((unsigned long long)cost << 32) | idx1; }

/* one CTA per candidate row; thread per candidate column; block then global min */
__global__ void k_me_full_cu(const xg_pix *in, int w, int h, const xg_pix *win, int wp, int x0, int y0, int nx, int ny,
                             int mvpx, int mvpy, uint32_t lambda, unsigned long long *best)
{
    __shared__ unsigned long long red[32];
    int row = blockIdx.x;
    unsigned long long k = ~0ull;
    if (row < ny) {
        for (int col = threadIdx.x; col < nx; col += blockDim.x) {
            const xg_pix *r = win + (intptr_t)row * wp + col;
            uint32_t sad = 0;
            for (int y = 0; y < h; y++)
                for (int x = 0; x < w; x++) sad += (uint32_t)abs((int)in[y * w + x] - (int)r[(intptr_t)y * wp + x]);
            int mvx = (x0 + col) * 4, mvy = (y0 + row) * 4;
            uint32_t c = (sad << XG_COST_FRACTION) + (xg_mvd_bits(mvx - mvpx) + xg_mvd_bits(mvy - mvpy)) * lambda;
            unsigned long long kk = xg_key(c, (uint32_t)(row * nx + col) + 1u);
            k = kk < k ? kk : k;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { unsigned long long v = __shfl_xor_sync(0xffffffffu, k, o); k = v < k ? v : k; }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); i++) k = red[i] < k ? red[i] : k;
        atomicMin(best, k);
    }
}

extern "C" void XinGpuMotionEstFull(struct xin_me_struct *meSetOpaque)
{
    xin_gpu_me_struct *me = (xin_gpu_me_struct *)meSetOpaque;
    XG_BEGIN(t);
    XG_ARG(me && me->input && me->ref, "MotionEstFull: null state");
    int w = (int)me->width, h = (int)me->height;
    XG_ARG(w >= 1 && h >= 1 && w <= 128 && h <= 128, "MotionEstFull: bad block size");
    int rx = me->searchWidth, ry = me->searchHeight;
    XG_ARG(rx >= 0 && ry >= 0 && rx <= 512 && ry <= 512, "MotionEstFull: bad search range");
    int mvpx = me->predMv.mv.mvX, mvpy = me->predMv.mv.mvY;
    int cx = mvpx >> 2, cy = mvpy >> 2;
    int x0 = max(cx - rx, (int)me->minMv.mv.mvX), x1 = min(cx + rx, (int)me->maxMv.mv.mvX);
    int y0 = max(cy - ry, (int)me->minMv.mv.mvY), y1 = min(cy + ry, (int)me->maxMv.mv.mvY);
    if (x1 < x0 || y1 < y0) return;   /* empty window: state unchanged */
    int nx = x1 - x0 + 1, ny = y1 - y0 + 1;
    const xg_pix *din = (const xg_pix *)xg_stage_in(t, me->input, me->inputStride, w, h, sizeof(xg_pix)); XG_TRY(din);
    int wp = nx + w - 1, wh = ny + h - 1;
    const xg_pix *dwin = (const xg_pix *)xg_stage_in(t, me->ref + (intptr_t)y0 * me->refStride + x0, me->refStride, wp, wh,
                                                     sizeof(xg_pix));
    XG_TRY(dwin);
    unsigned long long *dbest = (unsigned long long *)xg_dalloc(t, 8); XG_TRY(dbest);
    unsigned long long init = xg_key(me->bestCost, 0);
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(dbest, &init, 8, cudaMemcpyHostToDevice, t->stream), "h2d") == 0);
    k_me_full_cu<<<ny, 128, 0, t->stream>>>(din, w, h, dwin, wp, x0, y0, nx, ny, mvpx, mvpy, me->sadLambda, dbest);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dbest, 8, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    unsigned long long k = *(unsigned long long *)t->hbuf;
    uint32_t idx1 = (uint32_t)k;
    if (idx1 == 0) return;             /* nothing beat the incoming best */
    int row = (int)(idx1 - 1) / nx, col = (int)(idx1 - 1) % nx;
    int mvx = (x0 + col) * 4, mvy = (y0 + row) * 4;
    uint32_t cost = (uint32_t)(k >> 32);
    uint32_t bits = 0;
    {
        unsigned u = mvx - mvpx > 0 ? (unsigned)(2 * (mvx - mvpx) - 1) : (unsigned)(-2 * (mvx - mvpx));
        unsigned l = 0; for (unsigned v = u + 1; v > 1; v >>= 1) l++;
        bits += 2 * l + 1;
        u = mvy - mvpy > 0 ? (unsigned)(2 * (mvy - mvpy) - 1) : (unsigned)(-2 * (mvy - mvpy));
        l = 0; for (unsigned v = u + 1; v > 1; v >>= 1) l++;
        bits += 2 * l + 1;
    }
    me->bestMv.mv.mvX = (int16_t)mvx;
    me->bestMv.mv.mvY = (int16_t)mvy;
    me->bestCost = cost;
    me->bestSad = (cost - bits * me->sadLambda) >> XG_COST_FRACTION;
}

/* luma sample of the reference at quarter-pel MV (tx, ty) relative to the block
 * origin, by the table dispatch pfXinLumaInterp[!!fx][!!fy] with filter 0 */
__device__ __forceinline__ int xg_luma_qpel(const xg_pix *org, intptr_t pitch, int x, int y, int tx, int ty)
{
    int fx = (tx << 2) & 15, fy = (ty << 2) & 15;
    const xg_pix *p = org + (intptr_t)(y + ((ty << 2) >> 4)) * pitch + x + ((tx << 2) >> 4);
    const int8_t *th = c_luma_taps[0][fx], *tv = c_luma_taps[0][fy];
    if (!fx && !fy) return p[0];
    if (fx && !fy) return xg_if_pix<8>(p, 1, th);
    if (!fx && fy) return xg_if_pix<8>(p, pitch, tv);
    return xg_if_hv<8, false>(p, pitch, th, tv);
}

/* one CTA: 8 half-pel then 8 quarter-pel candidates, SADs reduced per candidate */
__global__ void k_full_subpel(const xg_pix *in, int w, int h, const xg_pix *org, int pitch, int mvx, int mvy, int mvpx, int mvpy,
                              uint32_t lambda, uint32_t cost0, int *out)
{
    __shared__ uint32_t sads[8][33];
    __shared__ int best[3];
    const int offx[8] = { -1, 1, 0, 0, -1, 1, -1, 1 }, offy[8] = { 0, 0, -1, 1, -1, -1, 1, 1 };
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) { best[0] = mvx; best[1] = mvy; best[2] = (int)cost0; }
    __syncthreads();
    for (int step = 2; step >= 1; step--) {
        int cx = best[0], cy = best[1];
        for (int c = 0; c < 8; c++) {
            int tx = cx + offx[c] * step, ty = cy + offy[c] * step;
            uint32_t s = 0;
            for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
                int x = i % w, y = i / w;
                s += (uint32_t)abs((int)in[i] - xg_luma_qpel(org, pitch, x, y, tx, ty));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) sads[c][warp] = s;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t bc = (uint32_t)best[2];
            int bx = cx, by = cy;
            for (int c = 0; c < 8; c++) {
                uint32_t s = 0;
                for (int i = 0; i < nw; i++) s += sads[c][i];
                int tx = cx + offx[c] * step, ty = cy + offy[c] * step;
                uint32_t cost = (s << XG_COST_FRACTION) + (xg_mvd_bits(tx - mvpx) + xg_mvd_bits(ty - mvpy)) * lambda;
                if (cost < bc) { bc = cost; bx = tx; by = ty; }
            }
            best[0] = bx; best[1] = by; best[2] = (int)bc;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = best[0]; out[1] = best[1]; out[2] = best[2]; }
}

extern "C" void XinGpuFullSubPelMe(struct xin_me_struct *meSetOpaque)
{
    xin_gpu_me_struct *me = (xin_gpu_me_struct *)meSetOpaque;
    XG_BEGIN(t);
    XG_ARG(me && me->input && me->ref, "FullSubPelMe: null state");
    int w = (int)me->width, h = (int)me->height;
    XG_ARG(w >= 1 && h >= 1 && w <= 128 && h <= 128 && (w & (w - 1)) == 0, "FullSubPelMe: bad block size");
    int mvx = me->bestMv.mv.mvX, mvy = me->bestMv.mv.mvY;
    if (!((mvx >> 2) >= me->minMv.mv.mvX && (mvy >> 2) >= me->minMv.mv.mvY && (mvx >> 2) <= me->maxMv.mv.mvX &&
          (mvy >> 2) <= me->maxMv.mv.mvY))
        return;   /* Xin266FullSubPelMe returns unchanged (h266_sub_pel_refine.c:117-120) */
    /* integer positions reached by the 16 candidates: within +-3 quarter-pel of the start */
    int ix0 = (mvx - 3) >> 2, ix1 = (mvx + 3) >> 2, iy0 = (mvy - 3) >> 2, iy1 = (mvy + 3) >> 2;
    int ox = ix0 - 3, oy = iy0 - 3;                      /* window origin relative to the block */
    int ww = (ix1 - ix0) + w + 7, wh = (iy1 - iy0) + h + 7;
    const xg_pix *din = (const xg_pix *)xg_stage_in(t, me->input, me->inputStride, w, h, sizeof(xg_pix)); XG_TRY(din);
    const xg_pix *dwin = (const xg_pix *)xg_stage_in(t, me->ref + (intptr_t)oy * me->refStride + ox, me->refStride, ww, wh,
                                                     sizeof(xg_pix));
    XG_TRY(dwin);
    int *dout = (int *)xg_dalloc(t, 16); XG_TRY(dout);
    const xg_pix *org = dwin + (intptr_t)(-oy) * ww + (-ox);  /* block origin inside the window */
    k_full_subpel<<<1, 256, 0, t->stream>>>(din, w, h, org, ww, mvx, mvy, me->predMv.mv.mvX, me->predMv.mv.mvY, me->sadLambda,
                                            me->bestCost, dout);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dout, 12, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    int *r = (int *)t->hbuf;
    me->bestMv.mv.mvX = (int16_t)r[0];
    me->bestMv.mv.mvY = (int16_t)r[1];
    me->bestCost = (uint32_t)r[2];
}
