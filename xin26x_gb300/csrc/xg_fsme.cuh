/*
 * xg_fsme.cuh -- fast sub-pel search by variance (the preset-6 sub-pel search,
 * fastSubMe 1: h266_encoder/source/h266_encoder_create.c:2007, called at
 * h266_analyze_inter_cu.c:1078-1083):
 *
 *   XinGpuFastSubPelMeVar  Xin266FastSubPelMeVar (h266_encoder/source/h266_sub_pel_refine.c:214-361)
 *   XinGpuInterpoHalfPel   pfXinInterpoHalfPel (typedef XinInterpHalfPel,
 *                          h26x_core/include/h26x_me_func_struct.h:143; closed in the
 *                          reference, restated: the luma filter's half-pel phase)
 *
 * The search evaluates the eight half-pel neighbours of an integer start by the
 * variance of the difference, then (without AMVR) the eight quarter-pel
 * neighbours of the best, each quarter-pel prediction the rounded average of
 * two half-grid samples: for a diagonal step around the centre or a diagonal
 * half position the two points on the other diagonal, otherwise the half
 * position and the point one half-sample further (the pairing of the
 * reference's qBufA / qBufB pointers, h266_encoder/source/h266_create_section.c:97-230).
 *
 * Half-grid planes: element (x, y), x in [-1, w], y in [-1, h], of plane k sits
 * at half-grid point (2x - dx_k, 2y - dy_k), (dx, dy) = (0,0) integer, (1,0)
 * horizontal, (0,1) vertical, (1,1) both; one kernel fills them, a second runs
 * the search in one CTA.
 */

/* sample at half-grid point (gx, gy) relative to o (half-sample units) */
__device__ __forceinline__ int xg_half_grid_at(const xg_pix *o, int op, int gx, int gy, int fi)
{
    const xg_pix *s = o + (long long)(gy >> 1) * op + (gx >> 1);
    const int8_t *t8 = c_luma_taps[fi][8];
    if (!(gx & 1) && !(gy & 1)) return s[0];
    if (!(gy & 1)) return xg_if_pix<8>(s, 1, t8);
    if (!(gx & 1)) return xg_if_pix<8>(s, op, t8);
    return xg_if_hv<8, false>(s, op, t8, t8);
}

/* the four planes, (w + 2) x (h + 2) each, packed one after the other; o: the
 * block origin inside the staged window */
__global__ void k_half_planes(const xg_pix *o, int op, int w, int h, int fi, xg_pix *planes)
{
    const int pw = w + 2, ph = h + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 4 * pw * ph) return;
    const int k = i / (pw * ph), j = i - k * pw * ph, y = j / pw - 1, x = j % pw - 1;
    planes[i] = (xg_pix)xg_half_grid_at(o, op, 2 * x - (k & 1), 2 * y - (k >> 1), fi);
}

/* plane sample at half-grid point (gx, gy), gx in [-2, 2w], gy in [-2, 2h] */
__device__ __forceinline__ int xg_plane_at(const xg_pix *planes, int w, int h, int gx, int gy)
{
    const int dx = gx & 1, dy = gy & 1, pw = w + 2;
    const int k = dx | (dy << 1), x = (gx + dx) >> 1, y = (gy + dy) >> 1;
    return planes[(long long)k * pw * (h + 2) + (long long)(y + 1) * pw + x + 1];
}

/* (gx0, gy0) / (gx1, gy1): the prediction's half-grid offsets; the second only when avg */
__device__ void xg_fsme_var(const xg_pix *in, const xg_pix *planes, int w, int h, int gx0, int gy0, int gx1, int gy1, bool avg,
                            long long *red, uint32_t *out)
{
    long long s = 0, s2 = 0;
    for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
        const int y = i / w, x = i - y * w;
        int p = xg_plane_at(planes, w, h, gx0 + 2 * x, gy0 + 2 * y);
        if (avg) p = (p + xg_plane_at(planes, w, h, gx1 + 2 * x, gy1 + 2 * y) + 1) >> 1;
        const int d = (int)in[i] - p;
        s += d;
        s2 += (long long)d * d;
    }
#pragma unroll
    for (int o2 = 16; o2 > 0; o2 >>= 1) { s += __shfl_xor_sync(0xffffffffu, s, o2); s2 += __shfl_xor_sync(0xffffffffu, s2, o2); }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = s; red[32 + (threadIdx.x >> 5)] = s2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long a = 0, b = 0;
        for (int j = 0; j < (int)(blockDim.x >> 5); j++) { a += red[j]; b += red[32 + j]; }
        *out = (uint32_t)(b - ((a * a) >> (31 - __clz(w * h))));
    }
}

__device__ __forceinline__ unsigned long long xg_fsme_cost(uint32_t var, int mvx, int mvy, int mvpx, int mvpy, int shift,
                                                           unsigned long long lambda)
{
    const unsigned long long bits = (unsigned long long)(xg_mvd_bits((mvx - mvpx) >> shift) + xg_mvd_bits((mvy - mvpy) >> shift)) << 15;
    return (unsigned long long)(uint32_t)(var << XG_COST_FRACTION) + ((lambda * bits + (1ull << 22)) >> 23);
}

/* io: mvx, mvy in; mvx, mvy, best position out */
__global__ void k_fsme_search(const xg_pix *in, const xg_pix *planes, int w, int h, int mvpx, int mvpy, unsigned long long lambda,
                              int imv, int *io)
{
    __shared__ long long red[64];
    __shared__ uint32_t var[9];
    __shared__ int hb[3];
    const int off[9][2] = { { -1, 0 }, { 1, 0 }, { 0, -1 }, { 0, 1 }, { -1, -1 }, { 1, -1 }, { -1, 1 }, { 1, 1 }, { 0, 0 } };
    const int shift = imv == 3 ? 1 : imv << 1;
    const int mvx = io[0], mvy = io[1];
    /* the integer start and its eight half-pel neighbours */
    for (int p = 0; p < 9; p++) xg_fsme_var(in, planes, w, h, off[p][0], off[p][1], 0, 0, false, red, &var[p]);
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long best = xg_fsme_cost(var[8], mvx, mvy, mvpx, mvpy, shift, lambda);
        int bp = 8;
        for (int p = 0; p < 8; p++) {
            const unsigned long long c = xg_fsme_cost(var[p], mvx + 2 * off[p][0], mvy + 2 * off[p][1], mvpx, mvpy, shift, lambda);
            if (c < best) { best = c; bp = p; }
        }
        hb[0] = bp;
        red[63] = (long long)best;
    }
    __syncthreads();
    const int bp = hb[0], hx = off[bp][0], hy = off[bp][1];
    if (imv != 0) {
        if (threadIdx.x == 0) { io[0] = mvx + 2 * hx; io[1] = mvy + 2 * hy; io[2] = bp; }
        return;
    }
    const unsigned long long best0 = (unsigned long long)red[63];
    __syncthreads();
    for (int p = 0; p < 8; p++) {
        const int qx = off[p][0], qy = off[p][1];
        const bool other = qx && qy && !((hx ^ hy) & 1);
        const int ax = hx + qx, ay = other ? hy : hy + qy, bx = other ? hx : hx, by = other ? hy + qy : hy;
        xg_fsme_var(in, planes, w, h, ax, ay, bx, by, true, red, &var[p]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long best = best0;
        int qp = 8;
        const int mx = mvx + 2 * hx, my = mvy + 2 * hy;
        for (int p = 0; p < 8; p++) {
            const unsigned long long c = xg_fsme_cost(var[p], mx + off[p][0], my + off[p][1], mvpx, mvpy, shift, lambda);
            if (c < best) { best = c; qp = p; }
        }
        io[0] = mx + off[qp][0]; io[1] = my + off[qp][1]; io[2] = qp;
    }
}

/* stage the window the half-grid planes read (samples -5 .. w + 3 around the
 * block: the filter's 3 before / 4 after around positions -2 .. w - 1) and fill
 * the planes */
static xg_pix *xg_half_planes(XgThread *t, const XG_PIXEL *ref, intptr_t rs, int w, int h, int fi)
{
    const int ww = w + 9, wh = h + 9;
    const xg_pix *win = (const xg_pix *)xg_stage_in(t, ref - 5 * rs - 5, rs, ww, wh, sizeof(xg_pix));
    if (!win) return nullptr;
    const int n = 4 * (w + 2) * (h + 2);
    xg_pix *planes = (xg_pix *)xg_dalloc(t, (size_t)n * sizeof(xg_pix));
    if (!planes) return nullptr;
    k_half_planes<<<(n + 255) / 256, 256, 0, t->stream>>>(win + 5 * ww + 5, ww, w, h, fi, planes);
    if (!xg_after_launch(t)) return nullptr;
    return planes;
}

extern "C" void XinGpuFastSubPelMeVar(struct xin_me_struct *meSetOpaque, int32_t listIdx, int32_t refIdx)
{
    (void)listIdx;
    (void)refIdx;
    xin_gpu_me_struct *me = (xin_gpu_me_struct *)meSetOpaque;
    XG_BEGIN(t);
    XG_ARG(me && me->input && me->ref, "FastSubPelMeVar: null state");
    const int w = (int)me->width, h = (int)me->height;
    XG_ARG(w >= 1 && h >= 1 && w <= 128 && h <= 128 && !(w & (w - 1)) && !(h & (h - 1)), "FastSubPelMeVar: bad block size");
    XG_ARG(me->iMvMode == 0 || me->iMvMode == 3, "FastSubPelMeVar: AMVR mode other than off or half-pel");
    const int mvx = me->bestMv.mv.mvX, mvy = me->bestMv.mv.mvY, ix = mvx >> 2, iy = mvy >> 2;
    if (!(ix >= me->minMv.mv.mvX && iy >= me->minMv.mv.mvY && ix <= me->maxMv.mv.mvX && iy <= me->maxMv.mv.mvY))
        return;   /* h266_sub_pel_refine.c:262-265 */
    const xg_pix *din = (const xg_pix *)xg_stage_in(t, me->input, me->inputStride, w, h, sizeof(xg_pix)); XG_TRY(din);
    xg_pix *planes = xg_half_planes(t, me->ref + (intptr_t)iy * me->refStride + ix, me->refStride, w, h, me->iMvMode == 3);
    XG_TRY(planes);
    int *dio = (int *)xg_dalloc(t, 16); XG_TRY(dio);
    int hio[4] = { mvx, mvy, 0, 0 };
    memcpy(t->hbuf, hio, 16);
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(dio, t->hbuf, 16, cudaMemcpyHostToDevice, t->stream), "h2d") == 0);
    k_fsme_search<<<1, 256, 0, t->stream>>>(din, planes, w, h, me->predMv.mv.mvX, me->predMv.mv.mvY,
                                            (unsigned long long)me->sseLambda, me->iMvMode, dio);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_cuda_check(cudaMemcpyAsync((char *)t->hbuf + 16, dio, 12, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    const int *r = (const int *)((char *)t->hbuf + 16);
    me->bestMv.mv.mvX = (int16_t)r[0];
    me->bestMv.mv.mvY = (int16_t)r[1];
    me->bestPos = (uint32_t)r[2];
}

extern "C" void XinGpuInterpoHalfPel(XG_PIXEL *ref, intptr_t refStride, uint32_t width, uint32_t height, XG_PIXEL *integPel,
                                     XG_PIXEL *halfPelH, XG_PIXEL *halfPelV, XG_PIXEL *halfPelHv, intptr_t interpStride,
                                     int32_t interpAlt)
{
    XG_BEGIN(t);
    XG_ARG(ref && integPel && halfPelH && halfPelV && halfPelHv && width >= 1 && height >= 1 && width <= 128 && height <= 128 &&
           interpStride >= (intptr_t)width + 3, "InterpoHalfPel: bad argument");
    const int w = (int)width, h = (int)height;
    xg_pix *planes = xg_half_planes(t, ref, refStride, w, h, interpAlt ? 1 : 0); XG_TRY(planes);
    /* the layout the ME state's pointers assume (h266_create_section.c:74-86): the
     * integer plane from (-1, -1) at integPel, the horizontal plane from (0, -1) at
     * halfPelH + stride, the vertical plane from (-1, 0) at halfPelV, the diagonal
     * plane from (0, 0) at halfPelHv */
    const int pw = w + 2, pn = pw * (h + 2);
    XG_PIXEL *dst[4] = { integPel, halfPelH + interpStride, halfPelV, halfPelHv };
    const int x0[4] = { -1, 0, -1, 0 }, y0[4] = { -1, -1, 0, 0 };
    for (int k = 0; k < 4; k++) {
        const xg_pix *src = planes + (size_t)k * pn + (size_t)(y0[k] + 1) * pw + x0[k] + 1;
        XG_TRY(xg_cuda_check(cudaMemcpy2DAsync(dst[k], (size_t)interpStride * sizeof(xg_pix), src, (size_t)pw * sizeof(xg_pix),
                                               (size_t)(w + 1 - x0[k]) * sizeof(xg_pix), (size_t)(h + 1 - y0[k]),
                                               cudaMemcpyDeviceToHost, t->stream), "InterpoHalfPel d2h") == 0);
    }
    XG_TRY(xg_sync(t) == 0);
}
