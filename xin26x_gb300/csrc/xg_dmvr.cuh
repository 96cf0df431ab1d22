/*
 * xg_dmvr.cuh -- the encoder's emulation of the H.266 decoder-side MV
 * refinement (DMVR) of a bi-predicted CU, and the helpers it calls through the
 * function table:
 *
 *   XinGpuLumaMotionCompDmvr  Xin266LumaMotionCompDmvr with Xin266DeriveMvFromDmvr
 *                             and Xin266SubPelRefineDmvr
 *                             (h266_encoder/source/h266_inter_prediction.c:864-1420)
 *   XinGpuComputeSadS16       pfXinComputeSadS16 (the closed Xin26xComputeSadS16,
 *                             h26x_core/include/h26x_compute_dist.h:942; restated)
 *   XinGpuCopyAndPad(Uv)      pfXinCopyAndPad / pfXinCopyAndPadUv
 *                             (h266_encoder/source/h266_copy_and_pad.c:32-112, with
 *                             the closed Xin26xBlockCopy / Xin26xBlockPad1/2 restated)
 *
 * One CTA per 16 x 16 sub-block: the bilinear predictions of both lists around
 * the sub-block, the 25 row-subsampled costs of the 5 x 5 integer search in
 * parallel, the decision and the parabolic sub-pel offset on one thread, then
 * the refined 8-tap predictions of both lists and their average.  When a
 * refinement moves the integer position, the reference filters a copy of the
 * unrefined position's (s + 7)-sample region padded by 2 on every side; the
 * kernel reads the same samples through clamped coordinates.
 */

/* one bilinear DMVR sample (h266_core/source/h266_bilinear_filter.c:46-260), as k_bili */
__device__ __forceinline__ int xg_bili_at(const xg_pix *s, int sp, int fx, int fy)
{
    const int sh = XG_BITDEPTH - 6, off = 1 << (sh - 1);
    if (!fx && !fy) return (int)s[0] << (10 - XG_BITDEPTH);
    if (fx && !fy) return ((int)s[0] * (16 - fx) + (int)s[1] * fx + off) >> sh;
    if (!fx) return ((int)s[0] * (16 - fy) + (int)s[sp] * fy + off) >> sh;
    const int t0 = (int16_t)(((int)s[0] * (16 - fx) + (int)s[1] * fx + off) >> sh);
    const int t1 = (int16_t)(((int)s[sp] * (16 - fx) + (int)s[sp + 1] * fx + off) >> sh);
    return (t0 * (16 - fy) + t1 * fy + 8) >> 4;
}

/* one sample of the luma S16 stage (pfXinLumaInterpS16[!!fx][!!fy], h266_luma_mc.c:216-560) */
__device__ __forceinline__ int xg_luma_s16_at(const xg_pix *s, intptr_t sp, int frac, int fi)
{
    const int fx = frac & 15, fy = frac >> 4;
    const int8_t *th = c_luma_taps[fi][fx], *tv = c_luma_taps[fi][fy];
    if (!fx && !fy) return (int)(int16_t)(((int)s[0] << XG_IF_HEAD) - XG_IF_OFF14);
    if (fx && !fy) return (int)xg_if_to_s16<8>(s, 1, th);
    if (!fx) return (int)xg_if_to_s16<8>(s, sp, tv);
    return xg_if_hv<8, true>(s, sp, th, tv);
}

/* the parabolic offset in eighths of the cost difference (Xin266DivForMaxQ7, :864-907) */
__device__ __forceinline__ int xg_dmvr_div8(long long n, long long d)
{
    const bool neg = n < 0;
    if (neg) n = -n;
    int q = 0;
#pragma unroll
    for (int b = 2; b >= 0; b--) {
        const long long step = d << (b + 1);
        if (n >= step) { n -= step; q |= 1 << b; }
    }
    return neg ? -q : q;
}

struct XgDmvrArgs {
    const xg_pix *win[2];       /* staged reference windows: origin XG_DMVR_WOFF samples up-left of
                                   the CU's integer position under the clipped list MV */
    int wp;                     /* window pitch */
    int cu_x, cu_y, w, h, sw, sh, nsx;
    int mnx, mny, mxx, mxy;     /* window, full-pel */
    int mv[4];                  /* L0 x, y, L1 x, y (1/16) */
    int base[4];                /* the same clipped to the window */
    int fi;                     /* luma filter set: 1 = alternative half-pel */
};

#define XG_DMVR_PADP 27         /* pitch of the padded copy: 16 + 11 */
/* window margin: the refined filters reach 3 + 3 samples before the CU's
 * integer position (refinement up to 2.5 samples, filter taps 3 before) and
 * w + 6 after it; the window is (w + 13) x (h + 13) */
#define XG_DMVR_WOFF 6

__global__ void __launch_bounds__(256) k_dmvr(XgDmvrArgs a, int16_t *mvd, xg_pix *pred)
{
    __shared__ int16_t bil[2][20][20];
    __shared__ uint32_t part[25][8];
    __shared__ int16_t pp[2][16][16];
    __shared__ xg_pix padb[2][XG_DMVR_PADP * XG_DMVR_PADP];
    __shared__ int del_s[2];
    const int t = threadIdx.x, n = blockIdx.x;
    const int sw = a.sw, sh = a.sh, x0 = (n % a.nsx) * sw, y0 = (n / a.nsx) * sh;
    /* bilinear predictions of the sub-block and 2 samples around it (:1037-1085):
     * the prediction origin is 2 samples up-left of the integer position */
    for (int i = t; i < 2 * (sw + 4) * (sh + 4); i += blockDim.x) {
        const int l = i / ((sw + 4) * (sh + 4)), j = i - l * (sw + 4) * (sh + 4), r = j / (sw + 4), c = j - r * (sw + 4);
        const xg_pix *s = a.win[l] + (long long)(XG_DMVR_WOFF - 2 + y0 + r) * a.wp + XG_DMVR_WOFF - 2 + x0 + c;
        bil[l][r][c] = (int16_t)xg_bili_at(s, a.wp, a.base[2 * l] & 15, a.base[2 * l + 1] & 15);
    }
    __syncthreads();
    /* the 25 candidates' SADs over every second row (pfXinComputeSadS16 with subShift 1):
     * L0 displaced by (dx, dy), L1 by (-dx, -dy) */
    const int rows = sh >> 1;
    if (t < 25 * rows) {
        const int k = t / rows, j = t - k * rows, dx = k % 5 - 2, dy = k / 5 - 2, y = 2 * j;
        uint32_t s = 0;
        for (int x = 0; x < sw; x++)
            s = __usad((unsigned)(bil[0][2 + y + dy][2 + x + dx] + 32768), (unsigned)(bil[1][2 + y - dy][2 + x - dx] + 32768), s);
        part[k][j] = s;
    }
    __syncthreads();
    if (t == 0) {
        uint32_t cost[25];
        for (int k = 0; k < 25; k++) {
            uint32_t s = 0;
            for (int j = 0; j < rows; j++) s += part[k][j];
            cost[k] = (s << 1) >> 1;               /* (SadS16 << subShift) >> 1 */
        }
        /* one iteration of the integer search (:1087-1160) */
        int ctr = 12, non0 = 1, del[2] = { 0, 0 };
        uint32_t best = cost[12];
        best -= best >> 2;
        if (best < (uint32_t)(sh * sw) || best == 0) non0 = 0;
        else {
            cost[12] = best;
            int bk = 12;
            for (int k = 0; k < 25; k++)
                if (cost[k] < best) { best = cost[k]; bk = k; }
            del[0] = bk % 5 - 2; del[1] = bk / 5 - 2;
            ctr = bk;
        }
        del[0] *= 16; del[1] *= 16;
        /* sub-pel offset from the costs around the best (Xin266SubPelRefineDmvr, :941-973) */
        const int cx = ctr % 5, cy = ctr / 5;
        if (non0 && del[0] != 32 && del[0] != -32 && del[1] != 32 && del[1] != -32) {
            const long long c0 = cost[ctr];
            const long long nb[2][2] = { { cost[cy * 5 + cx - 1], cost[cy * 5 + cx + 1] }, { cost[ctr - 5], cost[ctr + 5] } };
            for (int hv = 0; hv < 2; hv++) {
                const long long num = (nb[hv][0] - nb[hv][1]) * 16, den = nb[hv][0] + nb[hv][1] - 2 * c0;
                if (den == 0) continue;
                if (nb[hv][0] != c0 && nb[hv][1] != c0) del[hv] += xg_dmvr_div8(num, den);
                else del[hv] += nb[hv][0] == c0 ? -8 : 8;
            }
        }
        del_s[0] = del[0]; del_s[1] = del[1];
        mvd[2 * n] = (int16_t)del[0];
        mvd[2 * n + 1] = (int16_t)del[1];
    }
    __syncthreads();
    /* the refined predictions (Xin266LumaMotionCompDmvr, :1260-1405) */
    int dix[2], diy[2], rx[2], ry[2];
#pragma unroll
    for (int l = 0; l < 2; l++) {
        const int sg = l ? -1 : 1;
        rx[l] = a.mv[2 * l] + sg * del_s[0];
        ry[l] = a.mv[2 * l + 1] + sg * del_s[1];
        dix[l] = (rx[l] >> 4) - (a.mv[2 * l] >> 4);
        diy[l] = (ry[l] >> 4) - (a.mv[2 * l + 1] >> 4);
    }
    /* padded copies (Xin266CopyAndPad: the unrefined position's region [-3, s + 4)
     * repeated outward by 2) for the lists whose integer position moved */
    for (int i = t; i < 2 * XG_DMVR_PADP * XG_DMVR_PADP; i += blockDim.x) {
        const int l = i / (XG_DMVR_PADP * XG_DMVR_PADP), j = i - l * XG_DMVR_PADP * XG_DMVR_PADP;
        if (!(dix[l] | diy[l])) continue;
        const int r = j / XG_DMVR_PADP, c = j - r * XG_DMVR_PADP;
        if (r >= sh + 11 || c >= sw + 11) continue;
        const int yy = min(max(r - 5, -3), sh + 3), xx = min(max(c - 5, -3), sw + 3);
        padb[l][j] = a.win[l][(long long)(XG_DMVR_WOFF + y0 + yy) * a.wp + XG_DMVR_WOFF + x0 + xx];
    }
    __syncthreads();
    if (t < sw * sh) {
        const int y = t / sw, x = t - y * sw;
#pragma unroll
        for (int l = 0; l < 2; l++) {
            int v;
            if (dix[l] | diy[l]) {
                const xg_pix *s = padb[l] + (5 + diy[l] + y) * XG_DMVR_PADP + 5 + dix[l] + x;
                v = xg_luma_s16_at(s, XG_DMVR_PADP, ((ry[l] & 15) << 4) | (rx[l] & 15), a.fi);
            } else {
                const int cx = min(max(rx[l], a.mnx * 16), a.mxx * 16), cy = min(max(ry[l], a.mny * 16), a.mxy * 16);
                const int ox = (a.cu_x + x0) * 16 + cx, oy = (a.cu_y + y0) * 16 + cy;
                const int bx = (a.cu_x * 16 + a.base[2 * l]) >> 4, by = (a.cu_y * 16 + a.base[2 * l + 1]) >> 4;
                const xg_pix *s = a.win[l] + (long long)((oy >> 4) - by + XG_DMVR_WOFF + y) * a.wp + (ox >> 4) - bx + XG_DMVR_WOFF + x;
                v = xg_luma_s16_at(s, a.wp, ((oy & 15) << 4) | (ox & 15), a.fi);
            }
            pp[l][y][x] = (int16_t)v;
        }
        /* pfXinInterpAvg (h266_luma_mc.c:561) */
        const int shb = XG_IF_HEAD + 1;
        pred[(long long)(y0 + y) * a.w + x0 + x] =
            (xg_pix)xg_clip_pix((pp[0][y][x] + pp[1][y][x] + (1 << (shb - 1)) + 2 * XG_IF_OFF14) >> shb);
    }
}

extern "C" void XinGpuLumaMotionCompDmvr(const XG_PIXEL *ref0, const XG_PIXEL *ref1, intptr_t refStride, int32_t cuX, int32_t cuY,
                                         int32_t minMvX, int32_t minMvY, int32_t maxMvX, int32_t maxMvY, uint32_t width,
                                         uint32_t height, const int32_t mv[4], int32_t useAltHpelIf, XG_PIXEL *pred,
                                         intptr_t predStride, int16_t *mvdL0SubPu)
{
    XG_BEGIN(t);
    XG_ARG(ref0 && ref1 && mv && pred && mvdL0SubPu, "LumaMotionCompDmvr: null pointer");
    XG_ARG(width >= 8 && height >= 8 && width <= 128 && height <= 128 && !(width & (width - 1)) && !(height & (height - 1)) &&
           predStride >= (intptr_t)width, "LumaMotionCompDmvr: bad block size or stride");
    XgDmvrArgs a;
    memset(&a, 0, sizeof a);
    a.cu_x = cuX; a.cu_y = cuY; a.w = (int)width; a.h = (int)height;
    a.sw = min((int)width, 16); a.sh = min((int)height, 16); a.nsx = (int)width / a.sw;
    a.mnx = minMvX; a.mny = minMvY; a.mxx = maxMvX; a.mxy = maxMvY;
    a.fi = useAltHpelIf ? 1 : 0;
    a.wp = (int)width + 2 * XG_DMVR_WOFF + 1;
    const XG_PIXEL *refs[2] = { ref0, ref1 };
    for (int l = 0; l < 2; l++) {
        a.mv[2 * l] = mv[2 * l]; a.mv[2 * l + 1] = mv[2 * l + 1];
        a.base[2 * l] = min(max(mv[2 * l], minMvX * 16), maxMvX * 16);
        a.base[2 * l + 1] = min(max(mv[2 * l + 1], minMvY * 16), maxMvY * 16);
        const int ix = (cuX * 16 + a.base[2 * l]) >> 4, iy = (cuY * 16 + a.base[2 * l + 1]) >> 4;
        a.win[l] = (const xg_pix *)xg_stage_in(t, refs[l] + (intptr_t)(iy - XG_DMVR_WOFF) * refStride + (ix - XG_DMVR_WOFF),
                                               refStride, width + 2 * XG_DMVR_WOFF + 1, height + 2 * XG_DMVR_WOFF + 1,
                                               sizeof(xg_pix));
        XG_TRY(a.win[l]);
    }
    const int nsub = (int)(width / a.sw) * (int)(height / a.sh);
    int16_t *dmvd = (int16_t *)xg_dalloc(t, (size_t)nsub * 4); XG_TRY(dmvd);
    xg_pix *dpred = (xg_pix *)xg_dalloc(t, (size_t)width * height * sizeof(xg_pix)); XG_TRY(dpred);
    k_dmvr<<<nsub, 256, 0, t->stream>>>(a, dmvd, dpred);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, pred, predStride, dpred, width, height, sizeof(xg_pix)) == 0);
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dmvd, (size_t)nsub * 4, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    memcpy(mvdL0SubPu, t->hbuf, (size_t)nsub * 4);
}

/* ---- table entries ---------------------------------------------------- */

__global__ void k_sad_s16(const int16_t *a, int ap, const int16_t *b, int bp, int w, int h, int sub, uint32_t *out)
{
    __shared__ uint32_t red[32];
    uint32_t s = 0;
    const int rows = (h + (1 << sub) - 1) >> sub;
    for (int i = threadIdx.x; i < rows * w; i += blockDim.x) {
        const int r = i / w, x = i - r * w, y = r << sub;
        s = __usad((unsigned)(a[y * ap + x] + 32768), (unsigned)(b[y * bp + x] + 32768), s);
    }
    s = xg_cta_sum(s, red);
    if (threadIdx.x == 0) *out = s << sub;
}

extern "C" void XinGpuComputeSadS16(int16_t *input, intptr_t inputStride, int16_t *pred, intptr_t predStride, uint32_t width,
                                    uint32_t height, uint32_t subShift, uint32_t *sad)
{
    XG_BEGIN(t);
    XG_ARG(input && pred && sad && width >= 1 && height >= 1 && width <= 256 && height <= 256 && subShift <= 4,
           "ComputeSadS16: bad argument");
    const int16_t *da = (const int16_t *)xg_stage_in(t, input, inputStride, width, height, 2); XG_TRY(da);
    const int16_t *db = (const int16_t *)xg_stage_in(t, pred, predStride, width, height, 2); XG_TRY(db);
    uint32_t *dout = (uint32_t *)xg_dalloc(t, 4); XG_TRY(dout);
    k_sad_s16<<<1, 256, 0, t->stream>>>(da, (int)width, db, (int)width, (int)width, (int)height, (int)subShift, dout);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dout, 4, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    *sad = *(uint32_t *)t->hbuf;
}

/* the (w + 2m + 2p) x (h + 2m + 2p) output: the staged (w + 2m + 1) x (h + 2m + 1)
 * region (m samples before, m + 1 after the block) repeated outward by p */
__global__ void k_copy_pad(const xg_pix *src, int sp, int rw, int rh, int p, xg_pix *dst)
{
    const int ow = rw + 2 * p, oh = rh + 2 * p;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ow * oh) return;
    const int y = i / ow, x = i - y * ow;
    const int sy = min(max(y - p, 0), rh - 1), sx = min(max(x - p, 0), rw - 1);
    dst[i] = src[sy * sp + sx];
}

static void xg_copy_and_pad(XgThread *t, const XG_PIXEL *ref, intptr_t rs, XG_PIXEL *pad, intptr_t ps, uint32_t w, uint32_t h,
                            int taps, int p)
{
    const int m = taps / 2 - 1, rw = (int)w + taps - 1, rh = (int)h + taps - 1;
    const xg_pix *d = (const xg_pix *)xg_stage_in(t, ref - m * rs - m, rs, rw, rh, sizeof(xg_pix)); XG_TRY(d);
    const int ow = rw + 2 * p, oh = rh + 2 * p;
    xg_pix *o = (xg_pix *)xg_dalloc(t, (size_t)ow * oh * sizeof(xg_pix)); XG_TRY(o);
    k_copy_pad<<<(ow * oh + 255) / 256, 256, 0, t->stream>>>(d, rw, rw, rh, p, o);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, pad - (m + p) * ps - (m + p), ps, o, ow, oh, sizeof(xg_pix)) == 0);
}

extern "C" void XinGpuCopyAndPad(XG_PIXEL *ref, intptr_t refStride, XG_PIXEL *pad, intptr_t padStride, uint32_t width,
                                 uint32_t height)
{
    XG_BEGIN(t);
    XG_ARG(ref && pad && width >= 1 && height >= 1 && width <= 128 && height <= 128 && padStride >= (intptr_t)width + 11,
           "CopyAndPad: bad argument");
    xg_copy_and_pad(t, ref, refStride, pad, padStride, width, height, 8, 2);
    if (xin_gpu_last_status() == XIN_GPU_OK) xg_sync(t);
}

extern "C" void XinGpuCopyAndPadUv(XG_PIXEL *refU, XG_PIXEL *refV, intptr_t refStride, XG_PIXEL *padU, XG_PIXEL *padV,
                                   intptr_t padStride, uint32_t width, uint32_t height)
{
    XG_BEGIN(t);
    XG_ARG(refU && refV && padU && padV && width >= 1 && height >= 1 && width <= 64 && height <= 64 &&
           padStride >= (intptr_t)width + 5, "CopyAndPadUv: bad argument");
    xg_copy_and_pad(t, refU, refStride, padU, padStride, width, height, 4, 1);
    if (xin_gpu_last_status() != XIN_GPU_OK) return;
    xg_copy_and_pad(t, refV, refStride, padV, padStride, width, height, 4, 1);
    if (xin_gpu_last_status() == XIN_GPU_OK) xg_sync(t);
}
