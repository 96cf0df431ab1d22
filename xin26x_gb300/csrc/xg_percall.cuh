/*
 * xg_percall.cuh -- the plain per-call GPU form: one kernel per reference call.
 *
 * Each XinGpu* entry point has the exact signature of the reference
 * function-pointer type it replaces (see include/xingpu.h).  It stages the
 * host input window the reference function reads into device memory, runs one
 * kernel on the calling thread's stream, copies the outputs back and
 * synchronises.  On failure the outputs are left untouched and the thread's
 * status / message are set.
 */
#include "xg_device.cuh"

/* ====================================================================
 * kernels
 * ==================================================================== */
enum { XG_D_SAD = 0, XG_D_AVG = 1, XG_D_WEIGHT = 2 };

__device__ __forceinline__ int xg_pred_sample(const xg_pix *a, const xg_pix *b, int i, int mode, int wa, int wb)
{
    if (mode == XG_D_SAD) return a[i];
    if (mode == XG_D_AVG) return (a[i] + b[i] + 1) >> 1;
    return xg_clip_pix((wa * a[i] + wb * b[i] + 4) >> 3);
}

template <typename T>
__device__ __forceinline__ T xg_block_sum(T v)
{
    __shared__ T red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    T s = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
    return s;
}

struct XgRefs { const xg_pix *a[8]; const xg_pix *b[8]; };

/* SAD / averaged SAD / weighted SAD / variance of in - pred over w x h packed
 * blocks; blockIdx.x selects the reference (Sadx8/x5/x3). */
__global__ void k_dist(const xg_pix *in, XgRefs refs, int w, int h, int mode, int wa, int wb, int var, uint32_t *out)
{
    const xg_pix *a = refs.a[blockIdx.x], *b = refs.b[blockIdx.x];
    long long s = 0, s2 = 0;
    for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
        int d = (int)in[i] - xg_pred_sample(a, b, i, mode, wa, wb);
        if (var) { s += d; s2 += (long long)d * d; }
        else s += abs(d);
    }
    s = xg_block_sum<long long>(s);
    if (var) s2 = xg_block_sum<long long>(s2);
    if (threadIdx.x == 0) {
        if (var) {
            int lg = 31 - __clz(w * h);
            out[blockIdx.x] = (uint32_t)(s2 - ((s * s) >> lg));
        } else {
            out[blockIdx.x] = (uint32_t)s;
        }
    }
}

/* Hadamard SATD: 8x8 tiles normalised (S+2)>>2 when w and h are multiples of
 * 8, else 4x4 tiles normalised (S+1)>>1 (HM xCalcHADs8x8 / xCalcHADs4x4). */
__global__ void k_satd(const xg_pix *in, const xg_pix *pa, const xg_pix *pb, int w, int h, int mode, int wa, int wb,
                       int pix_only, uint32_t *out)
{
    int t8 = (w % 8 == 0) && (h % 8 == 0);
    int ts = t8 ? 8 : 4, tx = w / ts, ntiles = tx * (h / ts);
    unsigned long long s = 0;
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
        int x0 = (t % tx) * ts, y0 = (t / tx) * ts;
        if (t8) {
            int d[64];
#pragma unroll
            for (int y = 0; y < 8; y++)
#pragma unroll
                for (int x = 0; x < 8; x++) {
                    int i = (y0 + y) * w + x0 + x;
                    d[y * 8 + x] = pix_only ? (int)in[i] : (int)in[i] - xg_pred_sample(pa, pb, i, mode, wa, wb);
                }
            s += (xg_had8(d) + 2) >> 2;
        } else {
            int d[16];
#pragma unroll
            for (int y = 0; y < 4; y++)
#pragma unroll
                for (int x = 0; x < 4; x++) {
                    int i = (y0 + y) * w + x0 + x;
                    d[y * 4 + x] = (int)in[i] - xg_pred_sample(pa, pb, i, mode, wa, wb);
                }
            s += (xg_had4(d) + 1) >> 1;
        }
    }
    s = xg_block_sum<unsigned long long>(s);
    if (threadIdx.x == 0) *out = (uint32_t)s;
}

/* interpolation: VARIANT 0 copy, 1 H, 2 V, 3 HV; SRC16 reads the intermediate
 * (VetS16U8 / VetS16S16); DST16 writes the intermediate. src points at the
 * block origin inside a staged window of row pitch sp. */
template <int NT, int VARIANT, bool SRC16, bool DST16>
__global__ void k_interp(const void *srcv, int sp, void *dstv, int w, int h, int frac, int fi)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const int8_t *th, *tv;
    if (NT == 8) { th = c_luma_taps[fi][frac & 15]; tv = c_luma_taps[fi][(frac >> 4) & 15]; }
    else { th = c_chroma_taps[frac & 31]; tv = c_chroma_taps[(frac >> 5) & 31]; }
    int v;
    if (SRC16) {
        const int16_t *s = (const int16_t *)srcv + (intptr_t)y * sp + x;
        int sum = xg_fir<NT>(s, sp, tv);
        v = DST16 ? (int)(int16_t)(sum >> XG_IF_SHIFT) : xg_s16_to_pix(sum);
    } else {
        const xg_pix *s = (const xg_pix *)srcv + (intptr_t)y * sp + x;
        if (VARIANT == 0) v = DST16 ? (int)(int16_t)(((int)s[0] << XG_IF_HEAD) - XG_IF_OFF14) : (int)s[0];
        else if (VARIANT == 1) v = DST16 ? (int)xg_if_to_s16<NT>(s, 1, th) : xg_if_pix<NT>(s, 1, th);
        else if (VARIANT == 2) v = DST16 ? (int)xg_if_to_s16<NT>(s, sp, tv) : xg_if_pix<NT>(s, sp, tv);
        else v = xg_if_hv<NT, DST16>(s, sp, th, tv);
    }
    if (DST16) ((int16_t *)dstv)[y * w + x] = (int16_t)v;
    else ((xg_pix *)dstv)[y * w + x] = (xg_pix)v;
}

/* bilinear DMVR prediction (h266_core/source/h266_bilinear_filter.c:46-260):
 * taps {16 - f, f} at 1/16 pel, 10-bit intermediate precision, output rows of
 * w + 4 samples.  VARIANT 0 copy (<< 10 - bd), 1 horizontal, 2 vertical,
 * 3 horizontal over h + 1 rows into 16 bits, then vertical with (+8) >> 4. */
template <int VARIANT>
__global__ void k_bili(const xg_pix *src, int sp, int16_t *dst, int w, int h, int frac)
{
    const int ow = w + 4;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= ow || y >= h) return;
    const int fx = frac & 15, fy = frac >> 4, sh = XG_BITDEPTH - 6, off = 1 << (sh - 1);
    const xg_pix *s = src + (intptr_t)y * sp + x;
    int v;
    if (VARIANT == 0) v = (int)s[0] << (10 - XG_BITDEPTH);
    else if (VARIANT == 1) v = ((int)s[0] * (16 - fx) + (int)s[1] * fx + off) >> sh;
    else if (VARIANT == 2) v = ((int)s[0] * (16 - fy) + (int)s[sp] * fy + off) >> sh;
    else {
        const int t0 = (int16_t)(((int)s[0] * (16 - fx) + (int)s[1] * fx + off) >> sh);
        const int t1 = (int16_t)(((int)s[sp] * (16 - fx) + (int)s[sp + 1] * fx + off) >> sh);
        v = (t0 * (16 - fy) + t1 * fy + 8) >> 4;
    }
    dst[y * ow + x] = (int16_t)v;
}

/* bi average / BCW blend of intermediates (h266_luma_mc.c:561,595) */
__global__ void k_interp_avg(const int16_t *a, const int16_t *b, xg_pix *dst, int n, int weighted, int wa, int wb)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!weighted) {
        const int sh = XG_IF_HEAD + 1;
        dst[i] = (xg_pix)xg_clip_pix((a[i] + b[i] + (1 << (sh - 1)) + 2 * XG_IF_OFF14) >> sh);
    } else {
        const int sh = XG_IF_HEAD + 3;
        dst[i] = (xg_pix)xg_clip_pix((a[i] * wa + b[i] * wb + (1 << (sh - 1)) + (XG_IF_OFF14 << 3)) >> sh);
    }
}

/* 1-D forward: line i (input row i, stride is) -> out[k * os + i] */
__global__ void k_fdct1d(int type, int lg, const xg_coef *in, int is, xg_coef *out, int os, int line, int shift)
{
    int n = 1 << lg;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * line) return;
    int k = idx / line, i = idx % line;
    const int16_t *m = xg_mat(type, lg) + k * n;
    int s = 0;
    for (int j = 0; j < n; j++) s += (int)m[j] * (int)in[i * is + j];
    out[k * os + i] = (xg_coef)xg_clip16(xg_rshift_rnd(s, shift));
}

/* 1-D inverse: column j (in[k * is + j]) -> out[j * os + x]; the last skip
 * lines come out zero */
__global__ void k_idct1d(int type, int lg, const xg_coef *in, int is, xg_coef *out, int os, int line, int skip, int shift)
{
    int n = 1 << lg;
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * line) return;
    int j = idx / n, x = idx % n;
    int v = 0;
    if (j < line - skip) {
        const int16_t *m = xg_mat(type, lg);
        int s = 0;
        for (int k = 0; k < n; k++) s += (int)m[k * n + x] * (int)in[k * is + j];
        v = xg_clip16(xg_rshift_rnd(s, shift));
    }
    out[j * os + x] = (xg_coef)v;
}

/* forward / inverse transform skip (Xin26xFSkipWxH restated; Xin266ISkipWxH, h266_inverse_trans.c:91) */
__global__ void k_skip(const xg_coef *in, xg_coef *out, int n, int sh, int inverse)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int v = in[i];
    if (inverse) out[i] = (xg_coef)(int16_t)(v >> sh);
    else out[i] = (xg_coef)xg_clip16(sh >= 0 ? v * (1 << sh) : xg_rshift_rnd(v, -sh));
}

__global__ void k_sub(const xg_pix *in, const xg_pix *pred, xg_coef *out, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (xg_coef)((int)in[i] - (int)pred[i]);
}

__global__ void k_add(const xg_coef *res, const xg_pix *pred, xg_pix *out, int n)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (xg_pix)xg_clip_pix((int)pred[i] + (int)res[i]);
}

/* Xin266QuantInvQuant (h266_quant_inv_quant.c:27-139): per coefficient q and r;
 * bit b of the map <-> coding group b in raster order */
__global__ void k_quant(xg_coef *q, const xg_coef *t, xg_coef *r, int w, int h, int cgw, int cgh, int qmult, int qadd,
                        int qshift, int iqmult, int iqadd, int iqshift, unsigned long long *nz)
{
    __shared__ unsigned long long map;
    if (threadIdx.x == 0) map = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < w * h; i += blockDim.x) {
        int x = i % w, y = i / w;
        int tv = t[i], a = abs(tv);
        int qv = (int)(((long long)a * qmult + qadd) >> qshift);
        qv = xg_clip16(tv < 0 ? -qv : qv);
        q[i] = (xg_coef)qv;
        int rv = (int)(((long long)qv * iqmult + iqadd) >> iqshift);
        r[i] = (xg_coef)xg_clip16(rv);
        if (qv) atomicOr(&map, 1ull << ((y / cgh) * (w / cgw) + x / cgw));
    }
    __syncthreads();
    if (threadIdx.x == 0) *nz = map;
}

/* Xin266PreRdoq (h266_quant_inv_quant.c:208-288): a sequential walk */
__global__ void k_prerdoq(const xg_coef *t, xg_coef *r, xg_coef *q, int w, int h, int cgw, int cgh, int thr,
                          const xin_gpu_scan_pos *scan, unsigned long long *nz)
{
    if (threadIdx.x) return;
    int nblk = w * h / (cgw * cgh), wcg = w / cgw;
    unsigned long long map = *nz;
    for (int i = nblk - 1; i >= 1; i--) {
        unsigned pos = scan[i].posIdx;
        if (!(map & (1ull << pos))) continue;
        int by = (int)pos / wcg, bx = (int)pos - by * wcg, big = 0;
        for (int y = 0; y < cgh; y++)
            for (int x = 0; x < 4; x++) big |= abs((int)t[(by * cgh + y) * w + bx * cgw + x]) > thr;
        if (big) break;
        for (int y = 0; y < 4; y++)
            for (int x = 0; x < cgw; x++) { int p = (by * cgh + y) * w + bx * cgw + x; r[p] = 0; q[p] = 0; }
        map &= ~(1ull << pos);
    }
    *nz = map;
}

/* ====================================================================
 * host wrappers
 * ==================================================================== */
#define XG_BEGIN(T)                     \
    XgThread *T = xg_thread();          \
    if (!T) return;                     \
    (void)cudaGetLastError();           \
    xin_gpu_clear_error();
#define XG_TRY(expr) do { if (!(expr)) return; } while (0)
#define XG_ARG(cond, msg) do { if (!(cond)) { xg_set_error(XIN_GPU_ERR_ARG, "%s", msg); return; } } while (0)

static bool xg_after_launch(XgThread *t, uint64_t n = 1)
{
    xg_count_launch(n);
    return XG_LAUNCH_CHECK("kernel launch") == XIN_GPU_OK;
}

static void xg_dist_call(XG_PIXEL *input, intptr_t is, XG_PIXEL *const *ra, XG_PIXEL *const *rb, int nref, intptr_t rs,
                         uint32_t w, uint32_t h, int mode, int wa, int wb, int var, uint32_t *out)
{
    XG_BEGIN(t);
    XG_ARG(w >= 1 && h >= 1 && w <= 128 && h <= 128 && input && out, "distortion: bad size or pointer");
    const xg_pix *din = (const xg_pix *)xg_stage_in(t, input, is, w, h, sizeof(xg_pix));
    XG_TRY(din);
    XgRefs refs;
    for (int i = 0; i < nref; i++) {
        refs.a[i] = (const xg_pix *)xg_stage_in(t, ra[i], rs, w, h, sizeof(xg_pix));
        XG_TRY(refs.a[i]);
        refs.b[i] = refs.a[i];
        if (rb) { refs.b[i] = (const xg_pix *)xg_stage_in(t, rb[i], rs, w, h, sizeof(xg_pix)); XG_TRY(refs.b[i]); }
    }
    uint32_t *dout = (uint32_t *)xg_dalloc(t, 8 * sizeof(uint32_t));
    XG_TRY(dout);
    k_dist<<<nref, 256, 0, t->stream>>>(din, refs, (int)w, (int)h, mode, wa, wb, var, dout);
    XG_TRY(xg_after_launch(t));
    uint32_t *hout = (uint32_t *)t->hbuf;
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(hout, dout, nref * sizeof(uint32_t), cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    for (int i = 0; i < nref; i++) out[i] = hout[i];
}

extern "C" void XinGpuComputeSad(XG_PIXEL *in, intptr_t is, XG_PIXEL *pred, intptr_t ps, uint32_t w, uint32_t h, uint32_t *sad)
{ xg_dist_call(in, is, &pred, nullptr, 1, ps, w, h, XG_D_SAD, 0, 0, 0, sad); }
extern "C" void XinGpuComputeAvgSad(XG_PIXEL *in, intptr_t is, XG_PIXEL *a, XG_PIXEL *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad)
{ xg_dist_call(in, is, &a, &b, 1, rs, w, h, XG_D_AVG, 0, 0, 0, sad); }
extern "C" void XinGpuComputeWeightSad(XG_PIXEL *in, intptr_t is, XG_PIXEL *a, XG_PIXEL *b, intptr_t rs, uint32_t w, uint32_t h,
                                       int32_t wa, int32_t wb, uint32_t *sad)
{ xg_dist_call(in, is, &a, &b, 1, rs, w, h, XG_D_WEIGHT, wa, wb, 0, sad); }
extern "C" void XinGpuComputeSadx8(XG_PIXEL *in, intptr_t is, XG_PIXEL *ref[8], intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad)
{ xg_dist_call(in, is, ref, nullptr, 8, rs, w, h, XG_D_SAD, 0, 0, 0, sad); }
extern "C" void XinGpuComputeSadx5(XG_PIXEL *in, intptr_t is, XG_PIXEL *r0, XG_PIXEL *r1, XG_PIXEL *r2, XG_PIXEL *r3, XG_PIXEL *r4,
                                   intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad)
{ XG_PIXEL *r[5] = { r0, r1, r2, r3, r4 }; xg_dist_call(in, is, r, nullptr, 5, rs, w, h, XG_D_SAD, 0, 0, 0, sad); }
extern "C" void XinGpuComputeSadx3(XG_PIXEL *in, intptr_t is, XG_PIXEL *r0, XG_PIXEL *r1, XG_PIXEL *r2, intptr_t rs,
                                   uint32_t w, uint32_t h, uint32_t *sad)
{ XG_PIXEL *r[3] = { r0, r1, r2 }; xg_dist_call(in, is, r, nullptr, 3, rs, w, h, XG_D_SAD, 0, 0, 0, sad); }
extern "C" void XinGpuComputeAvgSadx8(XG_PIXEL *in, intptr_t is, XG_PIXEL *a[8], XG_PIXEL *b[8], intptr_t rs, uint32_t w, uint32_t h,
                                      uint32_t *sad)
{ xg_dist_call(in, is, a, b, 8, rs, w, h, XG_D_AVG, 0, 0, 0, sad); }
extern "C" void XinGpuComputeVar(XG_PIXEL *in, intptr_t is, XG_PIXEL *pred, intptr_t ps, uint32_t w, uint32_t h, uint32_t *var)
{ xg_dist_call(in, is, &pred, nullptr, 1, ps, w, h, XG_D_SAD, 0, 0, 1, var); }
extern "C" void XinGpuComputeAvgVar(XG_PIXEL *in, intptr_t is, XG_PIXEL *a, XG_PIXEL *b, intptr_t ps, uint32_t w, uint32_t h, uint32_t *var)
{ xg_dist_call(in, is, &a, &b, 1, ps, w, h, XG_D_AVG, 0, 0, 1, var); }

static void xg_satd_call(XG_PIXEL *in, intptr_t is, XG_PIXEL *a, XG_PIXEL *b, intptr_t rs, uint32_t w, uint32_t h, int mode,
                         int wa, int wb, int pix_only, uint32_t *out)
{
    XG_BEGIN(t);
    XG_ARG(w >= 4 && h >= 4 && w <= 128 && h <= 128 && w % 4 == 0 && h % 4 == 0 && in && out, "SATD: sizes must be multiples of 4");
    const xg_pix *din = (const xg_pix *)xg_stage_in(t, in, is, w, h, sizeof(xg_pix));
    XG_TRY(din);
    const xg_pix *da = din, *db = din;
    if (!pix_only) {
        da = (const xg_pix *)xg_stage_in(t, a, rs, w, h, sizeof(xg_pix)); XG_TRY(da);
        db = da;
        if (b) { db = (const xg_pix *)xg_stage_in(t, b, rs, w, h, sizeof(xg_pix)); XG_TRY(db); }
    }
    uint32_t *dout = (uint32_t *)xg_dalloc(t, 4);
    XG_TRY(dout);
    k_satd<<<1, 128, 0, t->stream>>>(din, da, db, (int)w, (int)h, mode, wa, wb, pix_only, dout);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dout, 4, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    *out = *(uint32_t *)t->hbuf;
}

extern "C" void XinGpuComputeSatd(XG_PIXEL *in, intptr_t is, XG_PIXEL *pred, intptr_t ps, uint32_t w, uint32_t h, uint32_t *satd)
{ xg_satd_call(in, is, pred, nullptr, ps, w, h, XG_D_SAD, 0, 0, 0, satd); }
extern "C" void XinGpuComputeAvgSatd(XG_PIXEL *in, intptr_t is, XG_PIXEL *a, XG_PIXEL *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *satd)
{ xg_satd_call(in, is, a, b, rs, w, h, XG_D_AVG, 0, 0, 0, satd); }
extern "C" void XinGpuComputeWeightSatd(XG_PIXEL *in, intptr_t is, XG_PIXEL *a, XG_PIXEL *b, intptr_t rs, uint32_t w, uint32_t h,
                                        int32_t wa, int32_t wb, uint32_t *satd)
{ xg_satd_call(in, is, a, b, rs, w, h, XG_D_WEIGHT, wa, wb, 0, satd); }
extern "C" void XinGpuComputeHada8x8(XG_PIXEL *in, intptr_t is, uint32_t *satd)
{ xg_satd_call(in, is, nullptr, nullptr, 0, 8, 8, XG_D_SAD, 0, 0, 1, satd); }

/* interpolation: stage exactly the window the reference function reads */
template <int NT, int VARIANT, bool SRC16, bool DST16>
static void xg_interp_call(const void *src, intptr_t ss, void *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h,
                           uint32_t fi)
{
    XG_BEGIN(t);
    XG_ARG(src && dst && w >= 1 && h >= 1 && w <= 128 && h <= 128 && fi <= 2, "interpolation: bad size or pointer");
    const int lo = NT / 2 - 1, hi = NT / 2;
    const bool hx = !SRC16 && (VARIANT == 1 || VARIANT == 3), vy = SRC16 || VARIANT == 2 || VARIANT == 3;
    int mx0 = hx ? lo : 0, mx1 = hx ? hi : 0, my0 = vy ? lo : 0, my1 = vy ? hi : 0;
    size_t es = SRC16 ? sizeof(int16_t) : sizeof(xg_pix);
    size_t ww = w + mx0 + mx1, hh = h + my0 + my1;
    const char *origin = (const char *)src - ((intptr_t)my0 * ss + mx0) * (intptr_t)es;
    char *d = (char *)xg_stage_in(t, origin, ss, ww, hh, es);
    XG_TRY(d);
    size_t des = DST16 ? sizeof(int16_t) : sizeof(xg_pix);
    void *dout = xg_dalloc(t, (size_t)w * h * des);
    XG_TRY(dout);
    dim3 blk(32, 8), grd((w + 31) / 32, (h + 7) / 8);
    k_interp<NT, VARIANT, SRC16, DST16><<<grd, blk, 0, t->stream>>>(d + ((intptr_t)my0 * ww + mx0) * es, (int)ww, dout,
                                                                    (int)w, (int)h, frac, (int)fi);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, dst, ds, dout, w, h, des) == 0);
    XG_TRY(xg_sync(t) == 0);
}

#define XG_INTERP_DEF(NAME, NT, VAR, S16, D16, ST, DT)                                                               \
    extern "C" void NAME(const ST *src, intptr_t ss, DT *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h,      \
                         uint32_t fi)                                                                                \
    { xg_interp_call<NT, VAR, S16, D16>(src, ss, dst, ds, frac, w, h, NT == 8 ? fi : 0); }
XG_INTERP_DEF(XinGpuInterpCopy, 8, 0, false, false, XG_PIXEL, XG_PIXEL)
XG_INTERP_DEF(XinGpuInterpCopyU8S16, 8, 0, false, true, XG_PIXEL, int16_t)
XG_INTERP_DEF(XinGpuLumaInterpHor, 8, 1, false, false, XG_PIXEL, XG_PIXEL)
XG_INTERP_DEF(XinGpuLumaInterpVet, 8, 2, false, false, XG_PIXEL, XG_PIXEL)
XG_INTERP_DEF(XinGpuLumaInterpHorVet, 8, 3, false, false, XG_PIXEL, XG_PIXEL)
XG_INTERP_DEF(XinGpuLumaInterpHorU8S16, 8, 1, false, true, XG_PIXEL, int16_t)
XG_INTERP_DEF(XinGpuLumaInterpVetU8S16, 8, 2, false, true, XG_PIXEL, int16_t)
XG_INTERP_DEF(XinGpuLumaInterpHorVetU8S16, 8, 3, false, true, XG_PIXEL, int16_t)
XG_INTERP_DEF(XinGpuLumaInterpVetS16U8, 8, 2, true, false, int16_t, XG_PIXEL)
XG_INTERP_DEF(XinGpuLumaInterpVetS16S16, 8, 2, true, true, int16_t, int16_t)
XG_INTERP_DEF(XinGpuChromaInterpHor, 4, 1, false, false, XG_PIXEL, XG_PIXEL)
XG_INTERP_DEF(XinGpuChromaInterpVet, 4, 2, false, false, XG_PIXEL, XG_PIXEL)
XG_INTERP_DEF(XinGpuChromaInterpHorVet, 4, 3, false, false, XG_PIXEL, XG_PIXEL)
XG_INTERP_DEF(XinGpuChromaInterpHorU8S16, 4, 1, false, true, XG_PIXEL, int16_t)
XG_INTERP_DEF(XinGpuChromaInterpVetU8S16, 4, 2, false, true, XG_PIXEL, int16_t)
XG_INTERP_DEF(XinGpuChromaInterpHorVetU8S16, 4, 3, false, true, XG_PIXEL, int16_t)
XG_INTERP_DEF(XinGpuChromaInterpVetS16U8, 4, 2, true, false, int16_t, XG_PIXEL)
XG_INTERP_DEF(XinGpuChromaInterpVetS16S16, 4, 2, true, true, int16_t, int16_t)

/* bilinear DMVR prediction, typedef XinBiliInterp, table entry pfXinBiliInterp
 * (h266_encoder/include/h266_func_struct.h:150,741): writes h rows of w + 4
 * samples; reads (w + 4 + hx) x (h + vy) samples from src */
template <int VARIANT>
static void xg_bili_call(const XG_PIXEL *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h)
{
    XG_BEGIN(t);
    XG_ARG(src && dst && w >= 1 && h >= 1 && w <= 128 && h <= 128 && frac >= 0 && frac < 256 && ds >= (intptr_t)w + 4,
           "bilinear interpolation: bad size, phase or pointer");
    const size_t ww = w + 4 + (VARIANT & 1), hh = h + (VARIANT >> 1);
    const xg_pix *d = (const xg_pix *)xg_stage_in(t, src, ss, ww, hh, sizeof(xg_pix)); XG_TRY(d);
    int16_t *dout = (int16_t *)xg_dalloc(t, (size_t)(w + 4) * h * 2); XG_TRY(dout);
    dim3 blk(32, 8), grd((w + 4 + 31) / 32, (h + 7) / 8);
    k_bili<VARIANT><<<grd, blk, 0, t->stream>>>(d, (int)ww, dout, (int)w, (int)h, frac);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, dst, ds, dout, w + 4, h, 2) == 0);
    XG_TRY(xg_sync(t) == 0);
}
#define XG_BILI_DEF(NAME, VAR)                                                                                   \
    extern "C" void NAME(const XG_PIXEL *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w,  \
                         uint32_t h)                                                                             \
    { xg_bili_call<VAR>(src, ss, dst, ds, frac, w, h); }
XG_BILI_DEF(XinGpuBiliInterpCopy, 0)
XG_BILI_DEF(XinGpuBiliInterpHor, 1)
XG_BILI_DEF(XinGpuBiliInterpVet, 2)
XG_BILI_DEF(XinGpuBiliInterpHorVet, 3)

static void xg_avg_call(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, XG_PIXEL *dst, intptr_t ds, uint32_t w,
                        uint32_t h, int weighted, int wa, int wb)
{
    XG_BEGIN(t);
    XG_ARG(a && b && dst && w >= 1 && h >= 1 && w <= 128 && h <= 128, "interp average: bad size or pointer");
    const int16_t *da = (const int16_t *)xg_stage_in(t, a, as, w, h, 2); XG_TRY(da);
    const int16_t *db = (const int16_t *)xg_stage_in(t, b, bs, w, h, 2); XG_TRY(db);
    xg_pix *dout = (xg_pix *)xg_dalloc(t, (size_t)w * h * sizeof(xg_pix)); XG_TRY(dout);
    int n = (int)(w * h);
    k_interp_avg<<<(n + 255) / 256, 256, 0, t->stream>>>(da, db, dout, n, weighted, wa, wb);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, dst, ds, dout, w, h, sizeof(xg_pix)) == 0);
    XG_TRY(xg_sync(t) == 0);
}
extern "C" void XinGpuInterpAvgS16U8(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, XG_PIXEL *dst, intptr_t ds,
                                     uint32_t w, uint32_t h)
{ xg_avg_call(a, as, b, bs, dst, ds, w, h, 0, 0, 0); }
extern "C" void XinGpuInterpWeightS16U8(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, XG_PIXEL *dst, intptr_t ds,
                                        uint32_t w, uint32_t h, int32_t wa, int32_t wb)
{ xg_avg_call(a, as, b, bs, dst, ds, w, h, 1, wa, wb); }

/* 1-D transforms: the input window is line x n (forward: line rows of n) or
 * n x line (inverse: n rows of line columns) */
static void xg_fdct1d_call(int type, int lg, XG_COEFF *in, intptr_t is, XG_COEFF *out, intptr_t os, int32_t line, int32_t shift)
{
    XG_BEGIN(t);
    int n = 1 << lg;
    XG_ARG(in && out && line >= 1 && line <= 64, "forward 1-D transform: bad line count or pointer");
    const xg_coef *din = (const xg_coef *)xg_stage_in(t, in, is, n, line, sizeof(xg_coef)); XG_TRY(din);
    xg_coef *dout = (xg_coef *)xg_dalloc(t, (size_t)n * line * sizeof(xg_coef)); XG_TRY(dout);
    k_fdct1d<<<(n * line + 255) / 256, 256, 0, t->stream>>>(type, lg, din, n, dout, line, line, shift);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, out, os, dout, line, n, sizeof(xg_coef)) == 0);
    XG_TRY(xg_sync(t) == 0);
}
static void xg_idct1d_call(int type, int lg, XG_COEFF *in, intptr_t is, XG_COEFF *out, intptr_t os, int32_t line, int32_t skip,
                           int32_t shift)
{
    XG_BEGIN(t);
    int n = 1 << lg;
    XG_ARG(in && out && line >= 1 && line <= 64 && skip >= 0 && skip <= line, "inverse 1-D transform: bad line count or pointer");
    const xg_coef *din = (const xg_coef *)xg_stage_in(t, in, is, line, n, sizeof(xg_coef)); XG_TRY(din);
    xg_coef *dout = (xg_coef *)xg_dalloc(t, (size_t)n * line * sizeof(xg_coef)); XG_TRY(dout);
    k_idct1d<<<(n * line + 255) / 256, 256, 0, t->stream>>>(type, lg, din, line, dout, n, line, skip, shift);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, out, os, dout, n, line, sizeof(xg_coef)) == 0);
    XG_TRY(xg_sync(t) == 0);
}
#define XG_F1(NAME, TYPE, LG) extern "C" XG_FDCT1D(NAME) { xg_fdct1d_call(TYPE, LG, input, inputStride, output, outputStride, line, shift); }
#define XG_I1(NAME, TYPE, LG) extern "C" XG_IDCT1D(NAME) { xg_idct1d_call(TYPE, LG, input, inputStride, output, outputStride, line, skipLine, shift); }
XG_F1(XinGpuFDct2P2, 0, 1) XG_F1(XinGpuFDct2P4, 0, 2) XG_F1(XinGpuFDct2P8, 0, 3) XG_F1(XinGpuFDct2P16, 0, 4)
XG_F1(XinGpuFDct2P32, 0, 5) XG_F1(XinGpuFDct2P64, 0, 6)
XG_F1(XinGpuFDst7P4, 2, 2) XG_F1(XinGpuFDst7P8, 2, 3) XG_F1(XinGpuFDst7P16, 2, 4) XG_F1(XinGpuFDst7P32, 2, 5)
XG_F1(XinGpuFDct8P4, 1, 2) XG_F1(XinGpuFDct8P8, 1, 3) XG_F1(XinGpuFDct8P16, 1, 4) XG_F1(XinGpuFDct8P32, 1, 5)
XG_I1(XinGpuIDct2P2, 0, 1) XG_I1(XinGpuIDct2P4, 0, 2) XG_I1(XinGpuIDct2P8, 0, 3) XG_I1(XinGpuIDct2P16, 0, 4)
XG_I1(XinGpuIDct2P32, 0, 5) XG_I1(XinGpuIDct2P64, 0, 6)
XG_I1(XinGpuIDst7P4, 2, 2) XG_I1(XinGpuIDst7P8, 2, 3) XG_I1(XinGpuIDst7P16, 2, 4) XG_I1(XinGpuIDst7P32, 2, 5)
XG_I1(XinGpuIDct8P4, 1, 2) XG_I1(XinGpuIDct8P8, 1, 3) XG_I1(XinGpuIDct8P16, 1, 4) XG_I1(XinGpuIDct8P32, 1, 5)

static int xg_lg(uint32_t v) { int l = 0; while ((1u << l) < v) l++; return (1u << l) == v ? l : -1; }

/* 2-D DCT2: forward rows then columns through a transposed temporary
 * (Xin26xFDct2WxH restated); inverse columns first with the zero-out skip of
 * lines beyond 32 (Xin266IDct2WxH, h266_inverse_trans.c:52-88) */
extern "C" void XinGpuFDct2WxH(XG_COEFF *in, intptr_t is, XG_COEFF *out, intptr_t os, uint32_t w, uint32_t h, XG_COEFF *tmp,
                               int32_t s1, int32_t s2)
{
    (void)tmp;
    XG_BEGIN(t);
    int lw = xg_lg(w), lh = xg_lg(h);
    XG_ARG(in && out && lw >= 1 && lw <= 6 && lh >= 1 && lh <= 6, "2-D DCT2: sizes must be powers of two in 2..64");
    const xg_coef *din = (const xg_coef *)xg_stage_in(t, in, is, w, h, sizeof(xg_coef)); XG_TRY(din);
    xg_coef *dtmp = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dtmp);
    xg_coef *dout = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dout);
    int n = (int)(w * h);
    k_fdct1d<<<(n + 255) / 256, 256, 0, t->stream>>>(0, lw, din, (int)w, dtmp, (int)h, (int)h, s1);
    k_fdct1d<<<(n + 255) / 256, 256, 0, t->stream>>>(0, lh, dtmp, (int)h, dout, (int)w, (int)w, s2);
    XG_TRY(xg_after_launch(t, 2));
    XG_TRY(xg_stage_out(t, out, os, dout, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_sync(t) == 0);
}

extern "C" void XinGpuIDct2WxH(XG_COEFF *in, intptr_t is, XG_COEFF *out, intptr_t os, uint32_t w, uint32_t h, XG_COEFF *tmp,
                               int32_t s1, int32_t s2)
{
    (void)tmp;
    XG_BEGIN(t);
    int lw = xg_lg(w), lh = xg_lg(h);
    XG_ARG(in && out && lw >= 1 && lw <= 6 && lh >= 1 && lh <= 6, "2-D IDCT2: sizes must be powers of two in 2..64");
    const xg_coef *din = (const xg_coef *)xg_stage_in(t, in, is, w, h, sizeof(xg_coef)); XG_TRY(din);
    xg_coef *dtmp = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dtmp);
    xg_coef *dout = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dout);
    int n = (int)(w * h), skip = w > 32 ? (int)w - 32 : 0;
    k_idct1d<<<(n + 255) / 256, 256, 0, t->stream>>>(0, lh, din, (int)w, dtmp, (int)h, (int)w, skip, s1);
    k_idct1d<<<(n + 255) / 256, 256, 0, t->stream>>>(0, lw, dtmp, (int)h, dout, (int)w, (int)h, 0, s2);
    XG_TRY(xg_after_launch(t, 2));
    XG_TRY(xg_stage_out(t, out, os, dout, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_sync(t) == 0);
}

static void xg_skip_call(XG_COEFF *in, intptr_t is, XG_COEFF *out, intptr_t os, uint32_t w, uint32_t h, int inverse)
{
    XG_BEGIN(t);
    int lw = xg_lg(w), lh = xg_lg(h);
    XG_ARG(in && out && lw >= 0 && lw <= 7 && lh >= 0 && lh <= 7, "transform skip: sizes must be powers of two");
    const xg_coef *din = (const xg_coef *)xg_stage_in(t, in, is, w, h, sizeof(xg_coef)); XG_TRY(din);
    xg_coef *dout = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dout);
    int n = (int)(w * h);
    int sh = inverse ? 15 - 8 - ((lw + lh) >> 1) : 15 - XG_BITDEPTH - ((lw + lh) >> 1);
    k_skip<<<(n + 255) / 256, 256, 0, t->stream>>>(din, dout, n, sh, inverse);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, out, os, dout, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_sync(t) == 0);
}
extern "C" void XinGpuFSkipWxH(XG_COEFF *in, intptr_t is, XG_COEFF *out, intptr_t os, uint32_t w, uint32_t h, XG_COEFF *tmp)
{ (void)tmp; xg_skip_call(in, is, out, os, w, h, 0); }
extern "C" void XinGpuISkipWxH(XG_COEFF *in, intptr_t is, XG_COEFF *out, intptr_t os, uint32_t w, uint32_t h)
{ xg_skip_call(in, is, out, os, w, h, 1); }

extern "C" void XinGpuBlockSubForDct(XG_PIXEL *in, intptr_t is, XG_PIXEL *pred, intptr_t ps, XG_COEFF *diff, intptr_t ds,
                                     uint32_t w, uint32_t h)
{
    XG_BEGIN(t);
    XG_ARG(in && pred && diff && w >= 1 && h >= 1 && w <= 128 && h <= 128, "residual: bad size or pointer");
    const xg_pix *di = (const xg_pix *)xg_stage_in(t, in, is, w, h, sizeof(xg_pix)); XG_TRY(di);
    const xg_pix *dp = (const xg_pix *)xg_stage_in(t, pred, ps, w, h, sizeof(xg_pix)); XG_TRY(dp);
    xg_coef *dout = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dout);
    int n = (int)(w * h);
    k_sub<<<(n + 255) / 256, 256, 0, t->stream>>>(di, dp, dout, n);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, diff, ds, dout, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_sync(t) == 0);
}

extern "C" void XinGpuBlockAddForDct(XG_COEFF *res, intptr_t rs, XG_PIXEL *pred, intptr_t ps, XG_PIXEL *rec, intptr_t os,
                                     uint32_t w, uint32_t h)
{
    XG_BEGIN(t);
    XG_ARG(res && pred && rec && w >= 1 && h >= 1 && w <= 128 && h <= 128, "reconstruction: bad size or pointer");
    const xg_coef *dr = (const xg_coef *)xg_stage_in(t, res, rs, w, h, sizeof(xg_coef)); XG_TRY(dr);
    const xg_pix *dp = (const xg_pix *)xg_stage_in(t, pred, ps, w, h, sizeof(xg_pix)); XG_TRY(dp);
    xg_pix *dout = (xg_pix *)xg_dalloc(t, (size_t)w * h * sizeof(xg_pix)); XG_TRY(dout);
    int n = (int)(w * h);
    k_add<<<(n + 255) / 256, 256, 0, t->stream>>>(dr, dp, dout, n);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, rec, os, dout, w, h, sizeof(xg_pix)) == 0);
    XG_TRY(xg_sync(t) == 0);
}

extern "C" void XinGpuQuantInvQuant(XG_COEFF *q, XG_COEFF *tc, XG_COEFF *r, intptr_t cs, uint32_t w, uint32_t h, uint32_t cgw,
                                    uint32_t cgh, int32_t qmult, int32_t qadd, int32_t qshift, int32_t iqmult, int32_t iqadd,
                                    int32_t iqshift, uint64_t *nz)
{
    XG_BEGIN(t);
    XG_ARG(q && tc && r && nz && w >= 1 && h >= 1 && w <= 64 && h <= 64 && cgw >= 1 && cgh >= 1 && w % cgw == 0 && h % cgh == 0 &&
           (w / cgw) * (h / cgh) <= 64 && qshift >= 0 && qshift < 63 && iqshift >= 0 && iqshift < 63,
           "quant: bad size, coding-group shape or shift");
    const xg_coef *dt = (const xg_coef *)xg_stage_in(t, tc, cs, w, h, sizeof(xg_coef)); XG_TRY(dt);
    xg_coef *dq = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dq);
    xg_coef *dr = (xg_coef *)xg_dalloc(t, (size_t)w * h * sizeof(xg_coef)); XG_TRY(dr);
    unsigned long long *dnz = (unsigned long long *)xg_dalloc(t, 8); XG_TRY(dnz);
    k_quant<<<1, 1024, 0, t->stream>>>(dq, dt, dr, (int)w, (int)h, (int)cgw, (int)cgh, qmult, qadd, qshift, iqmult, iqadd, iqshift, dnz);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, q, cs, dq, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_stage_out(t, r, cs, dr, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dnz, 8, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    *nz = *(uint64_t *)t->hbuf;
}

extern "C" void XinGpuPreRdoq(XG_COEFF *tc, XG_COEFF *r, XG_COEFF *q, intptr_t cs, uint32_t w, uint32_t h, uint32_t cgw, uint32_t cgh,
                              int32_t thr, xin_gpu_scan_pos *scan, uint64_t *nz)
{
    XG_BEGIN(t);
    XG_ARG(tc && r && q && scan && nz && w >= 4 && h >= 4 && w <= 64 && h <= 64 && cgw == 4 && cgh == 4,
           "pre-RDOQ: 4x4 coding groups and sizes 4..64 required");
    int nblk = (int)(w * h / 16);
    XG_ARG(nblk <= 64, "pre-RDOQ: at most 64 coding groups");
    for (int i = 0; i < nblk; i++) XG_ARG(scan[i].posIdx < (uint32_t)nblk, "pre-RDOQ: scan position out of range");
    const xg_coef *dt = (const xg_coef *)xg_stage_in(t, tc, cs, w, h, sizeof(xg_coef)); XG_TRY(dt);
    xg_coef *dr = (xg_coef *)xg_stage_in(t, r, cs, w, h, sizeof(xg_coef)); XG_TRY(dr);
    xg_coef *dq = (xg_coef *)xg_stage_in(t, q, cs, w, h, sizeof(xg_coef)); XG_TRY(dq);
    xin_gpu_scan_pos *ds = (xin_gpu_scan_pos *)xg_stage_in(t, scan, nblk, nblk, 1, sizeof(xin_gpu_scan_pos)); XG_TRY(ds);
    unsigned long long *dnz = (unsigned long long *)xg_stage_in(t, nz, 1, 1, 1, 8); XG_TRY(dnz);
    k_prerdoq<<<1, 32, 0, t->stream>>>(dt, dr, dq, (int)w, (int)h, (int)cgw, (int)cgh, thr, ds, dnz);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, r, cs, dr, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_stage_out(t, q, cs, dq, w, h, sizeof(xg_coef)) == 0);
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dnz, 8, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    *nz = *(uint64_t *)t->hbuf;
}
