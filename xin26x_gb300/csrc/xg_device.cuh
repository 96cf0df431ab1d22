/*
 * xg_device.cuh -- device building blocks shared by the per-call and the
 * batched kernels: H.266 interpolation stages, Hadamard SATD, separable
 * integer transforms over shared-memory tiles, MVD bit counts.
 * Arithmetic follows the reference functions cited at each helper.
 */
#ifndef XG_DEVICE_CUH
#define XG_DEVICE_CUH

#include "xg_runtime.cuh"

__device__ __forceinline__ int xg_clip_pix(int v) { return min(max(v, 0), XG_MAX_PIX); }
__device__ __forceinline__ int xg_clip16(int v) { return min(max(v, -32768), 32767); }
__device__ __forceinline__ int xg_rshift_rnd(int v, int s) { return s > 0 ? (v + (1 << (s - 1))) >> s : v; }

/* ---- interpolation ------------------------------------------------------
 * One output sample of each stage.  p points at the output position in the
 * source; step is 1 (horizontal) or the row pitch (vertical). */
template <int NT, typename T>
__device__ __forceinline__ int xg_fir(const T *p, intptr_t step, const int8_t *taps)
{
    p -= (NT / 2 - 1) * step;
    int s = 0;
#pragma unroll
    for (int k = 0; k < NT; k++) s += (int)p[k * step] * (int)taps[k];
    return s;
}

/* H or V only, to pixels: clip((sum + 32) >> 6)  (h266_luma_mc.c:100-214) */
template <int NT>
__device__ __forceinline__ int xg_if_pix(const xg_pix *p, intptr_t step, const int8_t *taps)
{
    return xg_clip_pix((xg_fir<NT>(p, step, taps) + (1 << (XG_IF_SHIFT - 1))) >> XG_IF_SHIFT);
}

/* first stage to the 14-bit intermediate: (sum - (8192 << s)) >> s, s = 6 - max(2, 14 - bd)
 * (Xin266LumaInterpHorU8S16, h266_luma_mc.c:216) */
template <int NT>
__device__ __forceinline__ int16_t xg_if_to_s16(const xg_pix *p, intptr_t step, const int8_t *taps)
{
    const int sh = XG_IF_SHIFT - XG_IF_HEAD;
    return (int16_t)((xg_fir<NT>(p, step, taps) - (XG_IF_OFF14 << sh)) >> sh);
}

/* second stage intermediate -> pixel: clip((sum + (1 << (s-1)) + (8192 << 6)) >> s), s = 6 + max(2, 14-bd)
 * (Xin266LumaInterpVetS16U8, h266_luma_mc.c:275) */
__device__ __forceinline__ int xg_s16_to_pix(int sum)
{
    const int sh = XG_IF_SHIFT + XG_IF_HEAD;
    return xg_clip_pix((sum + (1 << (sh - 1)) + (XG_IF_OFF14 << XG_IF_SHIFT)) >> sh);
}

/* full HV sample: horizontal first-stage values of the NT rows around the
 * output, then the vertical pass.  Equal to the reference's two-pass form,
 * whose intermediate sample depends only on its own position. */
template <int NT, bool TO_S16>
__device__ __forceinline__ int xg_if_hv(const xg_pix *p, intptr_t pitch, const int8_t *th, const int8_t *tv)
{
    const xg_pix *r = p - (NT / 2 - 1) * pitch;
    int s = 0;
#pragma unroll
    for (int k = 0; k < NT; k++) s += (int)xg_if_to_s16<NT>(r + k * pitch, 1, th) * (int)tv[k];
    return TO_S16 ? (int)(int16_t)(s >> XG_IF_SHIFT) : xg_s16_to_pix(s);
}

/* ---- Hadamard ---------------------------------------------------------- */
__device__ __forceinline__ unsigned xg_had4(const int d[16])
{
    int t[16], m[16];
#pragma unroll
    for (int r = 0; r < 4; r++) {
        int s01 = d[r * 4] + d[r * 4 + 1], d01 = d[r * 4] - d[r * 4 + 1];
        int s23 = d[r * 4 + 2] + d[r * 4 + 3], d23 = d[r * 4 + 2] - d[r * 4 + 3];
        t[r * 4] = s01 + s23; t[r * 4 + 1] = s01 - s23; t[r * 4 + 2] = d01 + d23; t[r * 4 + 3] = d01 - d23;
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        int s01 = t[c] + t[4 + c], d01 = t[c] - t[4 + c], s23 = t[8 + c] + t[12 + c], d23 = t[8 + c] - t[12 + c];
        m[c] = s01 + s23; m[4 + c] = s01 - s23; m[8 + c] = d01 + d23; m[12 + c] = d01 - d23;
    }
    unsigned s = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) s += (unsigned)abs(m[i]);
    return s;
}

__device__ __forceinline__ void xg_wht8(int *v)
{
    int a[8];
#pragma unroll
    for (int i = 0; i < 4; i++) { a[i] = v[i] + v[i + 4]; a[i + 4] = v[i] - v[i + 4]; }
#pragma unroll
    for (int g = 0; g < 8; g += 4) {
        int b0 = a[g] + a[g + 2], b1 = a[g + 1] + a[g + 3], b2 = a[g] - a[g + 2], b3 = a[g + 1] - a[g + 3];
        v[g] = b0 + b1; v[g + 1] = b0 - b1; v[g + 2] = b2 + b3; v[g + 3] = b2 - b3;
    }
}

__device__ __forceinline__ unsigned xg_had8(int d[64])
{
#pragma unroll
    for (int r = 0; r < 8; r++) xg_wht8(d + r * 8);
    unsigned s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        int col[8];
#pragma unroll
        for (int r = 0; r < 8; r++) col[r] = d[r * 8 + c];
        xg_wht8(col);
#pragma unroll
        for (int r = 0; r < 8; r++) s += (unsigned)abs(col[r]);
    }
    return s;
}

/* ---- transforms -------------------------------------------------------- */
/* matrix of type (0 DCT2, 1 DCT8, 2 DST7) and log2 size, row = basis function */
__device__ __forceinline__ const int16_t *xg_mat(int type, int lg) { return d_mats + c_mat_off[type][lg]; }

/* ---- MVD bits: signed Exp-Golomb length of v (CALC_MVD_BIT,
 * common/include/h26x_definition.h:176; table values restated) */
__device__ __forceinline__ unsigned xg_mvd_bits(int v)
{
    unsigned u = v > 0 ? (unsigned)(2 * v - 1) : (unsigned)(-2 * v);
    return 2u * (31u - (unsigned)__clz(u + 1)) + 1u;
}

#endif
