/*
 * xin_oracle.c -- CPU oracle (checker) for the xin26x VVC encoder pixel hot path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU legs of bench.py to check the CUDA library.  The product never links it.
 * See xin_oracle.h for the parity status legend ("pinned (open C)",
 * "pinned (H.266)", "unpinned").  Reference citations are path:line inside the
 * xin26x source tree.
 */
#include "xin_oracle.h"
#include <stdlib.h>
#include <string.h>

#define CLIP3(lo, hi, v) ((v) < (lo) ? (lo) : ((v) > (hi) ? (hi) : (v)))
#define IABS(v) ((v) < 0 ? -(v) : (v))

int orc_bitdepth(void) { return ORC_BITDEPTH; }

static inline opix clip_pix(int32_t v) { return (opix)CLIP3(0, ORC_MAX_PIX, v); }
static inline int32_t clip16(int32_t v) { return CLIP3(-32768, 32767, v); }
static inline uint32_t lg2u(uint32_t v) { uint32_t l = 0; while ((1u << l) < v) l++; return l; }

/* ======================================================================
 * Distortion.  The reference ships these only as a closed binary
 * (declarations h26x_core/include/h26x_compute_dist.h:27-1096).
 * ====================================================================== */

/* SAD: sum |in - ref| over w x h.  Unpinned but unambiguous (Xin26xComputeSad,
 * h26x_compute_dist.h:27). */
void orc_sad(const opix *in, intptr_t is, const opix *ref, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad)
{
    uint32_t s = 0;
    for (uint32_t y = 0; y < h; y++, in += is, ref += rs)
        for (uint32_t x = 0; x < w; x++) s += (uint32_t)IABS((int32_t)in[x] - (int32_t)ref[x]);
    *sad = s;
}

/* n SADs of one input against n references (Xin26xComputeSadx8/x5/x3,
 * h26x_compute_dist.h:400,482,625).  Unpinned, unambiguous. */
void orc_sad_xn(const opix *in, intptr_t is, const opix *const *ref, int n, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad)
{
    for (int i = 0; i < n; i++) orc_sad(in, is, ref[i], rs, w, h, sad + i);
}

/* bi-prediction average (a + b + 1) >> 1, the H.266 default-weight rounding.
 * Used by Xin26xComputeAvgSad/AvgSatd/AvgVar (h26x_compute_dist.h:153,880,1008).
 * Unpinned (closed). */
static inline int32_t avg2(int32_t a, int32_t b) { return (a + b + 1) >> 1; }

void orc_avg_sad(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad)
{
    uint32_t s = 0;
    for (uint32_t y = 0; y < h; y++, in += is, a += rs, b += rs)
        for (uint32_t x = 0; x < w; x++) s += (uint32_t)IABS((int32_t)in[x] - avg2(a[x], b[x]));
    *sad = s;
}

void orc_avg_sad_xn(const opix *in, intptr_t is, const opix *const *a, const opix *const *b, int n, intptr_t rs, uint32_t w, uint32_t h, uint32_t *sad)
{
    for (int i = 0; i < n; i++) orc_avg_sad(in, is, a[i], b[i], rs, w, h, sad + i);
}

/* BCW blend of two pixel predictions, weights in units of 1/8
 * (XIN_BCW_LOG_WGT_BASE = 3, h266_core/include/h266_constant.h:24):
 * clip((wa*a + wb*b + 4) >> 3).  Unpinned (closed Xin26xComputeWeightSad/Satd,
 * h26x_compute_dist.h:1048,1060). */
static inline int32_t wblend(int32_t a, int32_t b, int32_t wa, int32_t wb)
{
    return CLIP3(0, ORC_MAX_PIX, (wa * a + wb * b + 4) >> 3);
}

void orc_weight_sad(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, int32_t wa, int32_t wb, uint32_t *sad)
{
    uint32_t s = 0;
    for (uint32_t y = 0; y < h; y++, in += is, a += rs, b += rs)
        for (uint32_t x = 0; x < w; x++) s += (uint32_t)IABS((int32_t)in[x] - wblend(a[x], b[x], wa, wb));
    *sad = s;
}

/* Walsh-Hadamard SATD of a difference block.  Published method: HM's
 * TComRdCost::xCalcHADs4x4 / xCalcHADs8x8 -- sum of |H D H^T| over 4x4 tiles
 * normalised (S + 1) >> 1, over 8x8 tiles normalised (S + 2) >> 2; 8x8 tiles
 * when both sides are multiples of 8, else 4x4 tiles.  The sum of absolute
 * values does not depend on the butterfly order.  Unpinned (closed
 * Xin26xComputeSatd, h26x_compute_dist.h:806-936). */
static uint32_t had4(const int32_t *d, int ds)
{
    int32_t m[16], t[16];
    for (int r = 0; r < 4; r++) {
        const int32_t *p = d + r * ds;
        int32_t s01 = p[0] + p[1], d01 = p[0] - p[1], s23 = p[2] + p[3], d23 = p[2] - p[3];
        t[r * 4 + 0] = s01 + s23; t[r * 4 + 1] = s01 - s23; t[r * 4 + 2] = d01 + d23; t[r * 4 + 3] = d01 - d23;
    }
    for (int c = 0; c < 4; c++) {
        int32_t s01 = t[c] + t[4 + c], d01 = t[c] - t[4 + c], s23 = t[8 + c] + t[12 + c], d23 = t[8 + c] - t[12 + c];
        m[c] = s01 + s23; m[4 + c] = s01 - s23; m[8 + c] = d01 + d23; m[12 + c] = d01 - d23;
    }
    uint32_t s = 0;
    for (int i = 0; i < 16; i++) s += (uint32_t)IABS(m[i]);
    return s;
}

static uint32_t had8(const int32_t *d, int ds)
{
    int32_t t[64];
    for (int r = 0; r < 8; r++) {
        const int32_t *p = d + r * ds;
        int32_t a[8], b[8];
        for (int i = 0; i < 4; i++) { a[i] = p[i] + p[i + 4]; a[i + 4] = p[i] - p[i + 4]; }
        for (int g = 0; g < 8; g += 4) { b[g] = a[g] + a[g + 2]; b[g + 1] = a[g + 1] + a[g + 3]; b[g + 2] = a[g] - a[g + 2]; b[g + 3] = a[g + 1] - a[g + 3]; }
        for (int i = 0; i < 8; i += 2) { t[r * 8 + i] = b[i] + b[i + 1]; t[r * 8 + i + 1] = b[i] - b[i + 1]; }
    }
    uint32_t s = 0;
    for (int c = 0; c < 8; c++) {
        int32_t a[8], b[8];
        for (int i = 0; i < 4; i++) { a[i] = t[i * 8 + c] + t[(i + 4) * 8 + c]; a[i + 4] = t[i * 8 + c] - t[(i + 4) * 8 + c]; }
        for (int g = 0; g < 8; g += 4) { b[g] = a[g] + a[g + 2]; b[g + 1] = a[g + 1] + a[g + 3]; b[g + 2] = a[g] - a[g + 2]; b[g + 3] = a[g + 1] - a[g + 3]; }
        for (int i = 0; i < 8; i += 2) s += (uint32_t)IABS(b[i] + b[i + 1]) + (uint32_t)IABS(b[i] - b[i + 1]);
    }
    return s;
}

static uint32_t satd_of_diff(const int32_t *d, int ds, uint32_t w, uint32_t h)
{
    uint32_t s = 0;
    if ((w % 8) == 0 && (h % 8) == 0) {
        for (uint32_t y = 0; y < h; y += 8)
            for (uint32_t x = 0; x < w; x += 8) s += (had8(d + y * ds + x, ds) + 2) >> 2;
    } else {
        for (uint32_t y = 0; y < h; y += 4)
            for (uint32_t x = 0; x < w; x += 4) s += (had4(d + y * ds + x, ds) + 1) >> 1;
    }
    return s;
}

void orc_satd(const opix *in, intptr_t is, const opix *ref, intptr_t rs, uint32_t w, uint32_t h, uint32_t *satd)
{
    int32_t *d = (int32_t *)malloc(sizeof(int32_t) * w * h);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) d[y * w + x] = (int32_t)in[y * is + x] - (int32_t)ref[y * rs + x];
    *satd = satd_of_diff(d, (int)w, w, h);
    free(d);
}

void orc_avg_satd(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *satd)
{
    int32_t *d = (int32_t *)malloc(sizeof(int32_t) * w * h);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) d[y * w + x] = (int32_t)in[y * is + x] - avg2(a[y * rs + x], b[y * rs + x]);
    *satd = satd_of_diff(d, (int)w, w, h);
    free(d);
}

void orc_weight_satd(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, int32_t wa, int32_t wb, uint32_t *satd)
{
    int32_t *d = (int32_t *)malloc(sizeof(int32_t) * w * h);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) d[y * w + x] = (int32_t)in[y * is + x] - wblend(a[y * rs + x], b[y * rs + x], wa, wb);
    *satd = satd_of_diff(d, (int)w, w, h);
    free(d);
}

/* Hadamard activity of one 8x8 pixel block (no prediction), normalised like
 * the 8x8 SATD.  Unpinned (closed Xin26xComputeHada8x8, h26x_compute_dist.h:937). */
void orc_hada8x8(const opix *in, intptr_t is, uint32_t *satd)
{
    int32_t d[64];
    for (int y = 0; y < 8; y++) for (int x = 0; x < 8; x++) d[y * 8 + x] = in[y * is + x];
    *satd = (had8(d, 8) + 2) >> 2;
}

/* Variance of the difference in - pred: sum(d^2) - (sum d)^2 / (w*h), the
 * division done as a shift by log2(w*h) on the magnitude.  Unpinned (closed
 * Xin26xComputeVar/AvgVar, h26x_compute_dist.h:972,1008). */
static uint32_t var_of(int64_t s, int64_t s2, uint32_t w, uint32_t h)
{
    uint32_t lg = lg2u(w * h);
    int64_t mean2 = (s * s) >> lg;
    return (uint32_t)(s2 - mean2);
}

void orc_var(const opix *in, intptr_t is, const opix *ref, intptr_t rs, uint32_t w, uint32_t h, uint32_t *var)
{
    int64_t s = 0, s2 = 0;
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) { int32_t d = (int32_t)in[y * is + x] - (int32_t)ref[y * rs + x]; s += d; s2 += (int64_t)d * d; }
    *var = var_of(s, s2, w, h);
}

void orc_avg_var(const opix *in, intptr_t is, const opix *a, const opix *b, intptr_t rs, uint32_t w, uint32_t h, uint32_t *var)
{
    int64_t s = 0, s2 = 0;
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) { int32_t d = (int32_t)in[y * is + x] - avg2(a[y * rs + x], b[y * rs + x]); s += d; s2 += (int64_t)d * d; }
    *var = var_of(s, s2, w, h);
}

/* ======================================================================
 * Interpolation.  Pinned (open C): h266_core/source/h266_luma_mc.c and
 * h266_chroma_mc.c.  Filter taps are the H.266 normative tables; only the
 * first half of each table is written, the second half is the mirror image
 * (phase P = reverse of phase N - P), which is how the standard's tables are
 * built.
 * ====================================================================== */
#define IF_SHIFT 6                                   /* INTERP_SHIFT, h266_inter_pred_context.h:31 */
#define IF_PREC 14                                   /* INTERP_PRECISION, :37 */
#define IF_OFF14 (1 << (IF_PREC - 1))                /* INTERP_PREC_OFFSET, :38 */
#define IF_HEAD (IF_PREC - ORC_BITDEPTH > 2 ? IF_PREC - ORC_BITDEPTH : 2)  /* max(2, 14 - bd) */

static const int8_t luma_half[9][8] = {             /* H.266 luma 1/16 phases 0..8 */
    { 0, 0, 0, 64, 0, 0, 0, 0 }, { 0, 1, -3, 63, 4, -2, 1, 0 }, { -1, 2, -5, 62, 8, -3, 1, 0 },
    { -1, 3, -8, 60, 13, -4, 1, 0 }, { -1, 4, -10, 58, 17, -5, 1, 0 }, { -1, 4, -11, 52, 26, -8, 3, -1 },
    { -1, 3, -9, 47, 31, -10, 4, -1 }, { -1, 4, -11, 45, 34, -10, 4, -1 }, { -1, 4, -11, 40, 40, -11, 4, -1 } };
static const int8_t luma4x4_half[9][8] = {          /* H.266 affine 4x4 luma phases 0..8 */
    { 0, 0, 0, 64, 0, 0, 0, 0 }, { 0, 1, -3, 63, 4, -2, 1, 0 }, { 0, 1, -5, 62, 8, -3, 1, 0 },
    { 0, 2, -8, 60, 13, -4, 1, 0 }, { 0, 3, -10, 58, 17, -5, 1, 0 }, { 0, 3, -11, 52, 26, -8, 2, 0 },
    { 0, 2, -9, 47, 31, -10, 3, 0 }, { 0, 3, -11, 45, 34, -10, 3, 0 }, { 0, 3, -11, 40, 40, -11, 3, 0 } };
static const int8_t luma_alt_hpel[8] = { 0, 3, 9, 20, 20, 9, 3, 0 };  /* H.266 alternative half-pel */
static const int8_t chroma_half[17][4] = {          /* H.266 chroma 1/32 phases 0..16 */
    { 0, 64, 0, 0 }, { -1, 63, 2, 0 }, { -2, 62, 4, 0 }, { -2, 60, 7, -1 }, { -2, 58, 10, -2 },
    { -3, 57, 12, -2 }, { -4, 56, 14, -2 }, { -4, 55, 15, -2 }, { -4, 54, 16, -2 }, { -5, 53, 18, -2 },
    { -6, 52, 20, -2 }, { -6, 49, 24, -3 }, { -6, 46, 28, -4 }, { -5, 44, 29, -4 }, { -4, 42, 30, -4 },
    { -4, 39, 33, -4 }, { -4, 36, 36, -4 } };

/* fills taps[8] for a 1/16 luma phase and filterIndex (0 default, 1 alt half-pel, 2 affine 4x4),
 * following the selection at h266_luma_mc.c:117-128 */
static void luma_taps(int phase, uint32_t fi, int32_t *taps)
{
    if (fi == 1 && phase == 8) { for (int i = 0; i < 8; i++) taps[i] = luma_alt_hpel[i]; return; }
    const int8_t (*tab)[8] = (fi == 2) ? luma4x4_half : luma_half;
    if (phase <= 8) for (int i = 0; i < 8; i++) taps[i] = tab[phase][i];
    else for (int i = 0; i < 8; i++) taps[i] = tab[16 - phase][7 - i];
}

static void chroma_taps(int phase, int32_t *taps)
{
    if (phase <= 16) for (int i = 0; i < 4; i++) taps[i] = chroma_half[phase][i];
    else for (int i = 0; i < 4; i++) taps[i] = chroma_half[32 - phase][3 - i];
}

/* generic separable FIR pass: NT taps, input element type selected by the caller */
#define FIR_ROW(SRC, STEP, T, NT) ({ int32_t _s = 0; for (int _k = 0; _k < (NT); _k++) _s += (int32_t)(SRC)[_k * (STEP)] * (T)[_k]; _s; })

/* Copy (Xin266InterpCopy, h266_luma_mc.c:72) */
void orc_interp_copy(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{
    (void)frac; (void)fi;
    for (uint32_t y = 0; y < h; y++, src += ss, dst += ds) memcpy(dst, src, w * sizeof(opix));
}

/* Copy to the 14-bit intermediate: (p << max(2,14-bd)) - 8192 (Xin266InterpCopyU8S16, h266_luma_mc.c:430) */
void orc_interp_copy_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{
    (void)frac; (void)fi;
    for (uint32_t y = 0; y < h; y++, src += ss, dst += ds)
        for (uint32_t x = 0; x < w; x++) dst[x] = (int16_t)(((int32_t)src[x] << IF_HEAD) - IF_OFF14);
}

/* One-pass filter to pixels: clip((sum + 32) >> 6).  NT = 8 (luma) or 4 (chroma);
 * dir 0 = horizontal, 1 = vertical.  Xin266LumaInterpHor/Vet (h266_luma_mc.c:100,157),
 * Xin266ChromaInterpHor/Vet (h266_chroma_mc.c:62,99). */
static void fir_pix(const opix *src, intptr_t ss, opix *dst, intptr_t ds, const int32_t *t, int nt, int dir, uint32_t w, uint32_t h)
{
    intptr_t step = dir ? ss : 1;
    src -= (nt / 2 - 1) * step;
    for (uint32_t y = 0; y < h; y++, src += ss, dst += ds)
        for (uint32_t x = 0; x < w; x++) dst[x] = clip_pix((FIR_ROW(src + x, step, t, nt) + (1 << (IF_SHIFT - 1))) >> IF_SHIFT);
}

/* One-pass filter from pixels to the 14-bit intermediate: (sum - (8192 << s)) >> s,
 * s = 6 - max(2, 14 - bd).  Xin266LumaInterpHorU8S16 / VetU8S16 (h266_luma_mc.c:216,465). */
static void fir_pix_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, const int32_t *t, int nt, int dir, uint32_t w, uint32_t h)
{
    intptr_t step = dir ? ss : 1;
    int32_t shift = IF_SHIFT - IF_HEAD, offset = -IF_OFF14 * (1 << shift);
    src -= (nt / 2 - 1) * step;
    for (uint32_t y = 0; y < h; y++, src += ss, dst += ds)
        for (uint32_t x = 0; x < w; x++) dst[x] = (int16_t)((FIR_ROW(src + x, step, t, nt) + offset) >> shift);
}

/* Vertical pass from the intermediate to pixels: clip((sum + (1 << (s-1)) + (8192 << 6)) >> s),
 * s = 6 + max(2, 14 - bd).  Xin266LumaInterpVetS16U8 (h266_luma_mc.c:275). */
static void fir_s16_pix(const int16_t *src, intptr_t ss, opix *dst, intptr_t ds, const int32_t *t, int nt, uint32_t w, uint32_t h)
{
    int32_t shift = IF_SHIFT + IF_HEAD, offset = (1 << (shift - 1)) + (IF_OFF14 << IF_SHIFT);
    src -= (nt / 2 - 1) * ss;
    for (uint32_t y = 0; y < h; y++, src += ss, dst += ds)
        for (uint32_t x = 0; x < w; x++) dst[x] = clip_pix((FIR_ROW(src + x, ss, t, nt) + offset) >> shift);
}

/* Vertical pass intermediate -> intermediate: sum >> 6.  Xin266LumaInterpVetS16S16 (h266_luma_mc.c:338). */
static void fir_s16_s16(const int16_t *src, intptr_t ss, int16_t *dst, intptr_t ds, const int32_t *t, int nt, uint32_t w, uint32_t h)
{
    src -= (nt / 2 - 1) * ss;
    for (uint32_t y = 0; y < h; y++, src += ss, dst += ds)
        for (uint32_t x = 0; x < w; x++) dst[x] = (int16_t)(FIR_ROW(src + x, ss, t, nt) >> IF_SHIFT);
}

/* Two-pass HV: horizontal to the intermediate over h + nt - 1 rows, then vertical.
 * Xin266LumaInterpHorVet (h266_luma_mc.c:394), HorVetU8S16 (:525). */
static void fir_hv(const opix *src, intptr_t ss, void *dst, intptr_t ds, const int32_t *th, const int32_t *tv, int nt,
                   uint32_t w, uint32_t h, int to_s16)
{
    int16_t *tmp = (int16_t *)malloc(sizeof(int16_t) * w * (h + nt - 1));
    fir_pix_s16(src - (nt / 2 - 1) * ss, ss, tmp, w, th, nt, 0, w, h + nt - 1);
    if (to_s16) fir_s16_s16(tmp + (nt / 2 - 1) * w, w, (int16_t *)dst, ds, tv, nt, w, h);
    else fir_s16_pix(tmp + (nt / 2 - 1) * w, w, (opix *)dst, ds, tv, nt, w, h);
    free(tmp);
}

/* luma: horizontal phase = frac & 15 (h266_luma_mc.c:116), vertical phase = frac >> 4 (:173) */
void orc_luma_hor(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t t[8]; luma_taps(frac & 15, fi, t); fir_pix(src, ss, dst, ds, t, 8, 0, w, h); }
void orc_luma_vet(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t t[8]; luma_taps(frac >> 4, fi, t); fir_pix(src, ss, dst, ds, t, 8, 1, w, h); }
void orc_luma_hv(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t th[8], tv[8]; luma_taps(frac & 15, fi, th); luma_taps(frac >> 4, fi, tv); fir_hv(src, ss, dst, ds, th, tv, 8, w, h, 0); }
void orc_luma_hor_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t t[8]; luma_taps(frac & 15, fi, t); fir_pix_s16(src, ss, dst, ds, t, 8, 0, w, h); }
void orc_luma_vet_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t t[8]; luma_taps(frac >> 4, fi, t); fir_pix_s16(src, ss, dst, ds, t, 8, 1, w, h); }
void orc_luma_hv_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t th[8], tv[8]; luma_taps(frac & 15, fi, th); luma_taps(frac >> 4, fi, tv); fir_hv(src, ss, dst, ds, th, tv, 8, w, h, 1); }
void orc_luma_vet_s16_pix(const int16_t *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t t[8]; luma_taps(frac >> 4, fi, t); fir_s16_pix(src, ss, dst, ds, t, 8, w, h); }
void orc_luma_vet_s16_s16(const int16_t *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ int32_t t[8]; luma_taps(frac >> 4, fi, t); fir_s16_s16(src, ss, dst, ds, t, 8, w, h); }

/* chroma: horizontal phase = frac & 31 (h266_chroma_mc.c:72), vertical phase = frac >> 5 (:109) */
void orc_chroma_hor(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t t[4]; chroma_taps(frac & 31, t); fir_pix(src, ss, dst, ds, t, 4, 0, w, h); }
void orc_chroma_vet(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t t[4]; chroma_taps(frac >> 5, t); fir_pix(src, ss, dst, ds, t, 4, 1, w, h); }
void orc_chroma_hv(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t th[4], tv[4]; chroma_taps(frac & 31, th); chroma_taps(frac >> 5, tv); fir_hv(src, ss, dst, ds, th, tv, 4, w, h, 0); }
void orc_chroma_hor_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t t[4]; chroma_taps(frac & 31, t); fir_pix_s16(src, ss, dst, ds, t, 4, 0, w, h); }
void orc_chroma_vet_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t t[4]; chroma_taps(frac >> 5, t); fir_pix_s16(src, ss, dst, ds, t, 4, 1, w, h); }
void orc_chroma_hv_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t th[4], tv[4]; chroma_taps(frac & 31, th); chroma_taps(frac >> 5, tv); fir_hv(src, ss, dst, ds, th, tv, 4, w, h, 1); }
void orc_chroma_vet_s16_pix(const int16_t *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t t[4]; chroma_taps(frac >> 5, t); fir_s16_pix(src, ss, dst, ds, t, 4, w, h); }
void orc_chroma_vet_s16_s16(const int16_t *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h, uint32_t fi)
{ (void)fi; int32_t t[4]; chroma_taps(frac >> 5, t); fir_s16_s16(src, ss, dst, ds, t, 4, w, h); }

/* bi average of two intermediates: clip((a + b + (1 << (s-1)) + 2*8192) >> s), s = max(2,14-bd) + 1
 * (Xin266InterpAvgS16U8, h266_luma_mc.c:561) */
void orc_interp_avg(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, opix *dst, intptr_t ds, uint32_t w, uint32_t h)
{
    int32_t shift = IF_HEAD + 1, offset = (1 << (shift - 1)) + 2 * IF_OFF14;
    for (uint32_t y = 0; y < h; y++, a += as, b += bs, dst += ds)
        for (uint32_t x = 0; x < w; x++) dst[x] = clip_pix(((int32_t)a[x] + b[x] + offset) >> shift);
}

/* BCW blend of two intermediates: clip((a*wa + b*wb + (1 << (s-1)) + (8192 << 3)) >> s),
 * s = max(2,14-bd) + 3 (Xin266InterpWeightS16U8, h266_luma_mc.c:595) */
void orc_interp_weight(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, opix *dst, intptr_t ds, uint32_t w, uint32_t h, int32_t wa, int32_t wb)
{
    int32_t shift = IF_HEAD + 3, offset = (1 << (shift - 1)) + (IF_OFF14 << 3);
    for (uint32_t y = 0; y < h; y++, a += as, b += bs, dst += ds)
        for (uint32_t x = 0; x < w; x++) dst[x] = clip_pix(((int32_t)a[x] * wa + (int32_t)b[x] * wb + offset) >> shift);
}

/* Bilinear DMVR prediction (h266_core/source/h266_bilinear_filter.c:46-260), pinned (open C):
 * two taps {16 - f, f} at 1/16 pel into a 10-bit intermediate; every form
 * writes h rows of w + 4 (DMVR_PADING_SIZE) samples.  variant 0 copy, 1 H, 2 V,
 * 3 H over h + 1 rows (16-bit) then V with (+8) >> 4. */
void orc_bili_interp(int variant, const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h)
{
    int fx = frac & 15, fy = frac >> 4, sh = ORC_BITDEPTH - 6, off = 1 << (sh - 1);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w + 4; x++) {
            const opix *p = src + (intptr_t)y * ss + x;
            int v;
            if (variant == 0) v = (int)p[0] << (10 - ORC_BITDEPTH);
            else if (variant == 1) v = ((int)p[0] * (16 - fx) + (int)p[1] * fx + off) >> sh;
            else if (variant == 2) v = ((int)p[0] * (16 - fy) + (int)p[ss] * fy + off) >> sh;
            else {
                int a = (int16_t)(((int)p[0] * (16 - fx) + (int)p[1] * fx + off) >> sh);
                int b = (int16_t)(((int)p[ss] * (16 - fx) + (int)p[ss + 1] * fx + off) >> sh);
                v = (a * (16 - fy) + b * fy + 8) >> 4;
            }
            dst[(intptr_t)y * ds + x] = (int16_t)v;
        }
}

/* Table dispatch pfXinLumaInterp[!!fx][!!fy][lgW] (h266_encoder/source/h266_inter_prediction.c:143-169).
 * The 8-argument form is the one h266_sub_pel_refine.c calls through the header
 * h266_encoder/include/h266_inter_prediction.h:43; the filter index is the
 * caller's (0 in that call path). */
void orc_luma_interpolation(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t lgw, uint32_t h, uint32_t fi)
{
    int fx = frac & 15, fy = (frac >> 4) & 15;
    uint32_t w = 1u << lgw;
    if (!fx && !fy) orc_interp_copy(src, ss, dst, ds, frac, w, h, fi);
    else if (fx && !fy) orc_luma_hor(src, ss, dst, ds, frac, w, h, fi);
    else if (!fx && fy) orc_luma_vet(src, ss, dst, ds, frac, w, h, fi);
    else orc_luma_hv(src, ss, dst, ds, frac, w, h, fi);
}

/* h266_inter_prediction.c:171 Xin266ChromaInterpolation (frac = fy << 5 | fx) */
void orc_chroma_interpolation(const opix *src, intptr_t ss, opix *dst, intptr_t ds, int32_t frac, uint32_t lgw, uint32_t h)
{
    uint32_t w = 1u << lgw;
    if (!frac) orc_interp_copy(src, ss, dst, ds, frac, w, h, 0);
    else if (!(frac & (31 << 5))) orc_chroma_hor(src, ss, dst, ds, frac, w, h, 0);
    else if (!(frac & 31)) orc_chroma_vet(src, ss, dst, ds, frac, w, h, 0);
    else orc_chroma_hv(src, ss, dst, ds, frac, w, h, 0);
}

/* Xin266LumaInterPred (h266_inter_prediction.c:302-351): clamp the 1/16-pel MV to the
 * CU's window, split into integer offset and phase, dispatch. */
void orc_luma_inter_pred(const opix *ref_origin, intptr_t rs, opix *pred, intptr_t ps, int32_t mvx16, int32_t mvy16,
                         int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                         uint32_t w, uint32_t h, uint32_t fi)
{
    int32_t mvx = CLIP3(min_mvx * 16, max_mvx * 16, mvx16), mvy = CLIP3(min_mvy * 16, max_mvy * 16, mvy16);
    int32_t ox = cu_x * 16 + mvx, oy = cu_y * 16 + mvy;
    int32_t frac = ((oy & 15) << 4) + (ox & 15);
    orc_luma_interpolation(ref_origin + (intptr_t)(oy >> 4) * rs + (ox >> 4), rs, pred, ps, frac, lg2u(w), h, fi);
}

/* Uni-prediction branch of Xin266ChromaMotionComp (h266_inter_prediction.c:784-818):
 * chroma phase is the 1/32 remainder (mask 31) of the luma 1/16 position. */
void orc_chroma_motion_comp(const opix *ref_origin, intptr_t rs, opix *pred, intptr_t ps, int32_t mvx16, int32_t mvy16,
                            int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                            uint32_t w, uint32_t h)
{
    int32_t mvx = CLIP3(min_mvx * 16, max_mvx * 16, mvx16), mvy = CLIP3(min_mvy * 16, max_mvy * 16, mvy16);
    int32_t ox = cu_x * 16 + mvx, oy = cu_y * 16 + mvy;
    int32_t fx = ox & 31, fy = oy & 31, frac = (fy << 5) + fx;
    const opix *src = ref_origin + (intptr_t)(oy >> 5) * rs + (ox >> 5);
    uint32_t cw = w >> 1, ch = h >> 1;
    if (!fx && !fy) orc_interp_copy(src, rs, pred, ps, frac, cw, ch, 0);
    else if (fx && !fy) orc_chroma_hor(src, rs, pred, ps, frac, cw, ch, 0);
    else if (!fx && fy) orc_chroma_vet(src, rs, pred, ps, frac, cw, ch, 0);
    else orc_chroma_hv(src, rs, pred, ps, frac, cw, ch, 0);
}

/* Bi-prediction branch of Xin266LumaMotionComp (h266_inter_prediction.c:473-552):
 * each list's 1/16-pel MV clamped to the window, its 14-bit intermediate
 * prediction (pfXinLumaInterpS16 by phase), then Xin266InterpAvgS16U8. */
void orc_luma_motion_comp_bi(const opix *ref0, const opix *ref1, intptr_t rs, opix *pred, intptr_t ps, const int32_t *mv16,
                             int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                             uint32_t w, uint32_t h)
{
    int16_t *b[2];
    for (int l = 0; l < 2; l++) {
        b[l] = (int16_t *)malloc(sizeof(int16_t) * w * h);
        int32_t mvx = CLIP3(min_mvx * 16, max_mvx * 16, mv16[2 * l]), mvy = CLIP3(min_mvy * 16, max_mvy * 16, mv16[2 * l + 1]);
        int32_t ox = cu_x * 16 + mvx, oy = cu_y * 16 + mvy, fx = ox & 15, fy = oy & 15, frac = (fy << 4) + fx;
        const opix *src = (l ? ref1 : ref0) + (intptr_t)(oy >> 4) * rs + (ox >> 4);
        if (!fx && !fy) orc_interp_copy_s16(src, rs, b[l], w, frac, w, h, 0);
        else if (fx && !fy) orc_luma_hor_s16(src, rs, b[l], w, frac, w, h, 0);
        else if (!fx && fy) orc_luma_vet_s16(src, rs, b[l], w, frac, w, h, 0);
        else orc_luma_hv_s16(src, rs, b[l], w, frac, w, h, 0);
    }
    orc_interp_avg(b[0], w, b[1], w, pred, ps, w, h);
    free(b[0]); free(b[1]);
}

/* Bi-prediction branch of Xin266ChromaMotionComp (h266_inter_prediction.c:658-755):
 * the 1/32 chroma phase (mask 31) of each list, the 14-bit intermediate
 * (pfXinChromaInterpS16), then Xin266InterpAvgS16U8 over the (w/2) x (h/2) block. */
void orc_chroma_motion_comp_bi(const opix *ref0, const opix *ref1, intptr_t rs, opix *pred, intptr_t ps, const int32_t *mv16,
                               int32_t cu_x, int32_t cu_y, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                               uint32_t w, uint32_t h)
{
    uint32_t cw = w >> 1, ch = h >> 1;
    int16_t *b[2];
    for (int l = 0; l < 2; l++) {
        b[l] = (int16_t *)malloc(sizeof(int16_t) * cw * ch);
        int32_t mvx = CLIP3(min_mvx * 16, max_mvx * 16, mv16[2 * l]), mvy = CLIP3(min_mvy * 16, max_mvy * 16, mv16[2 * l + 1]);
        int32_t ox = cu_x * 16 + mvx, oy = cu_y * 16 + mvy, fx = ox & 31, fy = oy & 31, frac = (fy << 5) + fx;
        const opix *src = (l ? ref1 : ref0) + (intptr_t)(oy >> 5) * rs + (ox >> 5);
        if (!fx && !fy) orc_interp_copy_s16(src, rs, b[l], cw, frac, cw, ch, 0);
        else if (fx && !fy) orc_chroma_hor_s16(src, rs, b[l], cw, frac, cw, ch, 0);
        else if (!fx && fy) orc_chroma_vet_s16(src, rs, b[l], cw, frac, cw, ch, 0);
        else orc_chroma_hv_s16(src, rs, b[l], cw, frac, cw, ch, 0);
    }
    orc_interp_avg(b[0], cw, b[1], cw, pred, ps, cw, ch);
    free(b[0]); free(b[1]);
}

/* Target of the bi refinement, clip(2 in - pred).  The default-weight
 * constructor (Xin26xConstructBiMeInput) is closed; the open weighted form
 * Xin266ConstructWeightBiMeInput (h266_construct_weight_input.c:24-58) at the
 * default weight 4 of 8 computes (8192 in - 4096 pred + 2048) >> 12, which is
 * 2 in - pred exactly, clipped to the sample range. */
void orc_bi_me_input(const opix *in, intptr_t is, const opix *pred, intptr_t ps, opix *out, intptr_t os, uint32_t w, uint32_t h)
{
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) out[y * os + x] = clip_pix(2 * (int32_t)in[y * is + x] - (int32_t)pred[y * ps + x]);
}

/* ======================================================================
 * Transforms.
 * Matrices: H.266 clause 8.7.4.5 transMatrix (DCT-II up to 64 points) and the
 * DST-VII / DCT-VIII matrices for 4..32 points.  They are generated here from
 * the standard's unique coefficient magnitudes and the trigonometric sign /
 * index structure of each transform:
 *   DCT-II : T64[k][n] = g(k*(2n+1) mod 256), g(m) ~ 64*sqrt(2)*cos(m*pi/128),
 *            row 0 = 64, and the N-point matrix is rows 0, 64/N, 2*64/N ... of T64.
 *   DST-VII: T[k][n] = a((2k+1)(n+1)), a(m) ~ sin(m*pi/(2N+1)) with period 2(2N+1).
 *   DCT-VIII: T[k][n] = (-1)^k * DST-VII[k][N-1-n].
 * The 1-D routines (closed in the reference, h26x_core/include/h26x_forward_1d_trans.h,
 * h26x_inverse_1d_trans.h) follow the reference's call contract read from the open
 * 2-D wrappers h266_encoder/source/h266_forward_trans.c:100-151 and
 * h266_inverse_trans.c:52-88,184-229:
 *   forward: line i of input (stride is) -> out[k*os + i]   (transposing)
 *   inverse: column j: coefficients in[k*is + j] -> out[j*os + n] (transposing);
 *            the last skip_line lines are not transformed and come out zero.
 * Rounding (x + 2^(s-1)) >> s.  Forward outputs saturate to 16 bits (unpinned);
 * inverse outputs clip to 16 bits after each stage (H.266 8.7.4.1 intermediate clip).
 * ====================================================================== */
static const uint8_t dct2_c64[65] = {
    /* m = 0..64 : magnitude for angle m*pi/128 (m = 0 only reached by row 0) */
    64, 91, 90, 90, 90, 90, 90, 90, 89, 88, 88, 87, 87, 86, 85, 84,
    83, 83, 82, 81, 80, 79, 78, 77, 75, 73, 73, 71, 70, 69, 67, 65,
    64, 62, 61, 59, 57, 56, 54, 52, 50, 48, 46, 44, 43, 41, 38, 37,
    36, 33, 31, 28, 25, 24, 22, 20, 18, 15, 13, 11, 9, 7, 4, 2, 0 };
static const uint8_t dst7_a4[4]  = { 29, 55, 74, 84 };
static const uint8_t dst7_a8[8]  = { 17, 32, 46, 60, 71, 78, 85, 86 };
static const uint8_t dst7_a16[16] = { 8, 17, 25, 33, 40, 48, 55, 62, 68, 73, 77, 81, 85, 87, 88, 88 };
static const uint8_t dst7_a32[32] = { 4, 9, 13, 17, 21, 26, 30, 34, 38, 42, 46, 50, 53, 56, 60, 63,
                                      66, 68, 72, 74, 77, 78, 80, 82, 84, 85, 86, 88, 88, 89, 90, 90 };

static int16_t mat_dct2[7][64 * 64];   /* index lg 1..6 */
static int16_t mat_dst7[6][32 * 32];   /* index lg 2..5 */
static int16_t mat_dct8[6][32 * 32];
static int mats_ready = 0;

static int dct2_g(int m)
{
    m &= 255;
    if (m <= 64) return dct2_c64[m];
    if (m <= 128) return -dct2_c64[128 - m];
    if (m <= 192) return -dct2_c64[m - 128];
    return dct2_c64[256 - m];
}

static void build_mats(void)
{
    if (mats_ready) return;
    for (int lg = 1; lg <= 6; lg++) {
        int n = 1 << lg, step = 64 / n;
        for (int k = 0; k < n; k++)
            for (int i = 0; i < n; i++) {
                int kk = k * step;
                mat_dct2[lg][k * n + i] = (int16_t)(kk == 0 ? 64 : dct2_g(kk * (2 * i + 1)));
            }
    }
    for (int lg = 2; lg <= 5; lg++) {
        int n = 1 << lg, period = 2 * (2 * n + 1);
        const uint8_t *a = lg == 2 ? dst7_a4 : lg == 3 ? dst7_a8 : lg == 4 ? dst7_a16 : dst7_a32;
        for (int k = 0; k < n; k++)
            for (int i = 0; i < n; i++) {
                int m = ((2 * k + 1) * (i + 1)) % period, v;
                int half = 2 * n + 1;
                if (m == 0 || m == half) v = 0;
                else if (m < half) v = a[(m <= n ? m : half - m) - 1];
                else { int mm = m - half; v = -a[(mm <= n ? mm : half - mm) - 1]; }
                mat_dst7[lg][k * n + i] = (int16_t)v;
            }
        for (int k = 0; k < n; k++)
            for (int i = 0; i < n; i++)
                mat_dct8[lg][k * n + i] = (int16_t)((k & 1 ? -1 : 1) * mat_dst7[lg][k * n + (n - 1 - i)]);
    }
    mats_ready = 1;
}

/* type: 0 DCT2, 1 DCT8, 2 DST7 (XIN_DCT2/DCT8/DST7, h26x_core/include/h26x_trans_context.h:33-40) */
const int16_t *orc_tr_matrix(int type, int n)
{
    build_mats();
    int lg = (int)lg2u((uint32_t)n);
    if (type == 0 && lg >= 1 && lg <= 6) return mat_dct2[lg];
    if (type == 1 && lg >= 2 && lg <= 5) return mat_dct8[lg];
    if (type == 2 && lg >= 2 && lg <= 5) return mat_dst7[lg];
    return NULL;
}

static inline int32_t rshift_rnd(int32_t v, int32_t s) { return s > 0 ? (v + (1 << (s - 1))) >> s : v; }

void orc_fdct1d(int type, int lg, const ocoef *in, intptr_t is, ocoef *out, intptr_t os, int32_t line, int32_t shift)
{
    int n = 1 << lg;
    const int16_t *m = orc_tr_matrix(type, n);
    for (int i = 0; i < line; i++)
        for (int k = 0; k < n; k++) {
            int32_t s = 0;
            for (int j = 0; j < n; j++) s += (int32_t)m[k * n + j] * (int32_t)in[i * is + j];
            out[k * os + i] = (ocoef)clip16(rshift_rnd(s, shift));
        }
}

void orc_idct1d(int type, int lg, const ocoef *in, intptr_t is, ocoef *out, intptr_t os, int32_t line, int32_t skip_line, int32_t shift)
{
    int n = 1 << lg;
    const int16_t *m = orc_tr_matrix(type, n);
    for (int j = 0; j < line; j++)
        for (int x = 0; x < n; x++) {
            int32_t s = 0;
            if (j < line - skip_line)
                for (int k = 0; k < n; k++) s += (int32_t)m[k * n + x] * (int32_t)in[k * is + j];
            out[j * os + x] = (ocoef)(j < line - skip_line ? clip16(rshift_rnd(s, shift)) : 0);
        }
}

/* Xin26xFDct2WxH (closed, h26x_core/include/h26x_forward_2d_trans.h): rows then columns
 * through a transposed temporary, the same composition Xin266FDctWxH uses for the
 * separable types (h266_forward_trans.c:112-128).  Unpinned. */
void orc_fdct2_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h, int32_t s1, int32_t s2)
{
    ocoef *tmp = (ocoef *)malloc(sizeof(ocoef) * w * h);
    orc_fdct1d(0, (int)lg2u(w), in, is, tmp, h, (int32_t)h, s1);
    orc_fdct1d(0, (int)lg2u(h), tmp, h, out, os, (int32_t)w, s2);
    free(tmp);
}

/* Xin266IDct2WxH (open, h266_inverse_trans.c:52-88): columns first with the zero-out
 * skip of lines beyond 32, then rows. */
void orc_idct2_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h, int32_t s1, int32_t s2)
{
    ocoef *tmp = (ocoef *)malloc(sizeof(ocoef) * w * h);
    int32_t skip = w > 32 ? (int32_t)w - 32 : 0;
    orc_idct1d(0, (int)lg2u(h), in, is, tmp, h, (int32_t)w, skip, s1);
    orc_idct1d(0, (int)lg2u(w), tmp, h, out, os, (int32_t)h, 0, s2);
    free(tmp);
}

/* Forward transform skip: r << (15 - bd - (lgW + lgH)/2) (H.266 transform-skip scaling,
 * mirror of the open inverse Xin266ISkipWxH).  Unpinned (closed Xin26xFSkipWxH). */
void orc_fskip_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h)
{
    int32_t sh = 15 - ORC_BITDEPTH - (int32_t)((lg2u(w) + lg2u(h)) >> 1);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) {
            int32_t v = in[y * is + x];
            out[y * os + x] = (ocoef)clip16(sh >= 0 ? v * (1 << sh) : rshift_rnd(v, -sh));
        }
}

/* Xin266ISkipWxH (open, h266_inverse_trans.c:91-115): v >> (15 - 8 - (lgW+lgH)/2), truncated to 16 bits. */
void orc_iskip_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h)
{
    int32_t sh = 15 - 8 - (int32_t)((lg2u(w) + lg2u(h)) >> 1);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) out[y * os + x] = (ocoef)(int16_t)((int32_t)in[y * is + x] >> sh);
}

/* MTS index -> (horizontal, vertical) type; XIN_MTS_* order at
 * h26x_core/include/h26x_trans_context.h:42-51 (1 = transform skip, coded as 4). */
static const int8_t mts_tx[6][2] = { { 0, 0 }, { 4, 4 }, { 2, 2 }, { 1, 2 }, { 2, 1 }, { 1, 1 } };

/* Xin266FDctWxH (open, h266_forward_trans.c:45-151) */
void orc_fdct_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t comp, uint32_t w, uint32_t h,
                  uint32_t mts, int is_intra, int enable_mts)
{
    int hor = mts_tx[mts][0], ver = mts_tx[mts][1];
    int lgw = (int)lg2u(w), lgh = (int)lg2u(h);
    int32_t s1 = lgw + ORC_BITDEPTH + 6 - 15, s2 = lgh + 6;
    if (is_intra && comp == 0 && enable_mts && mts == 0) {
        if (w >= 4 && w <= 16) hor = 2;
        if (h >= 4 && h <= 16) ver = 2;
    }
    if (lgw > 0 && lgh > 0 && hor == 0 && ver == 0) { orc_fdct2_wxh(in, is, out, os, w, h, s1, s2); return; }
    if (hor == 4) { orc_fskip_wxh(in, is, out, os, w, h); return; }
    if (lgw > 0 && lgh > 0) {
        ocoef *tmp = (ocoef *)malloc(sizeof(ocoef) * w * h);
        orc_fdct1d(hor, lgw, in, is, tmp, h, (int32_t)h, s1);
        orc_fdct1d(ver, lgh, tmp, h, out, os, (int32_t)w, s2);
        free(tmp);
    } else if (lgw > 0) orc_fdct1d(hor, lgw, in, is, out, os, (int32_t)h, s1);
    else orc_fdct1d(ver, lgh, in, is, out, os, (int32_t)w, s2);
}

/* Xin266IDctWxH (open, h266_inverse_trans.c:117-229).  The two degenerate 1-D branches
 * write into the reference's scratch buffer and leave the output untouched; here the
 * same result goes to the scratch and the output is left untouched too. */
void orc_idct_wxh(const ocoef *in, intptr_t is, ocoef *out, intptr_t os, uint32_t w, uint32_t h,
                  int is_intra, uint32_t comp, uint32_t mts, int enable_mts)
{
    int hor = mts_tx[mts][0], ver = mts_tx[mts][1];
    int lgw = (int)lg2u(w), lgh = (int)lg2u(h);
    int32_t s1 = 6 + 1, s2 = 6 + 15 - 1 - ORC_BITDEPTH;
    int32_t skip = (hor != 0 && w == 32) ? 16 : (w > 32 ? (int32_t)w - 32 : 0);
    if (is_intra && comp == 0 && enable_mts && mts == 0) {
        if (w >= 4 && w <= 16) hor = 2;
        if (h >= 4 && h <= 16) ver = 2;
    }
    if (lgw > 0 && lgh > 0 && hor == 0 && ver == 0) { orc_idct2_wxh(in, is, out, os, w, h, s1, s2); return; }
    if (hor == 4) { orc_iskip_wxh(in, is, out, os, w, h); return; }
    if (lgw > 0 && lgh > 0) {
        ocoef *tmp = (ocoef *)malloc(sizeof(ocoef) * w * h);
        orc_idct1d(ver, lgh, in, is, tmp, h, (int32_t)w, skip, s1);
        orc_idct1d(hor, lgw, tmp, h, out, os, (int32_t)h, 0, s2);
        free(tmp);
    }
}

/* residual = input - prediction (closed Xin26xBlockSubForDct, h26x_core/include/h26x_block_utility.h).
 * Unpinned, unambiguous. */
void orc_block_sub(const opix *in, intptr_t is, const opix *pred, intptr_t ps, ocoef *diff, intptr_t ds, uint32_t w, uint32_t h)
{
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) diff[y * ds + x] = (ocoef)((int32_t)in[y * is + x] - (int32_t)pred[y * ps + x]);
}

/* recon = clip(pred + residual) (closed Xin26xBlockRecon via pfXinBlockAddForDct,
 * h266_idct_add.c:94).  Unpinned, unambiguous. */
void orc_block_add(const ocoef *res, intptr_t rs, const opix *pred, intptr_t ps, opix *rec, intptr_t os, uint32_t w, uint32_t h)
{
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) rec[y * os + x] = clip_pix((int32_t)pred[y * ps + x] + (int32_t)res[y * rs + x]);
}

/* Xin266SubFDctWxH (open, h266_sub_dct.c:47-107), LMCS chroma scaling off */
void orc_sub_fdct_wxh(const opix *in, intptr_t is, const opix *pred, intptr_t ps, ocoef *out, intptr_t os,
                      uint32_t comp, uint32_t mts, int32_t w, int32_t h, int is_intra, int enable_mts)
{
    ocoef *res = (ocoef *)malloc(sizeof(ocoef) * (size_t)(w * h));
    orc_block_sub(in, is, pred, ps, res, w, (uint32_t)w, (uint32_t)h);
    orc_fdct_wxh(res, w, out, os, comp, (uint32_t)w, (uint32_t)h, mts, is_intra, enable_mts);
    free(res);
}

/* Xin266IDctAdd (open, h266_idct_add.c:45-105), LMCS chroma scaling off */
void orc_idct_add(const ocoef *in, intptr_t is, const opix *pred, intptr_t ps, opix *out, intptr_t os,
                  int is_intra, uint32_t comp, uint32_t mts, uint32_t w, uint32_t h, int enable_mts)
{
    ocoef *buf = (ocoef *)calloc(64 * 64, sizeof(ocoef));
    orc_idct_wxh(in, is, buf, 64, w, h, is_intra, comp, mts, enable_mts);
    orc_block_add(buf, 64, pred, ps, out, os, w, h);
    free(buf);
}

/* ======================================================================
 * Quantisation.  Pinned (open C).
 * ====================================================================== */

/* Xin266QuantInvQuant + Xin266QIQCodingGroup (h266_quant_inv_quant.c:27-139):
 * coding groups visited from the last (bottom-right) to the first in raster order;
 * bit 0 of the map is CG 0 (raster), i.e. bit b <-> CG b. */
void orc_quant_inv_quant(ocoef *q, const ocoef *t, ocoef *r, intptr_t stride, uint32_t w, uint32_t h,
                         uint32_t cgw, uint32_t cgh, int32_t qmult, int32_t qadd, int32_t qshift,
                         int32_t iqmult, int32_t iqadd, int32_t iqshift, uint64_t *nz)
{
    uint32_t wcg = w / cgw, hcg = h / cgh;
    uint64_t map = 0;
    for (int by = (int)hcg - 1; by >= 0; by--)
        for (int bx = (int)wcg - 1; bx >= 0; bx--) {
            int any = 0;
            for (uint32_t y = 0; y < cgh; y++)
                for (uint32_t x = 0; x < cgw; x++) {
                    intptr_t p = (intptr_t)(by * (int)cgh + (int)y) * stride + bx * (int)cgw + (int)x;
                    int32_t tv = t[p], a = IABS(tv);
                    int32_t qv = (int32_t)(((int64_t)a * qmult + qadd) >> qshift);
                    qv = CLIP3(-32768, 32767, tv < 0 ? -qv : qv);
                    q[p] = (ocoef)qv;
                    int32_t rv = (int32_t)(((int64_t)qv * iqmult + iqadd) >> iqshift);
                    r[p] = (ocoef)CLIP3(-32768, 32767, rv);
                    any |= qv != 0;
                }
            map = (map << 1) | (uint64_t)any;
        }
    *nz = map;
}

/* Xin266PreRdoq (h266_quant_inv_quant.c:208-288): walking the CG scan backwards,
 * zero each non-zero CG whose |t| are all <= thr, stop at the first that is not. */
void orc_pre_rdoq(const ocoef *t, ocoef *r, ocoef *q, intptr_t stride, uint32_t w, uint32_t h,
                  uint32_t cgw, uint32_t cgh, int32_t thr, const orc_scan_pos *scan_cg, uint64_t *nz)
{
    int32_t nblk = (int32_t)(w * h / (cgw * cgh)), wcg = (int32_t)(w / cgw);
    uint64_t map = *nz;
    for (int32_t i = nblk - 1; i >= 1; i--) {
        uint32_t pos = scan_cg[i].posIdx;
        if (!(map & ((uint64_t)1 << pos))) continue;
        int32_t by = (int32_t)pos / wcg, bx = (int32_t)pos - by * wcg;
        int big = 0;
        for (uint32_t y = 0; y < cgh; y++)
            for (uint32_t x = 0; x < 4; x++) {
                int32_t v = t[(by * (int32_t)cgh + (int32_t)y) * stride + bx * (int32_t)cgw + (int32_t)x];
                big |= IABS(v) > thr;
            }
        if (big) break;
        for (uint32_t y = 0; y < 4; y++)
            for (uint32_t x = 0; x < cgw; x++) {
                intptr_t p = (intptr_t)(by * (int32_t)cgh + (int32_t)y) * stride + bx * (int32_t)cgw + (int32_t)x;
                r[p] = 0; q[p] = 0;
            }
        map &= ~((uint64_t)1 << pos);
    }
    *nz = map;
}

/* Quant parameters of one TU.  qMult/iqMult tables and shift bases from
 * Xin266ConstructQuantParam (h266_encoder_create.c:94-105,1677-1707); the per-TU
 * adjustment, qAdd and iqAdd from Xin266Transform (h266_trans_quant.c:107-120).
 * qp is the slice QP; the 10-bit build adds XIN_QP_SHIFT = 12 like :101. */
void orc_quant_params(int32_t qp, uint32_t lgw, uint32_t lgh, uint32_t mts, int rdoq, int intra_frame, orc_qparams *p)
{
    static const int32_t qm[2][6] = { { 26214, 23302, 20560, 18396, 16384, 14564 }, { 18396, 16384, 14564, 13107, 11651, 10280 } };
    static const int32_t iqm[2][6] = { { 40, 45, 51, 57, 64, 72 }, { 57, 64, 72, 80, 90, 102 } };
    if (ORC_BITDEPTH == 10) qp += 12;
    uint32_t lgt = lgw + lgh;
    int adj = (int)(lgt & 1) && mts != 1;
    int32_t lgs = (int32_t)(lgt >> 1);
    int32_t per = qp / 6, rem = qp % 6;
    p->qmult = qm[adj][rem];
    p->iqmult = iqm[adj][rem] << per;
    p->qshift = 14 + (15 - ORC_BITDEPTH) + per - lgs - adj;
    p->iqshift = 6 - (15 - ORC_BITDEPTH) + lgs + adj;
    p->qadd = (rdoq && mts != 1) ? (1 << (p->qshift - 1)) : ((intra_frame ? 171 : 85) << (p->qshift - 9));
    p->iqadd = (mts != 1) ? (1 << (p->iqshift - 1)) : (1 << ((p->iqshift - lgs) + (15 - ORC_BITDEPTH) - 1));
}

/* One TU of Xin266Transform without dependent quantisation and without the
 * pre-RDOQ pass (h266_trans_quant.c:131-220): residual + forward transform into t,
 * zero-out of r beyond 32, quant/dequant over the low min(w,32) x min(h,32) part
 * with 4x4 coding groups.  Output strides are cs. */
void orc_transform_tu(const opix *in, intptr_t is, const opix *pred, intptr_t ps,
                      ocoef *t, ocoef *q, ocoef *r, intptr_t cs, uint32_t w, uint32_t h, uint32_t comp,
                      uint32_t mts, int32_t qp, int rdoq, int intra_frame, int is_intra, int enable_mts, uint64_t *nz)
{
    orc_qparams p;
    orc_quant_params(qp, lg2u(w), lg2u(h), mts, rdoq, intra_frame, &p);
    orc_sub_fdct_wxh(in, is, pred, ps, t, cs, comp, mts, (int32_t)w, (int32_t)h, is_intra, enable_mts);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++)
            if (x >= 32 || y >= 32) { r[y * cs + x] = 0; q[y * cs + x] = 0; }
    orc_quant_inv_quant(q, t, r, cs, w < 32 ? w : 32, h < 32 ? h : 32, 4, 4, p.qmult, p.qadd, p.qshift,
                        p.iqmult, p.iqadd, p.iqshift, nz);
}

void orc_tq_block(const ocoef *res, intptr_t rs, uint32_t w, uint32_t h, uint32_t comp, uint32_t mts, int32_t qp,
                  int rdoq, int intra_frame, int is_intra, int enable_mts,
                  ocoef *q, ocoef *r, ocoef *res_out, intptr_t os, uint64_t *nz)
{
    orc_qparams p;
    ocoef *t = (ocoef *)malloc(sizeof(ocoef) * w * h);
    orc_quant_params(qp, lg2u(w), lg2u(h), mts, rdoq, intra_frame, &p);
    orc_fdct_wxh(res, rs, t, w, comp, w, h, mts, is_intra, enable_mts);
    for (uint32_t y = 0; y < h; y++)
        for (uint32_t x = 0; x < w; x++) { q[y * os + x] = 0; r[y * os + x] = 0; }
    {   /* quant over the low part with the outputs' stride */
        ocoef *tq = (ocoef *)malloc(sizeof(ocoef) * w * h);
        for (uint32_t i = 0; i < w * h; i++) tq[i] = t[i];
        ocoef *qq = (ocoef *)calloc(w * h, sizeof(ocoef)), *rr = (ocoef *)calloc(w * h, sizeof(ocoef));
        orc_quant_inv_quant(qq, tq, rr, w, w < 32 ? w : 32, h < 32 ? h : 32, 4, 4, p.qmult, p.qadd, p.qshift,
                            p.iqmult, p.iqadd, p.iqshift, nz);
        for (uint32_t y = 0; y < h; y++)
            for (uint32_t x = 0; x < w; x++) { q[y * os + x] = qq[y * w + x]; r[y * os + x] = rr[y * w + x]; }
        free(tq); free(qq); free(rr);
    }
    orc_idct_wxh(r, os, res_out, os, w, h, is_intra, comp, mts, enable_mts);
    free(t);
}

/* ======================================================================
 * Motion estimation.
 * ====================================================================== */

/* Signed Exp-Golomb code length of v: 2*floor(log2(u+1)) + 1 with u = 2v-1 (v > 0)
 * or -2v (v <= 0).  Stands in for the closed table ExpGolombBits
 * (h26x_core/include/h26x_common_data.h:23) read through
 * CALC_MVD_BIT (common/include/h26x_definition.h:176).  Unpinned. */
uint32_t orc_mvd_bits(int32_t v)
{
    uint32_t u = v > 0 ? (uint32_t)(2 * v - 1) : (uint32_t)(-2 * v), l = 0;
    u += 1;
    while (u > 1) { u >>= 1; l++; }
    return 2 * l + 1;
}

void orc_exp_golomb_table(uint32_t *tab)
{
    for (int32_t i = 0; i < 32767; i++) tab[i] = orc_mvd_bits(i - 16383);
}

static inline uint32_t mv_cost(int32_t mvx, int32_t mvy, int32_t mvpx, int32_t mvpy, uint32_t lambda)
{
    return (orc_mvd_bits(mvx - mvpx) + orc_mvd_bits(mvy - mvpy)) * lambda;
}

/* Per-CU integer MV window from the reference-plane padding (ctu + 16 on each side):
 * h266_encoder/source/h266_enc_init.c:1462-1465. */
void orc_mv_window(int32_t frame_w, int32_t frame_h, int32_t ctu, int32_t cu_x, int32_t cu_y, int32_t cu_w, int32_t cu_h,
                   int32_t *min_mvx, int32_t *min_mvy, int32_t *max_mvx, int32_t *max_mvy)
{
    *min_mvx = (int16_t)(-cu_x - ctu - (16 - 8));
    *min_mvy = (int16_t)(-cu_y - ctu - (16 - 8));
    *max_mvx = (int16_t)(frame_w + (ctu - cu_w + 16 - 8) - cu_x);
    *max_mvy = (int16_t)(frame_h + (ctu - cu_h + 16 - 8) - cu_y);
}

/* Exhaustive integer search (stands in for the closed Xin26xMotionEstFull,
 * h26x_core/include/h26x_motion_est.h:23-36): every integer MV in
 * [c - range, c + range]^2 intersected with [min, max], c = predictor >> 2, visited
 * in raster order (y outer, x inner) with a strict '<' on
 * cost = (SAD << 8) + (bits(mvd_x) + bits(mvd_y)) * lambda, mvd in quarter-pel,
 * the cost form of the open sub-pel search (h266_sub_pel_refine.c:155-156).
 * The search starts from io->best_cost (the caller's running best).  Unpinned
 * (the closed drivers' search order is not visible). */
void orc_me_full(const opix *in, intptr_t is, const opix *ref_at_pu, intptr_t rs, uint32_t w, uint32_t h,
                 int32_t mvpx, int32_t mvpy, int32_t range, uint32_t lambda,
                 int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy, orc_me_io *io)
{
    int32_t cx = mvpx >> 2, cy = mvpy >> 2;
    int32_t x0 = cx - range > min_mvx ? cx - range : min_mvx, x1 = cx + range < max_mvx ? cx + range : max_mvx;
    int32_t y0 = cy - range > min_mvy ? cy - range : min_mvy, y1 = cy + range < max_mvy ? cy + range : max_mvy;
    uint32_t best = io->best_cost, bsad = io->best_sad;
    int32_t bx = io->best_mvx, by = io->best_mvy;
    for (int32_t y = y0; y <= y1; y++)
        for (int32_t x = x0; x <= x1; x++) {
            uint32_t sad;
            orc_sad(in, is, ref_at_pu + (intptr_t)y * rs + x, rs, w, h, &sad);
            uint32_t c = (sad << 8) + mv_cost(x * 4, y * 4, mvpx, mvpy, lambda);
            if (c < best) { best = c; bsad = sad; bx = x * 4; by = y * 4; }
        }
    io->best_cost = best; io->best_sad = bsad; io->best_mvx = bx; io->best_mvy = by;
}

/* ---- integer search by resolution levels --------------------------------
 * The reference's hierarchical search (Xin26xMotionEstHier, its level searches
 * Xin26xMotionSearchHier1/2 and the 2x2 downscale Xin26xDownscale2x2;
 * h26x_core/include/h26x_motion_est.h:23-36,
 * h26x_core/include/h26x_hierarchic_motion_search.h:29,42,
 * h26x_core/include/h26x_downscale_subs.h:23) exists only in the closed
 * library: its order is not published.  Restated here; parity unpinned. */

/* 2x2 downscale (typedef XinDownscale2x2, h266_encoder/include/h266_func_struct.h:425):
 * out(x, y) = (a + b + c + d + 2) >> 2 over in(2x..2x+1, 2y..2y+1).  Every open
 * caller passes FALSE for both row flags (h266_enc_init.c:2804-2824,
 * h266_scene_cut.c:64); only that form is defined here. */
void orc_downscale2x2(const opix *in, intptr_t is, int row_above, int row_below, opix *out, intptr_t os,
                      uint32_t ow, uint32_t oh)
{
    (void)row_above; (void)row_below;
    for (uint32_t y = 0; y < oh; y++)
        for (uint32_t x = 0; x < ow; x++) {
            const opix *a = in + (intptr_t)(2 * y) * is + 2 * x;
            out[(intptr_t)y * os + x] = (opix)((a[0] + a[1] + a[is] + a[is + 1] + 2) >> 2);
        }
}

/* one level (typedef XinHierMotionSearch, h266_func_struct.h:435): every MV of
 * [min_x, max_x] x [min_y, max_y] at the level's resolution, raster order
 * (y outer), strict '<' on the SAD of the w x h block; an empty window leaves
 * the output untouched */
void orc_hier_search(const opix *in, intptr_t is, const opix *ref, intptr_t rs, int32_t min_x, int32_t max_x,
                     int32_t min_y, int32_t max_y, uint32_t w, uint32_t h, int32_t *best_x, int32_t *best_y)
{
    uint32_t best = 0xFFFFFFFFu;
    for (int32_t y = min_y; y <= max_y; y++)
        for (int32_t x = min_x; x <= max_x; x++) {
            uint32_t sad;
            orc_sad(in, is, ref + (intptr_t)y * rs + x, rs, w, h, &sad);
            if (sad < best) { best = sad; *best_x = x; *best_y = y; }
        }
}

static int32_t ceil_shr(int32_t v, int s) { return -((-v) >> s); }

/* The driver:
 *  window   [c - range, c + range] intersected with [min, max], c = predictor >> 2
 *           (full-pel); at level L (1/2, 1/4) its ends become ceil(lo / 2^L) and
 *           floor(hi / 2^L)
 *  start    the incoming best, then every candidate (quarter-pel MV >> 2,
 *           clipped to the window) with the full cost, list order, strict '<'
 *  1/4      exhaustive SAD over the level window, block (w/4) x (h/4); b2
 *  1/2      +-1 around 2 * b2 within the level window, block (w/2) x (h/2); b1
 *  full     the 3 x 3 MVs around 2 * b1 within the window, raster order, full
 *           cost (SAD << 8) + (bits(mvd x) + bits(mvd y)) * lambda against the
 *           running best, strict '<'
 * A level whose window is empty keeps the centre it was given (c >> L). */
void orc_me_hier(const orc_hier_in *hi, uint32_t w, uint32_t h, int32_t mvpx, int32_t mvpy, int32_t range_x,
                 int32_t range_y, uint32_t lambda, int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy,
                 orc_me_io *io)
{
    const int32_t cx = mvpx >> 2, cy = mvpy >> 2;
    const int32_t x0 = cx - range_x > min_mvx ? cx - range_x : min_mvx, x1 = cx + range_x < max_mvx ? cx + range_x : max_mvx;
    const int32_t y0 = cy - range_y > min_mvy ? cy - range_y : min_mvy, y1 = cy + range_y < max_mvy ? cy + range_y : max_mvy;
    uint32_t best = io->best_cost, bsad = io->best_sad;
    int32_t bx = io->best_mvx, by = io->best_mvy;
    for (uint32_t i = 0; i < hi->ncand; i++) {
        int32_t x = CLIP3(x0, x1, hi->cand[2 * i] >> 2), y = CLIP3(y0, y1, hi->cand[2 * i + 1] >> 2);
        uint32_t sad;
        orc_sad(hi->in[0], hi->in_stride[0], hi->ref[0] + (intptr_t)y * hi->ref_stride[0] + x, hi->ref_stride[0], w, h, &sad);
        uint32_t c = (sad << 8) + mv_cost(x * 4, y * 4, mvpx, mvpy, lambda);
        if (c < best) { best = c; bsad = sad; bx = x * 4; by = y * 4; }
    }
    int32_t b2x = cx >> 2, b2y = cy >> 2;
    orc_hier_search(hi->in[2], hi->in_stride[2], hi->ref[2], hi->ref_stride[2], ceil_shr(x0, 2), x1 >> 2,
                    ceil_shr(y0, 2), y1 >> 2, w >> 2, h >> 2, &b2x, &b2y);
    const int32_t l1x0 = ceil_shr(x0, 1), l1x1 = x1 >> 1, l1y0 = ceil_shr(y0, 1), l1y1 = y1 >> 1;
    int32_t b1x = cx >> 1, b1y = cy >> 1;
    orc_hier_search(hi->in[1], hi->in_stride[1], hi->ref[1], hi->ref_stride[1],
                    2 * b2x - 1 > l1x0 ? 2 * b2x - 1 : l1x0, 2 * b2x + 1 < l1x1 ? 2 * b2x + 1 : l1x1,
                    2 * b2y - 1 > l1y0 ? 2 * b2y - 1 : l1y0, 2 * b2y + 1 < l1y1 ? 2 * b2y + 1 : l1y1,
                    w >> 1, h >> 1, &b1x, &b1y);
    for (int32_t y = 2 * b1y - 1; y <= 2 * b1y + 1; y++)
        for (int32_t x = 2 * b1x - 1; x <= 2 * b1x + 1; x++) {
            if (x < x0 || x > x1 || y < y0 || y > y1) continue;
            uint32_t sad;
            orc_sad(hi->in[0], hi->in_stride[0], hi->ref[0] + (intptr_t)y * hi->ref_stride[0] + x, hi->ref_stride[0], w, h, &sad);
            uint32_t c = (sad << 8) + mv_cost(x * 4, y * 4, mvpx, mvpy, lambda);
            if (c < best) { best = c; bsad = sad; bx = x * 4; by = y * 4; }
        }
    io->best_cost = best; io->best_sad = bsad; io->best_mvx = bx; io->best_mvy = by;
}

/* ---- fast sub-pel search by variance -----------------------------------
 * Xin266FastSubPelMeVar (open, h266_encoder/source/h266_sub_pel_refine.c:214-361):
 * the eight half-pel neighbours of an integer start, then (without AMVR) the
 * eight quarter-pel neighbours of the best, each quarter-pel prediction the
 * rounded average of two half-grid samples (the pointer pairs qBufA / qBufB set
 * up by Xin266ConstructMe, h266_encoder/source/h266_create_section.c:45-230);
 * cost (variance << 8) + (lambda * bits << 15 + 2^22) >> 23.  The half-pel
 * planes come from the closed pfXinInterpoHalfPel
 * (h26x_core/include/h26x_me_func_struct.h:143), restated here with the
 * luma filter's half-pel phase (the alternative half-pel filter under half-pel
 * AMVR, as the driver's interpAlt argument selects); parity of those samples is
 * unpinned, the driver and the pairing are pinned. */

/* the w x h block at half-grid point (px, py) in half-sample units relative to
 * ref: integer, horizontal, vertical or both-direction half-pel samples */
void orc_half_grid_block(const opix *ref, intptr_t rs, int32_t px, int32_t py, uint32_t w, uint32_t h, uint32_t fi,
                         opix *out, intptr_t os)
{
    const opix *src = ref + (intptr_t)(py >> 1) * rs + (px >> 1);
    const int32_t frac = ((py & 1) ? 8 << 4 : 0) | ((px & 1) ? 8 : 0);
    if (!(px & 1) && !(py & 1)) orc_interp_copy(src, rs, out, os, frac, w, h, fi);
    else if (!(py & 1)) orc_luma_hor(src, rs, out, os, frac, w, h, fi);
    else if (!(px & 1)) orc_luma_vet(src, rs, out, os, frac, w, h, fi);
    else orc_luma_hv(src, rs, out, os, frac, w, h, fi);
}

/* the two half-grid points averaged for the quarter-pel position h + q / 2
 * (half-sample units): for a diagonal q around the centre or around a
 * diagonal h, the two points on the other diagonal; otherwise h + q and h */
void orc_qpel_pair(int32_t hx, int32_t hy, int32_t qx, int32_t qy, int32_t p[4])
{
    const int h_same_parity = ((hx ^ hy) & 1) == 0;      /* the centre or a diagonal half position */
    if (qx && qy && h_same_parity) { p[0] = hx + qx; p[1] = hy; p[2] = hx; p[3] = hy + qy; }
    else { p[0] = hx + qx; p[1] = hy + qy; p[2] = hx; p[3] = hy; }
}

/* the four planes in the layout the driver's pointers assume: plane k's
 * element (x, y), x in [-1, w], y in [-1, h], sits at half-grid point
 * (2x - dx_k, 2y - dy_k) with (dx, dy) = (0,0) integer, (1,0) H, (0,1) V, (1,1) HV;
 * origins: integer at integ + stride + 1, H at hb + 2 stride, V at vb + 1, HV at
 * hvb (h266_create_section.c:74-86) */
void orc_interpo_half_pel(const opix *ref, intptr_t rs, uint32_t w, uint32_t h, opix *integ, opix *hb, opix *vb, opix *hvb,
                          intptr_t stride, int alt)
{
    opix *org[4] = { integ + stride + 1, hb + 2 * stride, vb + 1, hvb };
    static const int d[4][2] = { { 0, 0 }, { 1, 0 }, { 0, 1 }, { 1, 1 } };
    for (int k = 0; k < 4; k++) {
        /* rows -1 .. h of every plane fit the buffer except above the V and HV
         * origins (row 0 of their buffers), whose row -1 is not read */
        const int y0 = (k >= 2) ? 0 : -1, x0 = (k == 1 || k == 3) ? 0 : -1;
        orc_half_grid_block(ref, rs, 2 * x0 - d[k][0], 2 * y0 - d[k][1], (uint32_t)(w + 1 - x0), (uint32_t)(h + 1 - y0),
                            alt ? 1u : 0u, org[k] + (intptr_t)y0 * stride + x0, stride);
    }
}

static uint64_t fsme_cost(uint32_t var, int32_t mvx, int32_t mvy, int32_t mvpx, int32_t mvpy, int shift, uint64_t lambda)
{
    const uint64_t bits = (uint64_t)(orc_mvd_bits((mvx - mvpx) >> shift) + orc_mvd_bits((mvy - mvpy) >> shift)) << 15;
    return (uint64_t)(uint32_t)(var << 8) + ((lambda * bits + (1ull << 22)) >> 23);
}

void orc_fast_subpel_me_var(const opix *in, intptr_t is, const opix *ref_at_pu, intptr_t rs, uint32_t w, uint32_t h,
                            int32_t mvpx, int32_t mvpy, uint64_t lambda, int32_t imv, int32_t min_mvx, int32_t min_mvy,
                            int32_t max_mvx, int32_t max_mvy, int32_t *io)
{
    static const int8_t off[9][2] = { { -1, 0 }, { 1, 0 }, { 0, -1 }, { 0, 1 }, { -1, -1 }, { 1, -1 }, { -1, 1 }, { 1, 1 }, { 0, 0 } };
    int32_t mvx = io[0], mvy = io[1];
    const int32_t ix = mvx >> 2, iy = mvy >> 2;
    if (!(ix >= min_mvx && iy >= min_mvy && ix <= max_mvx && iy <= max_mvy)) return;
    const int shift = imv == 3 ? 1 : imv << 1;
    const uint32_t fi = imv == 3 ? 1u : 0u;
    const opix *r0 = ref_at_pu + (intptr_t)iy * rs + ix;
    opix *a = (opix *)malloc(sizeof(opix) * w * h), *b = (opix *)malloc(sizeof(opix) * w * h);
    uint32_t var;
    orc_var(in, is, r0, rs, w, h, &var);
    uint64_t best = fsme_cost(var, mvx, mvy, mvpx, mvpy, shift, lambda);
    int bp = 8;
    for (int p = 0; p < 8; p++) {
        orc_half_grid_block(r0, rs, off[p][0], off[p][1], w, h, fi, a, w);
        orc_var(in, is, a, w, w, h, &var);
        const uint64_t c = fsme_cost(var, mvx + 2 * off[p][0], mvy + 2 * off[p][1], mvpx, mvpy, shift, lambda);
        if (c < best) { best = c; bp = p; }
    }
    const int hx = off[bp][0], hy = off[bp][1];
    mvx += 2 * hx; mvy += 2 * hy;
    if (imv == 0) {
        int qp = 8;
        for (int p = 0; p < 8; p++) {
            int32_t pr[4];
            orc_qpel_pair(hx, hy, off[p][0], off[p][1], pr);
            orc_half_grid_block(r0, rs, pr[0], pr[1], w, h, fi, a, w);
            orc_half_grid_block(r0, rs, pr[2], pr[3], w, h, fi, b, w);
            orc_avg_var(in, is, a, b, w, w, h, &var);
            const uint64_t c = fsme_cost(var, mvx + off[p][0], mvy + off[p][1], mvpx, mvpy, shift, lambda);
            if (c < best) { best = c; qp = p; }
        }
        mvx += off[qp][0]; mvy += off[qp][1];
        bp = qp;
    }
    free(a); free(b);
    io[0] = mvx; io[1] = mvy; io[2] = bp;
}

/* ---- DMVR ------------------------------------------------------------
 * The encoder's emulation of the H.266 decoder-side MV refinement:
 * Xin266DeriveMvFromDmvr + Xin266SubPelRefineDmvr and Xin266LumaMotionCompDmvr
 * (open, h266_encoder/source/h266_inter_prediction.c:864-1420) and
 * Xin266CopyAndPad / Xin266CopyAndPadUv (open, h266_copy_and_pad.c:32-112).
 * Their closed helpers are restated: Xin26xComputeSadS16
 * (h26x_core/include/h26x_compute_dist.h:942), Xin26xBlockCopy and
 * Xin26xBlockPad1/2 (h26x_core/include/h26x_block_utility.h:23,335,343). */

/* SAD over every (1 << sub)-th row, scaled back by 1 << sub (the row-subsampled
 * distortion of the standard's DMVR).  Restated; unpinned. */
void orc_sad_s16(const int16_t *a, intptr_t as, const int16_t *b, intptr_t bs, uint32_t w, uint32_t h, uint32_t sub,
                 uint32_t *sad)
{
    uint32_t s = 0;
    for (uint32_t y = 0; y < h; y += 1u << sub)
        for (uint32_t x = 0; x < w; x++) {
            int d = a[(intptr_t)y * as + x] - b[(intptr_t)y * bs + x];
            s += (uint32_t)(d < 0 ? -d : d);
        }
    *sad = s << sub;
}

void orc_block_copy(const opix *src, intptr_t ss, opix *dst, intptr_t ds, uint32_t w, uint32_t h)
{
    for (uint32_t y = 0; y < h; y++) memcpy(dst + (intptr_t)y * ds, src + (intptr_t)y * ss, w * sizeof(opix));
}

/* extend the w x h block outward by pw columns and ph rows, repeating its edge
 * samples (the standard's DMVR reference padding).  Restated; unpinned. */
void orc_block_pad(opix *buf, intptr_t bs, uint32_t w, uint32_t h, uint32_t pw, uint32_t ph)
{
    for (uint32_t y = 0; y < h; y++) {
        opix *row = buf + (intptr_t)y * bs;
        for (uint32_t i = 1; i <= pw; i++) { row[-(intptr_t)i] = row[0]; row[w - 1 + i] = row[w - 1]; }
    }
    for (uint32_t i = 1; i <= ph; i++) {
        memcpy(buf - (intptr_t)i * bs - pw, buf - pw, (w + 2 * pw) * sizeof(opix));
        memcpy(buf + (intptr_t)(h - 1 + i) * bs - pw, buf + (intptr_t)(h - 1) * bs - pw, (w + 2 * pw) * sizeof(opix));
    }
}

/* h266_copy_and_pad.c:32-57: the (w + 7) x (h + 7) luma region the 8-tap filter
 * reads, padded by 2 (DMVR_NUM_ITERATION) on every side */
void orc_copy_and_pad(const opix *ref, intptr_t rs, opix *pad, intptr_t ps, uint32_t w, uint32_t h)
{
    orc_block_copy(ref - 3 * rs - 3, rs, pad - 3 * ps - 3, ps, w + 7, h + 7);
    orc_block_pad(pad - 3 * ps - 3, ps, w + 7, h + 7, 2, 2);
}

/* h266_copy_and_pad.c:59-112: the (w + 3) x (h + 3) chroma regions of the 4-tap
 * filter, padded by 1 */
void orc_copy_and_pad_uv(const opix *ref_u, const opix *ref_v, intptr_t rs, opix *pad_u, opix *pad_v, intptr_t ps,
                         uint32_t w, uint32_t h)
{
    orc_block_copy(ref_u - rs - 1, rs, pad_u - ps - 1, ps, w + 3, h + 3);
    orc_block_copy(ref_v - rs - 1, rs, pad_v - ps - 1, ps, w + 3, h + 3);
    orc_block_pad(pad_u - ps - 1, ps, w + 3, h + 3, 1, 1);
    orc_block_pad(pad_v - ps - 1, ps, w + 3, h + 3, 1, 1);
}

/* Xin266DivForMaxQ7 (:864-907): |n| / d in eighths as three quotient bits (4, 2, 1), sign of n */
static int32_t dmvr_div8(int64_t n, int64_t d)
{
    const int neg = n < 0;
    if (neg) n = -n;
    int32_t q = 0;
    for (int b = 2; b >= 0; b--) {
        const int64_t step = d << (b + 1);
        if (n >= step) { n -= step; q |= 1 << b; }
    }
    return neg ? -q : q;
}

/* Xin266SubPelErrorSrfc + Xin266SubPelRefineDmvr (:909-973): the parabolic
 * sub-pel offset from the costs around the best integer position */
static void dmvr_subpel(int non0, int32_t del[2], const uint32_t *c, int cs)
{
    if (!non0 || del[0] == 32 || del[0] == -32 || del[1] == 32 || del[1] == -32) return;
    const int64_t c0 = c[0];
    const int64_t nb[2][2] = { { c[-1], c[1] }, { c[-cs], c[cs] } };   /* (before, after) per direction */
    for (int hv = 0; hv < 2; hv++) {
        const int64_t num = (nb[hv][0] - nb[hv][1]) * 16, den = nb[hv][0] + nb[hv][1] - 2 * c0;
        if (den == 0) continue;
        if (nb[hv][0] != c0 && nb[hv][1] != c0) del[hv] += dmvr_div8(num, den);
        else del[hv] += nb[hv][0] == c0 ? -8 : 8;
    }
}

static void dmvr_luma_s16(const opix *src, intptr_t ss, int16_t *dst, intptr_t ds, int32_t frac, uint32_t w, uint32_t h,
                          uint32_t fi)
{
    const int fx = frac & 15, fy = frac >> 4;
    if (!fx && !fy) orc_interp_copy_s16(src, ss, dst, ds, frac, w, h, fi);
    else if (fx && !fy) orc_luma_hor_s16(src, ss, dst, ds, frac, w, h, fi);
    else if (!fx && fy) orc_luma_vet_s16(src, ss, dst, ds, frac, w, h, fi);
    else orc_luma_hv_s16(src, ss, dst, ds, frac, w, h, fi);
}

void orc_dmvr_luma(const opix *ref0, const opix *ref1, intptr_t rs, int32_t cu_x, int32_t cu_y, int32_t min_mvx,
                   int32_t min_mvy, int32_t max_mvx, int32_t max_mvy, uint32_t w, uint32_t h, const int32_t mv16[4],
                   int alt_hpel, int16_t *mvd, opix *pred, intptr_t ps)
{
    enum { BS = 256, CS = 5 };                               /* bilinear buffer stride; cost grid side */
    const uint32_t sw = w < 16 ? w : 16, sh = h < 16 ? h : 16;
    const opix *refs[2] = { ref0, ref1 };
    int16_t *bil = (int16_t *)malloc(sizeof(int16_t) * 2 * BS * BS);
    int32_t base[2][2];                                      /* clipped MVs, 1/16 */
    /* bilinear predictions of both lists over (w + 4) x (h + 4), from 2 samples up and left (:1037-1085) */
    for (int l = 0; l < 2; l++) {
        base[l][0] = CLIP3(min_mvx * 16, max_mvx * 16, mv16[2 * l]);
        base[l][1] = CLIP3(min_mvy * 16, max_mvy * 16, mv16[2 * l + 1]);
        const int32_t ox = cu_x * 16 + base[l][0] - 32, oy = cu_y * 16 + base[l][1] - 32;
        const int32_t fx = ox & 15, fy = oy & 15;
        orc_bili_interp((fx ? 1 : 0) | (fy ? 2 : 0), refs[l] + (intptr_t)(oy >> 4) * rs + (ox >> 4), rs, bil + l * BS * BS, BS,
                        (fy << 4) + fx, w, h + 4);
    }
    /* per 16 x 16 sub-block: the 5 x 5 integer search of one iteration and the
     * sub-pel offset (:1087-1175) */
    int n = 0;
    for (uint32_t y0 = 0; y0 < h; y0 += sh)
        for (uint32_t x0 = 0; x0 < w; x0 += sw, n++) {
            const int16_t *c0 = bil + (2 + y0) * BS + x0 + 2, *c1 = bil + BS * BS + (2 + y0) * BS + x0 + 2;
            uint32_t cost[CS * CS];
            for (int i = 0; i < CS * CS; i++) cost[i] = 0xFFFFFFFFu;
            int ctr = CS * CS / 2, non0 = 1;
            int32_t del[2] = { 0, 0 };
            uint32_t best;
            orc_sad_s16(c0, BS, c1, BS, sw, sh, 1, &best);
            best >>= 1;
            best -= best >> 2;
            if (best < sh * sw || best == 0) non0 = 0;
            else {
                cost[ctr] = best;
                int bdx = 0, bdy = 0;
                for (int dy = -2; dy <= 2; dy++)
                    for (int dx = -2; dx <= 2; dx++) {
                        uint32_t *c = &cost[ctr + dy * CS + dx];
                        if (*c == 0xFFFFFFFFu) {
                            orc_sad_s16(c0 + dy * BS + dx, BS, c1 - dy * BS - dx, BS, sw, sh, 1, c);
                            *c >>= 1;
                        }
                        if (*c < best) { best = *c; bdx = dx; bdy = dy; }
                    }
                del[0] = bdx; del[1] = bdy;
                ctr += bdy * CS + bdx;
            }
            del[0] *= 16; del[1] *= 16;
            dmvr_subpel(non0, del, &cost[ctr], CS);
            mvd[2 * n] = (int16_t)del[0];
            mvd[2 * n + 1] = (int16_t)del[1];
            /* the refined prediction of the sub-block (Xin266LumaMotionCompDmvr, :1260-1420):
             * L0 moves by +del, L1 by -del; when the integer part moved, the 8-tap
             * filter reads a copy of the unrefined position's region padded by 2 */
            int16_t p[2][16 * 16];
            for (int l = 0; l < 2; l++) {
                const int32_t sg = l ? -1 : 1;
                const int32_t rx = mv16[2 * l] + sg * del[0], ry = mv16[2 * l + 1] + sg * del[1];
                const int32_t dix = (rx >> 4) - (mv16[2 * l] >> 4), diy = (ry >> 4) - (mv16[2 * l + 1] >> 4);
                if (dix || diy) {
                    const int32_t ix = (((cu_x + (int32_t)x0) * 16) + base[l][0]) >> 4, iy = (((cu_y + (int32_t)y0) * 16) + base[l][1]) >> 4;
                    opix padb[32 * 32];
                    opix *pb = padb + 8 * 32;
                    orc_copy_and_pad(refs[l] + (intptr_t)iy * rs + ix, rs, pb, 32, sw, sh);
                    dmvr_luma_s16(pb + diy * 32 + dix, 32, p[l], 16, ((ry & 15) << 4) + (rx & 15), sw, sh, (uint32_t)alt_hpel);
                } else {
                    const int32_t cx = CLIP3(min_mvx * 16, max_mvx * 16, rx), cy = CLIP3(min_mvy * 16, max_mvy * 16, ry);
                    const int32_t ox = (cu_x + (int32_t)x0) * 16 + cx, oy = (cu_y + (int32_t)y0) * 16 + cy;
                    dmvr_luma_s16(refs[l] + (intptr_t)(oy >> 4) * rs + (ox >> 4), rs, p[l], 16, ((oy & 15) << 4) + (ox & 15), sw,
                                  sh, (uint32_t)alt_hpel);
                }
            }
            orc_interp_avg(p[0], 16, p[1], 16, pred + (intptr_t)y0 * ps + x0, ps, sw, sh);
        }
    free(bil);
}

/* Xin266FullSubPelMe (open, h266_sub_pel_refine.c:81-212): 8 half-pel then 8
 * quarter-pel neighbours in the fixed order of :47-55, luma interpolation with the
 * default filter into a W x H block, SAD, strict '<'.  Returns unchanged when the
 * integer part of the start MV is outside the window (:117-120). */
void orc_full_subpel_me(const opix *in, intptr_t is, const opix *ref_at_pu, intptr_t rs, uint32_t w, uint32_t h,
                        int32_t mvpx, int32_t mvpy, uint32_t lambda,
                        int32_t min_mvx, int32_t min_mvy, int32_t max_mvx, int32_t max_mvy, orc_me_io *io)
{
    static const int8_t off[8][2] = { { -1, 0 }, { 1, 0 }, { 0, -1 }, { 0, 1 }, { -1, -1 }, { 1, -1 }, { -1, 1 }, { 1, 1 } };
    int32_t mvx = io->best_mvx, mvy = io->best_mvy;
    if (!((mvx >> 2) >= min_mvx && (mvy >> 2) >= min_mvy && (mvx >> 2) <= max_mvx && (mvy >> 2) <= max_mvy)) return;
    opix *pred = (opix *)malloc(sizeof(opix) * w * h);
    uint32_t best = io->best_cost;
    int32_t bx = mvx, by = mvy;
    for (int step = 2; step >= 1; step--) {
        int32_t cxm = bx, cym = by;
        for (int p = 0; p < 8; p++) {
            int32_t tx = cxm + off[p][0] * step, ty = cym + off[p][1] * step;
            int32_t frac = (((ty << 2) & 15) << 4) + ((tx << 2) & 15);
            uint32_t sad;
            orc_luma_interpolation(ref_at_pu + (intptr_t)((ty << 2) >> 4) * rs + ((tx << 2) >> 4), rs, pred, w, frac, lg2u(w), h, 0);
            orc_sad(in, is, pred, w, w, h, &sad);
            uint32_t c = (sad << 8) + mv_cost(tx, ty, mvpx, mvpy, lambda);
            if (c < best) { best = c; bx = tx; by = ty; }
        }
    }
    free(pred);
    io->best_cost = best; io->best_mvx = bx; io->best_mvy = by;
}

/* ======================================================================
 * Frame hot path of one CU (the checker of the batched GPU frame stages):
 *   window (h266_enc_init.c:1462) -> exhaustive integer search around MVP 0
 *   -> Xin266FullSubPelMe -> Xin266LumaInterPred / uni Xin266ChromaMotionComp
 *   -> per plane Xin266Transform TU (DCT2, TU = CU, 4x4 CGs, no RDOQ)
 *   -> Xin266IDctAdd recon; SSD(recon, input) per plane.
 * The integer search starts from cost UINT32_MAX at MV (0,0).
 * ====================================================================== */
/* The preset-4 TU of one CU (tu_mode 1), TU = CU: every transform candidate the
 * reference's mode decision may evaluate, each through the dependent-quantisation
 * branch of Xin266Transform (h266_encoder/source/h266_trans_quant.c:61-245:
 * Xin266SubFDctWxH, then pfXinDepQuant with QP + 12 at 10 bits) and
 * Xin266IDctAdd (h266_idct_add.c:45): luma DCT2 and, for CUs up to 32, the
 * explicit MTS pairs 2..5 (enableMts at preset 4,
 * app/common/source/xin_encoder_option.c:196); chroma DCT2.  The rate tables
 * come from the frame's context set; luma carries the root cbf (an inter CU
 * coded as one TU).  The choice among the candidates (the host's rate
 * estimation) is not made: each candidate's non-zero map and SSD are returned,
 * and the coefficient / reconstructed planes hold the DCT2 candidate.  Also
 * the cost of the final luma prediction with SATD as the distortion (satdMd
 * at preset 4, h266_encoder_create.c:1938; the recomputation at
 * h266_analyze_inter_cu.c:1109-1131 with predictor 0 and one reference). */
static void orc_cu_tu_p4(const orc_frame_desc *f, int32_t cu_x, int32_t cu_y, int32_t size, int32_t mnx, int32_t mny,
                         int32_t mxx, int32_t mxy, int32_t dir, const int32_t *mv16, ocoef *q[3], intptr_t q_stride[2],
                         opix *rec[3], intptr_t rec_stride[2], opix *pred, ocoef *t, ocoef *qb, ocoef *r, orc_cu_out *out)
{
    static const uint32_t mts_list[5] = { 0, 2, 3, 4, 5 };
    const int32_t cs = size >> 1;
    opix *rb = (opix *)malloc(sizeof(opix) * (size_t)(size * size));
    out->ncand = size <= 32 ? 5 : 1;
    for (int pl = 0; pl < 3; pl++) {
        const int32_t bs = pl ? cs : size, px = pl ? cu_x >> 1 : cu_x, py = pl ? cu_y >> 1 : cu_y;
        const intptr_t istr = f->in_stride[pl ? 1 : 0], qstr = q_stride[pl ? 1 : 0], rstr = rec_stride[pl ? 1 : 0];
        const opix *const *lref = dir == 2 ? f->ref1 : f->ref;
        if (dir == 3 && pl == 0)
            orc_luma_motion_comp_bi(f->ref[0], f->ref1[0], f->ref_stride[0], pred, bs, mv16, cu_x, cu_y, mnx, mny, mxx, mxy,
                                    (uint32_t)size, (uint32_t)size);
        else if (dir == 3)
            orc_chroma_motion_comp_bi(f->ref[pl], f->ref1[pl], f->ref_stride[1], pred, bs, mv16, cu_x, cu_y, mnx, mny, mxx,
                                      mxy, (uint32_t)size, (uint32_t)size);
        else if (pl == 0)
            orc_luma_inter_pred(lref[0], f->ref_stride[0], pred, bs, mv16[0], mv16[1], cu_x, cu_y,
                                mnx, mny, mxx, mxy, (uint32_t)size, (uint32_t)size, 0);
        else
            orc_chroma_motion_comp(lref[pl], f->ref_stride[1], pred, bs, mv16[0], mv16[1], cu_x, cu_y,
                                   mnx, mny, mxx, mxy, (uint32_t)size, (uint32_t)size);
        const opix *src = f->in[pl] + (intptr_t)py * istr + px;
        if (pl == 0) {
            /* the coded prediction's MV bits: one MV, or both of the pair */
            uint32_t satd, bits = orc_mvd_bits(mv16[0] >> 2) + orc_mvd_bits(mv16[1] >> 2);
            if (dir == 3) bits += orc_mvd_bits(mv16[2] >> 2) + orc_mvd_bits(mv16[3] >> 2);
            orc_satd(src, istr, pred, bs, (uint32_t)bs, (uint32_t)bs, &satd);
            out->satd_cost = (satd << 8) + bits * f->sad_lambda;
        }
        const int32_t qp = (pl ? f->uv_qp : f->qp) + (ORC_BITDEPTH == 10 ? 12 : 0);
        const uint32_t nc = pl ? 1 : out->ncand;
        for (uint32_t c = 0; c < nc; c++) {
            uint64_t nz = 0;
            orc_sub_fdct_wxh(src, istr, pred, bs, t, bs, pl ? 1u : 0u, mts_list[c], bs, bs, 0, 1);
            /* beyond the low 32 x 32 the dequantised values are zero (Xin266ZeroOutCoeff,
             * h266_trans_quant.c:155-189) and no level is coded; the trellis writes the
             * low 32 x 32 */
            memset(r, 0, sizeof(ocoef) * (size_t)(bs * bs));
            memset(qb, 0, sizeof(ocoef) * (size_t)(bs * bs));
            orc_dep_quant(t, bs, bs, bs, qp, pl, f->ctx, pl == 0, qb, r, &nz);
            orc_idct_add(r, bs, pred, bs, rb, bs, 0, pl ? 1u : 0u, mts_list[c], (uint32_t)bs, (uint32_t)bs, 1);
            uint64_t ssd = 0;
            for (int32_t y = 0; y < bs; y++)
                for (int32_t x = 0; x < bs; x++) {
                    const int64_t d = (int64_t)src[y * istr + x] - (int64_t)rb[y * bs + x];
                    ssd += (uint64_t)(d * d);
                }
            if (pl == 0) { out->nz_mts[c] = nz; out->ssd_mts[c] = ssd; }
            if (c == 0) {
                out->nz[pl] = nz; out->ssd[pl] = ssd;
                for (int32_t y = 0; y < bs; y++)
                    for (int32_t x = 0; x < bs; x++) {
                        q[pl][(intptr_t)(py + y) * qstr + px + x] = qb[y * bs + x];
                        rec[pl][(intptr_t)(py + y) * rstr + px + x] = rb[y * bs + x];
                    }
            }
        }
    }
    free(rb);
}

/* integer search and Xin266FullSubPelMe of one list (ref: the list's padded luma
 * at picture (0,0); ref_lo its downscaled planes for search_mode 1) */
static void orc_uni_search(const orc_frame_desc *f, const opix *ref, const opix *const *ref_lo, int32_t cu_x, int32_t cu_y,
                           int32_t size, int32_t mnx, int32_t mny, int32_t mxx, int32_t mxy, orc_me_io *io, uint32_t *int_cost)
{
    const opix *in_y = f->in[0] + (intptr_t)cu_y * f->in_stride[0] + cu_x;
    const opix *ref_y = ref + (intptr_t)cu_y * f->ref_stride[0] + cu_x;
    orc_me_io z = { 0, 0, 0xFFFFFFFFu, 0 };
    *io = z;
    if (f->search_mode == 1) {
        /* predictor 0, one candidate: the zero MV (Xin266FillMeCand's meCand[0],
         * h266_analyze_inter_cu.c:168) */
        static const int32_t zero[2] = { 0, 0 };
        orc_hier_in hin;
        hin.in[0] = in_y; hin.in_stride[0] = f->in_stride[0];
        hin.ref[0] = ref_y; hin.ref_stride[0] = f->ref_stride[0];
        for (int l = 1; l <= 2; l++) {
            hin.in[l] = f->in_lo[l - 1] + (intptr_t)(cu_y >> l) * f->in_lo_stride[l - 1] + (cu_x >> l);
            hin.in_stride[l] = f->in_lo_stride[l - 1];
            hin.ref[l] = ref_lo[l - 1] + (intptr_t)(cu_y >> l) * f->ref_lo_stride[l - 1] + (cu_x >> l);
            hin.ref_stride[l] = f->ref_lo_stride[l - 1];
        }
        hin.cand = zero; hin.ncand = 1;
        orc_me_hier(&hin, (uint32_t)size, (uint32_t)size, 0, 0, f->search_range, f->search_range, f->sad_lambda,
                    mnx, mny, mxx, mxy, io);
    } else
        orc_me_full(in_y, f->in_stride[0], ref_y, f->ref_stride[0], (uint32_t)size, (uint32_t)size, 0, 0,
                    f->search_range, f->sad_lambda, mnx, mny, mxx, mxy, io);
    *int_cost = io->best_cost;
    orc_full_subpel_me(in_y, f->in_stride[0], ref_y, f->ref_stride[0], (uint32_t)size, (uint32_t)size, 0, 0,
                       f->sad_lambda, mnx, mny, mxx, mxy, io);
}

/* Integer step of the bi refinement.  The reference runs the closed
 * Xin26xMotionEstBbdgs with searchWidth = searchHeight = 4 around the list's
 * uni MV (h266_analyze_inter_cu.c:607-608,665-677); restated here as every
 * integer MV in [c - 4, c + 4]^2 within the window, raster order, strict '<'
 * from UINT32_MAX, cost (SAD << 8) + bits(mv) * lambda with predictor 0.
 * Unpinned (the closed search's order is not visible). */
static void orc_me_square(const opix *in, intptr_t is, const opix *ref_at_pu, intptr_t rs, uint32_t w, uint32_t h,
                          int32_t cx, int32_t cy, int32_t range, uint32_t lambda,
                          int32_t mnx, int32_t mny, int32_t mxx, int32_t mxy, orc_me_io *io)
{
    uint32_t best = 0xFFFFFFFFu, bsad = 0;
    int32_t bx = 0, by = 0;
    for (int32_t y = cy - range; y <= cy + range; y++)
        for (int32_t x = cx - range; x <= cx + range; x++) {
            if (x < mnx || x > mxx || y < mny || y > mxy) continue;
            uint32_t sad;
            orc_sad(in, is, ref_at_pu + (intptr_t)y * rs + x, rs, w, h, &sad);
            uint32_t c = (sad << 8) + mv_cost(x * 4, y * 4, 0, 0, lambda);
            if (c < best) { best = c; bsad = sad; bx = x * 4; by = y * 4; }
        }
    io->best_cost = best; io->best_sad = bsad; io->best_mvx = bx; io->best_mvy = by;
}

/* Xin266InterBiSearch (h266_analyze_inter_cu.c:507-870) for one reference per
 * list, the default BCW weight, mvdL1Zero off (two iterations) and predictor 0:
 * the list with the larger uni cost is refined first (:580-591), each time
 * against clip(2 in - the other list's prediction) (:617-641) from the integer
 * part of its uni MV (:665-671), integer step then Xin266FullSubPelMe
 * (:676-701); the pair's cost is the SAD against the average of the two
 * predictions (pfXinComputeAvgDist, :718-729) plus both MVs' bits (:780-782),
 * kept when it improves (:784-794).  The prediction buffers keep each
 * iteration's last MV, and the final cost is taken on them (:815-852).  Ref-index,
 * predictor-index, BCW and direction bits are left out (one reference per
 * list, predictor 0).  Returns the bi pair and cost. */
static void orc_cu_bi(const orc_frame_desc *f, int32_t cu_x, int32_t cu_y, int32_t size, int32_t mnx, int32_t mny,
                      int32_t mxx, int32_t mxy, const int32_t uni[2][2], uint32_t ucost[2], int32_t bmv[2][2],
                      uint32_t *bi_cost)
{
    const opix *in_y = f->in[0] + (intptr_t)cu_y * f->in_stride[0] + cu_x;
    const intptr_t is = f->in_stride[0], rs = f->ref_stride[0];
    const opix *refo[2] = { f->ref[0], f->ref1[0] };
    const uint32_t n = (uint32_t)(size * size), lambda = f->sad_lambda;
    opix *bp[2], *tgt = (opix *)malloc(sizeof(opix) * n);
    for (int l = 0; l < 2; l++) {
        bp[l] = (opix *)malloc(sizeof(opix) * n);
        orc_luma_inter_pred(refo[l], rs, bp[l], size, uni[l][0] * 4, uni[l][1] * 4, cu_x, cu_y, mnx, mny, mxx, mxy,
                            (uint32_t)size, (uint32_t)size, 0);
        bmv[l][0] = uni[l][0]; bmv[l][1] = uni[l][1];
    }
    /* tu_mode 1 (preset 4, satdMd): the distortion of the mode decision is SATD --
     * pfXinComputeAvgDist is pfXinComputeAvgSatd (h266_encoder_create.c:3336-3345),
     * and each list's uni cost is its final prediction's SATD cost (the
     * recomputation at h266_analyze_inter_cu.c:1103-1131) */
    const int satd = f->tu_mode == 1;
    if (satd)
        for (int l = 0; l < 2; l++) {
            uint32_t d;
            orc_satd(in_y, is, bp[l], size, (uint32_t)size, (uint32_t)size, &d);
            ucost[l] = (d << 8) + (orc_mvd_bits(uni[l][0]) + orc_mvd_bits(uni[l][1])) * lambda;
        }
    int li = ucost[0] <= ucost[1] ? 1 : 0;
    uint32_t best = 0xFFFFFFFFu, sad;
    for (int it = 0; it < 2; it++, li = 1 - li) {
        orc_bi_me_input(in_y, is, bp[1 - li], size, tgt, size, (uint32_t)size, (uint32_t)size);
        const opix *ref_y = refo[li] + (intptr_t)cu_y * rs + cu_x;
        orc_me_io io;
        orc_me_square(tgt, size, ref_y, rs, (uint32_t)size, (uint32_t)size, uni[li][0] >> 2, uni[li][1] >> 2, 4, lambda,
                      mnx, mny, mxx, mxy, &io);
        orc_full_subpel_me(tgt, size, ref_y, rs, (uint32_t)size, (uint32_t)size, 0, 0, lambda, mnx, mny, mxx, mxy, &io);
        orc_luma_inter_pred(refo[li], rs, bp[li], size, io.best_mvx * 4, io.best_mvy * 4, cu_x, cu_y, mnx, mny, mxx, mxy,
                            (uint32_t)size, (uint32_t)size, 0);
        if (satd) orc_avg_satd(in_y, is, bp[0], bp[1], size, (uint32_t)size, (uint32_t)size, &sad);
        else orc_avg_sad(in_y, is, bp[0], bp[1], size, (uint32_t)size, (uint32_t)size, &sad);
        const uint32_t c = (sad << 8) + (orc_mvd_bits(io.best_mvx) + orc_mvd_bits(io.best_mvy) +
                                         orc_mvd_bits(bmv[1 - li][0]) + orc_mvd_bits(bmv[1 - li][1])) * lambda;
        if (c < best) { best = c; bmv[li][0] = io.best_mvx; bmv[li][1] = io.best_mvy; }
    }
    if (satd) orc_avg_satd(in_y, is, bp[0], bp[1], size, (uint32_t)size, (uint32_t)size, &sad);
    else orc_avg_sad(in_y, is, bp[0], bp[1], size, (uint32_t)size, (uint32_t)size, &sad);
    *bi_cost = (sad << 8) + (orc_mvd_bits(bmv[0][0]) + orc_mvd_bits(bmv[0][1]) + orc_mvd_bits(bmv[1][0]) +
                             orc_mvd_bits(bmv[1][1])) * lambda;
    free(bp[0]); free(bp[1]); free(tgt);
}

void orc_cu_hotpath(const orc_frame_desc *f, int32_t cu_x, int32_t cu_y, int32_t size,
                    ocoef *q[3], intptr_t q_stride[2], opix *rec[3], intptr_t rec_stride[2], orc_cu_out *out)
{
    int32_t mnx, mny, mxx, mxy;
    orc_mv_window(f->width, f->height, f->ctu, cu_x, cu_y, size, size, &mnx, &mny, &mxx, &mxy);
    orc_me_io io;
    orc_uni_search(f, f->ref[0], f->ref_lo, cu_x, cu_y, size, mnx, mny, mxx, mxy, &io, &out->int_cost);
    out->mvx = io.best_mvx; out->mvy = io.best_mvy; out->cost = io.best_cost;
    /* the prediction that is coded: list 0 (refs 1), or the choice among list 0,
     * list 1 and the pair (lowest cost, strict '<' in that order) */
    int32_t dir = 1, mv16[4] = { io.best_mvx * 4, io.best_mvy * 4, 0, 0 };
    if (f->refs == 2) {
        orc_me_io io1;
        orc_uni_search(f, f->ref1[0], f->ref1_lo, cu_x, cu_y, size, mnx, mny, mxx, mxy, &io1, &out->int_cost1);
        out->mvx1 = io1.best_mvx; out->mvy1 = io1.best_mvy; out->cost1 = io1.best_cost;
        const int32_t uni[2][2] = { { io.best_mvx, io.best_mvy }, { io1.best_mvx, io1.best_mvy } };
        uint32_t ucost[2] = { io.best_cost, io1.best_cost };
        int32_t bmv[2][2];
        orc_cu_bi(f, cu_x, cu_y, size, mnx, mny, mxx, mxy, uni, ucost, bmv, &out->bi_cost);
        for (int l = 0; l < 2; l++) { out->bmv[2 * l] = bmv[l][0]; out->bmv[2 * l + 1] = bmv[l][1]; }
        uint32_t best = ucost[0];
        if (ucost[1] < best) { best = ucost[1]; dir = 2; }
        if (out->bi_cost < best) dir = 3;
        if (dir == 2) { mv16[0] = io1.best_mvx * 4; mv16[1] = io1.best_mvy * 4; }
        if (dir == 3)
            for (int k = 0; k < 4; k++) mv16[k] = out->bmv[k] * 4;
        out->inter_dir = (uint32_t)dir;
    }
    const opix *lref[3] = { f->ref[0], f->ref[1], f->ref[2] };
    if (dir == 2)
        for (int p = 0; p < 3; p++) lref[p] = f->ref1[p];

    int32_t cs = size >> 1;
    opix *pred = (opix *)malloc(sizeof(opix) * (size_t)(size * size));
    ocoef *t = (ocoef *)malloc(sizeof(ocoef) * (size_t)(size * size));
    ocoef *qb = (ocoef *)malloc(sizeof(ocoef) * (size_t)(size * size));
    ocoef *r = (ocoef *)malloc(sizeof(ocoef) * (size_t)(size * size));
    if (f->tu_mode == 1) {
        orc_cu_tu_p4(f, cu_x, cu_y, size, mnx, mny, mxx, mxy, dir, mv16, q, q_stride, rec, rec_stride, pred, t, qb, r, out);
        free(pred); free(t); free(qb); free(r);
        return;
    }
    for (int pl = 0; pl < 3; pl++) {
        int32_t bs = pl ? cs : size, px = pl ? cu_x >> 1 : cu_x, py = pl ? cu_y >> 1 : cu_y;
        intptr_t istr = f->in_stride[pl ? 1 : 0], qstr = q_stride[pl ? 1 : 0], rstr = rec_stride[pl ? 1 : 0];
        if (dir == 3 && pl == 0)
            orc_luma_motion_comp_bi(f->ref[0], f->ref1[0], f->ref_stride[0], pred, bs, mv16, cu_x, cu_y, mnx, mny, mxx, mxy,
                                    (uint32_t)size, (uint32_t)size);
        else if (dir == 3)
            orc_chroma_motion_comp_bi(f->ref[pl], f->ref1[pl], f->ref_stride[1], pred, bs, mv16, cu_x, cu_y, mnx, mny, mxx,
                                      mxy, (uint32_t)size, (uint32_t)size);
        else if (pl == 0)
            orc_luma_inter_pred(lref[0], f->ref_stride[0], pred, bs, mv16[0], mv16[1], cu_x, cu_y,
                                mnx, mny, mxx, mxy, (uint32_t)size, (uint32_t)size, 0);
        else
            orc_chroma_motion_comp(lref[pl], f->ref_stride[1], pred, bs, mv16[0], mv16[1], cu_x, cu_y,
                                   mnx, mny, mxx, mxy, (uint32_t)size, (uint32_t)size);
        /* the CU's TUs: the CU itself up to the largest transform (64 luma, 32 chroma);
         * a 128 x 128 CU is four TUs per plane in raster order (the reference's implicit
         * split): its non-zero maps are OR-ed, its SSDs added */
        const int32_t tb = bs < (pl ? 32 : 64) ? bs : (pl ? 32 : 64);
        out->nz[pl] = 0;
        out->ssd[pl] = 0;
        for (int32_t oy = 0; oy < bs; oy += tb)
            for (int32_t ox = 0; ox < bs; ox += tb) {
                const opix *src = f->in[pl] + (intptr_t)(py + oy) * istr + px + ox;
                const opix *pr = pred + oy * bs + ox;
                ocoef *qo = q[pl] + (intptr_t)(py + oy) * qstr + px + ox;
                opix *ro = rec[pl] + (intptr_t)(py + oy) * rstr + px + ox;
                uint64_t nz = 0;
                orc_transform_tu(src, istr, pr, bs, t, qb, r, tb, (uint32_t)tb, (uint32_t)tb,
                                 pl ? 1u : 0u, 0, pl ? f->uv_qp : f->qp, 0, f->intra_frame, 0, 0, &nz);
                out->nz[pl] |= nz;
                for (int32_t y = 0; y < tb; y++)
                    for (int32_t x = 0; x < tb; x++) qo[y * qstr + x] = qb[y * tb + x];
                orc_idct_add(r, tb, pr, bs, ro, rstr, 0, pl ? 1u : 0u, 0, (uint32_t)tb, (uint32_t)tb, 0);
                uint64_t ssd = 0;
                for (int32_t y = 0; y < tb; y++)
                    for (int32_t x = 0; x < tb; x++) {
                        int64_t d = (int64_t)src[y * istr + x] - (int64_t)ro[y * rstr + x];
                        ssd += (uint64_t)(d * d);
                    }
                out->ssd[pl] += ssd;
            }
    }
    free(pred); free(t); free(qb); free(r);
}
