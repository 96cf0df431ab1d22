/*
 * xg_runtime.cu -- library runtime: device selection, coefficient tables,
 * per-thread error state and per-thread staging for the per-call form.
 */
#include "xg_runtime.cuh"

#include <atomic>
#include <mutex>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

int8_t  h_luma_taps[3][16][8];
int8_t  h_chroma_taps[32][4];
int16_t h_mats[8192];
int32_t h_mat_off[3][7];

static std::atomic<uint64_t> g_launches{0};
static std::once_flag g_init_once;
static int g_init_status = XIN_GPU_FAIL;
static int g_device = 0;

void xg_count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

/* ---------------------------------------------------------------- errors */
static thread_local int  t_status = XIN_GPU_OK;
static thread_local char t_msg[256] = "";

void xg_set_error(int status, const char *fmt, ...)
{
    t_status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_msg, sizeof t_msg, fmt, ap);
    va_end(ap);
}

int xg_cuda_check(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return XIN_GPU_OK;
    xg_set_error(XIN_GPU_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return XIN_GPU_ERR_CUDA;
}

/* ---------------------------------------------------------------- tables
 * H.266 interpolation filters (luma 8-tap 1/16 pel, affine 4x4 variant,
 * alternative half-pel; chroma 4-tap 1/32 pel).  Only phases up to the half
 * are written; phase P of the upper half is the mirror image of phase N - P.
 * Transform matrices: H.266 DCT-II up to 64 points and DST-VII / DCT-VIII up to
 * 32 points, generated from the standard's coefficient magnitudes and the sign
 * and index structure of each transform (see build_mats). */
static const int8_t luma_half[9][8] = {
    { 0, 0, 0, 64, 0, 0, 0, 0 }, { 0, 1, -3, 63, 4, -2, 1, 0 }, { -1, 2, -5, 62, 8, -3, 1, 0 },
    { -1, 3, -8, 60, 13, -4, 1, 0 }, { -1, 4, -10, 58, 17, -5, 1, 0 }, { -1, 4, -11, 52, 26, -8, 3, -1 },
    { -1, 3, -9, 47, 31, -10, 4, -1 }, { -1, 4, -11, 45, 34, -10, 4, -1 }, { -1, 4, -11, 40, 40, -11, 4, -1 } };
static const int8_t luma_affine_half[9][8] = {
    { 0, 0, 0, 64, 0, 0, 0, 0 }, { 0, 1, -3, 63, 4, -2, 1, 0 }, { 0, 1, -5, 62, 8, -3, 1, 0 },
    { 0, 2, -8, 60, 13, -4, 1, 0 }, { 0, 3, -10, 58, 17, -5, 1, 0 }, { 0, 3, -11, 52, 26, -8, 2, 0 },
    { 0, 2, -9, 47, 31, -10, 3, 0 }, { 0, 3, -11, 45, 34, -10, 3, 0 }, { 0, 3, -11, 40, 40, -11, 3, 0 } };
static const int8_t luma_alt_half_pel[8] = { 0, 3, 9, 20, 20, 9, 3, 0 };
static const int8_t chroma_half[17][4] = {
    { 0, 64, 0, 0 }, { -1, 63, 2, 0 }, { -2, 62, 4, 0 }, { -2, 60, 7, -1 }, { -2, 58, 10, -2 },
    { -3, 57, 12, -2 }, { -4, 56, 14, -2 }, { -4, 55, 15, -2 }, { -4, 54, 16, -2 }, { -5, 53, 18, -2 },
    { -6, 52, 20, -2 }, { -6, 49, 24, -3 }, { -6, 46, 28, -4 }, { -5, 44, 29, -4 }, { -4, 42, 30, -4 },
    { -4, 39, 33, -4 }, { -4, 36, 36, -4 } };

/* DCT-II magnitudes g(m) ~ 64*sqrt(2)*cos(m*pi/128), m = 0..64 (m = 0 only for row 0 -> 64) */
static const uint8_t dct2_mag[65] = {
    64, 91, 90, 90, 90, 90, 90, 90, 89, 88, 88, 87, 87, 86, 85, 84,
    83, 83, 82, 81, 80, 79, 78, 77, 75, 73, 73, 71, 70, 69, 67, 65,
    64, 62, 61, 59, 57, 56, 54, 52, 50, 48, 46, 44, 43, 41, 38, 37,
    36, 33, 31, 28, 25, 24, 22, 20, 18, 15, 13, 11, 9, 7, 4, 2, 0 };
/* DST-VII magnitudes a(i) ~ sin(i*pi/(2N+1)), i = 1..N */
static const uint8_t dst7_mag4[4] = { 29, 55, 74, 84 };
static const uint8_t dst7_mag8[8] = { 17, 32, 46, 60, 71, 78, 85, 86 };
static const uint8_t dst7_mag16[16] = { 8, 17, 25, 33, 40, 48, 55, 62, 68, 73, 77, 81, 85, 87, 88, 88 };
static const uint8_t dst7_mag32[32] = { 4, 9, 13, 17, 21, 26, 30, 34, 38, 42, 46, 50, 53, 56, 60, 63,
                                        66, 68, 72, 74, 77, 78, 80, 82, 84, 85, 86, 88, 88, 89, 90, 90 };

static int dct2_entry(int m)
{
    m &= 255;
    if (m <= 64) return dct2_mag[m];
    if (m <= 128) return -dct2_mag[128 - m];
    if (m <= 192) return -dct2_mag[m - 128];
    return dct2_mag[256 - m];
}

static void build_tables(void)
{
    for (int set = 0; set < 3; set++)
        for (int p = 0; p < 16; p++)
            for (int k = 0; k < 8; k++) {
                const int8_t (*half)[8] = set == 2 ? luma_affine_half : luma_half;
                int v = p <= 8 ? half[p][k] : half[16 - p][7 - k];
                if (set == 1 && p == 8) v = luma_alt_half_pel[k];
                h_luma_taps[set][p][k] = (int8_t)v;
            }
    for (int p = 0; p < 32; p++)
        for (int k = 0; k < 4; k++)
            h_chroma_taps[p][k] = p <= 16 ? chroma_half[p][k] : chroma_half[32 - p][3 - k];

    int off = 0;
    memset(h_mat_off, 0xff, sizeof h_mat_off);
    for (int lg = 1; lg <= 6; lg++) {           /* DCT2 */
        int n = 1 << lg, step = 64 / n;
        h_mat_off[0][lg] = off;
        for (int k = 0; k < n; k++)
            for (int i = 0; i < n; i++)
                h_mats[off + k * n + i] = (int16_t)(k == 0 ? 64 : dct2_entry(k * step * (2 * i + 1)));
        off += n * n;
    }
    for (int lg = 2; lg <= 5; lg++) {           /* DST7 (type 2) and DCT8 (type 1) */
        int n = 1 << lg, half = 2 * n + 1;
        const uint8_t *a = lg == 2 ? dst7_mag4 : lg == 3 ? dst7_mag8 : lg == 4 ? dst7_mag16 : dst7_mag32;
        int o7 = off, o8 = off + n * n;
        h_mat_off[2][lg] = o7;
        h_mat_off[1][lg] = o8;
        for (int k = 0; k < n; k++)
            for (int i = 0; i < n; i++) {
                int m = ((2 * k + 1) * (i + 1)) % (2 * half), v;
                if (m == 0 || m == half) v = 0;
                else if (m < half) v = a[(m <= n ? m : half - m) - 1];
                else { int mm = m - half; v = -a[(mm <= n ? mm : half - mm) - 1]; }
                h_mats[o7 + k * n + i] = (int16_t)v;
            }
        for (int k = 0; k < n; k++)
            for (int i = 0; i < n; i++)
                h_mats[o8 + k * n + i] = (int16_t)((k & 1 ? -1 : 1) * h_mats[o7 + k * n + (n - 1 - i)]);
        off += 2 * n * n;
    }
}

static void do_init(void)
{
    build_tables();
    cudaError_t e = cudaSetDevice(g_device);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_luma_taps, h_luma_taps, sizeof h_luma_taps);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_chroma_taps, h_chroma_taps, sizeof h_chroma_taps);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(d_mats, h_mats, sizeof h_mats);
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_mat_off, h_mat_off, sizeof h_mat_off);
    g_init_status = xg_cuda_check(e, "xin_gpu_init");
}

int xg_ensure_init(void)
{
    std::call_once(g_init_once, do_init);
    if (g_init_status != XIN_GPU_OK) xg_set_error(XIN_GPU_ERR_CUDA, "libxingpu: CUDA initialisation failed");
    return g_init_status;
}

/* ------------------------------------------------------------ per thread */
static thread_local XgThread *t_ctx = nullptr;

XgThread *xg_thread(void)
{
    if (xg_ensure_init() != XIN_GPU_OK) return nullptr;
    if (t_ctx) { t_ctx->dtop = 0; return t_ctx; }
    XgThread *t = new XgThread();
    t->dcap = 64u << 20;
    t->hcap = 16u << 20;
    t->dtop = 0;
    if (xg_cuda_check(cudaSetDevice(g_device), "cudaSetDevice") ||
        xg_cuda_check(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking), "cudaStreamCreate")) { delete t; return nullptr; }
    if (cudaMalloc((void **)&t->dbuf, t->dcap) != cudaSuccess || cudaMallocHost((void **)&t->hbuf, t->hcap) != cudaSuccess) {
        xg_set_error(XIN_GPU_ERR_NOMEM, "per-thread staging allocation failed");
        delete t;
        return nullptr;
    }
    t_ctx = t;
    return t;
}

void *xg_dalloc(XgThread *t, size_t bytes)
{
    size_t a = (t->dtop + 255) & ~(size_t)255;
    if (a + bytes > t->dcap) { xg_set_error(XIN_GPU_ERR_ARG, "per-call staging exhausted (%zu bytes)", bytes); return nullptr; }
    t->dtop = a + bytes;
    return t->dbuf + a;
}

void *xg_stage_in(XgThread *t, const void *src, intptr_t pitch, size_t w, size_t h, size_t esize)
{
    void *d = xg_dalloc(t, w * h * esize);
    if (!d) return nullptr;
    if (xg_cuda_check(cudaMemcpy2DAsync(d, w * esize, src, (size_t)pitch * esize, w * esize, h, cudaMemcpyHostToDevice, t->stream),
                      "stage in"))
        return nullptr;
    return d;
}

int xg_stage_out(XgThread *t, void *dst, intptr_t pitch, const void *dsrc, size_t w, size_t h, size_t esize)
{
    return xg_cuda_check(cudaMemcpy2DAsync(dst, (size_t)pitch * esize, dsrc, w * esize, w * esize, h, cudaMemcpyDeviceToHost, t->stream),
                         "stage out");
}

int xg_sync(XgThread *t)
{
    return xg_cuda_check(cudaStreamSynchronize(t->stream), "cudaStreamSynchronize");
}

/* ------------------------------------------------------------ public API */
extern "C" int xin_gpu_init(int device)
{
    if (g_init_status == XIN_GPU_OK) return XIN_GPU_OK;
    g_device = device;
    return xg_ensure_init();
}
extern "C" int xin_gpu_bitdepth(void) { return XG_BITDEPTH; }
extern "C" int xin_gpu_last_status(void) { return t_status; }
extern "C" const char *xin_gpu_last_error(void) { return t_msg; }
extern "C" void xin_gpu_clear_error(void) { t_status = XIN_GPU_OK; t_msg[0] = 0; }
extern "C" uint64_t xin_gpu_kernel_launches(void) { return g_launches.load(); }
