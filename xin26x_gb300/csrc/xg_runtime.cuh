/*
 * xg_runtime.cuh -- runtime shared by every translation unit of libxingpu:
 * per-thread error state, per-thread CUDA stream and staging buffers for the
 * per-call form, the kernel launch counter, and the coefficient tables
 * (interpolation taps in constant memory, transform matrices in global memory).
 */
#ifndef XG_RUNTIME_CUH
#define XG_RUNTIME_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "xg_config.h"
#include "../../include/xingpu.h"

/* ---- tables (defined once: the library is a single translation unit) ---- */
/* luma taps [filter set][phase][tap]: set 0 default, set 1 default except the
 * alternative half-pel filter at phase 8, set 2 affine 4x4 (the selection of
 * h266_core/source/h266_luma_mc.c:117-128) */
__constant__ int8_t c_luma_taps[3][16][8];
__constant__ int8_t c_chroma_taps[32][4];
/* transform matrices, row k = basis function k: DCT2 n = 2..64 at offsets
 * c_mat_off[0][lg], DCT8 / DST7 n = 4..32 at c_mat_off[1|2][lg] */
__device__ int16_t d_mats[8192];
__constant__ int32_t c_mat_off[3][7];

/* host copies (built once by xg_tables_init) */
extern int8_t  h_luma_taps[3][16][8];
extern int8_t  h_chroma_taps[32][4];
extern int16_t h_mats[8192];
extern int32_t h_mat_off[3][7];

/* ---- errors ------------------------------------------------------------ */
void xg_set_error(int status, const char *fmt, ...);
int  xg_cuda_check(cudaError_t e, const char *what);
int  xg_ensure_init(void);
void xg_count_launch(uint64_t n);

/* ---- per-thread per-call context --------------------------------------- */
struct XgThread {
    cudaStream_t stream;
    char  *dbuf;         /* device staging */
    size_t dcap;
    size_t dtop;         /* bump pointer, reset per call */
    char  *hbuf;         /* pinned host staging for outputs */
    size_t hcap;
};
XgThread *xg_thread(void);   /* NULL on failure (error already set) */
void *xg_dalloc(XgThread *t, size_t bytes);   /* from the bump area, 256-byte aligned; NULL if full */

/* copy a w x h window (elements of esize bytes, row pitch in elements) starting
 * at host pointer src to a packed device buffer; returns the device pointer */
void *xg_stage_in(XgThread *t, const void *src, intptr_t pitch, size_t w, size_t h, size_t esize);
int   xg_stage_out(XgThread *t, void *dst, intptr_t pitch, const void *dsrc, size_t w, size_t h, size_t esize);
int   xg_sync(XgThread *t);

#define XG_LAUNCH_CHECK(what) xg_cuda_check(cudaGetLastError(), what)

#endif
