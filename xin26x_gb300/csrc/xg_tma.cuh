/*
 * xg_tma.cuh -- tensor-memory-accelerator (TMA) tile loads into shared memory.
 *
 * Host: tensor maps over 2-D sample planes (cuTensorMapEncodeTiled, reached
 * through the runtime's driver entry point, so the library does not link the
 * driver library).  Device: an mbarrier per load group, one thread issuing
 * cp.async.bulk.tensor.2d with complete_tx, and a bounded wait.
 *
 * Alignment (checked by the callers on the host): the plane's base address
 * and row pitch are multiples of 16 bytes; the inner extent of a box is a
 * multiple of 16 bytes; every x coordinate a kernel passes is a multiple of 16
 * bytes of samples.  Coordinates outside the plane read zeros.
 */
#ifndef XG_TMA_CUH
#define XG_TMA_CUH

#include <cuda.h>
#include <mutex>

typedef CUresult (*XgTmaEncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static XgTmaEncodeFn xg_tma_encoder(void)
{
    static XgTmaEncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (XgTmaEncodeFn)p;
        else
            cudaGetLastError();
    });
    return fn;
}

/* a tensor map over a w x h plane of es-byte samples (pitch in samples) with
 * box bw x bh; false (error set) when the encoder is missing or refuses */
static bool xg_tma_map_2d(CUtensorMap *map, const void *base, int es, long long w, long long h, long long pitch, int bw, int bh)
{
    XgTmaEncodeFn enc = xg_tma_encoder();
    if (!enc) { xg_set_error(XIN_GPU_ERR_CUDA, "tensor map: cuTensorMapEncodeTiled unavailable"); return false; }
    if (((uintptr_t)base & 15) || ((pitch * es) & 15) || ((bw * es) & 15) || bw > 256 || bh > 256 || bw < 1 || bh < 1) {
        xg_set_error(XIN_GPU_ERR_ARG, "tensor map: base, pitch or box not 16-byte aligned, or box above 256");
        return false;
    }
    const cuuint64_t dims[2] = { (cuuint64_t)w, (cuuint64_t)h };
    const cuuint64_t strides[1] = { (cuuint64_t)(pitch * es) };
    const cuuint32_t box[2] = { (cuuint32_t)bw, (cuuint32_t)bh };
    const cuuint32_t estr[2] = { 1, 1 };
    const CUresult r = enc(map, es == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16, 2,
                           const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { xg_set_error(XIN_GPU_ERR_CUDA, "tensor map: encode failed (%d)", (int)r); return false; }
    return true;
}

/* ------------------------------------------------------------------ device */

__device__ __forceinline__ uint32_t xg_smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void xg_mbar_init(unsigned long long *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(xg_smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void xg_mbar_expect_tx(unsigned long long *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(xg_smem_u32(bar)), "r"(bytes) : "memory");
}

/* box at (x, y) of the map into dst (128-byte aligned), completing on bar */
__device__ __forceinline__ void xg_tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(xg_smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(xg_smem_u32(bar)) : "memory");
}

/* default bound of a wait for a TMA load: about a second */
#define XG_TMA_WAIT_TRIES (1LL << 26)

/* bounded wait for phase `parity` of bar; false after `tries` polls */
__device__ __forceinline__ bool xg_mbar_wait(unsigned long long *bar, uint32_t parity, long long tries)
{
    uint32_t done = 0;
    for (long long it = 0; it < tries && !done; it++)
        asm volatile("{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n\tselp.u32 %0, 1, 0, q;\n\t}"
                     : "=r"(done) : "r"(xg_smem_u32(bar)), "r"(parity) : "memory");
    return done != 0;
}

#endif
