/*
 * xingpu.h -- C ABI of libxingpu: the xin26x VVC encoder pixel hot path on a
 * GB300 GPU (sm_103a).
 *
 * Three layers, all plain C with host pointers and sizes:
 *
 *  1. Per-call functions ("plain per-call GPU form").  Each has exactly the
 *     signature of the reference function-pointer type it replaces, so it can
 *     be stored in the reference's tables xin_func_struct
 *     (h266_encoder/include/h266_func_struct.h:719-799) and xin_me_func
 *     (h26x_core/include/h26x_me_func_struct.h:174-191).  Arguments are host
 *     pointers; every call copies its inputs to the GPU, runs one kernel, copies
 *     the outputs back and synchronises.  The reference types return void and
 *     have no error channel, so failures are reported through
 *     xin_gpu_last_status() / xin_gpu_last_error() (per calling thread) and the
 *     outputs are left untouched.  Calls are re-entrant: each host thread gets
 *     its own CUDA stream and staging buffers.
 *
 *  2. Motion-estimation drivers taking the reference's xin_me_struct
 *     (h26x_core/include/h26x_me_struct.h:60-131, mirrored in xingpu_me.h).
 *
 *  3. The batched frame form: a stream handle keeps reference pictures, padded
 *     planes, quarter-pel planes and outputs resident on the GPU and runs the
 *     whole hot path of a picture (integer search, sub-pel search, motion
 *     compensation, transform, quantisation, reconstruction for every CU of
 *     every quadtree level) as a few launches captured in a CUDA graph.
 *
 * PIXEL / COEFF follow the reference's compile switch ENABLE_10BIT_ENCODER
 * (video_api/video_common/include/xin_typedef.h:72-96): libxingpu8.so is the
 * 8-bit build, libxingpu10.so the 10-bit build.
 *
 * Status codes mirror XIN_SUCCESS / XIN_FAIL (xin_typedef.h:36-37): 0 is
 * success, negative values are errors.
 */
#ifndef XINGPU_H
#define XINGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifdef ENABLE_10BIT_ENCODER
typedef uint16_t XG_PIXEL;
typedef int32_t  XG_COEFF;
#else
typedef uint8_t  XG_PIXEL;
typedef int16_t  XG_COEFF;
#endif

/* ---------------------------------------------------------------- status */
#define XIN_GPU_OK            0
#define XIN_GPU_FAIL         -1   /* generic failure (XIN_FAIL) */
#define XIN_GPU_ERR_ARG      -2   /* invalid argument (size, stride, pointer) */
#define XIN_GPU_ERR_CUDA     -3   /* CUDA runtime error; message in xin_gpu_last_error() */
#define XIN_GPU_ERR_NOMEM    -4   /* device or pinned allocation failed */
#define XIN_GPU_ERR_TIMEOUT  -5   /* wait limit reached */
#define XIN_GPU_ERR_STATE    -6   /* call not valid in the current state */
#define XIN_GPU_ERR_ADMIT    -7   /* serving: not enough device memory to admit */

int         xin_gpu_init(int device);          /* select the CUDA device; idempotent */
int         xin_gpu_bitdepth(void);            /* 8 or 10: the build of this library */
int         xin_gpu_last_status(void);         /* status of this thread's last call */
const char *xin_gpu_last_error(void);          /* message of this thread's last failure */
void        xin_gpu_clear_error(void);
uint64_t    xin_gpu_kernel_launches(void);     /* kernels launched by this library so far */

/* ------------------------------------------------------ distortion (a2-a6)
 * replaces Xin26xComputeSad / Sadx8 / Sadx5 / Sadx3 / AvgSad / AvgSadx8 /
 * Satd / AvgSatd / WeightSad / WeightSatd / Var / AvgVar / ComputeHada8x8
 * (h26x_core/include/h26x_compute_dist.h:27-1096); typedefs XinComputeDist,
 * XinComputeAvgDist, XinComputeWeightDist, XinComputeSadx8/x5/x3,
 * XinComputeAvgSadx8, XinComputeHada8x8 (h266_func_struct.h:56-128,459). */
void XinGpuComputeSad(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *pred, intptr_t predStride,
                      uint32_t width, uint32_t height, uint32_t *sad);
void XinGpuComputeSatd(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *pred, intptr_t predStride,
                       uint32_t width, uint32_t height, uint32_t *satd);
void XinGpuComputeAvgSad(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *refA, XG_PIXEL *refB, intptr_t refStride,
                         uint32_t width, uint32_t height, uint32_t *sad);
void XinGpuComputeAvgSatd(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *refA, XG_PIXEL *refB, intptr_t refStride,
                          uint32_t width, uint32_t height, uint32_t *satd);
void XinGpuComputeWeightSad(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *refA, XG_PIXEL *refB, intptr_t refStride,
                            uint32_t width, uint32_t height, int32_t weightA, int32_t weightB, uint32_t *sad);
void XinGpuComputeWeightSatd(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *refA, XG_PIXEL *refB, intptr_t refStride,
                             uint32_t width, uint32_t height, int32_t weightA, int32_t weightB, uint32_t *satd);
void XinGpuComputeSadx8(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *ref[8], intptr_t refStride,
                        uint32_t width, uint32_t height, uint32_t *sad);
void XinGpuComputeSadx5(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *ref0, XG_PIXEL *ref1, XG_PIXEL *ref2,
                        XG_PIXEL *ref3, XG_PIXEL *ref4, intptr_t refStride, uint32_t width, uint32_t height, uint32_t *sad);
void XinGpuComputeSadx3(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *ref0, XG_PIXEL *ref1, XG_PIXEL *ref2,
                        intptr_t refStride, uint32_t width, uint32_t height, uint32_t *sad);
void XinGpuComputeAvgSadx8(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *refA[8], XG_PIXEL *refB[8],
                           intptr_t refStride, uint32_t width, uint32_t height, uint32_t *sad);
void XinGpuComputeVar(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *pred, intptr_t predStride,
                      uint32_t width, uint32_t height, uint32_t *var);
void XinGpuComputeAvgVar(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *predA, XG_PIXEL *predB, intptr_t predStride,
                         uint32_t width, uint32_t height, uint32_t *var);
void XinGpuComputeHada8x8(XG_PIXEL *input, intptr_t inputStride, uint32_t *satd);

/* ----------------------------------------------- interpolation (a10-a12)
 * replaces Xin266InterpCopy, Xin266LumaInterpHor/Vet/HorVet and the U8S16 /
 * S16U8 / S16S16 stages (h266_core/source/h266_luma_mc.c:72-630),
 * Xin266ChromaInterp* (h266_core/source/h266_chroma_mc.c:62-386),
 * Xin266InterpAvgS16U8 / Xin266InterpWeightS16U8 (h266_luma_mc.c:561,595);
 * typedefs XinMotionInterp, XinMotionInterpS16, XinMotionInterpAvg,
 * XinMotionInterpWeight (h266_func_struct.h:130-179).  Luma frac = fy << 4 | fx
 * (1/16 pel), chroma frac = fy << 5 | fx (1/32 pel); filterIndex 0 default,
 * 1 alternative half-pel, 2 affine 4x4. */
#define XG_INTERP_ARGS(SRC_T, DST_T) const SRC_T *src, intptr_t srcStride, DST_T *dst, intptr_t dstStride, \
                                     int32_t frac, uint32_t width, uint32_t height, uint32_t filterIndex
void XinGpuInterpCopy(XG_INTERP_ARGS(XG_PIXEL, XG_PIXEL));
void XinGpuInterpCopyU8S16(XG_INTERP_ARGS(XG_PIXEL, int16_t));
void XinGpuLumaInterpHor(XG_INTERP_ARGS(XG_PIXEL, XG_PIXEL));
void XinGpuLumaInterpVet(XG_INTERP_ARGS(XG_PIXEL, XG_PIXEL));
void XinGpuLumaInterpHorVet(XG_INTERP_ARGS(XG_PIXEL, XG_PIXEL));
void XinGpuLumaInterpHorU8S16(XG_INTERP_ARGS(XG_PIXEL, int16_t));
void XinGpuLumaInterpVetU8S16(XG_INTERP_ARGS(XG_PIXEL, int16_t));
void XinGpuLumaInterpHorVetU8S16(XG_INTERP_ARGS(XG_PIXEL, int16_t));
void XinGpuLumaInterpVetS16U8(XG_INTERP_ARGS(int16_t, XG_PIXEL));
void XinGpuLumaInterpVetS16S16(XG_INTERP_ARGS(int16_t, int16_t));
void XinGpuChromaInterpHor(XG_INTERP_ARGS(XG_PIXEL, XG_PIXEL));
void XinGpuChromaInterpVet(XG_INTERP_ARGS(XG_PIXEL, XG_PIXEL));
void XinGpuChromaInterpHorVet(XG_INTERP_ARGS(XG_PIXEL, XG_PIXEL));
void XinGpuChromaInterpHorU8S16(XG_INTERP_ARGS(XG_PIXEL, int16_t));
void XinGpuChromaInterpVetU8S16(XG_INTERP_ARGS(XG_PIXEL, int16_t));
void XinGpuChromaInterpHorVetU8S16(XG_INTERP_ARGS(XG_PIXEL, int16_t));
void XinGpuChromaInterpVetS16U8(XG_INTERP_ARGS(int16_t, XG_PIXEL));
void XinGpuChromaInterpVetS16S16(XG_INTERP_ARGS(int16_t, int16_t));
/* bilinear DMVR prediction, typedef XinBiliInterp, table entry
 * pfXinBiliInterp[!!fx][!!fy][lgW] (h266_encoder/include/h266_func_struct.h:150,741;
 * h266_core/source/h266_bilinear_filter.c:46-260):
 * frac = fy << 4 | fx (1/16 pel), taps {16 - f, f}, 10-bit intermediate; each
 * writes h rows of w + 4 int16 samples (DMVR_PADING_SIZE extra columns). */
void XinGpuBiliInterpCopy(const XG_PIXEL *src, intptr_t srcStride, int16_t *dst, intptr_t dstStride, int32_t frac,
                          uint32_t width, uint32_t height);
void XinGpuBiliInterpHor(const XG_PIXEL *src, intptr_t srcStride, int16_t *dst, intptr_t dstStride, int32_t frac,
                         uint32_t width, uint32_t height);
void XinGpuBiliInterpVet(const XG_PIXEL *src, intptr_t srcStride, int16_t *dst, intptr_t dstStride, int32_t frac,
                         uint32_t width, uint32_t height);
void XinGpuBiliInterpHorVet(const XG_PIXEL *src, intptr_t srcStride, int16_t *dst, intptr_t dstStride, int32_t frac,
                            uint32_t width, uint32_t height);
void XinGpuInterpAvgS16U8(const int16_t *src0, intptr_t src0Stride, const int16_t *src1, intptr_t src1Stride,
                          XG_PIXEL *dst, intptr_t dstStride, uint32_t width, uint32_t height);
void XinGpuInterpWeightS16U8(const int16_t *src0, intptr_t src0Stride, const int16_t *src1, intptr_t src1Stride,
                             XG_PIXEL *dst, intptr_t dstStride, uint32_t width, uint32_t height,
                             int32_t weightA, int32_t weightB);

/* ------------------------------------------------------- transforms (a14-a19)
 * 1-D forward: replaces Xin26xFDct2P2..P64, Xin26xFDst7P4..P32, Xin26xFDct8P4..P32
 * (h26x_core/include/h26x_forward_1d_trans.h), typedef XinFor1dDct
 * (h266_func_struct.h:198).  1-D inverse: replaces Xin26xIDct2P2..P64,
 * Xin26xIDst7P4..P32, Xin26xIDct8P4..P32 (h26x_core/include/h26x_inverse_1d_trans.h),
 * typedef XinInv1dDct (h266_func_struct.h:280). */
#define XG_FDCT1D(NAME) void NAME(XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride, \
                                  int32_t line, int32_t shift)
#define XG_IDCT1D(NAME) void NAME(XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride, \
                                  int32_t line, int32_t skipLine, int32_t shift)
XG_FDCT1D(XinGpuFDct2P2); XG_FDCT1D(XinGpuFDct2P4); XG_FDCT1D(XinGpuFDct2P8); XG_FDCT1D(XinGpuFDct2P16);
XG_FDCT1D(XinGpuFDct2P32); XG_FDCT1D(XinGpuFDct2P64);
XG_FDCT1D(XinGpuFDst7P4); XG_FDCT1D(XinGpuFDst7P8); XG_FDCT1D(XinGpuFDst7P16); XG_FDCT1D(XinGpuFDst7P32);
XG_FDCT1D(XinGpuFDct8P4); XG_FDCT1D(XinGpuFDct8P8); XG_FDCT1D(XinGpuFDct8P16); XG_FDCT1D(XinGpuFDct8P32);
XG_IDCT1D(XinGpuIDct2P2); XG_IDCT1D(XinGpuIDct2P4); XG_IDCT1D(XinGpuIDct2P8); XG_IDCT1D(XinGpuIDct2P16);
XG_IDCT1D(XinGpuIDct2P32); XG_IDCT1D(XinGpuIDct2P64);
XG_IDCT1D(XinGpuIDst7P4); XG_IDCT1D(XinGpuIDst7P8); XG_IDCT1D(XinGpuIDst7P16); XG_IDCT1D(XinGpuIDst7P32);
XG_IDCT1D(XinGpuIDct8P4); XG_IDCT1D(XinGpuIDct8P8); XG_IDCT1D(XinGpuIDct8P16); XG_IDCT1D(XinGpuIDct8P32);

/* 2-D DCT2: replaces Xin26xFDct2WxH (XinFor2dDct2, h266_func_struct.h:206) and
 * Xin266IDct2WxH (XinInv2dDct2, :269; h266_encoder/source/h266_inverse_trans.c:52).
 * tempBuf is accepted for signature compatibility and not used. */
void XinGpuFDct2WxH(XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride,
                    uint32_t width, uint32_t height, XG_COEFF *tempBuf, int32_t shift1st, int32_t shift2nd);
void XinGpuIDct2WxH(XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride,
                    uint32_t width, uint32_t height, XG_COEFF *tempBuf, int32_t shift1st, int32_t shift2nd);
/* Allocation-free variant of XinGpuFDct2WxH; no counterpart in the reference.
 * For callers that cannot call cudaMalloc (a real-time host thread, where
 * cudaMalloc may synchronise the device; code recording a CUDA graph; a fixed
 * memory budget): input and output are device pointers, the work is queued on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and the call returns
 * without waiting.  The intermediate between the two 1-D passes lives in a
 * file-scope device array of 64 x 64 coefficients (held by every GPU that loads
 * the library until exit); larger blocks are rejected with XIN_GPU_ERR_ARG.
 * xin_gpu_init must have been called (XIN_GPU_ERR_STATE otherwise: this entry
 * point never initialises the library itself), and the current device must be
 * the one given to it (XIN_GPU_ERR_STATE otherwise).  The first call on a
 * device looks up that array's device address; it must come before any stream
 * capture (XIN_GPU_ERR_STATE if `stream` is capturing then).  All calls share
 * the array, so calls that overlap on the GPU race; serialise them. */
int  xin_gpu_fdct2_wxh_noalloc(const XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride,
                               uint32_t width, uint32_t height, int32_t shift1st, int32_t shift2nd, void *stream);
/* transform skip: replaces Xin26xFSkipWxH (XinFor2dSkip, :217) and Xin266ISkipWxH
 * (XinInv2dSkip, :635; h266_inverse_trans.c:91) */
void XinGpuFSkipWxH(XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride,
                    uint32_t width, uint32_t height, XG_COEFF *tempBuf);
void XinGpuISkipWxH(XG_COEFF *input, intptr_t inputStride, XG_COEFF *output, intptr_t outputStride,
                    uint32_t width, uint32_t height);
/* residual / reconstruction: replaces Xin26xBlockSubForDct (XinBlockSubForDct, :520) and
 * Xin26xBlockRecon (XinBlockAddForDct, :530) */
void XinGpuBlockSubForDct(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *recon, intptr_t reconStride,
                          XG_COEFF *diff, intptr_t diffStride, uint32_t width, uint32_t height);
void XinGpuBlockAddForDct(XG_COEFF *input, intptr_t inputStride, XG_PIXEL *pred, intptr_t predStride,
                          XG_PIXEL *recon, intptr_t reconStride, uint32_t width, uint32_t height);

/* ----------------------------------------------------------- quant (a16-a17)
 * replaces Xin266QuantInvQuant (XinQuantInvQuant, h266_func_struct.h:181;
 * h266_encoder/source/h266_quant_inv_quant.c:80) and Xin266PreRdoq (XinPreRdoq,
 * :622; h266_quant_inv_quant.c:208).  xin_gpu_scan_pos has the layout of
 * xin_scan_pos (h266_encoder/include/h266_trans_unit_struct.h:23-28). */
typedef struct xin_gpu_scan_pos { uint32_t posX, posY, posIdx; } xin_gpu_scan_pos;
void XinGpuQuantInvQuant(XG_COEFF *qCoeff, XG_COEFF *tCoeff, XG_COEFF *rCoeff, intptr_t coeffStride,
                         uint32_t width, uint32_t height, uint32_t cGWidth, uint32_t cGHeight,
                         int32_t qMult, int32_t qAdd, int32_t qShift, int32_t iqMult, int32_t iqAdd, int32_t iqShift,
                         uint64_t *nzCGBitMapRs);
void XinGpuPreRdoq(XG_COEFF *tCoeff, XG_COEFF *rCoeff, XG_COEFF *qCoeff, intptr_t coeffStride,
                   uint32_t width, uint32_t height, uint32_t cGWidth, uint32_t cGHeight, int32_t rdoqThrVal,
                   xin_gpu_scan_pos *scanOrderCG, uint64_t *nzCGBitMapRs);

/* ------------------------------------------------ batched transform / quant
 * Many residual blocks of mixed sizes and transform types in one call: per
 * block the TU arithmetic of Xin266Transform (h266_encoder/source/h266_trans_quant.c:61;
 * forward DCT2 / DST7 / DCT8 / skip by MTS index with the implicit-MTS rule of
 * h266_forward_trans.c:75-86, zero-out beyond 32, quant / dequant with 4x4
 * coding groups, no dependent quantisation or pre-RDOQ) followed by
 * Xin266IDctWxH (h266_inverse_trans.c:117).  Block b reads resid[offset ..
 * offset + w*h) (row-major, stride w) and writes q, r (dequantised) and
 * resid_out (inverse-transformed r) at the same offsets, nz[b] = non-zero-CG map.
 * tile: -1 autotune the thread-group size per block-size class (timed on the
 * first call for each class, then cached), 0 fixed heuristic, or 32/64/128/256. */
typedef struct xin_gpu_tq_block {
    uint32_t offset;            /* element offset of the block in every array */
    uint8_t  log2w, log2h;      /* 2..6 (skip, DST7 / DCT8: 2..5) */
    uint8_t  mts;               /* 0 DCT2, 1 transform skip, 2 DST7/DST7, 3 DCT8/DST7, 4 DST7/DCT8, 5 DCT8/DCT8 */
    uint8_t  flags;             /* XIN_GPU_TQ_* */
    int32_t  qp;                /* slice QP 0..63 (the 10-bit build adds 12 internally) */
} xin_gpu_tq_block;
#define XIN_GPU_TQ_INTRA_CU     1u   /* intra CU: implicit MTS for luma DCT2 when MTS is enabled */
#define XIN_GPU_TQ_CHROMA       2u
#define XIN_GPU_TQ_RDOQ_ROUND   4u   /* qAdd = 1 << (qShift - 1) (RDOQ enabled) */
#define XIN_GPU_TQ_INTRA_PIC    8u   /* qAdd = 171 << (qShift - 9) instead of 85 << (qShift - 9) */
#define XIN_GPU_TQ_MTS_ENABLED 16u
/* tile: the CUDA-core kernel's thread-group size (-1 autotune, 0 fixed, 32..256),
 * or XIN_GPU_TQ_TENSOR: transform passes on the tensor cores (tcgen05, exact
 * f16 halves, f32 accumulation), transform-skip blocks on the CUDA cores; the
 * tensor form needs the four coefficient arrays 16-byte aligned */
#define XIN_GPU_TQ_TENSOR      (-2)
/* host arrays of ncoeffs samples; samples that no block covers are returned as zeros */
int  xin_gpu_tq_batch(const xin_gpu_tq_block *blocks, int32_t nblocks, const XG_COEFF *resid, XG_COEFF *q, XG_COEFF *r,
                      XG_COEFF *resid_out, uint64_t *nz, size_t ncoeffs, int32_t tile);
/* the same on device arrays (blocks stay a host array); tiles_used (optional,
 * 49 entries indexed log2w * 7 + log2h) reports the group size of each class */
int  xin_gpu_tq_batch_device(const xin_gpu_tq_block *blocks, int32_t nblocks, const XG_COEFF *resid, XG_COEFF *q,
                             XG_COEFF *r, XG_COEFF *resid_out, uint64_t *nz, size_t ncoeffs, int32_t tile, void *stream,
                             int32_t *tiles_used);
/* A plan keeps a validated block list, sorted by size class, on the device so
 * that one list can run on new residuals without host work: run only enqueues
 * launches on `stream` (device arrays).  Runs of one plan must not overlap in
 * time (the tensor form's tile queue and timeout flag belong to the plan):
 * enqueue them on one stream, or create a plan per stream.  With tile -1 the first run of a class
 * not tuned yet times the candidates and synchronises; later runs are
 * asynchronous.  tiles: 49 entries, 0 for classes not resolved yet. */
typedef struct xin_gpu_tq_plan xin_gpu_tq_plan;
int  xin_gpu_tq_plan_create(const xin_gpu_tq_block *blocks, int32_t nblocks, size_t ncoeffs, int32_t tile,
                            xin_gpu_tq_plan **plan);
int  xin_gpu_tq_plan_run(xin_gpu_tq_plan *plan, const XG_COEFF *resid, XG_COEFF *q, XG_COEFF *r, XG_COEFF *resid_out,
                         uint64_t *nz, void *stream);
int  xin_gpu_tq_plan_tiles(const xin_gpu_tq_plan *plan, int32_t *tiles);
/* synchronises; XIN_GPU_ERR_TIMEOUT if a tensor-core wait of a run since the
 * last status call gave up (the outputs of that run are not valid; the flag is
 * cleared by this call) */
int  xin_gpu_tq_plan_status(xin_gpu_tq_plan *plan);
/* Polls of one tensor-core wait before it gives up (default 2^26, about a
 * second).  A wait that gives up sets the plan's timeout flag, waits (bounded
 * by the default) for its MMA to finish, releases its tensor memory and ends its
 * CTA.  0 makes every wait give up at once: a way to exercise that path. */
int  xin_gpu_tq_plan_set_wait_tries(xin_gpu_tq_plan *plan, int64_t tries);
void xin_gpu_tq_plan_destroy(xin_gpu_tq_plan *plan);

/* ---------------------------------------------------- dependent quantisation
 * The trellis quantiser Xin266DepQuant (h266_encoder/source/h266_dep_quant.c:1789,
 * table entry pfXinDepQuant, h266_encoder/include/h266_func_struct.h:664-676,795)
 * on batches of transform blocks.  Rates come from CABAC context states in the
 * reference's layout: a context set is the array xin_prob_model[XIN_NUM_OF_CTX]
 * of the encoder's cabac context (h266_encoder/include/h266_cabac_struct.h:225-235),
 * 6-byte records.  Block b reads t at offset (row stride `stride`) and writes
 * q (signed levels) and r (dequantised) at the same places over the whole
 * w x h block (zeros beyond the low 32 x 32), nz[b] = map of non-zero 4x4
 * groups (raster order of the low 32 x 32 region).  Bit-exact with the
 * reference's C for every block size 4..64, QP 0..51 and component. */
typedef struct xin_gpu_prob { uint16_t state[2]; uint8_t rate; } xin_gpu_prob;    /* xin_prob_model */
#define XIN_GPU_NUM_CTX 401                                                        /* XIN_NUM_OF_CTX */
typedef struct xin_gpu_dq_block {
    uint32_t offset;            /* element offset of the block's top-left coefficient in t, q and r */
    uint16_t stride;            /* elements between rows (>= w) */
    uint8_t  log2_w, log2_h;    /* 2..6 */
    uint8_t  qp;                /* 0..51: the QP the reference passes (10-bit: slice QP + 12, h266_trans_quant.c:104) */
    uint8_t  comp;              /* 0 luma, 1 Cb, 2 Cr */
    uint8_t  root_cbf;          /* luma of an inter CU coded as one TU: the cbf rate is the root cbf's */
    uint8_t  reserved;
    uint32_t ctx_set;           /* index of the block's context set */
} xin_gpu_dq_block;
/* host arrays: t, q, r hold ncoeffs samples, ctx_sets nsets x XIN_GPU_NUM_CTX records */
int  xin_gpu_dep_quant_batch(const xin_gpu_dq_block *blocks, int32_t nblocks, const XG_COEFF *t, XG_COEFF *q, XG_COEFF *r,
                             uint64_t *nz, size_t ncoeffs, const xin_gpu_prob *ctx_sets, int32_t nsets);
/* device arrays (blocks stay a host array); synchronises */
int  xin_gpu_dep_quant_batch_device(const xin_gpu_dq_block *blocks, int32_t nblocks, const XG_COEFF *t, XG_COEFF *q,
                                    XG_COEFF *r, uint64_t *nz, size_t ncoeffs, const xin_gpu_prob *ctx_sets,
                                    int32_t nsets, void *stream);
/* a plan keeps a validated block list on the device; run only enqueues on
 * `stream` (device arrays, device context sets) */
typedef struct xin_gpu_dq_plan xin_gpu_dq_plan;
int  xin_gpu_dq_plan_create(const xin_gpu_dq_block *blocks, int32_t nblocks, size_t ncoeffs, int32_t nsets,
                            xin_gpu_dq_plan **plan);
int  xin_gpu_dq_plan_run(xin_gpu_dq_plan *plan, const XG_COEFF *t, XG_COEFF *q, XG_COEFF *r, uint64_t *nz,
                         const xin_gpu_prob *ctx_sets, void *stream);
void xin_gpu_dq_plan_destroy(xin_gpu_dq_plan *plan);
/* Per-call form with the XinDepQuant signature.  It reads three fields of the
 * reference's structures: xin_dep_quant.context, xin_fast_md_buf.type and
 * .fullBuf, xin_full_md_buf.tuNum (h266_encoder/include/h266_dep_quant_struct.h:135,
 * h266_md_buffer_struct.h:65,71,109); tu is not read (standard scans).  A Cr
 * block's rates are built from the current contexts (the reference reuses the
 * tables of its previous call, the Cb block of the same TU, h266_dep_quant.c:296). */
#define XIN_GPU_DQ_CONTEXT_OFFSET      8
#define XIN_GPU_FASTBUF_FULLBUF_OFFSET 0
#define XIN_GPU_FASTBUF_TYPE_OFFSET    880
#define XIN_GPU_FULLBUF_TUNUM_OFFSET   2184
#define XIN_GPU_INTRA_MODE             3      /* XIN_INTRA_MODE */
void XinGpuDepQuant(void *depQuant, void *fastBuf, void *tu, XG_COEFF *tCoeff, XG_COEFF *rCoeff, XG_COEFF *qCoeff,
                    intptr_t coeffStride, uint32_t qp, int32_t width, int32_t height, uint64_t *nzCGBitMapRs,
                    uint32_t compId);

/* ------------------------------------------------------- motion search (a7-a8)
 * xin_me_struct is the reference's ME state (h26x_core/include/h26x_me_struct.h:60-131);
 * xingpu_me.h mirrors its layout.  Pass a pointer to the reference's struct.
 *
 * XinGpuMotionEstFull: stands in for Xin26xMotionEstFull (h26x_motion_est.h:23-36):
 *   exhaustive integer search of every MV within searchWidth x searchHeight of
 *   predMv >> 2, clipped to [minMv, maxMv], raster order, strict '<' on
 *   (SAD << 8) + (bits(mvd_x) + bits(mvd_y)) * sadLambda; starts from bestMv /
 *   bestCost; writes bestMv (quarter-pel), bestCost, bestSad.
 * XinGpuFullSubPelMe: the search of Xin266FullSubPelMe
 *   (h266_encoder/source/h266_sub_pel_refine.c:81), reading its inputs from the
 *   ME state instead of the section state. */
struct xin_me_struct;
void XinGpuMotionEstFull(struct xin_me_struct *meSet);
void XinGpuFullSubPelMe(struct xin_me_struct *meSet);

/* ------------------------------------------- fast sub-pel by variance (a9)
 * XinGpuFastSubPelMeVar: Xin266FastSubPelMeVar (h266_encoder/source/h266_sub_pel_refine.c:214-361),
 *   the same signature, on the ME state: the eight half-pel neighbours of the
 *   integer start (bestMv, quarter-pel, a multiple of 4) by the variance of the
 *   difference, then without AMVR (iMvMode 0) the eight quarter-pel neighbours
 *   of the best, each predicted by the rounded average of two half-grid samples
 *   (the pairing of the reference's qBufA / qBufB, h266_create_section.c:97-230);
 *   cost (variance << 8) + (sseLambda * bits << 15 + 2^22) >> 23, strict '<'.
 *   Writes bestMv and bestPos (as the reference, not bestCost); returns unchanged
 *   when the start is outside [minMv, maxMv].  It computes its half-pel samples
 *   itself: the ME state's interpolation buffers are neither read nor written.
 * XinGpuInterpoHalfPel: pfXinInterpoHalfPel (typedef XinInterpHalfPel,
 *   h26x_core/include/h26x_me_func_struct.h:143; closed in the reference,
 *   restated with the luma filter's half-pel phase, the alternative half-pel
 *   filter when interpAlt): the integer, horizontal, vertical and diagonal
 *   half-pel planes of the block in the layout the ME state's pointers assume
 *   (h266_create_section.c:74-86). */
struct xin_me_struct;
void XinGpuFastSubPelMeVar(struct xin_me_struct *meSet, int32_t listIdx, int32_t refIdx);
void XinGpuInterpoHalfPel(XG_PIXEL *ref, intptr_t refStride, uint32_t width, uint32_t height, XG_PIXEL *integPel,
                          XG_PIXEL *halfPelH, XG_PIXEL *halfPelV, XG_PIXEL *halfPelHv, intptr_t interpStride,
                          int32_t interpAlt);

/* ---------------------------------------- search by resolution levels (a7)
 * The reference's hierarchical search (motionSearchMode 2, the preset-4/6
 * default; h266_encoder/source/h266_analyze_inter_cu.c:1063-1067) and its
 * helpers exist only in the closed library; their order is restated here (the
 * oracle states the same, parity unpinned).
 *
 * XinGpuDownscale2x2: stands in for Xin26xDownscale2x2 (typedef XinDownscale2x2,
 *   h266_encoder/include/h266_func_struct.h:425; table entries
 *   xin_func_struct.pfXinDownscale2x2 and xin_me_func.pfXinDownscale2x2).
 *   out(x, y) = (a + b + c + d + 2) >> 2 over the 2x2 input block at (2x, 2y).
 *   The row flags must be 0, as every open caller passes them
 *   (h266_enc_init.c:2804-2824, h266_scene_cut.c:64); else XIN_GPU_ERR_ARG.
 * XinGpuMotionSearchHier: stands in for Xin26xMotionSearchHier1 / 2 (typedef
 *   XinHierMotionSearch, h266_func_struct.h:435; xin_me_func.pfXinMotionSearchHier1/2,
 *   h26x_core/include/h26x_hierarchic_motion_search.h:29,42): the SAD of every MV
 *   of [minMvX, maxMvX] x [minMvY, maxMvY] (units of the level), raster order,
 *   strict '<'; writes the best to *bestMv (a xin_mv_u); an empty window
 *   leaves it unchanged.
 * XinGpuMotionEstHier: stands in for Xin26xMotionEstHier (h26x_motion_est.h:23-36)
 *   on the ME state (input1/ref1 at 1/2, input2/ref2 at 1/4 resolution):
 *     window  [c - searchWidth, c + searchWidth] x [c - searchHeight, ...] within
 *             [minMv, maxMv], c = predMv >> 2; at level L its ends become
 *             ceil(lo / 2^L) and floor(hi / 2^L)
 *     start   bestMv / bestCost as given, then meCand[0 .. candNum) (quarter-pel,
 *             >> 2, clipped to the window) with the full cost, strict '<'
 *     1/4     exhaustive SAD over the level window, block (w/4) x (h/4)
 *     1/2     +-1 around twice the 1/4 best, block (w/2) x (h/2)
 *     full    3 x 3 around twice the 1/2 best, cost (SAD << 8) +
 *             (bits(mvd x) + bits(mvd y)) * sadLambda, strict '<'
 *   writes bestMv (quarter-pel), bestCost, bestSad.  width and height are
 *   multiples of 4. */
void XinGpuDownscale2x2(XG_PIXEL *input, intptr_t inputStride, int32_t haveRowAbove, int32_t haveRowBelow,
                        XG_PIXEL *output, intptr_t outputStride, uint32_t outWidth, uint32_t outHeight);
void XinGpuMotionSearchHier(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *ref, intptr_t refStride, int32_t minMvX,
                            int32_t maxMvX, int32_t minMvY, int32_t maxMvY, uint32_t width, uint32_t height, void *bestMv);
void XinGpuMotionEstHier(struct xin_me_struct *meSet);

/* ------------------------------------------------------------------- DMVR
 * The encoder's emulation of the H.266 decoder-side MV refinement of a
 * bi-predicted CU (Xin266LumaMotionCompDmvr with Xin266DeriveMvFromDmvr and
 * Xin266SubPelRefineDmvr, h266_encoder/source/h266_inter_prediction.c:864-1420),
 * and the table entries it calls.
 *
 * XinGpuLumaMotionCompDmvr: the arguments of Xin266LumaMotionCompDmvr unpacked
 *   from the section state: ref0 / ref1 are the L0 / L1 reference pictures
 *   (pointers at picture (0, 0) inside their padding, pictureRead[list][refIdx]
 *   ->refBuf[PLANE_LUMA]), (cuX, cuY) the CU position, [minMv, maxMv] the CU's
 *   window (secSet->minMv / maxMv, full-pel), mv the L0 and L1 MVs (1/16 pel, x, y
 *   pairs).  Per 16 x 16 sub-block (raster order): bilinear predictions of both
 *   lists, the 5 x 5 integer search on row-subsampled SADs (L0 moved by +d, L1
 *   by -d), the parabolic sub-pel offset; then the refined 8-tap bi-prediction.
 *   Writes pred (width x height) and mvdL0SubPu (x, y pairs of 1/16-pel L0
 *   refinements, one per sub-block; xin_mv_s).  width, height: powers of two
 *   8..128.
 * XinGpuComputeSadS16: pfXinComputeSadS16 (typedef XinComputeDistS16,
 *   h266_func_struct.h:540; the closed Xin26xComputeSadS16, restated): the SAD of
 *   int16 blocks over every (1 << subShift)-th row, times 1 << subShift.
 * XinGpuCopyAndPad / XinGpuCopyAndPadUv: pfXinCopyAndPad / pfXinCopyAndPadUv
 *   (typedefs XinCopyAndPad / XinCopyAndPadUv, h266_func_struct.h:604,612;
 *   h266_encoder/source/h266_copy_and_pad.c:32-112): the region an 8-tap (4-tap)
 *   filter reads around a w x h block, padded by 2 (1) samples on every side by
 *   repeating its edge (the closed Xin26xBlockPad2/1, restated). */
void XinGpuLumaMotionCompDmvr(const XG_PIXEL *ref0, const XG_PIXEL *ref1, intptr_t refStride, int32_t cuX, int32_t cuY,
                              int32_t minMvX, int32_t minMvY, int32_t maxMvX, int32_t maxMvY, uint32_t width,
                              uint32_t height, const int32_t mv[4], int32_t useAltHpelIf, XG_PIXEL *pred,
                              intptr_t predStride, int16_t *mvdL0SubPu);
void XinGpuComputeSadS16(int16_t *input, intptr_t inputStride, int16_t *pred, intptr_t predStride, uint32_t width,
                         uint32_t height, uint32_t subShift, uint32_t *sad);
void XinGpuCopyAndPad(XG_PIXEL *ref, intptr_t refStride, XG_PIXEL *pad, intptr_t padStride, uint32_t width,
                      uint32_t height);
void XinGpuCopyAndPadUv(XG_PIXEL *refU, XG_PIXEL *refV, intptr_t refStride, XG_PIXEL *padU, XG_PIXEL *padV,
                        intptr_t padStride, uint32_t width, uint32_t height);

/* ------------------------------------------------------------- frame form
 * One stream = one sequence.  Pictures are submitted in coding order; each
 * picture after the first uses the previously submitted picture as its
 * reference (low-delay P, one reference), which stays resident on the GPU
 * together with its padded planes and its 15 quarter-pel luma planes.
 *
 * For every quadtree level in level_mask (bit s set = s x s CUs, s in
 * {8,16,32,64}) and every s x s CU that lies inside the picture, in raster
 * order per level, the frame pipeline computes:
 *   window  [minMv, maxMv] from the padding (h266_encoder/source/h266_enc_init.c:1462)
 *   integer exhaustive search around MV 0 (as XinGpuMotionEstFull, predictor 0)
 *   Xin266FullSubPelMe refinement
 *   luma MC (Xin266LumaInterPred) and chroma MC (uni branch of Xin266ChromaMotionComp)
 *   per plane: residual, DCT2 (TU = CU), quant/dequant with 4x4 CGs (no RDOQ,
 *   qAdd = 85 << (qShift - 9) for P), inverse DCT2, reconstruction, SSD
 * Outputs per CU: mv (quarter-pel), cost after sub-pel, integer cost,
 * non-zero-CG map and SSD per plane; per level and plane: quantised
 * coefficient plane and reconstructed plane (picture layout). */
typedef struct xin_gpu_stream xin_gpu_stream;

#define XIN_GPU_OUT_Q     1u   /* copy the quantised coefficient planes back */
#define XIN_GPU_OUT_REC   2u   /* copy the reconstructed planes back */

typedef struct xin_gpu_stream_cfg {
    int32_t  width, height;      /* luma size, even */
    int32_t  ctu_size;           /* 64 or 128: reference padding = ctu_size + 16 */
    int32_t  search_range;       /* integer search radius, 1..256 */
    uint32_t level_mask;         /* bit s (8,16,32,64) set = evaluate s x s CUs */
    uint32_t out_flags;          /* XIN_GPU_OUT_* */
    int32_t  use_graph;          /* 1: capture the per-picture launches in a CUDA graph */
    int32_t  device_io;          /* 1: picture planes are device pointers and results stay on the
                                    device (xin_gpu_stream_device_results); for callers whose
                                    pictures already live in GPU memory */
    int32_t  input_bitdepth;     /* 0 (or the library's depth): planes of XG_PIXEL.  8 in the 10-bit
                                    library: planes of 8-bit samples (uint8_t, cast to the plane
                                    pointer type), coded at 10 bits as samples << 2 -- the
                                    reference's 10-bit build on 8-bit input.  The integer search
                                    then runs on the 8-bit samples with SADs x 4, which equals the
                                    10-bit SAD of those samples. */
    int32_t  search_mode;        /* 0: exhaustive integer search (as XinGpuMotionEstFull);
                                    1: by resolution levels (as XinGpuMotionEstHier with predictor
                                    0 and the zero MV as its candidate, the reference picture
                                    and the current picture downscaled by 2 and 4 with
                                    XinGpuDownscale2x2's arithmetic) */
    int32_t  tu_mode;            /* 0: DCT2, TU = CU, quant / dequant (no RDOQ).
                                    1: the preset-4 TU work: per CU (TU = CU) every transform
                                    candidate the mode decision may evaluate -- luma DCT2 and,
                                    for CUs up to 32, the MTS pairs 2..5; chroma DCT2 -- each
                                    through dependent quantisation (Xin266Transform's DepQuant
                                    branch, h266_trans_quant.c:61-245, QP + 12 at 10 bits, rates
                                    from the stream's context set, xin_gpu_stream_set_contexts)
                                    and the inverse transform and reconstruction
                                    (Xin266IDctAdd); plus the final luma prediction's cost with
                                    SATD as the distortion.  The choice among the candidates
                                    stays with the caller (its rate estimate): the per-CU
                                    records give each candidate's non-zero map and SSD
                                    (xin_gpu_results.mts); the coefficient and reconstructed
                                    planes and xin_gpu_cu_result's nz / ssd hold the DCT2
                                    candidate.  Slice QPs up to 51 (39 at 10 bits). */
    int32_t  refs;               /* 0 or 1: one reference, the previous picture (list 0).
                                    2: two references, list 0 = the previous picture and list 1 =
                                    the one before it (the second picture uses the previous one
                                    for both).  Per CU: the integer and sub-pel search in each
                                    list, the bi search of Xin266InterBiSearch
                                    (h266_analyze_inter_cu.c:507; default BCW weight, predictor 0,
                                    a +-4 integer step in place of the closed BBDGS step), the
                                    choice of the lowest of the list-0, list-1 and bi costs (strict,
                                    in that order), and the prediction, transform and
                                    reconstruction of that choice (the bi prediction:
                                    Xin266LumaMotionComp / Xin266ChromaMotionComp's average of the
                                    14-bit predictions).  xin_gpu_cu_result keeps list 0's search;
                                    xin_gpu_results.bi the rest.  With tu_mode 1 (satdMd) the
                                    decision's distortion is SATD: each list's uni cost is its final
                                    prediction's SATD cost and the pair's the averaged prediction's
                                    SATD (pfXinComputeAvgSatd); the TU stage takes the coded
                                    prediction, and its satd_cost the coded MVs' bits.  CU levels up
                                    to 64. */
    int32_t  dpb;                /* pictures kept as references: 0 = refs + 1 (the previous one or
                                    two), up to 32.  Picture k occupies slot k % dpb, so a picture
                                    may reference any of the dpb - 1 pictures submitted before it
                                    (xin_gpu_frame_submit_refs): the random-access GOP structures
                                    (in GOP 16 coding order a B picture reaches up to 20 submissions
                                    back: dpb 21 or more; 32 repeats the graph pattern every two
                                    GOPs). */
} xin_gpu_stream_cfg;

typedef struct xin_gpu_picture {
    const XG_PIXEL *plane[3];    /* host Y, U, V */
    intptr_t stride[3];          /* elements */
    int32_t  qp, uv_qp;          /* slice QPs */
    uint32_t sad_lambda;         /* 0 .. 2^20 */
} xin_gpu_picture;

typedef struct xin_gpu_cu_result {
    int32_t  mvx, mvy;           /* quarter-pel */
    uint32_t cost;               /* after sub-pel */
    uint32_t int_cost;           /* after the integer search */
    uint64_t nz[3];
    uint64_t ssd[3];
} xin_gpu_cu_result;

/* tu_mode 1: the transform candidates of a CU */
typedef struct xin_gpu_cu_mts {
    uint32_t satd_cost;          /* (SATD << 8) + (bits(mvx) + bits(mvy)) * sad_lambda of the final
                                    luma prediction (h266_analyze_inter_cu.c:1109-1131 with SATD) */
    uint32_t ncand;              /* luma candidates: 1 (64 x 64) or 5 */
    uint64_t nz[5];              /* luma non-zero-CG map per candidate: DCT2, then MTS index 2..5
                                    (DST7/DST7, DCT8/DST7, DST7/DCT8, DCT8/DCT8) */
    uint64_t ssd[5];             /* luma SSD of each candidate's reconstruction */
} xin_gpu_cu_mts;

/* refs 2: list 1's search, the bi pair and the choice of a CU */
typedef struct xin_gpu_cu_bi {
    int32_t  mvx1, mvy1;         /* list 1, quarter-pel */
    uint32_t cost1;              /* list 1 after sub-pel */
    uint32_t int_cost1;          /* list 1 after the integer search */
    int32_t  bmv[4];             /* the bi pair: list 0 (x, y), list 1 (x, y), quarter-pel */
    uint32_t bi_cost;            /* (averaged-prediction SAD << 8) + both MVs' bits * sad_lambda */
    uint32_t inter_dir;          /* the prediction coded: 1 list 0, 2 list 1, 3 bi */
} xin_gpu_cu_bi;

typedef struct xin_gpu_results {
    xin_gpu_cu_result *cu;       /* [xin_gpu_stream_num_cus()], levels from 64 down to 8 */
    XG_COEFF *q[3];              /* [levels][plane height][plane width] when XIN_GPU_OUT_Q; zero where
                                    the level's CUs do not reach (right and bottom edges of pictures
                                    that are not multiples of the CU size) */
    XG_PIXEL *rec[3];            /* same layout when XIN_GPU_OUT_REC */
    float    gpu_ms;             /* device time of the picture's launches */
    xin_gpu_cu_mts *mts;         /* tu_mode 1: [xin_gpu_stream_num_cus()] (NULL: a view is returned) */
    xin_gpu_cu_bi  *bi;          /* refs 2: [xin_gpu_stream_num_cus()] (NULL: a view is returned) */
} xin_gpu_results;

int  xin_gpu_stream_open(const xin_gpu_stream_cfg *cfg, xin_gpu_stream **out);
int  xin_gpu_stream_close(xin_gpu_stream *s);
int  xin_gpu_stream_num_cus(const xin_gpu_stream *s);             /* CUs per picture over all levels */
int  xin_gpu_stream_level_info(const xin_gpu_stream *s, int level, int32_t *size, int32_t *first_cu,
                               int32_t *cus_x, int32_t *cus_y);      /* level 0 = largest size */
int  xin_gpu_stream_num_levels(const xin_gpu_stream *s);
/* Autotune the exhaustive search's geometry (search_mode 0): the number of
 * candidate-row bands per 64 x 64 tile, which sets the CTAs of a launch, the
 * reference rows each CTA stages in shared memory and the buffered passes of
 * the 32 x 32 / 64 x 64 sums.  Times the search of the last picture against
 * its reference for the stream's default and up to five other band counts,
 * keeps the fastest for later pictures and re-captures the graphs.  The search
 * results do not depend on the geometry.  Call between pictures, after at
 * least two submitted and none in flight; bands = the chosen count, ms[0] /
 * ms[1] = the default's and the chosen geometry's search time (ms). */
int  xin_gpu_stream_tune_search(xin_gpu_stream *s, int32_t *bands, float ms[2]);
/* Autotune the CUs per CTA of the plain tails of the 16 x 16 and 8 x 8 levels (a
 * warp per CU; 2, 4 or 8 CUs a CTA): times those levels' tails of the last
 * picture for each, keeps the fastest for later pictures and re-captures the
 * graphs.  Results do not depend on it.  Streams with one reference; call
 * between pictures, after at least two submitted and none in flight.  cpb = the
 * choice for 16 x 16 and 8 x 8; ms[3 level + option] = each option's time (ms,
 * 0 for a level that is off). */
int  xin_gpu_stream_tune_tails(xin_gpu_stream *s, int32_t cpb[2], float ms[6]);
/* the geometries the last tune_search timed (n <= 6): band counts and search times (ms) */
int  xin_gpu_stream_tune_table(const xin_gpu_stream *s, int32_t *n, int32_t bands[6], float ms[6]);
/* Upload a picture and queue its hot path (asynchronous).  The first picture of
 * a stream only becomes the reference (no CU results).  Up to two pictures may
 * be in flight (the next one's upload and kernels overlap the previous one's
 * result copies); a third submit before a frame_wait is XIN_GPU_ERR_STATE. */
int  xin_gpu_frame_submit(xin_gpu_stream *s, const xin_gpu_picture *pic);
/* The same with the references named: ref0 (list 0) and ref1 (list 1, refs 2)
 * are picture numbers (0 = the stream's first submitted picture) of earlier
 * pictures at most dpb - 1 submissions back; -1 takes the default (the previous
 * picture for list 0, the one before it for list 1).  For a random-access GOP
 * the encoder submits in coding order and names each B picture's past and
 * future references.  XIN_GPU_ERR_ARG when a reference is out of reach. */
int  xin_gpu_frame_submit_refs(xin_gpu_stream *s, const xin_gpu_picture *pic, int32_t ref0, int32_t ref1);
/* Wait for the oldest picture in flight (bounded by timeout_ms; < 0 waits
 * without limit) and copy its results into the caller's buffers.  Members of res
 * left NULL receive views of the stream's pinned result buffers instead, valid
 * until the second frame_submit after this call.  Every submitted picture is
 * collected once, the first one included. */
int  xin_gpu_frame_wait(xin_gpu_stream *s, xin_gpu_results *res, int32_t timeout_ms);
/* Bound of the waits inside a stream's kernels (the quarter-pel planes wait
 * for their TMA tile loads), in polls of the barrier; -1 restores the default
 * (about a second).  A picture whose wait reaches the bound is reported by
 * xin_gpu_frame_wait as XIN_GPU_ERR_TIMEOUT (the kernel stages with plain
 * loads once the copies have landed); the stream stays usable.
 * XIN_GPU_ERR_STATE while pictures are in flight.  No counterpart in the
 * reference (a GPU wait bound). */
int  xin_gpu_stream_set_wait_tries(xin_gpu_stream *s, int64_t tries);
/* Device time of the stages of the last collected picture:
 * ms[0] upload + padding + quarter-pel planes, ms[1] integer search,
 * ms[2] sub-pel search + MC + transform/quant + reconstruction, ms[3] result copies. */
int  xin_gpu_stream_stage_ms(const xin_gpu_stream *s, float ms[4]);
/* Device pointers of the result arrays of the last collected picture (same
 * layouts as xin_gpu_results), valid until the second submit after it. */
int  xin_gpu_stream_device_results(const xin_gpu_stream *s, void **cu, void *q[3], void *rec[3]);

/* tu_mode 1: the CABAC context set (XIN_GPU_NUM_CTX records, the reference's
 * xin_prob_model array) the trellis takes its rates from, for the pictures
 * submitted after this call; XIN_GPU_ERR_STATE while pictures are in flight.
 * Until it is called, every context holds probability one half. */
int  xin_gpu_stream_set_contexts(xin_gpu_stream *s, const xin_gpu_prob *ctx);

/* Device and pinned-host bytes a stream of this configuration allocates
 * (before the CUDA allocator's rounding); no GPU needed. */
int  xin_gpu_stream_footprint(const xin_gpu_stream_cfg *cfg, uint64_t *device_bytes, uint64_t *host_bytes);

/* ------------------------------------------------------------ serving
 * Many live streams on one GPU.  join admits a stream only if its device
 * footprint fits the HBM budget and, when mpix_budget > 0, the luma Mpixel/s
 * already promised plus width*height*fps stays within it; otherwise
 * XIN_GPU_ERR_ADMIT and nothing is allocated.  submit copies the picture and
 * queues it (the caller's planes are free on return; cu_out must hold
 * xin_gpu_stream_num_cus records of that configuration and stay valid until the
 * picture is reported by poll; it may be NULL for a stream's first picture).
 * One scheduler thread runs up to max_inflight pictures of different streams
 * at once and starts the oldest waiting picture whenever one finishes; the
 * pictures of one stream run in order.  Streams of the plain form (exhaustive
 * search, one reference, tu_mode 0) with the same picture size, CTU size,
 * search range, levels and input depth share launches: the oldest waiting
 * picture takes up to batch_max - 1 waiting pictures of such streams into one
 * batch, one launch per stage over all of them (each picture still counts
 * toward max_inflight), as long as the batch's integer search stays within two
 * waves of the GPU's SMs: a batch completes its pictures together, so pictures
 * whose search fills the GPU on its own run alone.  A stream's results are the same as
 * when it runs alone.  leave drains the stream's queue, then frees it.  A
 * served stream keeps XIN_GPU_OUT_Q of its cfg.out_flags (its coefficient
 * planes, through xin_gpu_server_submit_planes); the other output flags are
 * cleared. */
typedef struct xin_gpu_server xin_gpu_server;
typedef struct xin_gpu_server_cfg {
    uint64_t hbm_budget;         /* device bytes for streams; 0 = 90 % of the free memory at open */
    double   mpix_budget;        /* sustained luma Mpixel/s admission may promise; 0 = no limit */
    uint32_t max_inflight;       /* pictures on the GPU at once; 0 = 8 */
    uint32_t max_streams;        /* 0 = 256 */
    uint32_t max_queue;          /* pictures a stream may have waiting; 0 = 4 */
    uint32_t batch_max;          /* pictures of different streams one launch per stage may carry
                                    (cross-stream batches); 0 = 8, 1 = one picture a launch */
    uint32_t batch_window_us;    /* how long the oldest waiting picture may be held for others to
                                    join its batch; 0 = launch at once with what is waiting */
    uint32_t reserved;
} xin_gpu_server_cfg;
typedef struct xin_gpu_server_done {
    int32_t  stream_id;
    uint32_t frame_index;        /* per stream, from 0 */
    uint64_t user_tag;
    int32_t  status;             /* XIN_GPU_OK or this picture's error */
    int32_t  has_results;        /* 0 for a stream's first picture (it only becomes the reference) */
    float    gpu_ms;             /* device time of the picture */
    float    reserved;
    double   queue_ms;           /* submit -> start on the GPU */
    double   latency_ms;         /* submit -> results in cu_out */
} xin_gpu_server_done;
typedef struct xin_gpu_server_stats {
    int32_t  streams, running, queued, reserved;
    uint64_t hbm_budget, hbm_used;
    double   mpix_used;
    uint64_t launched, completed;
    uint64_t batches;            /* launches that carried pictures of two or more streams */
    uint64_t batched_pictures;   /* pictures those launches carried */
} xin_gpu_server_stats;
int  xin_gpu_server_open(const xin_gpu_server_cfg *cfg, xin_gpu_server **srv);     /* cfg may be NULL */
int  xin_gpu_server_join(xin_gpu_server *srv, const xin_gpu_stream_cfg *cfg, double fps, int32_t *stream_id);
int  xin_gpu_server_submit(xin_gpu_server *srv, int32_t stream_id, const xin_gpu_picture *pic,
                           xin_gpu_cu_result *cu_out, uint64_t user_tag);
/* The same, with the picture's coefficient planes returned too: q_out[3] are
 * caller buffers laid out as xin_gpu_results.q ([levels][plane height][plane
 * width]), filled straight from the device when the picture completes (the
 * latency a poll reports includes that copy).  Pinned host memory
 * (cudaHostAlloc) keeps the copies asynchronous.  The stream must have been
 * joined with XIN_GPU_OUT_Q in its out_flags; a buffer must stay untouched
 * until its picture is polled. */
int  xin_gpu_server_submit_planes(xin_gpu_server *srv, int32_t stream_id, const xin_gpu_picture *pic,
                                  xin_gpu_cu_result *cu_out, XG_COEFF *const q_out[3], uint64_t user_tag);
/* up to max completed pictures; waits up to timeout_ms (< 0: until one completes) */
int  xin_gpu_server_poll(xin_gpu_server *srv, xin_gpu_server_done *out, int32_t max, int32_t timeout_ms, int32_t *n);
int  xin_gpu_server_leave(xin_gpu_server *srv, int32_t stream_id, int32_t timeout_ms);
int  xin_gpu_server_get_stats(xin_gpu_server *srv, xin_gpu_server_stats *stats);
int  xin_gpu_server_close(xin_gpu_server *srv);     /* finishes queued pictures, frees every stream */

/* Measured throughput of this GPU's packed SAD instructions on
 * register-resident data, in absolute differences per second: the ceiling of
 * the integer search kernel, used as its roofline.  8-bit library: the faster
 * of vabsdiff4 + dp4a and vabsdiff4 with add-reduction; 10-bit library: the
 * packed 16-bit add-then-max form its search issues. */
int  xin_gpu_measure_sad_peak(double *absdiff_per_s);

#ifdef __cplusplus
}
#endif
#endif
