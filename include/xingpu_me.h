/*
 * xingpu_me.h -- layout mirror of the reference's motion-estimation state
 * xin_me_struct (h26x_core/include/h26x_me_struct.h:60-131) and its embedded
 * function table xin_me_func (h26x_core/include/h26x_me_func_struct.h:174-191).
 *
 * XinGpuMotionEstFull / XinGpuFullSubPelMe take a pointer to the reference's
 * own struct; the library reads and writes it through this mirror.  The member
 * order and types must stay identical to the reference; tests/test_boundary.py
 * compiles both definitions and compares every offset.  Function-table entries
 * are opaque pointers here (the library never calls them).
 */
#ifndef XINGPU_ME_H
#define XINGPU_ME_H

#include "xingpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef union xin_gpu_mv { int32_t s32x1; int16_t s16x2[2]; struct { int16_t mvX, mvY; } mv; } xin_gpu_mv;
typedef struct xin_gpu_mv_s { int16_t mvX, mvY; } xin_gpu_mv_s;

typedef struct xin_gpu_me_func {
    void *pfXinComputeSad[8];
    void *pfXinComputeAvgSad[8];
    void *pfXinComputeSadx8[8];
    void *pfXinComputeSadx5[8];
    void *pfXinComputeSadx3[8];
    void *pfXinComputeAvgSadx8[8];
    void *pfXinHorMotionSearch[8];
    void *pfXinVerMotionSearch[8];
    void *pfXinComputeVar[8];
    void *pfXinComputeAvgVar[8];
    void *pfXinMotionSearchHier2[8];
    void *pfXinMotionSearchHier1[8];
    void *pfXinConstructBiMeInput[8];
    void *pfXinInterpoHalfPel;
    void *pfXinDownscale2x2;
} xin_gpu_me_func;

typedef struct xin_gpu_me_struct {
    xin_gpu_me_func funcSet;
    uint32_t     width;
    uint32_t     height;
    xin_gpu_mv   minMv;
    xin_gpu_mv   maxMv;
    xin_gpu_mv   meCand[12];
    uint32_t     candNum;
    int32_t      biMe;
    int32_t      oneDimMe;
    xin_gpu_mv   bestMv;
    xin_gpu_mv   predMv;
    uint32_t     bestCost;
    uint32_t     bestSad;
    uint32_t     bestPos;
    int32_t      searchWidth;
    int32_t      searchHeight;
    int32_t      iMvMode;
    int32_t      bestRound;
    int32_t      bestDist;
    int32_t      maxLgTZDist;
    int32_t      rasterDist;
    int32_t      bestMvX;
    int32_t      bestMvY;
    int32_t      numSearchRound;
    xin_gpu_mv_s searchOffset[16][13];
    uint32_t     searchRadius[16];
    uint32_t     searchPoints[16];
    uint32_t     skippedSR;
    uint32_t     refinedSR;
    uint32_t     sadLambda;
    uint64_t     sseLambda;
    int32_t      refIdx;
    int32_t      listIdx;
    XG_PIXEL    *input;
    intptr_t     inputStride;
    XG_PIXEL    *input1;
    intptr_t     input1Stride;
    XG_PIXEL    *input2;
    intptr_t     input2Stride;
    XG_PIXEL    *ref;
    intptr_t     refStride;
    XG_PIXEL    *ref1;
    intptr_t     ref1Stride;
    XG_PIXEL    *ref2;
    intptr_t     ref2Stride;
    XG_PIXEL    *interpBuf;
    XG_PIXEL    *halfPelH;
    XG_PIXEL    *halfPelV;
    XG_PIXEL    *halfPelHv;
    XG_PIXEL    *integPel;
    intptr_t     interpStride;
    XG_PIXEL    *halfPel[9];
    XG_PIXEL    *qBufA[9][8];
    XG_PIXEL    *qBufB[9][8];
} xin_gpu_me_struct;

#ifdef __cplusplus
}
#endif
#endif
