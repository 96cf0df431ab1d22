/*
 * xingpu_install.h -- fills the reference encoder's primitive tables with
 * libxingpu's per-call GPU forms.
 *
 * xin_gpu_func_struct mirrors the layout of the reference's xin_func_struct
 * (h266_encoder/include/h266_func_struct.h:719-799): every member is a function
 * pointer or an array of them, so the mirror lists the members in order with
 * their array shapes (tests/test_boundary.py compiles both and compares the
 * offsets).  The ME table xin_me_func is mirrored in xingpu_me.h.
 *
 * xin_gpu_install runs right after the reference's own table set-up:
 * Xin266FuncInit + Xin266FuncUpdate (h266_encoder/source/h266_encoder_create.c:3882,3332)
 * for xin_func_struct, Xin26xMeFuncInit (h266_encoder/source/h266_create_section.c:65)
 * for xin_me_func.  pfXinComputeDist / AvgDist / WeightDist point at SAD or SATD
 * depending on the preset; the installer keeps that choice by comparing each
 * with the SATD entry before replacing them.
 */
#ifndef XINGPU_INSTALL_H
#define XINGPU_INSTALL_H

#include <stdint.h>
#include "xingpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef void (*xin_gpu_fn)(void);

typedef struct xin_gpu_func_struct {
    xin_gpu_fn pfXinBlockCopy[8];
    xin_gpu_fn pfXinBlockAvg[8];
    xin_gpu_fn pfXinPictureCopy;
    xin_gpu_fn pfXinPictureScaleCopy;
    xin_gpu_fn pfXinComputeSad[8];
    xin_gpu_fn pfXinComputeSadS16[8];
    xin_gpu_fn pfXinComputeSatd[8];
    xin_gpu_fn pfXinComputeDist[8];
    xin_gpu_fn pfXinComputeAvgSad[8];
    xin_gpu_fn pfXinComputeAvgSatd[8];
    xin_gpu_fn pfXinComputeAvgDist[8];
    xin_gpu_fn pfXinComputeWeightSad[8];
    xin_gpu_fn pfXinComputeWeightSatd[8];
    xin_gpu_fn pfXinComputeWeightDist[8];
    xin_gpu_fn pfXinComputeSadx8[8];
    xin_gpu_fn pfXinComputeSadx5[8];
    xin_gpu_fn pfXinComputeSadx3[8];
    xin_gpu_fn pfXinComputeAvgSadx8[8];
    xin_gpu_fn pfXinLumaInterp[2][2][8];
    xin_gpu_fn pfXinChromaInterp[2][2][8];
    xin_gpu_fn pfXinBiliInterp[2][2][8];
    xin_gpu_fn pfXinLumaInterpS16[2][2][8];
    xin_gpu_fn pfXinChromaInterpS16[2][2][8];
    xin_gpu_fn pfXinInterpAvg[8];
    xin_gpu_fn pfXinInterpWeight[8];
    xin_gpu_fn pfXinQuantInvQuant[8];
    xin_gpu_fn pfXinFor2dDct2[8][8];
    xin_gpu_fn pfXinFor2dSkip[8];
    xin_gpu_fn pfXinInv2dSkip[8];
    xin_gpu_fn pfXinFor1dDct[3][8];
    xin_gpu_fn pfXinIDctAdd[8];
    xin_gpu_fn pfXinIDctAddDc[8];
    xin_gpu_fn pfXinInv2dDct2[8][8];
    xin_gpu_fn pfXinInv1dDct[3][8];
    xin_gpu_fn pfXinComputeSsd[8];
    xin_gpu_fn pfXinComputeSsdFd[8];
    xin_gpu_fn pfXinLinearTransform[8];
    xin_gpu_fn pfXinIntraPredDc[8];
    xin_gpu_fn pfXinIntraPredPlanar[8];
    xin_gpu_fn pfXinIntraPredHor[8];
    xin_gpu_fn pfXinIntraPredVer[8];
    xin_gpu_fn pfXinApplyPDPC[8];
    xin_gpu_fn pfXinApplyHorPDPC[8];
    xin_gpu_fn pfXinApplyVerPDPC[8];
    xin_gpu_fn pfXinApplyAngPDPC[2][8];
    xin_gpu_fn pfXinSaoStatEo[8];
    xin_gpu_fn pfXinCoeffScanCG[2];
    xin_gpu_fn pfXinSaoEo0[2];
    xin_gpu_fn pfXinSaoEo45[2];
    xin_gpu_fn pfXinSaoEo90[2];
    xin_gpu_fn pfXinSaoEo135[2];
    xin_gpu_fn pfXinBlockSub[8];
    xin_gpu_fn pfXinBlockSubForDct[8];
    xin_gpu_fn pfXinBlockAddForDct[8];
    xin_gpu_fn pfXinLumaIntraFilter[8];
    xin_gpu_fn pfXinChromaIntraFilter[8];
    xin_gpu_fn pfXinComputeBlockSsd;
    xin_gpu_fn pfXinEstimateTuCoeff;
    xin_gpu_fn pfXinDownscale2x2;
    xin_gpu_fn pfXinConstructBiMeInput[8];
    xin_gpu_fn pfXinConstructWeightBiMeInput[8];
    xin_gpu_fn pfXinComputeHada8x8;
    xin_gpu_fn pfXinGetBlockDeltaU[2];
    xin_gpu_fn pfXinCalcBlockDeltaU[2];
    xin_gpu_fn pfXinUpdateQuantOffset;
    xin_gpu_fn pfXinComputeVar8x8;
    xin_gpu_fn pfXinLaComputeDist[8];
    xin_gpu_fn pfXinCopyAndPad;
    xin_gpu_fn pfXinCopyAndPadUv;
    xin_gpu_fn pfXinComputeGradient[8];
    xin_gpu_fn pfXinLumaLoopFilter;
    xin_gpu_fn pfXinComputeFrameAct;
    xin_gpu_fn pfXinPreRdoq;
    xin_gpu_fn pfXinPreDepQuant;
    xin_gpu_fn pfXinDepQuant;
    xin_gpu_fn pfXinBlockTranspose;
    xin_gpu_fn pfXinExtendIntraRef;
    xin_gpu_fn pfXinFilterIntraNB;
} xin_gpu_func_struct;

#define XIN_GPU_INSTALL_DIST      1u   /* SAD / SATD / Var families, Hadamard 8x8 */
#define XIN_GPU_INSTALL_INTERP    2u   /* luma / chroma interpolation, bi average, BCW blend */
#define XIN_GPU_INSTALL_TRANSFORM 4u   /* 1-D / 2-D transforms, skip, residual, reconstruction */
#define XIN_GPU_INSTALL_QUANT     8u   /* quant / dequant, pre-RDOQ, dependent quantisation */
#define XIN_GPU_INSTALL_ALL       15u

/* funcSet: the reference's xin_func_struct *, meFunc: its xin_me_func *
 * (either may be NULL).  Does not touch the GPU.  Returns XIN_GPU_OK or
 * XIN_GPU_ERR_ARG when both are NULL. */
int xin_gpu_install(void *funcSet, void *meFunc, uint32_t what);

#ifdef __cplusplus
}
#endif
#endif
