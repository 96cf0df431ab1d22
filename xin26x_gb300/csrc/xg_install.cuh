/*
 * xg_install.cuh -- xin_gpu_install: writes the per-call GPU forms into the
 * reference's xin_func_struct / xin_me_func through their layout mirrors
 * (include/xingpu_install.h, include/xingpu_me.h).  Host code only.
 */
#include "../../include/xingpu_install.h"
#include "../../include/xingpu_me.h"

#define XG_FN(f) ((xin_gpu_fn)(void (*)(void))(f))

extern "C" int xin_gpu_install(void *funcSet, void *meFunc, uint32_t what)
{
    xin_gpu_func_struct *fs = (xin_gpu_func_struct *)funcSet;
    xin_gpu_me_func *mf = (xin_gpu_me_func *)meFunc;
    if (!fs && !mf) return XIN_GPU_ERR_ARG;
    const xin_gpu_fn fdct[3][8] = {
        { nullptr, XG_FN(XinGpuFDct2P2), XG_FN(XinGpuFDct2P4), XG_FN(XinGpuFDct2P8), XG_FN(XinGpuFDct2P16), XG_FN(XinGpuFDct2P32), XG_FN(XinGpuFDct2P64), nullptr },
        { nullptr, nullptr, XG_FN(XinGpuFDct8P4), XG_FN(XinGpuFDct8P8), XG_FN(XinGpuFDct8P16), XG_FN(XinGpuFDct8P32), nullptr, nullptr },
        { nullptr, nullptr, XG_FN(XinGpuFDst7P4), XG_FN(XinGpuFDst7P8), XG_FN(XinGpuFDst7P16), XG_FN(XinGpuFDst7P32), nullptr, nullptr } };
    const xin_gpu_fn idct[3][8] = {
        { nullptr, XG_FN(XinGpuIDct2P2), XG_FN(XinGpuIDct2P4), XG_FN(XinGpuIDct2P8), XG_FN(XinGpuIDct2P16), XG_FN(XinGpuIDct2P32), XG_FN(XinGpuIDct2P64), nullptr },
        { nullptr, nullptr, XG_FN(XinGpuIDct8P4), XG_FN(XinGpuIDct8P8), XG_FN(XinGpuIDct8P16), XG_FN(XinGpuIDct8P32), nullptr, nullptr },
        { nullptr, nullptr, XG_FN(XinGpuIDst7P4), XG_FN(XinGpuIDst7P8), XG_FN(XinGpuIDst7P16), XG_FN(XinGpuIDst7P32), nullptr, nullptr } };
    if (fs) {
        for (int lg = 0; lg < 8; lg++) {
            if (what & XIN_GPU_INSTALL_DIST) {
                bool dist_satd = fs->pfXinComputeDist[lg] && fs->pfXinComputeDist[lg] == fs->pfXinComputeSatd[lg];
                bool avg_satd = fs->pfXinComputeAvgDist[lg] && fs->pfXinComputeAvgDist[lg] == fs->pfXinComputeAvgSatd[lg];
                bool wgt_satd = fs->pfXinComputeWeightDist[lg] && fs->pfXinComputeWeightDist[lg] == fs->pfXinComputeWeightSatd[lg];
                fs->pfXinComputeSad[lg] = XG_FN(XinGpuComputeSad);
                fs->pfXinComputeSadx8[lg] = XG_FN(XinGpuComputeSadx8);
                fs->pfXinComputeSadx5[lg] = XG_FN(XinGpuComputeSadx5);
                fs->pfXinComputeSadx3[lg] = XG_FN(XinGpuComputeSadx3);
                fs->pfXinComputeAvgSadx8[lg] = XG_FN(XinGpuComputeAvgSadx8);
                fs->pfXinComputeSadS16[lg] = XG_FN(XinGpuComputeSadS16);
                if (lg >= 2) {   /* SATD, bi and BCW forms exist from width 4 (h266_func_init.c:182-208,648-655) */
                    fs->pfXinComputeSatd[lg] = XG_FN(XinGpuComputeSatd);
                    fs->pfXinComputeAvgSad[lg] = XG_FN(XinGpuComputeAvgSad);
                    fs->pfXinComputeAvgSatd[lg] = XG_FN(XinGpuComputeAvgSatd);
                    fs->pfXinComputeWeightSad[lg] = XG_FN(XinGpuComputeWeightSad);
                    fs->pfXinComputeWeightSatd[lg] = XG_FN(XinGpuComputeWeightSatd);
                    fs->pfXinComputeAvgDist[lg] = avg_satd ? XG_FN(XinGpuComputeAvgSatd) : XG_FN(XinGpuComputeAvgSad);
                    fs->pfXinComputeWeightDist[lg] = wgt_satd ? XG_FN(XinGpuComputeWeightSatd) : XG_FN(XinGpuComputeWeightSad);
                }
                fs->pfXinComputeDist[lg] = (dist_satd && lg >= 2) ? XG_FN(XinGpuComputeSatd) : XG_FN(XinGpuComputeSad);
            }
            if (what & XIN_GPU_INSTALL_INTERP) {
                fs->pfXinLumaInterp[0][0][lg] = XG_FN(XinGpuInterpCopy);
                fs->pfXinLumaInterp[1][0][lg] = XG_FN(XinGpuLumaInterpHor);
                fs->pfXinLumaInterp[0][1][lg] = XG_FN(XinGpuLumaInterpVet);
                fs->pfXinLumaInterp[1][1][lg] = XG_FN(XinGpuLumaInterpHorVet);
                fs->pfXinLumaInterpS16[0][0][lg] = XG_FN(XinGpuInterpCopyU8S16);
                fs->pfXinLumaInterpS16[1][0][lg] = XG_FN(XinGpuLumaInterpHorU8S16);
                fs->pfXinLumaInterpS16[0][1][lg] = XG_FN(XinGpuLumaInterpVetU8S16);
                fs->pfXinLumaInterpS16[1][1][lg] = XG_FN(XinGpuLumaInterpHorVetU8S16);
                fs->pfXinChromaInterp[0][0][lg] = XG_FN(XinGpuInterpCopy);
                fs->pfXinChromaInterp[1][0][lg] = XG_FN(XinGpuChromaInterpHor);
                fs->pfXinChromaInterp[0][1][lg] = XG_FN(XinGpuChromaInterpVet);
                fs->pfXinChromaInterp[1][1][lg] = XG_FN(XinGpuChromaInterpHorVet);
                fs->pfXinChromaInterpS16[0][0][lg] = XG_FN(XinGpuInterpCopyU8S16);
                fs->pfXinChromaInterpS16[1][0][lg] = XG_FN(XinGpuChromaInterpHorU8S16);
                fs->pfXinChromaInterpS16[0][1][lg] = XG_FN(XinGpuChromaInterpVetU8S16);
                fs->pfXinChromaInterpS16[1][1][lg] = XG_FN(XinGpuChromaInterpHorVetU8S16);
                fs->pfXinInterpAvg[lg] = XG_FN(XinGpuInterpAvgS16U8);
                fs->pfXinBiliInterp[0][0][lg] = XG_FN(XinGpuBiliInterpCopy);
                fs->pfXinBiliInterp[1][0][lg] = XG_FN(XinGpuBiliInterpHor);
                fs->pfXinBiliInterp[0][1][lg] = XG_FN(XinGpuBiliInterpVet);
                fs->pfXinBiliInterp[1][1][lg] = XG_FN(XinGpuBiliInterpHorVet);
                fs->pfXinInterpWeight[lg] = XG_FN(XinGpuInterpWeightS16U8);
            }
            if (what & XIN_GPU_INSTALL_TRANSFORM) {
                for (int ty = 0; ty < 3; ty++) { fs->pfXinFor1dDct[ty][lg] = fdct[ty][lg]; fs->pfXinInv1dDct[ty][lg] = idct[ty][lg]; }
                fs->pfXinFor2dSkip[lg] = XG_FN(XinGpuFSkipWxH);
                fs->pfXinInv2dSkip[lg] = XG_FN(XinGpuISkipWxH);
                fs->pfXinBlockSubForDct[lg] = XG_FN(XinGpuBlockSubForDct);
                fs->pfXinBlockAddForDct[lg] = XG_FN(XinGpuBlockAddForDct);
                for (int lh = 0; lh < 8; lh++) {
                    fs->pfXinFor2dDct2[lg][lh] = XG_FN(XinGpuFDct2WxH);
                    fs->pfXinInv2dDct2[lg][lh] = XG_FN(XinGpuIDct2WxH);
                }
            }
            if (what & XIN_GPU_INSTALL_QUANT) fs->pfXinQuantInvQuant[lg] = XG_FN(XinGpuQuantInvQuant);
        }
        if (what & XIN_GPU_INSTALL_DIST) {
            fs->pfXinComputeHada8x8 = XG_FN(XinGpuComputeHada8x8);
            fs->pfXinDownscale2x2 = XG_FN(XinGpuDownscale2x2);
        }
        if (what & XIN_GPU_INSTALL_INTERP) {
            fs->pfXinCopyAndPad = XG_FN(XinGpuCopyAndPad);
            fs->pfXinCopyAndPadUv = XG_FN(XinGpuCopyAndPadUv);
        }
        if (what & XIN_GPU_INSTALL_QUANT) {
            fs->pfXinPreRdoq = XG_FN(XinGpuPreRdoq);
            fs->pfXinDepQuant = XG_FN(XinGpuDepQuant);
        }
    }
    if (mf && (what & XIN_GPU_INSTALL_DIST)) {
        for (int lg = 0; lg < 8; lg++) {
            mf->pfXinComputeSad[lg] = (void *)XinGpuComputeSad;
            mf->pfXinComputeAvgSad[lg] = (void *)XinGpuComputeAvgSad;
            mf->pfXinComputeSadx8[lg] = (void *)XinGpuComputeSadx8;
            mf->pfXinComputeSadx5[lg] = (void *)XinGpuComputeSadx5;
            mf->pfXinComputeSadx3[lg] = (void *)XinGpuComputeSadx3;
            mf->pfXinComputeAvgSadx8[lg] = (void *)XinGpuComputeAvgSadx8;
            mf->pfXinComputeVar[lg] = (void *)XinGpuComputeVar;
            mf->pfXinComputeAvgVar[lg] = (void *)XinGpuComputeAvgVar;
            mf->pfXinMotionSearchHier1[lg] = (void *)XinGpuMotionSearchHier;
            mf->pfXinMotionSearchHier2[lg] = (void *)XinGpuMotionSearchHier;
        }
        mf->pfXinDownscale2x2 = (void *)XinGpuDownscale2x2;
        mf->pfXinInterpoHalfPel = (void *)XinGpuInterpoHalfPel;
    }
    return XIN_GPU_OK;
}
