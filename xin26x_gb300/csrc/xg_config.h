/*
 * xg_config.h -- compile-time configuration shared by host and device code.
 *
 * The library is built once per internal bit depth, like the reference's
 * ENABLE_10BIT_ENCODER switch (video_api/video_common/include/xin_typedef.h:72-96):
 *   XG_BITDEPTH=8  -> PIXEL uint8_t,  COEFF int16_t   (libxingpu8.so)
 *   XG_BITDEPTH=10 -> PIXEL uint16_t, COEFF int32_t   (libxingpu10.so)
 */
#ifndef XG_CONFIG_H
#define XG_CONFIG_H

#include <stdint.h>

#ifndef XG_BITDEPTH
#define XG_BITDEPTH 8
#endif

#if XG_BITDEPTH == 10 && !defined(ENABLE_10BIT_ENCODER)
#define ENABLE_10BIT_ENCODER   /* selects the 10-bit PIXEL / COEFF of include/xingpu.h */
#endif

#if XG_BITDEPTH == 10
typedef uint16_t xg_pix;
typedef int32_t  xg_coef;
#else
typedef uint8_t  xg_pix;
typedef int16_t  xg_coef;
#endif

#define XG_MAX_PIX ((1 << XG_BITDEPTH) - 1)

/* interpolation constants (h266_core/include/h266_inter_pred_context.h:31-38) */
#define XG_IF_SHIFT 6
#define XG_IF_OFF14 (1 << 13)
#define XG_IF_HEAD (14 - XG_BITDEPTH > 2 ? 14 - XG_BITDEPTH : 2)

/* cost precision (common/include/h26x_definition.h:88) */
#define XG_COST_FRACTION 8

#endif
