/*
 * xingpu.cu -- single translation unit of libxingpu (one build per bit depth,
 * -DXG_BITDEPTH=8 or 10).  The component files share constant-memory tables,
 * so they are compiled together.
 */
#include "xg_config.h"
#if XG_BITDEPTH == 10 && !defined(ENABLE_10BIT_ENCODER)
#define ENABLE_10BIT_ENCODER
#endif
#include "xg_runtime_impl.cuh"
#include "xg_percall.cuh"
#include "xg_me_percall.cuh"
#include "xg_frame.cuh"
#include "xg_batch.cuh"
#include "xg_dmvr.cuh"
#include "xg_fsme.cuh"
#include "xg_server.cuh"
#include "xg_install.cuh"
#include "xg_tq_batch.cuh"
#include "xg_noalloc.cuh"
#include "xg_dq.cuh"
#include "xg_tu.cuh"
