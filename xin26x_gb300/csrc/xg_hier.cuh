/*
 * xg_hier.cuh -- integer motion search by resolution levels (the preset-4/6
 * search mode, motionSearchMode 2 = XIN_ME_HIER_SEARCH,
 * common/include/h26x_definition.h:93, selected at
 * h266_encoder/source/h266_analyze_inter_cu.c:1063-1067) and the 2x2 downscale
 * that builds its reference levels (h266_encoder/source/h266_enc_init.c:2802-2824).
 *
 * The reference's search (Xin26xMotionEstHier, its level searches
 * Xin26xMotionSearchHier1/2 and Xin26xDownscale2x2) ships only in the closed
 * library, so its order is restated, the same way in the oracle
 * (oracle/xin_oracle.c, orc_me_hier):
 *   window  [c - range, c + range] within [minMv, maxMv], c = predictor >> 2;
 *           at level L (1/2, 1/4) its ends become ceil(lo / 2^L), floor(hi / 2^L)
 *   start   the incoming best, then the candidates (quarter-pel MVs >> 2,
 *           clipped to the window), full cost, list order, strict '<'
 *   1/4     exhaustive SAD over the level window (block w/4 x h/4)
 *   1/2     +-1 around twice the 1/4 best (block w/2 x h/2)
 *   full    the 3 x 3 MVs around twice the 1/2 best, full cost
 *           (SAD << 8) + (bits(mvd x) + bits(mvd y)) * lambda, strict '<'
 *
 * Entry points: XinGpuDownscale2x2 (pfXinDownscale2x2), XinGpuMotionSearchHier
 * (pfXinMotionSearchHier1/2: one exhaustive level), XinGpuMotionEstHier (the
 * driver on xin_me_struct), and k_hier_frame, the frame form's search when a
 * stream is opened with search_mode 1.
 */

/* (a + b + c + d + 2) >> 2 over the 2x2 block at (2x, 2y) */
__global__ void k_downscale2x2(const xg_pix *in, long long ip, xg_pix *out, long long op, int ow, int oh)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= ow || y >= oh) return;
    const xg_pix *a = in + (long long)(2 * y) * ip + 2 * x;
    out[(long long)y * op + x] = (xg_pix)(((int)a[0] + (int)a[1] + (int)a[ip] + (int)a[ip + 1] + 2) >> 2);
}

__host__ __device__ __forceinline__ int xg_ceil_shr(int v, int s) { return -((-v) >> s); }

/* this thread's share of the SAD of a w x h block: samples i = t, t + nt, ... */
__device__ __forceinline__ uint32_t xg_sad_part(const xg_pix *c, long long cp, const xg_pix *r, long long rp, int w, int h,
                                                int t, int nt)
{
    uint32_t s = 0;
    for (int i = t; i < w * h; i += nt) {
        const int y = i / w, x = i - y * w;
        s += (uint32_t)abs((int)c[(long long)y * cp + x] - (int)r[(long long)y * rp + x]);
    }
    return s;
}

__device__ __forceinline__ uint32_t xg_warp_sum(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long xg_warp_min64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o); v = u < v ? u : v; }
    return v;
}

/* whole-CTA reductions through a shared scratch of 32 entries (all threads call) */
__device__ uint32_t xg_cta_sum(uint32_t v, uint32_t *red)
{
    v = xg_warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t s = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
    return s;
}
__device__ unsigned long long xg_cta_min64(unsigned long long v, unsigned long long *red)
{
    v = xg_warp_min64(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    unsigned long long m = ~0ull;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) m = red[i] < m ? red[i] : m;
    return m;
}

/* ------------------------------------------------------------ per call */

/* one level: every MV of an nx x ny window (the window's top-left candidate at
 * ref), raster order, strict '<' on the SAD; out = 1 + index of the best, or 0
 * for an empty window */
__global__ void k_hier_level(const xg_pix *in, int w, int h, const xg_pix *ref, int rp, int nx, int ny, unsigned long long *out)
{
    __shared__ unsigned long long red[32];
    unsigned long long k = ~0ull;
    for (int i = threadIdx.x; i < nx * ny; i += blockDim.x) {
        const int y = i / nx, x = i - y * nx;
        const uint32_t s = xg_sad_part(in, w, ref + (long long)y * rp + x, rp, w, h, 0, 1);
        const unsigned long long kk = ((unsigned long long)s << 32) | (uint32_t)(i + 1);
        k = kk < k ? kk : k;
    }
    k = xg_cta_min64(k, red);
    if (threadIdx.x == 0) *out = (nx > 0 && ny > 0) ? k : 0ull;
}

/* The driver in one CTA.  Windows are staged per level: w0 (full resolution,
 * top-left MV (x0, y0)), w1 (1/2, top-left (x0 >> 1 rounded up)), w2 (1/4).
 * io in: best mvx, mvy (quarter-pel), cost, sad; out: the same. */
struct XgHierArgs {
    const xg_pix *in[3];            /* current block at the three levels, packed (pitch = width) */
    const xg_pix *win[3];           /* reference windows, packed */
    int wp[3];                      /* window pitches */
    int x0[3], x1[3], y0[3], y1[3]; /* window MV range per level (level units) */
    int w, h;
    int mvpx, mvpy;                 /* quarter-pel predictor */
    uint32_t lambda;
    int ncand;
    int cand[12][2];                /* quarter-pel candidates */
};

__device__ __forceinline__ uint32_t xg_full_cost(uint32_t sad, int mvx4, int mvy4, int mvpx, int mvpy, uint32_t lambda)
{
    return (sad << XG_COST_FRACTION) + (xg_mvd_bits(mvx4 - mvpx) + xg_mvd_bits(mvy4 - mvpy)) * lambda;
}

__global__ void k_me_hier_cu(XgHierArgs a, int *io)
{
    __shared__ uint32_t red[32];
    __shared__ unsigned long long red64[32];
    const int t = threadIdx.x, nt = blockDim.x;
    int bx = io[0], by = io[1];
    uint32_t best = (uint32_t)io[2], bsad = (uint32_t)io[3];
    /* the full-resolution SAD at integer MV (x, y) */
    auto sad0 = [&](int x, int y) {
        const xg_pix *r = a.win[0] + (long long)(y - a.y0[0]) * a.wp[0] + (x - a.x0[0]);
        return xg_cta_sum(xg_sad_part(a.in[0], a.w, r, a.wp[0], a.w, a.h, t, nt), red);
    };
    for (int i = 0; i < a.ncand; i++) {
        const int x = min(max(a.cand[i][0] >> 2, a.x0[0]), a.x1[0]), y = min(max(a.cand[i][1] >> 2, a.y0[0]), a.y1[0]);
        const uint32_t s = sad0(x, y), c = xg_full_cost(s, 4 * x, 4 * y, a.mvpx, a.mvpy, a.lambda);
        if (c < best) { best = c; bsad = s; bx = 4 * x; by = 4 * y; }
    }
    /* 1/4: exhaustive over the level window */
    int b2x = (a.mvpx >> 2) >> 2, b2y = (a.mvpy >> 2) >> 2;
    {
        const int nx = a.x1[2] - a.x0[2] + 1, ny = a.y1[2] - a.y0[2] + 1, bw = a.w >> 2, bh = a.h >> 2;
        unsigned long long k = ~0ull;
        if (nx > 0 && ny > 0)
            for (int i = t; i < nx * ny; i += nt) {
                const int y = i / nx, x = i - y * nx;
                const uint32_t s = xg_sad_part(a.in[2], bw, a.win[2] + (long long)y * a.wp[2] + x, a.wp[2], bw, bh, 0, 1);
                const unsigned long long kk = ((unsigned long long)s << 32) | (uint32_t)i;
                k = kk < k ? kk : k;
            }
        k = xg_cta_min64(k, red64);
        if (nx > 0 && ny > 0) { const int i = (int)(uint32_t)k; b2x = a.x0[2] + i % nx; b2y = a.y0[2] + i / nx; }
    }
    /* 1/2: +-1 around 2 * b2 */
    int b1x = (a.mvpx >> 2) >> 1, b1y = (a.mvpy >> 2) >> 1;
    {
        const int lx = max(2 * b2x - 1, a.x0[1]), hx = min(2 * b2x + 1, a.x1[1]);
        const int ly = max(2 * b2y - 1, a.y0[1]), hy = min(2 * b2y + 1, a.y1[1]);
        uint32_t bs1 = 0xFFFFFFFFu;
        for (int y = ly; y <= hy; y++)
            for (int x = lx; x <= hx; x++) {
                const xg_pix *r = a.win[1] + (long long)(y - a.y0[1]) * a.wp[1] + (x - a.x0[1]);
                const uint32_t s = xg_cta_sum(xg_sad_part(a.in[1], a.w >> 1, r, a.wp[1], a.w >> 1, a.h >> 1, t, nt), red);
                if (s < bs1) { bs1 = s; b1x = x; b1y = y; }
            }
    }
    /* full resolution: 3 x 3 around 2 * b1 */
    for (int y = 2 * b1y - 1; y <= 2 * b1y + 1; y++)
        for (int x = 2 * b1x - 1; x <= 2 * b1x + 1; x++) {
            if (x < a.x0[0] || x > a.x1[0] || y < a.y0[0] || y > a.y1[0]) continue;
            const uint32_t s = sad0(x, y), c = xg_full_cost(s, 4 * x, 4 * y, a.mvpx, a.mvpy, a.lambda);
            if (c < best) { best = c; bsad = s; bx = 4 * x; by = 4 * y; }
        }
    if (t == 0) { io[0] = bx; io[1] = by; io[2] = (int)best; io[3] = (int)bsad; }
}

extern "C" void XinGpuDownscale2x2(XG_PIXEL *input, intptr_t inputStride, int32_t haveRowAbove, int32_t haveRowBelow,
                                   XG_PIXEL *output, intptr_t outputStride, uint32_t outWidth, uint32_t outHeight)
{
    XG_BEGIN(t);
    XG_ARG(input && output && outWidth >= 1 && outHeight >= 1 && outWidth <= 8192 && outHeight <= 8192 &&
           inputStride >= (intptr_t)(2 * outWidth) && outputStride >= (intptr_t)outWidth,
           "Downscale2x2: bad pointer, size or stride");
    /* every open caller passes FALSE for both (h266_enc_init.c:2804-2824, h266_scene_cut.c:64) */
    XG_ARG(!haveRowAbove && !haveRowBelow, "Downscale2x2: only the form without the neighbouring rows is defined");
    const xg_pix *din = (const xg_pix *)xg_stage_in(t, input, inputStride, 2 * outWidth, 2 * outHeight, sizeof(xg_pix));
    XG_TRY(din);
    xg_pix *dout = (xg_pix *)xg_dalloc(t, (size_t)outWidth * outHeight * sizeof(xg_pix)); XG_TRY(dout);
    dim3 grd((outWidth + 127) / 128, outHeight);
    k_downscale2x2<<<grd, 128, 0, t->stream>>>(din, 2 * outWidth, dout, outWidth, (int)outWidth, (int)outHeight);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_stage_out(t, output, outputStride, dout, outWidth, outHeight, sizeof(xg_pix)) == 0);
    XG_TRY(xg_sync(t) == 0);
}

extern "C" void XinGpuMotionSearchHier(XG_PIXEL *input, intptr_t inputStride, XG_PIXEL *ref, intptr_t refStride, int32_t minMvX,
                                       int32_t maxMvX, int32_t minMvY, int32_t maxMvY, uint32_t width, uint32_t height,
                                       void *bestMv)
{
    XG_BEGIN(t);
    XG_ARG(input && ref && bestMv && width >= 1 && height >= 1 && width <= 128 && height <= 128, "MotionSearchHier: bad argument");
    XG_ARG(maxMvX - minMvX <= 1024 && maxMvY - minMvY <= 1024, "MotionSearchHier: window too large");
    if (maxMvX < minMvX || maxMvY < minMvY) return;    /* empty window: output unchanged */
    const int nx = maxMvX - minMvX + 1, ny = maxMvY - minMvY + 1, wp = nx + (int)width - 1, wh = ny + (int)height - 1;
    const xg_pix *din = (const xg_pix *)xg_stage_in(t, input, inputStride, width, height, sizeof(xg_pix)); XG_TRY(din);
    const xg_pix *dwin = (const xg_pix *)xg_stage_in(t, ref + (intptr_t)minMvY * refStride + minMvX, refStride, wp, wh,
                                                     sizeof(xg_pix));
    XG_TRY(dwin);
    unsigned long long *dk = (unsigned long long *)xg_dalloc(t, 8); XG_TRY(dk);
    k_hier_level<<<1, 256, 0, t->stream>>>(din, (int)width, (int)height, dwin, wp, nx, ny, dk);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(t->hbuf, dk, 8, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    const uint32_t i1 = (uint32_t)*(unsigned long long *)t->hbuf;
    if (!i1) return;
    xin_gpu_mv *mv = (xin_gpu_mv *)bestMv;
    mv->mv.mvX = (int16_t)(minMvX + (int)(i1 - 1) % nx);
    mv->mv.mvY = (int16_t)(minMvY + (int)(i1 - 1) / nx);
}

extern "C" void XinGpuMotionEstHier(struct xin_me_struct *meSetOpaque)
{
    xin_gpu_me_struct *me = (xin_gpu_me_struct *)meSetOpaque;
    XG_BEGIN(t);
    XG_ARG(me && me->input && me->ref && me->input1 && me->ref1 && me->input2 && me->ref2, "MotionEstHier: null state");
    const int w = (int)me->width, h = (int)me->height;
    XG_ARG(w >= 4 && h >= 4 && w <= 128 && h <= 128 && !(w & 3) && !(h & 3), "MotionEstHier: bad block size");
    const int rx = me->searchWidth, ry = me->searchHeight;
    XG_ARG(rx >= 0 && ry >= 0 && rx <= 512 && ry <= 512, "MotionEstHier: bad search range");
    XG_ARG(me->candNum <= 12, "MotionEstHier: more than 12 candidates");
    XgHierArgs a;
    memset(&a, 0, sizeof a);
    a.w = w; a.h = h;
    a.mvpx = me->predMv.mv.mvX; a.mvpy = me->predMv.mv.mvY;
    a.lambda = me->sadLambda;
    const int cx = a.mvpx >> 2, cy = a.mvpy >> 2;
    a.x0[0] = max(cx - rx, (int)me->minMv.mv.mvX); a.x1[0] = min(cx + rx, (int)me->maxMv.mv.mvX);
    a.y0[0] = max(cy - ry, (int)me->minMv.mv.mvY); a.y1[0] = min(cy + ry, (int)me->maxMv.mv.mvY);
    if (a.x1[0] < a.x0[0] || a.y1[0] < a.y0[0]) return;     /* empty window: state unchanged */
    for (int l = 1; l <= 2; l++) {
        a.x0[l] = xg_ceil_shr(a.x0[0], l); a.x1[l] = a.x1[0] >> l;
        a.y0[l] = xg_ceil_shr(a.y0[0], l); a.y1[l] = a.y1[0] >> l;
    }
    XG_PIXEL *ins[3] = { me->input, me->input1, me->input2 }, *refs[3] = { me->ref, me->ref1, me->ref2 };
    const intptr_t is[3] = { me->inputStride, me->input1Stride, me->input2Stride };
    const intptr_t rs[3] = { me->refStride, me->ref1Stride, me->ref2Stride };
    for (int l = 0; l < 3; l++) {
        const int bw = w >> l, bh = h >> l;
        a.in[l] = (const xg_pix *)xg_stage_in(t, ins[l], is[l], bw, bh, sizeof(xg_pix)); XG_TRY(a.in[l]);
        /* a level whose window is empty stages one block at its lower corner (never read) */
        const int nx = max(a.x1[l] - a.x0[l] + 1, 1), ny = max(a.y1[l] - a.y0[l] + 1, 1);
        a.wp[l] = nx + bw - 1;
        a.win[l] = (const xg_pix *)xg_stage_in(t, refs[l] + (intptr_t)a.y0[l] * rs[l] + a.x0[l], rs[l], a.wp[l], ny + bh - 1,
                                               sizeof(xg_pix));
        XG_TRY(a.win[l]);
    }
    a.ncand = (int)me->candNum;
    for (int i = 0; i < a.ncand; i++) { a.cand[i][0] = me->meCand[i].mv.mvX; a.cand[i][1] = me->meCand[i].mv.mvY; }
    int *dio = (int *)xg_dalloc(t, 16); XG_TRY(dio);
    int hio[4] = { me->bestMv.mv.mvX, me->bestMv.mv.mvY, (int)me->bestCost, (int)me->bestSad };
    memcpy(t->hbuf, hio, 16);
    XG_TRY(xg_cuda_check(cudaMemcpyAsync(dio, t->hbuf, 16, cudaMemcpyHostToDevice, t->stream), "h2d") == 0);
    k_me_hier_cu<<<1, 256, 0, t->stream>>>(a, dio);
    XG_TRY(xg_after_launch(t));
    XG_TRY(xg_cuda_check(cudaMemcpyAsync((char *)t->hbuf + 16, dio, 16, cudaMemcpyDeviceToHost, t->stream), "d2h") == 0);
    XG_TRY(xg_sync(t) == 0);
    const int *r = (const int *)((char *)t->hbuf + 16);
    me->bestMv.mv.mvX = (int16_t)r[0];
    me->bestMv.mv.mvY = (int16_t)r[1];
    me->bestCost = (uint32_t)r[2];
    me->bestSad = (uint32_t)r[3];
}

/* ------------------------------------------------------------ frame form
 * One CTA per (64 x 64 tile, CU level): the tile's CUs of that level.  The
 * quarter-resolution reference window of the whole tile (16 + 2 R4 samples
 * square, R4 = R >> 2, rows padded by 4 samples) and the tile's
 * quarter-resolution current samples are staged in shared memory.  A group of
 * G warps takes a CU (G = 8 / CUs a tile, at least 1): at 1/4 each lane
 * evaluates four horizontally adjacent candidates at a time from a sliding
 * window of reference samples; the 1/2 and full-resolution steps split the
 * block's samples over the group's lanes and read the planes directly.  Writes
 * the CU's key (cost << 32) | ((mvy + R) * (2R + 1) + mvx + R), the form the
 * tails read. */
struct XgHierFrameParams {
    XgPlane cur, ref;            /* full-resolution luma slots */
    XgPlane cur_lo[2], ref_lo[2];/* 1/2 and 1/4 resolution (pointers at picture (0, 0)) */
    int W, H, ctu, R;
    int level_size[4];           /* CU size of blockIdx.z */
    unsigned long long *keys[4];
    int cus_x[4];
};

#define XG_HIER_THREADS 256

/* this lane's shares of the SADs of a (1 << lgw) x h block against the 3 x 3
 * candidates around ctr (k = (dy + 1) * 3 + dx + 1, raster order) and, with
 * EXTRA, one more candidate at ext: one load of the current sample and
 * independent loads of the candidates' samples per position, so the loads of
 * all candidates are in flight together.  Samples i = t, t + nt, ... */
template <bool EXTRA>
__device__ __forceinline__ void xg_sad_3x3(const xg_pix *c, long long cp, const xg_pix *ctr, const xg_pix *ext, long long rp,
                                           int lgw, int h, int t, int nt, uint32_t s[10])
{
#pragma unroll
    for (int k = 0; k < 10; k++) s[k] = 0;
    const int n = h << lgw, wm = (1 << lgw) - 1;
    for (int i = t; i < n; i += nt) {
        const int y = i >> lgw, x = i & wm;
        const unsigned cv = c[(long long)y * cp + x];
        const xg_pix *r = ctr + (long long)y * rp + x;
#pragma unroll
        for (int k = 0; k < 9; k++) s[k] = __usad(cv, (unsigned)r[(k / 3 - 1) * rp + (k % 3 - 1)], s[k]);
        if (EXTRA) s[9] = __usad(cv, (unsigned)ext[(long long)y * rp + x], s[9]);
    }
}

/* TILE: 64 for CU levels 64 .. 8, 128 for the 128 x 128 level (CTU 128) */
template <int TILE>
__global__ void __launch_bounds__(XG_HIER_THREADS) k_hier_frame(XgHierFrameParams p, const XgPicParams *pp)
{
    constexpr int T4 = TILE / 4;                              /* the tile at 1/4 resolution */
    extern __shared__ __align__(16) xg_pix hs[];
    __shared__ unsigned long long wmin[8];
    __shared__ uint32_t wsum[8][10];
    const int S = p.level_size[blockIdx.z];
    const int lgS = S == 128 ? 7 : S == 64 ? 6 : S == 32 ? 5 : S == 16 ? 4 : 3;
    unsigned long long *keys = p.keys[blockIdx.z];
    const int cus_x = p.cus_x[blockIdx.z];
    const int R = p.R, R4 = R >> 2, WS = T4 + 2 * R4, WP = WS + 4;   /* window side, row pitch */
    const int tx0 = blockIdx.x * TILE, ty0 = blockIdx.y * TILE;
    xg_pix *win = hs, *cur4 = hs + WS * WP;                  /* [WS][WP], [T4][T4] */
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lambda = pp->lambda;
    /* a 128 tile holds one CU: without it (a partial tile) nothing is staged, so the
     * window never reaches past the planes' margins (R/4 + 18 samples at 1/4) */
    if (TILE == 128 && (tx0 + 128 > p.W || ty0 + 128 > p.H)) return;
    {
        const xg_pix *src = p.ref_lo[1].data + (long long)(ty0 / 4 - R4) * p.ref_lo[1].pitch + (tx0 / 4 - R4);
        for (int i = tid; i < WS * WP; i += XG_HIER_THREADS) {
            const int y = i / WP, x = i - y * WP;
            /* the four columns past the window feed only candidates beyond it */
            win[i] = x < WS ? src[(long long)y * p.ref_lo[1].pitch + x] : (xg_pix)0;
        }
        const xg_pix *cs = p.cur_lo[1].data + (long long)(ty0 / 4) * p.cur_lo[1].pitch + tx0 / 4;
        for (int i = tid; i < T4 * T4; i += XG_HIER_THREADS) cur4[i] = cs[(long long)(i / T4) * p.cur_lo[1].pitch + (i % T4)];
    }
    __syncthreads();
    const int per_row = TILE >> lgS, ncu = per_row * per_row;
    const int G = ncu >= 8 ? 1 : 8 / ncu;                     /* warps per CU */
    const int slots = 8 / G;                                  /* CUs in flight */
    const int b4 = S >> 2;
    const int grp = warp / G, gw = warp % G, gt = gw * 32 + lane, gn = 32 * G;   /* group, rank, thread in group */
    /* sums over the group of ten values per thread (every lane gets them) */
    auto gsum10 = [&](uint32_t v[10]) {
#pragma unroll
        for (int k = 0; k < 10; k++) v[k] = xg_warp_sum(v[k]);
        if (G == 1) return;
        if (lane < 10) {
#pragma unroll
            for (int k = 0; k < 10; k++) if (lane == k) wsum[warp][k] = v[k];
        }
        asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(gn) : "memory");
#pragma unroll
        for (int k = 0; k < 10; k++) {
            uint32_t t = 0;
            for (int j = 0; j < G; j++) t += wsum[grp * G + j][k];
            v[k] = t;
        }
        asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(gn) : "memory");
    };
    for (int c0 = 0; c0 < ncu; c0 += slots) {
        const int c = c0 + grp;
        const int cxi = (c % per_row) * S, cyi = (c / per_row) * S;
        const int cu_x = tx0 + cxi, cu_y = ty0 + cyi;
        const bool live = cu_x + S <= p.W && cu_y + S <= p.H;   /* uniform over the group */
        if (!live) continue;
        /* window (h266_enc_init.c:1462) within +-R */
        const int mnx = (int16_t)(-cu_x - p.ctu - 8), mny = (int16_t)(-cu_y - p.ctu - 8);
        const int mxx = (int16_t)(p.W + (p.ctu - S + 8) - cu_x), mxy = (int16_t)(p.H + (p.ctu - S + 8) - cu_y);
        const int lox = max(-R, mnx), hix = min(R, mxx), loy = max(-R, mny), hiy = min(R, mxy);
        /* ---- 1/4: exhaustive over the level window, four adjacent candidates a lane */
        const int lx4 = xg_ceil_shr(lox, 2), hx4 = hix >> 2, ly4 = xg_ceil_shr(loy, 2), hy4 = hiy >> 2;
        const int nx4 = hx4 - lx4 + 1, ny4 = hy4 - ly4 + 1;
        unsigned long long k = ~0ull;
        if (nx4 > 0 && ny4 > 0) {
            const int qpr = (nx4 + 3) >> 2, nq = qpr * ny4;      /* quads per row, quads */
            const xg_pix *cb = cur4 + (cyi >> 2) * T4 + (cxi >> 2);
            const xg_pix *wb = win + ((cyi >> 2) + R4 + ly4) * WP + (cxi >> 2) + R4 + lx4;
            int qy = gt / qpr, qx = gt - qy * qpr;              /* this lane's first quad */
            const int sy = gn / qpr, sx = gn - sy * qpr;        /* its step */
            for (int q = gt; q < nq; q += gn) {
                const xg_pix *r = wb + qy * WP + 4 * qx;
                uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                for (int yy = 0; yy < b4; yy++) {
                    const xg_pix *cr = cb + yy * T4, *rr = r + yy * WP;
                    unsigned w0 = rr[0], w1 = rr[1], w2 = rr[2];
                    for (int j = 0; j < b4; j++) {
                        const unsigned w3 = rr[j + 3], cv = cr[j];
                        s0 = __usad(cv, w0, s0); s1 = __usad(cv, w1, s1); s2 = __usad(cv, w2, s2); s3 = __usad(cv, w3, s3);
                        w0 = w1; w1 = w2; w2 = w3;
                    }
                }
                const int x0 = 4 * qx, i0 = qy * nx4 + x0;
                const uint32_t sv[4] = { s0, s1, s2, s3 };
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (x0 + u < nx4) {
                        const unsigned long long kk = ((unsigned long long)sv[u] << 32) | (uint32_t)(i0 + u);
                        k = kk < k ? kk : k;
                    }
                qx += sx; qy += sy;
                if (qx >= qpr) { qx -= qpr; qy++; }
            }
        }
        k = xg_warp_min64(k);
        if (G > 1) {
            if (lane == 0) wmin[warp] = k;
            asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(gn) : "memory");
            for (int j = 0; j < G; j++) { const unsigned long long v = wmin[grp * G + j]; k = v < k ? v : k; }
            asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(gn) : "memory");
        }
        int b2x = 0, b2y = 0;
        if (nx4 > 0 && ny4 > 0) { const int i = (int)(uint32_t)k; b2y = i / nx4; b2x = lx4 + (i - b2y * nx4); b2y += ly4; }
        /* ---- 1/2: +-1 around 2 * b2 (the nine SADs in one pass; candidates
         * outside the level window are computed and passed over: the planes'
         * margins hold them) */
        int b1x = 0, b1y = 0;
        {
            const int l1x = xg_ceil_shr(lox, 1), h1x = hix >> 1, l1y = xg_ceil_shr(loy, 1), h1y = hiy >> 1;
            const long long cpl = p.cur_lo[0].pitch, rpl = p.ref_lo[0].pitch;
            const xg_pix *cb = p.cur_lo[0].data + (long long)(cu_y >> 1) * cpl + (cu_x >> 1);
            const xg_pix *rc = p.ref_lo[0].data + (long long)((cu_y >> 1) + 2 * b2y) * rpl + (cu_x >> 1) + 2 * b2x;
            uint32_t sv[10];
            xg_sad_3x3<false>(cb, cpl, rc, rc, rpl, lgS - 1, S >> 1, gt, gn, sv);
            gsum10(sv);
            uint32_t bs = 0xFFFFFFFFu;
#pragma unroll
            for (int k = 0; k < 9; k++) {
                const int x = 2 * b2x + k % 3 - 1, y = 2 * b2y + k / 3 - 1;
                if (x < l1x || x > h1x || y < l1y || y > h1y) continue;
                if (sv[k] < bs) { bs = sv[k]; b1x = x; b1y = y; }
            }
        }
        /* ---- full resolution: the zero MV (the frame form's predictor and first
         * candidate), then 3 x 3 around 2 * b1, in one pass */
        const long long cp = p.cur.pitch, rp = p.ref.pitch;
        const xg_pix *cb = p.cur.data + (long long)cu_y * cp + cu_x;
        const xg_pix *rb = p.ref.data + (long long)cu_y * rp + cu_x;
        uint32_t sv[10];
        xg_sad_3x3<true>(cb, cp, rb + (long long)(2 * b1y) * rp + 2 * b1x, rb, rp, lgS, S, gt, gn, sv);
        gsum10(sv);
        uint32_t best = (sv[9] << XG_COST_FRACTION) + 2 * xg_mvd_bits(0) * lambda;
        int bx = 0, by = 0;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int x = 2 * b1x + k % 3 - 1, y = 2 * b1y + k / 3 - 1;
            if (x < lox || x > hix || y < loy || y > hiy) continue;
            const uint32_t cst = xg_full_cost(sv[k], 4 * x, 4 * y, 0, 0, lambda);
            if (cst < best) { best = cst; bx = x; by = y; }
        }
        if (gt == 0)
            keys[(cu_y >> lgS) * cus_x + (cu_x >> lgS)] = ((unsigned long long)best << 32) | (uint32_t)((by + R) * (2 * R + 1) + bx + R);
    }
}

/* shared memory of k_hier_frame<TILE> for search range R */
static size_t xg_hier_smem(int R, int tile = 64)
{
    const int t4 = tile / 4, ws = t4 + 2 * (R >> 2);
    return (size_t)(ws * (ws + 4) + t4 * t4) * sizeof(xg_pix);
}
