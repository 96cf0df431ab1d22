/*
 * xg_frame.cuh -- host side of the batched frame form (xin_gpu_stream_*,
 * xin_gpu_frame_*): device-resident picture slots, quarter-pel planes and
 * outputs; the per-picture launches captured once per slot into a CUDA graph.
 */
#include "xg_frame_kernels.cuh"
#include "xg_hier.cuh"

#include <chrono>
#include <new>
#include <string.h>
#include <map>
#include <mutex>
#include <thread>

/* CU levels: 64 .. 8 (every configuration), then 128 (CTU 128 with the search by
 * resolution levels): results are level-major in this order */
#define XG_NLEV 5
static const int XG_LEVEL_SIZE[XG_NLEV] = { 64, 32, 16, 8, 128 };

struct XgTuState;   /* the preset-4 TU stage (xg_tu.cuh) */

#define XG_MAX_DPB 32      /* picture slots a stream may keep */
/* captured graphs a stream keeps: one per (picture set, slot, list-0 slot, list-1
 * slot) met; beyond this the launches of a new combination run directly */
#define XG_MAX_GRAPHS 72

struct xin_gpu_stream {
    xin_gpu_stream_cfg cfg;
    int pad, pitch, cpad, cpitch, rows, crows;
    int lev_on[XG_NLEV], lev_first[XG_NLEV], lev_cx[XG_NLEV], lev_cy[XG_NLEV];
    int nlev, ncus;
    size_t plane_elems, cplane_elems;
    /* picture slots: picture k fills slot k % nslots; its references are the
     * slots of earlier pictures at most nslots - 1 back (by default list 0 the
     * previous picture, list 1 the one before) */
    int nslots;
    xg_pix *slot_base[XG_MAX_DPB][3];
    XgPlane slot[XG_MAX_DPB][3];
    xg_pix *qpel_base[XG_MAX_DPB];
    XgQpel qpel[XG_MAX_DPB];
    /* search_mode 1: luma at 1/2 and 1/4 resolution of each slot, downscaled from
     * the padded slot as a whole (the margins included) */
    xg_pix *lo_base[XG_MAX_DPB][2];
    XgPlane lo[XG_MAX_DPB][2];
    int lo_pitch[2], lo_rows[2];
    CUtensorMap tm_qp[XG_MAX_DPB];     /* TMA map of each slot's padded luma plane: quarter-pel tiles */
    long long wait_tries;  /* bound of the kernels' waits (polls) */
    /* the integer search's results, one buffer per picture set (so that a picture's
     * search may run beside the previous picture's tails); keys / keys1 point at
     * the buffers of the set being enqueued */
    unsigned long long *keys_base, *keys1_base;
    unsigned long long *keys;
    unsigned long long *keys1;         /* refs 2: list 1's integer search */
    /* what a picture in flight owns; picture k uses set k & 1 (its slot), so two
     * pictures can be in flight: one computing while the other's copies run */
    struct Set {
        xin_gpu_cu_result *dres;
        xin_gpu_cu_mts *dmts, *h_mts;    /* tu_mode 1: per-CU transform candidates */
        xin_gpu_cu_bi *dbi, *h_bi;       /* refs 2: per-CU list-1 search, bi pair and choice */
        xg_coef *dq[3];
        xg_pix *drec[3];
        XgPicParams *dpp;
        uint8_t *d_in8[3];     /* 8-bit input pictures (10-bit library, input_bitdepth 8): device staging */
        /* pinned host staging (input samples of in_es bytes) */
        xg_pix *h_in[3];
        XgPicParams *h_pp;
        int32_t *h_stat;       /* the picture's device status (XgPicParams.status), read back with the results */
        xin_gpu_cu_result *h_res;
        xg_coef *h_q[3];
        xg_coef *q_dst[3];     /* this picture's coefficient planes go here instead of h_q (caller buffers) */
        xg_pix *h_rec[3];
        cudaEvent_t ev0, ev1;  /* submitted; results in host memory */
        cudaEvent_t ev_kern;   /* kernels done (the copy stream waits on it) */
        cudaEvent_t ev_up;     /* the picture's parameters / staged samples are on the device */
        cudaEvent_t evs[5];    /* stage boundaries, recorded inside the picture's launches */
        cudaStream_t pst;      /* the picture's launches (a stream per set, so that the TU stage of
                                  one picture runs beside the next picture's search and tails) */
        cudaEvent_t ev_main;   /* the picture's reference planes, search and tails are done */
        cudaEvent_t ev_ref;    /* its slot, downscaled and quarter-pel planes are done (what the next
                                  picture reads of it) */
        int rd[3];             /* the slots the picture reads: its own, list 0's and list 1's */
    } set[2];
    cudaStream_t st;
    cudaStream_t cst;      /* result copies (device to host) */
    cudaStream_t ust;      /* uploads of the next picture's parameters and staged samples */
    cudaStream_t tst;      /* side branch that records the search's end (stage timing) */
    cudaEvent_t ev_tfork, ev_tjoin;
    cudaStream_t aux[XG_NLEV - 1];   /* the tails of levels 2..5 run beside the first level's */
    cudaStream_t auxq;     /* quarter-pel planes of the new picture, beside the search (low priority) */
    cudaEvent_t ev_fork, ev_join[XG_NLEV - 1], ev_qfork, ev_qjoin;
    /* captured graphs by (picture set, slot, list-0 slot, list-1 slot) */
    std::map<uint32_t, std::pair<cudaGraphExec_t, int>> graphs;   /* exec, kernels inside */
    int me_bands, me_band_rows, me_band_rows_alloc, me_row_words, me_nb;
    size_t me_smem;
    int sbd;               /* sample depth the integer search runs at (8 or 10) */
    bool widen;            /* 10-bit library fed 8-bit pictures: samples << 2 on the way in */
    size_t in_es;          /* bytes per input sample */
    int nsub;              /* pictures submitted */
    int ndone;             /* pictures collected by frame_wait (the oldest first) */
    XgTuState *tu[2];      /* tu_mode 1: per picture set */
    int prio_hi;           /* the most urgent stream priority (the tails' launches) */
    int tail_cpb[2];       /* CUs per CTA of the plain 16 x 16 and 8 x 8 tails (2, 4 or 8; warp per CU) */
    int tune_n;            /* the last xin_gpu_stream_tune_search: geometries timed */
    int32_t tune_bands[6];
    float tune_ms[6];
};

static int xg_tu_open(xin_gpu_stream *s, int set);
static void xg_tu_free(XgTuState *u);
static int xg_tu_enqueue(xin_gpu_stream *s, int set, int cur, xin_gpu_stream::Set &t, cudaStream_t st);
static uint64_t xg_tu_bytes(const xin_gpu_stream_cfg *c);
static int16_t *xg_tu_resid(XgTuState *u, int level, int plane);

static void xg_quant_params(int qp, int lg, int intra_frame, XgQuant *q)
{
    /* qMult / iqMult tables and shifts of Xin266ConstructQuantParam (h266_encoder_create.c:94-105,1677-1707),
     * per-TU adjustment and rounding of Xin266Transform (h266_trans_quant.c:107-120), square TU, DCT2, no RDOQ */
    static const int qm[6] = { 26214, 23302, 20560, 18396, 16384, 14564 };
    static const int iqm[6] = { 40, 45, 51, 57, 64, 72 };
    if (XG_BITDEPTH == 10) qp += 12;
    int per = qp / 6, rem = qp % 6;
    q->qmult = qm[rem];
    q->iqmult = iqm[rem] << per;
    q->qshift = 14 + (15 - XG_BITDEPTH) + per - lg;
    q->iqshift = 6 - (15 - XG_BITDEPTH) + lg;
    q->qadd = (intra_frame ? 171 : 85) << (q->qshift - 9);
    q->iqadd = 1 << (q->iqshift - 1);
}

static int xg_stream_free(xin_gpu_stream *s)
{
    if (!s) return XIN_GPU_OK;
    if (s->ust) cudaStreamSynchronize(s->ust);
    if (s->st) cudaStreamSynchronize(s->st);
    for (auto &t : s->set) if (t.pst) cudaStreamSynchronize(t.pst);
    if (s->cst) cudaStreamSynchronize(s->cst);
    for (auto &g : s->graphs) cudaGraphExecDestroy(g.second.first);
    s->graphs.clear();
    for (int i = 0; i < XG_MAX_DPB; i++) {
        for (int p = 0; p < 3; p++) cudaFree(s->slot_base[i][p]);
        cudaFree(s->qpel_base[i]);
        for (int l = 0; l < 2; l++) cudaFree(s->lo_base[i][l]);
    }
    cudaFree(s->keys_base);
    cudaFree(s->keys1_base);
    xg_tu_free(s->tu[0]);
    xg_tu_free(s->tu[1]);
    for (auto &t : s->set) {
        cudaFree(t.dres); cudaFree(t.dpp); cudaFree(t.dmts); cudaFreeHost(t.h_mts); cudaFree(t.dbi); cudaFreeHost(t.h_bi);
        for (int p = 0; p < 3; p++) { cudaFree(t.dq[p]); cudaFree(t.drec[p]); cudaFree(t.d_in8[p]); cudaFreeHost(t.h_in[p]); cudaFreeHost(t.h_q[p]); cudaFreeHost(t.h_rec[p]); }
        cudaFreeHost(t.h_pp); cudaFreeHost(t.h_res); cudaFreeHost(t.h_stat);
        for (int i = 0; i < 5; i++) if (t.evs[i]) cudaEventDestroy(t.evs[i]);
        if (t.ev0) cudaEventDestroy(t.ev0);
        if (t.ev1) cudaEventDestroy(t.ev1);
        if (t.ev_kern) cudaEventDestroy(t.ev_kern);
        if (t.ev_up) cudaEventDestroy(t.ev_up);
        if (t.ev_main) cudaEventDestroy(t.ev_main);
        if (t.ev_ref) cudaEventDestroy(t.ev_ref);
        if (t.pst) cudaStreamDestroy(t.pst);
    }
    if (s->cst) cudaStreamDestroy(s->cst);
    if (s->ust) cudaStreamDestroy(s->ust);
    if (s->tst) cudaStreamDestroy(s->tst);
    if (s->ev_tfork) cudaEventDestroy(s->ev_tfork);
    if (s->ev_tjoin) cudaEventDestroy(s->ev_tjoin);
    for (int i = 0; i < XG_NLEV - 1; i++) {
        if (s->ev_join[i]) cudaEventDestroy(s->ev_join[i]);
        if (s->aux[i]) cudaStreamDestroy(s->aux[i]);
    }
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    if (s->ev_qfork) cudaEventDestroy(s->ev_qfork);
    if (s->ev_qjoin) cudaEventDestroy(s->ev_qjoin);
    if (s->auxq) cudaStreamDestroy(s->auxq);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return XIN_GPU_OK;
}

/* integer-search band geometry from a starting number of candidate-row bands
 * per 64 x 64 tile (more bands: more CTAs, less reuse of each staged row):
 * shared memory within XG_ME_SMEM_MAX, taking more bands or fewer buffered
 * passes for the 32x32 / 64x64 sums (more barriers) when it does not fit;
 * false when no geometry fits */
static bool xg_me_geometry(xin_gpu_stream *s, int bands)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    const int R = c.search_range, ndy = 2 * R + 1;
    if (bands < 1) bands = 1;
    if (bands > ndy) bands = ndy;
    {
        /* word positions per band row; pitch congruent to nx (mod 32) */
        int nx = 2 * R + 1, relw = xg_me_relw(s->sbd, nx);
        s->me_row_words = relw + (((nx - relw) % 32) + 32) % 32;
    }
    for (;;) {
        s->me_band_rows = (ndy + bands - 1) / bands;
        const int dr = xg_me_d(s->sbd);
        int rows_rounded = (s->me_band_rows + dr - 1) / dr * dr;   /* rounded up to the per-lane chunk */
        s->me_band_rows_alloc = 64 + rows_rounded - 1;
        size_t fixed = (size_t)s->me_band_rows_alloc * s->me_row_words + (2 * R + 1) + s->me_band_rows_alloc + xg_me_cur_words(s->sbd);
        s->me_nb = 0;
        for (int nb = XG_ME_NB_MAX; nb >= 1 && !s->me_nb; nb /= 2)
            if (sizeof(uint32_t) * (fixed + xg_me_agg_words(s->sbd, nb)) <= XG_ME_SMEM_MAX) s->me_nb = nb;
        if (s->me_nb) {
            s->me_smem = sizeof(uint32_t) * (fixed + xg_me_agg_words(s->sbd, s->me_nb));
            break;
        }
        if (s->me_band_rows == 1) return false;
        bands++;
    }
    s->me_bands = (ndy + s->me_band_rows - 1) / s->me_band_rows;
    return true;
}

/* input_bitdepth: 0 or the library's depth, or 8 in the 10-bit library */
static bool xg_input_depth_ok(const xin_gpu_stream_cfg &c)
{
    return c.input_bitdepth == 0 || c.input_bitdepth == XG_BITDEPTH || (XG_BITDEPTH == 10 && c.input_bitdepth == 8);
}
/* bytes per input sample */
static size_t xg_in_es(const xin_gpu_stream_cfg &c)
{
    return (XG_BITDEPTH == 10 && c.input_bitdepth == 8) ? 1 : sizeof(xg_pix);
}

extern "C" int xin_gpu_stream_open(const xin_gpu_stream_cfg *cfg, xin_gpu_stream **out)
{
    xin_gpu_clear_error();
    if (!cfg || !out) { xg_set_error(XIN_GPU_ERR_ARG, "stream_open: null argument"); return XIN_GPU_ERR_ARG; }
    *out = nullptr;
    if (xg_ensure_init()) return XIN_GPU_ERR_CUDA;
    const xin_gpu_stream_cfg &c = *cfg;
    if (c.width < 16 || c.height < 16 || (c.width & 1) || (c.height & 1) || c.width > 8192 || c.height > 8192 ||
        (c.ctu_size != 64 && c.ctu_size != 128) || c.search_range < 1 || c.search_range > 256 ||
        !(c.level_mask & (8u | 16u | 32u | 64u | 128u)) || (c.level_mask & ~(8u | 16u | 32u | 64u | 128u)) ||
        !xg_input_depth_ok(c) || (c.search_mode != 0 && c.search_mode != 1) || (c.tu_mode != 0 && c.tu_mode != 1) ||
        ((c.level_mask & 128u) && (c.ctu_size != 128 || c.search_mode != 1 || c.tu_mode != 0)) || c.refs < 0 || c.refs > 2 ||
        (c.refs == 2 && (c.level_mask & 128u)) || c.dpb < 0 || c.dpb > XG_MAX_DPB || (c.dpb && c.dpb < (c.refs == 2 ? 3 : 2))) {
        xg_set_error(XIN_GPU_ERR_ARG, "stream_open: unsupported size, CTU, search range, level mask, input bit depth, search or "
                                      "TU mode, or references (the 128 x 128 level needs CTU 128, the search by levels and TU "
                                      "mode 0; two references need CU levels up to 64; dpb 0 or refs + 1 .. 32)");
        return XIN_GPU_ERR_ARG;
    }
    xin_gpu_stream *s = new (std::nothrow) xin_gpu_stream();
    if (!s) { xg_set_error(XIN_GPU_ERR_NOMEM, "stream_open: host allocation"); return XIN_GPU_ERR_NOMEM; }
    s->cfg = c;
    s->widen = XG_BITDEPTH == 10 && c.input_bitdepth == 8;
    s->sbd = s->widen ? 8 : XG_BITDEPTH;
    s->in_es = s->widen ? 1 : sizeof(xg_pix);
    s->nslots = c.dpb ? c.dpb : (c.refs == 2 ? 3 : 2);
    /* margin: the reference pads ctu + 16; the tile search also reads R + 64 + 8 around full tiles */
    int pad = c.ctu_size + 16 > c.search_range + 72 ? c.ctu_size + 16 : c.search_range + 72;
    pad = (pad + 31) & ~31;
    s->pad = pad;
    s->pitch = ((c.width + 2 * pad) + 127) & ~127;
    s->rows = c.height + 2 * pad;
    s->cpad = pad / 2;
    s->cpitch = ((c.width / 2 + 2 * s->cpad) + 127) & ~127;
    s->crows = c.height / 2 + 2 * s->cpad;
    s->plane_elems = (size_t)s->pitch * s->rows;
    s->cplane_elems = (size_t)s->cpitch * s->crows;
    int first = 0;
    for (int L = 0; L < XG_NLEV; L++) {
        int sz = XG_LEVEL_SIZE[L];
        s->lev_on[L] = (c.level_mask & (uint32_t)sz) != 0;
        s->lev_cx[L] = c.width / sz;
        s->lev_cy[L] = c.height / sz;
        s->lev_first[L] = first;
        if (s->lev_on[L]) { first += s->lev_cx[L] * s->lev_cy[L]; s->nlev++; }
    }
    s->ncus = first;

    cudaError_t e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cst, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->ust, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->tst, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_tfork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_tjoin, cudaEventDisableTiming);
    for (auto &t : s->set) {
        if (e == cudaSuccess) e = cudaEventCreate(&t.ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&t.ev1);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.ev_kern, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.ev_up, cudaEventDisableTiming);
        for (int i = 0; i < 5 && e == cudaSuccess; i++) e = cudaEventCreate(&t.evs[i]);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&t.pst, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.ev_main, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.ev_ref, cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_qfork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_qjoin, cudaEventDisableTiming);
    if (e == cudaSuccess) {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);    /* lo: the least urgent */
        s->prio_hi = hi;
        e = cudaStreamCreateWithPriority(&s->auxq, cudaStreamNonBlocking, lo);
    }
    for (int i = 0; i < XG_NLEV - 1 && e == cudaSuccess; i++) {
        e = cudaStreamCreateWithFlags(&s->aux[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join[i], cudaEventDisableTiming);
    }
    size_t ysz = s->plane_elems * sizeof(xg_pix), csz = s->cplane_elems * sizeof(xg_pix);
    size_t lq = (size_t)c.width * c.height, lc = lq / 4;
    for (int i = 0; i < s->nslots && e == cudaSuccess; i++) {
        for (int p = 0; p < 3 && e == cudaSuccess; p++) e = cudaMalloc(&s->slot_base[i][p], p ? csz : ysz);
        if (e == cudaSuccess) e = cudaMalloc(&s->qpel_base[i], 16 * ysz);
        for (int l = 0; l < 2 && e == cudaSuccess && c.search_mode == 1; l++) {
            s->lo_pitch[l] = (((c.width + 2 * pad) >> (l + 1)) + 127) & ~127;
            s->lo_rows[l] = (c.height + 2 * pad) >> (l + 1);
            e = cudaMalloc(&s->lo_base[i][l], (size_t)s->lo_pitch[l] * s->lo_rows[l] * sizeof(xg_pix));
        }
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->keys_base, 2 * sizeof(unsigned long long) * (s->ncus > 0 ? s->ncus : 1));
    if (e == cudaSuccess && c.refs == 2) e = cudaMalloc(&s->keys1_base, 2 * sizeof(unsigned long long) * (s->ncus > 0 ? s->ncus : 1));
    s->keys = s->keys_base;
    s->keys1 = s->keys1_base;
    for (auto &t : s->set) {
        if (e == cudaSuccess) e = cudaMalloc(&t.dres, sizeof(xin_gpu_cu_result) * s->ncus);
        if (e == cudaSuccess && c.refs == 2) e = cudaMalloc(&t.dbi, sizeof(xin_gpu_cu_bi) * s->ncus);
        if (e == cudaSuccess && c.refs == 2 && !c.device_io) e = cudaMallocHost(&t.h_bi, sizeof(xin_gpu_cu_bi) * s->ncus);
        if (e == cudaSuccess && c.tu_mode == 1) e = cudaMalloc(&t.dmts, sizeof(xin_gpu_cu_mts) * s->ncus);
        if (e == cudaSuccess && c.tu_mode == 1 && !c.device_io) e = cudaMallocHost(&t.h_mts, sizeof(xin_gpu_cu_mts) * s->ncus);
        if (e == cudaSuccess) e = cudaMalloc(&t.dpp, sizeof(XgPicParams));
        for (int p = 0; p < 3 && e == cudaSuccess; p++) {
            size_t n = (p ? lc : lq) * s->nlev;
            e = cudaMalloc(&t.dq[p], n * sizeof(xg_coef));
            if (e == cudaSuccess) e = cudaMalloc(&t.drec[p], n * sizeof(xg_pix));
            /* the kernels write only the area a level's CUs cover: the rest stays zero
             * (ordered on the stream, before any picture's launches) */
            if (e == cudaSuccess) e = cudaMemsetAsync(t.dq[p], 0, n * sizeof(xg_coef), t.pst);
            if (e == cudaSuccess) e = cudaMemsetAsync(t.drec[p], 0, n * sizeof(xg_pix), t.pst);
            if (c.device_io) continue;
            if (e == cudaSuccess && s->widen) e = cudaMalloc(&t.d_in8[p], p ? lc : lq);
            if (e == cudaSuccess) e = cudaMallocHost(&t.h_in[p], (p ? lc : lq) * s->in_es);
            if (e == cudaSuccess && (c.out_flags & XIN_GPU_OUT_Q)) e = cudaMallocHost(&t.h_q[p], n * sizeof(xg_coef));
            if (e == cudaSuccess && (c.out_flags & XIN_GPU_OUT_REC)) e = cudaMallocHost(&t.h_rec[p], n * sizeof(xg_pix));
        }
        if (e == cudaSuccess) e = cudaMallocHost(&t.h_pp, sizeof(XgPicParams));
        if (e == cudaSuccess) e = cudaMallocHost(&t.h_stat, sizeof(int32_t));
        if (e == cudaSuccess) *t.h_stat = 0;
        if (e == cudaSuccess) e = cudaMallocHost(&t.h_res, sizeof(xin_gpu_cu_result) * s->ncus);
    }
    if (e != cudaSuccess) {
        int st = (e == cudaErrorMemoryAllocation) ? XIN_GPU_ERR_NOMEM : XIN_GPU_ERR_CUDA;
        xg_set_error(st, "stream_open: %s", cudaGetErrorString(e));
        cudaGetLastError();
        xg_stream_free(s);
        return st;
    }
    for (int i = 0; i < s->nslots; i++) {
        for (int p = 0; p < 3; p++) {
            XgPlane &pl = s->slot[i][p];
            int pd = p ? s->cpad : s->pad, pt = p ? s->cpitch : s->pitch;
            pl.data = s->slot_base[i][p] + (size_t)pd * pt + pd;
            pl.pitch = pt;
            pl.w = p ? c.width / 2 : c.width;
            pl.h = p ? c.height / 2 : c.height;
            pl.pad = pd;
        }
        for (int l = 0; l < 2 && c.search_mode == 1; l++) {
            XgPlane &pl = s->lo[i][l];
            const int pd = pad >> (l + 1);
            pl.data = s->lo_base[i][l] + (size_t)pd * s->lo_pitch[l] + pd;
            pl.pitch = s->lo_pitch[l];
            pl.w = c.width >> (l + 1); pl.h = c.height >> (l + 1); pl.pad = pd;
        }
        XgQpel &q = s->qpel[i];
        for (int k = 0; k < 16; k++) q.plane[k] = s->qpel_base[i] + (size_t)k * s->plane_elems + (size_t)pad * s->pitch + pad;
        q.plane[0] = s->slot[i][0].data;
        q.pitch = s->pitch; q.w = c.width; q.h = c.height; q.pad = pad;
        /* the search stages reference rows with 16-byte loads from 8-sample-aligned columns */
        if (((uintptr_t)s->slot[i][0].data & 15) || (s->pitch & 7)) {
            xg_set_error(XIN_GPU_ERR_CUDA, "stream_open: luma slot not 16-byte aligned");
            xg_stream_free(s);
            return XIN_GPU_ERR_CUDA;
        }
    }
    /* the quarter-pel plane kernel's compile-time taps are the table's phases 4, 8, 12 */
    for (int f = 0; f < 3; f++)
        for (int k = 0; k < 8; k++)
            if (h_luma_taps[0][4 * (f + 1)][k] != xg_qp_tap(f, k)) {
                xg_set_error(XIN_GPU_FAIL, "stream_open: quarter-pel taps differ from the luma filter table");
                xg_stream_free(s);
                return XIN_GPU_FAIL;
            }
    /* integer-search band geometry: enough CTAs for the GPU; shared memory within
     * XG_ME_SMEM_MAX, taking more bands (less reuse of staged rows) or fewer
     * buffered passes for the 32x32 / 64x64 sums (more barriers) when it does not fit */
    int tiles = ((c.width + 63) / 64) * ((c.height + 63) / 64);
    if (!xg_me_geometry(s, (4 * 152 + tiles - 1) / tiles)) {
        xg_set_error(XIN_GPU_ERR_ARG, "stream_open: search range %d needs more shared memory than a CTA has", c.search_range);
        xg_stream_free(s);
        return XIN_GPU_ERR_ARG;
    }
    /* the limit is per kernel, not per launch: set it once to the most any
     * stream uses, so that streams of other sizes opened later (on any thread)
     * cannot lower it under a stream already running */
    static std::once_flag me_attr_once;
    static cudaError_t me_attr_err = cudaSuccess;
    std::call_once(me_attr_once, [] {
        me_attr_err = cudaFuncSetAttribute(k_me_tiles<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, XG_ME_SMEM_MAX);
#if XG_BITDEPTH == 10
        if (me_attr_err == cudaSuccess)
            me_attr_err = cudaFuncSetAttribute(k_me_tiles<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, XG_ME_SMEM_MAX);
#endif
    });
    if (xg_cuda_check(me_attr_err, "me smem attribute")) { xg_stream_free(s); return XIN_GPU_ERR_CUDA; }
    if (s->lev_on[4]) {
        /* the 128 x 128 level's kernels take more than the default 48 KB of shared memory */
        static std::once_flag l128_once;
        static cudaError_t l128_err = cudaSuccess;
        std::call_once(l128_once, [] {
            l128_err = cudaFuncSetAttribute(k_hier_frame<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)xg_hier_smem(256, 128));
            if (l128_err == cudaSuccess)
                l128_err = cudaFuncSetAttribute(k_cu_tail<128, 128, 1, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)xg_tail_smem<128, 128, 1>());
        });
        if (xg_cuda_check(l128_err, "128 x 128 level smem attribute")) { xg_stream_free(s); return XIN_GPU_ERR_CUDA; }
    }
    if (c.refs == 2) {
        /* the bi search's 64 x 64 tails take more than the default 48 KB of shared memory */
        static std::once_flag bi_once;
        static cudaError_t bi_err = cudaSuccess;
        std::call_once(bi_once, [] {
            bi_err = cudaFuncSetAttribute(k_cu_tail<64, 128, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)xg_tail_smem<64, 128, 1, true>());
        });
        if (xg_cuda_check(bi_err, "bi tail smem attribute")) { xg_stream_free(s); return XIN_GPU_ERR_CUDA; }
    }
    s->tail_cpb[0] = s->tail_cpb[1] = 4;
    s->wait_tries = XG_TMA_WAIT_TRIES;
    /* TMA maps of the padded luma slots for the quarter-pel tiles: the box of
     * tile (bx, by) starts at padded column XG_QP_TW bx (16-byte aligned) */
    for (int i = 0; i < s->nslots; i++)
        if (!xg_tma_map_2d(&s->tm_qp[i], s->slot_base[i][0], (int)sizeof(xg_pix), c.width + 2 * pad, c.height + 2 * pad,
                           s->pitch, XG_QP_BW, XG_QP_TH + 7)) {
            const int st = xin_gpu_last_status();
            xg_stream_free(s);
            return st;
        }
    if (c.tu_mode == 1)
        for (int i = 0; i < 2; i++) {
            const int st = xg_tu_open(s, i);
            if (st) { xg_stream_free(s); return st; }
        }
    *out = s;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_stream_close(xin_gpu_stream *s) { return xg_stream_free(s); }
extern "C" int xin_gpu_stream_num_cus(const xin_gpu_stream *s) { return s ? s->ncus : 0; }
extern "C" int xin_gpu_stream_num_levels(const xin_gpu_stream *s) { return s ? s->nlev : 0; }
extern "C" int xin_gpu_stream_level_info(const xin_gpu_stream *s, int level, int32_t *size, int32_t *first_cu, int32_t *cus_x,
                                         int32_t *cus_y)
{
    if (!s) return XIN_GPU_ERR_ARG;
    int k = 0;
    for (int L = 0; L < XG_NLEV; L++) {
        if (!s->lev_on[L]) continue;
        if (k++ != level) continue;
        if (size) *size = XG_LEVEL_SIZE[L];
        if (first_cu) *first_cu = s->lev_first[L];
        if (cus_x) *cus_x = s->lev_cx[L];
        if (cus_y) *cus_y = s->lev_cy[L];
        return XIN_GPU_OK;
    }
    return XIN_GPU_ERR_ARG;
}

/* stage-boundary event: inside a stream capture it must be an external record
 * node to be recorded when the graph runs; outside a capture a plain record */
static void xg_stage_event(cudaEvent_t e, cudaStream_t st, bool capturing)
{
    if (capturing) cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    else cudaEventRecord(e, st);
}

/* completion event of the last submitted picture */
static cudaEvent_t xg_stream_last_event(const xin_gpu_stream *s) { return s->set[(s->nsub - 1) & 1].ev1; }



/* quarter-pel planes of slot cur on the low-priority stream, after ev_qfork; then
 * `ready` (the picture's planes are all written, ev_ref) */
static void xg_stage_event(cudaEvent_t e, cudaStream_t st, bool capturing);
static int xg_enqueue_qpel(xin_gpu_stream *s, int cur, int *status, cudaEvent_t ready, bool capturing)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    cudaStreamWaitEvent(s->auxq, s->ev_qfork, 0);
    dim3 grd((c.width + 2 * s->pad - 8 + XG_QP_TW - 1) / XG_QP_TW, (c.height + 2 * s->pad - 8 + XG_QP_TH - 1) / XG_QP_TH);
    k_qpel_planes<<<grd, 256, 0, s->auxq>>>(s->tm_qp[cur], s->slot[cur][0], s->qpel[cur], status, s->wait_tries);
    xg_stage_event(ready, s->auxq, capturing);
    cudaEventRecord(s->ev_qjoin, s->auxq);
    return 1;
}

/* the exhaustive integer search of slot cur against slot ref into keys (the
 * stream's current band geometry) */
static XgMeParams xg_me_params(const xin_gpu_stream *s, int cur, int ref, unsigned long long *keys)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    XgMeParams mp;
    mp.cur = s->slot[cur][0];
    mp.ref = s->slot[ref][0];
    mp.W = c.width; mp.H = c.height; mp.ctu = c.ctu_size; mp.R = c.search_range;
    mp.band_rows = s->me_band_rows; mp.band_rows_alloc = s->me_band_rows_alloc; mp.row_words = s->me_row_words;
    mp.agg_passes = s->me_nb;
    mp.key_mul = 1u << (XG_COST_FRACTION + xg_me_db(s->sbd) + (XG_BITDEPTH - s->sbd));
    for (int L = 0; L < 4; L++) {
        mp.keys[L] = s->lev_on[L] ? keys + s->lev_first[L] : nullptr;
        mp.cus_x[L] = s->lev_cx[L];
    }
    return mp;
}

static void xg_enqueue_me_tiles(xin_gpu_stream *s, int cur, int ref, unsigned long long *keys, const XgPicParams *dpp,
                                cudaStream_t st)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    const XgMeParams mp = xg_me_params(s, cur, ref, keys);
    dim3 grd((c.width + 63) / 64, (c.height + 63) / 64, s->me_bands);
#if XG_BITDEPTH == 10
    if (s->sbd == 10) k_me_tiles<10><<<grd, XG_ME_THREADS, s->me_smem, st>>>(mp, dpp);
    else
#endif
        k_me_tiles<8><<<grd, XG_ME_THREADS, s->me_smem, st>>>(mp, dpp);
}

/* a kernel launch at the given stream priority (a node priority inside captured
 * graphs, which are instantiated with node priorities): the tails run at the
 * highest, so that the next picture's search, started beside them, does not
 * hold them back */
template <typename... KArgs, typename... Args>
static void xg_launch_prio(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, int prio, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid; cfg.blockDim = block; cfg.dynamicSmemBytes = smem; cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributePriority;
    at[0].val.priority = prio;
    cfg.attrs = at; cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

/* the plain tails of a 16 x 16 or 8 x 8 level: a warp per CU, cpb CUs per CTA */
template <int S>
static void xg_launch_small_tail(int cpb, const XgTailParams &tp, const XgPicParams *dpp, int n, cudaStream_t ls, int prio)
{
    static_assert(xg_tail_smem<S, 32, 8>() <= 48 * 1024, "eight CUs a CTA within the default shared memory");
    switch (cpb) {
    case 2: xg_launch_prio(k_cu_tail<S, 32, 2, false>, dim3((n + 1) / 2), dim3(64), xg_tail_smem<S, 32, 2>(), ls, prio, tp, dpp, n); break;
    case 8: xg_launch_prio(k_cu_tail<S, 32, 8, false>, dim3((n + 7) / 8), dim3(256), xg_tail_smem<S, 32, 8>(), ls, prio, tp, dpp, n); break;
    default: xg_launch_prio(k_cu_tail<S, 32, 4, false>, dim3((n + 3) / 4), dim3(128), xg_tail_smem<S, 32, 4>(), ls, prio, tp, dpp, n); break;
    }
}

/* the tails' parameters of level L (the li-th level on) of a picture of set
 * `set` in slot cur against slots l0 and l1 */
static XgTailParams xg_tail_params(xin_gpu_stream *s, int set, int cur, int l0, int l1, int L, int li)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    const xin_gpu_stream::Set &t = s->set[set];
    const size_t lq = (size_t)c.width * c.height, lc = lq / 4;
    XgTailParams tp;
    for (int p = 0; p < 3; p++) { tp.cur[p] = s->slot[cur][p]; tp.ref[p] = s->slot[l0][p]; tp.ref1[p] = s->slot[l1][p]; }
    tp.qpel = s->qpel[l0];
    tp.qpel1 = s->qpel[l1];
    tp.keys1 = c.refs == 2 ? s->keys1 + s->lev_first[L] : nullptr;
    tp.bi = t.dbi;
    tp.W = c.width; tp.H = c.height; tp.ctu = c.ctu_size; tp.R = c.search_range;
    tp.keys = s->keys + s->lev_first[L];
    tp.cus_x = s->lev_cx[L]; tp.first_cu = s->lev_first[L]; tp.size = XG_LEVEL_SIZE[L]; tp.level = L;
    for (int p = 0; p < 3; p++) {
        tp.q[p] = t.dq[p] + (p ? lc : lq) * li;
        tp.rec[p] = t.drec[p] + (p ? lc : lq) * li;
    }
    tp.res = t.dres;
    for (int p = 0; p < 3; p++) tp.resid[p] = nullptr;
    if (s->tu[set])
        for (int p = 0; p < 3; p++) tp.resid[p] = xg_tu_resid(s->tu[set], L, p);
    return tp;
}

/* point keys / keys1 at picture set `set`'s search buffers */
static void xg_use_set_keys(xin_gpu_stream *s, int set)
{
    const size_t n = s->ncus > 0 ? s->ncus : 1;
    s->keys = s->keys_base + set * n;
    if (s->keys1_base) s->keys1 = s->keys1_base + set * n;
}

/* the launches of one picture of picture set `set` into slot `cur`, against the
 * references in slots l0 (list 0) and l1 (list 1, refs 2) */
static int xg_enqueue_picture(xin_gpu_stream *s, int set, int cur, int l0, int l1, bool with_me, bool capturing,
                              bool early = false)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    xin_gpu_stream::Set &t = s->set[set];
    cudaStream_t st = t.pst;
    int nl = 0;
    xg_use_set_keys(s, set);
    /* the previous picture (the other set, on its own stream) must have written
     * the planes this picture reads of it (its slot, downscaled and quarter-pel
     * planes: ev_ref) and, unless this picture's slot is none of those it reads
     * (`early`), finished its search and tails (ev_main); its TU stage may still
     * run.  The search keys are per set. */
    const cudaEvent_t prev = early ? s->set[1 - set].ev_ref : s->set[1 - set].ev_main;
    if (capturing) cudaStreamWaitEvent(st, prev, cudaEventWaitExternal);
    else cudaStreamWaitEvent(st, prev, 0);
    /* upload and pad the current picture; it becomes the next picture's reference */
    xg_stage_event(t.evs[0], st, capturing);
    /* the parameters and (8-bit input) the staged samples were uploaded on the
     * upload stream before this picture's launches (xin_gpu_frame_submit) */
    int mode = XG_FILL_IN_PLACE;
    if (s->widen) {
        /* 8-bit samples into the 10-bit slot (<< 2) */
        mode = c.device_io ? XG_FILL_DEV8 : XG_FILL_STAGED8;
    } else if (c.device_io) {
        mode = XG_FILL_DEVPIX;
    } else {
        for (int p = 0; p < 3; p++) {
            XgPlane &pl = s->slot[cur][p];
            cudaMemcpy2DAsync(pl.data, (size_t)pl.pitch * sizeof(xg_pix), t.h_in[p], (size_t)pl.w * sizeof(xg_pix),
                              (size_t)pl.w * sizeof(xg_pix), pl.h, cudaMemcpyHostToDevice, st);
        }
    }
    {
        /* copy-in and edge replication of the three planes: 8 samples a thread */
        const XgPlane &ly = s->slot[cur][0];
        dim3 grd(((ly.w + 2 * ly.pad + 7) / 8 + 127) / 128, ly.h + 2 * ly.pad, 3);
        k_fill_slot<<<grd, 128, 0, st>>>(s->slot[cur][0], s->slot[cur][1], s->slot[cur][2], t.dpp, t.d_in8[0], t.d_in8[1],
                                         t.d_in8[2], mode);
        nl++;
    }
    if (c.search_mode == 1) {
        /* the new slot at 1/2 and 1/4 resolution: the current picture's levels now,
         * the reference's for the next picture */
        const xg_pix *src = s->slot_base[cur][0];
        long long sp = s->pitch;
        for (int l = 0; l < 2; l++) {
            const int ow = (c.width + 2 * s->pad) >> (l + 1), oh = s->lo_rows[l];
            dim3 grd((ow + 127) / 128, oh);
            k_downscale2x2<<<grd, 128, 0, st>>>(src, sp, s->lo_base[cur][l], s->lo_pitch[l], ow, oh);
            src = s->lo_base[cur][l];
            sp = s->lo_pitch[l];
            nl++;
        }
    }
    xg_stage_event(t.evs[1], st, capturing);
    /* the new picture's quarter-pel planes are read only by the next picture's
     * tails: build them on a low-priority stream beside the search */
    cudaEventRecord(s->ev_qfork, st);
    if (with_me) {
        /* the integer search of each list: list 0 into keys, list 1 (refs 2) into keys1 */
        for (int li = 0; li < (c.refs == 2 ? 2 : 1); li++) {
        const int ref = li ? l1 : l0;
        unsigned long long *keys = li ? s->keys1 : s->keys;
        cudaMemsetAsync(keys, 0xff, sizeof(unsigned long long) * s->ncus, st);
        if (c.search_mode == 1) {
            XgHierFrameParams hp;
            memset(&hp, 0, sizeof hp);
            hp.cur = s->slot[cur][0]; hp.ref = s->slot[ref][0];
            for (int l = 0; l < 2; l++) { hp.cur_lo[l] = s->lo[cur][l]; hp.ref_lo[l] = s->lo[ref][l]; }
            hp.W = c.width; hp.H = c.height; hp.ctu = c.ctu_size; hp.R = c.search_range;
            int nz = 0;
            for (int L = 0; L < 4; L++) {
                if (!s->lev_on[L]) continue;
                hp.level_size[nz] = XG_LEVEL_SIZE[L];
                hp.keys[nz] = keys + s->lev_first[L];
                hp.cus_x[nz] = s->lev_cx[L];
                nz++;
            }
            if (nz > 0) {
                dim3 grd((c.width + 63) / 64, (c.height + 63) / 64, nz);
                k_hier_frame<64><<<grd, XG_HIER_THREADS, xg_hier_smem(c.search_range, 64), st>>>(hp, t.dpp);
            }
            if (s->lev_on[4]) {
                /* the 128 x 128 level: 128 x 128 tiles */
                hp.level_size[0] = 128; hp.keys[0] = keys + s->lev_first[4]; hp.cus_x[0] = s->lev_cx[4];
                dim3 grd((c.width + 127) / 128, (c.height + 127) / 128, 1);
                k_hier_frame<128><<<grd, XG_HIER_THREADS, xg_hier_smem(c.search_range, 128), st>>>(hp, t.dpp);
                nl++;
            }
        } else {
            xg_enqueue_me_tiles(s, cur, ref, keys, t.dpp, st);
        }
        nl++;
        }
        nl += xg_enqueue_qpel(s, cur, &t.dpp->status, t.ev_ref, capturing);
        /* the search's end is recorded on a side branch joined at the picture's
         * end: a timing node between the search and the tails' fork held the tails
         * back by about 0.03 ms */
        cudaEventRecord(s->ev_tfork, st);
        cudaStreamWaitEvent(s->tst, s->ev_tfork, 0);
        xg_stage_event(t.evs[2], s->tst, capturing);
        cudaEventRecord(s->ev_tjoin, s->tst);
        /* the levels' tails are independent: fork them onto the auxiliary streams */
        cudaEventRecord(s->ev_fork, st);
        int li = 0, nfork = 0;
        for (int L = 0; L < XG_NLEV; L++) {
            if (!s->lev_on[L]) continue;
            cudaStream_t ls = st;
            if (li > 0) {
                ls = s->aux[li - 1];
                cudaStreamWaitEvent(ls, s->ev_fork, 0);
                nfork = li;
            }
            const XgTailParams tp = xg_tail_params(s, set, cur, l0, l1, L, li);
            int n = s->lev_cx[L] * s->lev_cy[L];
            if (n > 0 && c.refs == 2) {
                switch (XG_LEVEL_SIZE[L]) {
                case 64: xg_launch_prio(k_cu_tail<64, 128, 1, true>, dim3(n), dim3(128), xg_tail_smem<64, 128, 1, true>(), ls, s->prio_hi, tp, (const XgPicParams *)t.dpp, n); break;
                case 32: xg_launch_prio(k_cu_tail<32, 128, 1, true>, dim3(n), dim3(128), xg_tail_smem<32, 128, 1, true>(), ls, s->prio_hi, tp, (const XgPicParams *)t.dpp, n); break;
                case 16:
                    xg_launch_prio(k_cu_tail<16, 32, 4, true>, dim3((n + 3) / 4), dim3(128), xg_tail_smem<16, 32, 4, true>(), ls, s->prio_hi, tp, (const XgPicParams *)t.dpp, n);
                    break;
                default:
                    xg_launch_prio(k_cu_tail<8, 32, 4, true>, dim3((n + 3) / 4), dim3(128), xg_tail_smem<8, 32, 4, true>(), ls, s->prio_hi, tp, (const XgPicParams *)t.dpp, n);
                    break;
                }
                nl++;
            } else if (n > 0) {
                /* 64 and 32: a 128-thread CTA per CU; 16 and 8: a warp per CU, four CUs per
                 * CTA (the fastest of the shapes measured on GB300 at 1080p) */
                switch (XG_LEVEL_SIZE[L]) {
                case 128: xg_launch_prio(k_cu_tail<128, 128, 1, false>, dim3(n), dim3(128), xg_tail_smem<128, 128, 1>(), ls, s->prio_hi, tp, (const XgPicParams *)t.dpp, n); break;
                case 64: xg_launch_prio(k_cu_tail<64, 128, 1, false>, dim3(n), dim3(128), xg_tail_smem<64, 128, 1>(), ls, s->prio_hi, tp, (const XgPicParams *)t.dpp, n); break;
                case 32: xg_launch_prio(k_cu_tail<32, 128, 1, false>, dim3(n), dim3(128), xg_tail_smem<32, 128, 1>(), ls, s->prio_hi, tp, (const XgPicParams *)t.dpp, n); break;
                case 16: xg_launch_small_tail<16>(s->tail_cpb[0], tp, t.dpp, n, ls, s->prio_hi); break;
                default: xg_launch_small_tail<8>(s->tail_cpb[1], tp, t.dpp, n, ls, s->prio_hi); break;
                }
                nl++;
            }
            li++;
        }
        for (int i = 0; i < nfork; i++) {
            cudaEventRecord(s->ev_join[i], s->aux[i]);
            cudaStreamWaitEvent(st, s->ev_join[i], 0);
        }
        cudaStreamWaitEvent(st, s->ev_qjoin, 0);
        cudaStreamWaitEvent(st, s->ev_tjoin, 0);
        xg_stage_event(t.ev_main, st, capturing);
        if (s->tu[set]) nl += xg_tu_enqueue(s, set, cur, t, st);
        xg_stage_event(t.evs[3], st, capturing);
    } else {
        nl += xg_enqueue_qpel(s, cur, &t.dpp->status, t.ev_ref, capturing);
        cudaStreamWaitEvent(st, s->ev_qjoin, 0);
        xg_stage_event(t.ev_main, st, capturing);
        xg_stage_event(t.evs[2], st, capturing);
        xg_stage_event(t.evs[3], st, capturing);
    }
    return nl;
}

/* the result copies of picture set t on the copy stream, after the picture's
 * kernels, so that they overlap the next picture's kernels; then the picture's
 * completion event */
static void xg_enqueue_result_copies(xin_gpu_stream *s, xin_gpu_stream::Set &t, bool with_me, cudaStream_t cst)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    if (with_me && !c.device_io) {
        size_t lq = (size_t)c.width * c.height, lc = lq / 4;
        cudaMemcpyAsync(t.h_res, t.dres, sizeof(xin_gpu_cu_result) * s->ncus, cudaMemcpyDeviceToHost, cst);
        if (t.dmts) cudaMemcpyAsync(t.h_mts, t.dmts, sizeof(xin_gpu_cu_mts) * s->ncus, cudaMemcpyDeviceToHost, cst);
        if (t.dbi) cudaMemcpyAsync(t.h_bi, t.dbi, sizeof(xin_gpu_cu_bi) * s->ncus, cudaMemcpyDeviceToHost, cst);
        for (int p = 0; p < 3; p++) {
            size_t n = (p ? lc : lq) * s->nlev;
            if (c.out_flags & XIN_GPU_OUT_Q)
                cudaMemcpyAsync(t.q_dst[p] ? t.q_dst[p] : t.h_q[p], t.dq[p], n * sizeof(xg_coef), cudaMemcpyDeviceToHost, cst);
            if (c.out_flags & XIN_GPU_OUT_REC) cudaMemcpyAsync(t.h_rec[p], t.drec[p], n * sizeof(xg_pix), cudaMemcpyDeviceToHost, cst);
        }
    }
    /* the picture's device status (a wait bound reached) */
    cudaMemcpyAsync(t.h_stat, &t.dpp->status, sizeof(int32_t), cudaMemcpyDeviceToHost, cst);
    cudaEventRecord(t.evs[4], cst);
    cudaEventRecord(t.ev1, cst);
}

static void xg_enqueue_results(xin_gpu_stream *s, xin_gpu_stream::Set &t, bool with_me)
{
    cudaEventRecord(t.ev_kern, t.pst);
    cudaStreamWaitEvent(s->cst, t.ev_kern, 0);
    xg_enqueue_result_copies(s, t, with_me, s->cst);
}

static int xg_frame_submit(xin_gpu_stream *s, const xin_gpu_picture *pic, int32_t ref0, int32_t ref1, xg_coef *const *q_dst);
extern "C" int xin_gpu_frame_submit(xin_gpu_stream *s, const xin_gpu_picture *pic) { return xg_frame_submit(s, pic, -1, -1, nullptr); }
extern "C" int xin_gpu_frame_submit_refs(xin_gpu_stream *s, const xin_gpu_picture *pic, int32_t ref0, int32_t ref1)
{
    return xg_frame_submit(s, pic, ref0, ref1, nullptr);
}

/* picture nsub of stream s: the checks, the host staging of its samples and its
 * parameter block (in the picture set's pinned staging); its picture set and
 * slots */
struct XgSubmitPlan { int set, cur, l0, l1; };
static int xg_frame_prepare(xin_gpu_stream *s, const xin_gpu_picture *pic, int32_t ref0, int32_t ref1, XgSubmitPlan &plan)
{
    if (s->nsub - s->ndone >= 2) {
        xg_set_error(XIN_GPU_ERR_STATE, "frame_submit: two pictures in flight; collect one with frame_wait first");
        return XIN_GPU_ERR_STATE;
    }
    const xin_gpu_stream_cfg &c = s->cfg;
    if (pic->qp < 0 || pic->qp > 63 || pic->uv_qp < 0 || pic->uv_qp > 63) { xg_set_error(XIN_GPU_ERR_ARG, "frame_submit: QP out of range"); return XIN_GPU_ERR_ARG; }
    /* the search packs (cost << 2 | row) into 32 bits: costs must stay below 2^29 */
    if (pic->sad_lambda > (1u << 20)) { xg_set_error(XIN_GPU_ERR_ARG, "frame_submit: sad_lambda above 2^20"); return XIN_GPU_ERR_ARG; }
    /* picture set (in-flight resources) and slots: the picture's own, and its
     * references' -- named, or list 0 = the previous picture and list 1 = the one
     * before (the previous one again for the second picture) */
    const int set = s->nsub & 1, ns = s->nslots, k = s->nsub;
    if (ref0 < 0) ref0 = k - 1;
    if (ref1 < 0) ref1 = k >= 2 ? k - 2 : k - 1;
    if (k > 0 && (ref0 >= k || ref1 >= k || k - ref0 > ns - 1 || (c.refs == 2 && k - ref1 > ns - 1))) {
        xg_set_error(XIN_GPU_ERR_ARG, "frame_submit: reference pictures %d, %d out of reach of picture %d (dpb %d)", ref0, ref1, k, ns);
        return XIN_GPU_ERR_ARG;
    }
    const int cur = k % ns, l0 = k > 0 ? ref0 % ns : 0, l1 = c.refs == 2 && k > 0 ? ref1 % ns : l0;
    xin_gpu_stream::Set &t = s->set[set];
    /* set `set` was last used by picture nsub - 2, already collected by frame_wait
     * (at most two in flight), so its staging is free */
    XgPicParams pp;
    memset(&pp, 0, sizeof pp);
    for (int p = 0; p < 3; p++) {
        int w = p ? c.width / 2 : c.width, h = p ? c.height / 2 : c.height;
        if (!pic->plane[p] || pic->stride[p] < w) { xg_set_error(XIN_GPU_ERR_ARG, "frame_submit: bad plane"); return XIN_GPU_ERR_ARG; }
        if (c.device_io) {
            pp.src[p] = (const xg_pix *)pic->plane[p];
            pp.src_stride[p] = pic->stride[p];
            continue;
        }
        const size_t es = s->in_es;
        for (int y = 0; y < h; y++)
            memcpy((char *)t.h_in[p] + (size_t)y * w * es, (const char *)pic->plane[p] + (size_t)y * pic->stride[p] * es, (size_t)w * es);
    }
    pp.lambda = pic->sad_lambda;
    if (c.tu_mode == 1) {
        /* the trellis QP (h266_trans_quant.c:103-104): slice QP, + 12 at 10 bits; its
         * parameter table stops at 51 */
        pp.dq_qp[0] = pic->qp + (XG_BITDEPTH == 10 ? 12 : 0);
        pp.dq_qp[1] = pic->uv_qp + (XG_BITDEPTH == 10 ? 12 : 0);
        if (pp.dq_qp[0] > 51 || pp.dq_qp[1] > 51) {
            xg_set_error(XIN_GPU_ERR_ARG, "frame_submit: QP above %d for the dependent-quantisation stage", XG_BITDEPTH == 10 ? 39 : 51);
            return XIN_GPU_ERR_ARG;
        }
    }
    for (int L = 0; L < XG_NLEV; L++) {
        /* the TU's size: the CU's, at most 64 (a 128 x 128 CU has 64 x 64 TUs) */
        int lg = XG_LEVEL_SIZE[L] >= 64 ? 6 : XG_LEVEL_SIZE[L] == 32 ? 5 : XG_LEVEL_SIZE[L] == 16 ? 4 : 3;
        xg_quant_params(pic->qp, lg, 0, &pp.quant[L][0]);
        xg_quant_params(pic->uv_qp, lg - 1, 0, &pp.quant[L][1]);
        pp.quant[L][2] = pp.quant[L][1];
    }
    *t.h_pp = pp;
    plan.set = set; plan.cur = cur; plan.l0 = l0; plan.l1 = l1;
    return XIN_GPU_OK;
}

/* q_dst (optional): caller buffers that receive this picture's coefficient planes
 * (XIN_GPU_OUT_Q) straight from the device -- pinned host memory keeps the copy
 * asynchronous -- instead of the picture set's pinned staging */
static int xg_frame_submit(xin_gpu_stream *s, const xin_gpu_picture *pic, int32_t ref0, int32_t ref1, xg_coef *const *q_dst)
{
    xin_gpu_clear_error();
    (void)cudaGetLastError();   /* errors of earlier, unrelated calls are not this picture's */
    if (!s || !pic) { xg_set_error(XIN_GPU_ERR_ARG, "frame_submit: null argument"); return XIN_GPU_ERR_ARG; }
    XgSubmitPlan plan;
    if (int e = xg_frame_prepare(s, pic, ref0, ref1, plan)) return e;
    const int set = plan.set, cur = plan.cur, l0 = plan.l0, l1 = plan.l1;
    xin_gpu_stream::Set &t = s->set[set];
    const xin_gpu_stream_cfg &c = s->cfg;
    bool with_me = s->nsub > 0;
    cudaEventRecord(t.ev0, t.pst);
    /* uploads on their own stream, so that they overlap the previous picture's
     * kernels: set cur is not read by the picture in flight (it uses the other
     * set), and its last user, picture nsub - 2, has completed */
    cudaMemcpyAsync(t.dpp, t.h_pp, sizeof(XgPicParams), cudaMemcpyHostToDevice, s->ust);
    if (s->widen && !c.device_io)
        for (int p = 0; p < 3; p++) {
            const XgPlane &pl = s->slot[cur][p];
            cudaMemcpyAsync(t.d_in8[p], t.h_in[p], (size_t)pl.w * pl.h, cudaMemcpyHostToDevice, s->ust);
        }
    cudaEventRecord(t.ev_up, s->ust);
    cudaStreamWaitEvent(t.pst, t.ev_up, 0);
    /* a graph per (set, slot, list-0 slot, list-1 slot): the launches bake in the
     * slots' planes */
    /* the previous picture's tails may still run while this one starts when this
     * picture's slot is none of the slots it reads */
    const xin_gpu_stream::Set &pv = s->set[1 - set];
    const bool early = s->nsub >= 1 && s->nslots >= 3 && cur != pv.rd[0] && cur != pv.rd[1] && cur != pv.rd[2];
    t.rd[0] = cur; t.rd[1] = l0; t.rd[2] = l1;
    const uint32_t gkey = ((uint32_t)early << 20) | ((uint32_t)set << 15) | ((uint32_t)cur << 10) | ((uint32_t)l0 << 5) | (uint32_t)l1;
    auto git = s->graphs.find(gkey);
    if (with_me && c.use_graph && (git != s->graphs.end() || (int)s->graphs.size() < XG_MAX_GRAPHS)) {
        if (git == s->graphs.end()) {
            cudaGraph_t g;
            cudaGraphExec_t gx = nullptr;
            if (xg_cuda_check(cudaStreamBeginCapture(t.pst, cudaStreamCaptureModeThreadLocal), "begin capture")) return XIN_GPU_ERR_CUDA;
            const int n = xg_enqueue_picture(s, set, cur, l0, l1, true, true, early);
            if (xg_cuda_check(cudaStreamEndCapture(t.pst, &g), "end capture")) return XIN_GPU_ERR_CUDA;
            cudaError_t e = cudaGraphInstantiate(&gx, g, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(g);
            if (xg_cuda_check(e, "graph instantiate")) return XIN_GPU_ERR_CUDA;
            git = s->graphs.emplace(gkey, std::make_pair(gx, n)).first;
        }
        if (xg_cuda_check(cudaGraphLaunch(git->second.first, t.pst), "graph launch")) return XIN_GPU_ERR_CUDA;
        xg_count_launch((uint64_t)git->second.second);
    } else {
        xg_count_launch((uint64_t)xg_enqueue_picture(s, set, cur, l0, l1, with_me, false, early));
    }
    for (int p = 0; p < 3; p++) t.q_dst[p] = q_dst ? q_dst[p] : nullptr;
    xg_enqueue_results(s, t, with_me);
    if (xg_cuda_check(cudaGetLastError(), "frame_submit")) return XIN_GPU_ERR_CUDA;
    s->nsub++;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_frame_wait(xin_gpu_stream *s, xin_gpu_results *res, int32_t timeout_ms)
{
    xin_gpu_clear_error();
    if (!s) { xg_set_error(XIN_GPU_ERR_ARG, "frame_wait: null stream"); return XIN_GPU_ERR_ARG; }
    if (s->ndone == s->nsub) { xg_set_error(XIN_GPU_ERR_STATE, "frame_wait: no picture in flight"); return XIN_GPU_ERR_STATE; }
    const int k = s->ndone;                 /* the oldest picture in flight */
    xin_gpu_stream::Set &t = s->set[k & 1];
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaEventQuery(t.ev1);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return xg_cuda_check(e, "frame_wait");
        double el = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_ms >= 0 && el > timeout_ms) { xg_set_error(XIN_GPU_ERR_TIMEOUT, "frame_wait: timed out after %d ms", timeout_ms); return XIN_GPU_ERR_TIMEOUT; }
        std::this_thread::yield();
    }
    s->ndone++;
    if (*t.h_stat) {
        xg_set_error(XIN_GPU_ERR_TIMEOUT, "frame_wait: picture %d: a device wait reached its bound (status %d)", k, *t.h_stat);
        return XIN_GPU_ERR_TIMEOUT;
    }
    if (k == 0) {                           /* the first picture only becomes the reference */
        if (res) res->gpu_ms = 0;
        return XIN_GPU_OK;
    }
    if (!res) return XIN_GPU_OK;
    float ms = 0;
    if (cudaEventElapsedTime(&ms, t.evs[0], t.evs[4]) != cudaSuccess) { cudaGetLastError(); ms = -1.0f; }
    res->gpu_ms = ms;
    const xin_gpu_stream_cfg &c = s->cfg;
    if (c.device_io) return XIN_GPU_OK;
    size_t lq = (size_t)c.width * c.height, lc = lq / 4;
    /* caller buffers are filled; NULL members receive views of the picture set's
     * pinned buffers, valid until the second frame_submit after this call */
    if (res->cu) memcpy(res->cu, t.h_res, sizeof(xin_gpu_cu_result) * s->ncus);
    else res->cu = t.h_res;
    if (t.h_mts) {
        if (res->mts) memcpy(res->mts, t.h_mts, sizeof(xin_gpu_cu_mts) * s->ncus);
        else res->mts = t.h_mts;
    }
    if (t.h_bi) {
        if (res->bi) memcpy(res->bi, t.h_bi, sizeof(xin_gpu_cu_bi) * s->ncus);
        else res->bi = t.h_bi;
    }
    for (int p = 0; p < 3; p++) {
        size_t n = (p ? lc : lq) * s->nlev;
        if (c.out_flags & XIN_GPU_OUT_Q) {
            xg_coef *src = t.q_dst[p] ? t.q_dst[p] : t.h_q[p];    /* where the picture's planes were copied */
            if (res->q[p]) {
                if (res->q[p] != src) memcpy(res->q[p], src, n * sizeof(xg_coef));
            } else {
                res->q[p] = src;
            }
        }
        if (c.out_flags & XIN_GPU_OUT_REC) {
            if (res->rec[p]) memcpy(res->rec[p], t.h_rec[p], n * sizeof(xg_pix));
            else res->rec[p] = t.h_rec[p];
        }
    }
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_stream_set_wait_tries(xin_gpu_stream *s, int64_t tries)
{
    xin_gpu_clear_error();
    if (!s || tries < -1) { xg_set_error(XIN_GPU_ERR_ARG, "stream_set_wait_tries: null stream or tries below -1"); return XIN_GPU_ERR_ARG; }
    if (s->nsub != s->ndone) { xg_set_error(XIN_GPU_ERR_STATE, "stream_set_wait_tries: pictures in flight"); return XIN_GPU_ERR_STATE; }
    s->wait_tries = tries < 0 ? XG_TMA_WAIT_TRIES : tries;
    /* the bound is a parameter of the captured graphs: capture them again */
    for (auto &g : s->graphs) cudaGraphExecDestroy(g.second.first);
    s->graphs.clear();
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_stream_tune_search(xin_gpu_stream *s, int32_t *bands, float ms[2])
{
    xin_gpu_clear_error();
    if (!s) { xg_set_error(XIN_GPU_ERR_ARG, "stream_tune_search: null stream"); return XIN_GPU_ERR_ARG; }
    const xin_gpu_stream_cfg &c = s->cfg;
    if (c.search_mode != 0 || s->nsub < 2 || s->nsub != s->ndone) {
        xg_set_error(XIN_GPU_ERR_STATE, "stream_tune_search: needs the exhaustive search, two pictures submitted and none in flight");
        return XIN_GPU_ERR_STATE;
    }
    /* the last picture against its list-0 reference (the previous picture) */
    const int ns = s->nslots, k = s->nsub - 1, cur = k % ns, ref = (k + ns - 1) % ns;
    const XgPicParams *dpp = s->set[k & 1].dpp;
    cudaStream_t st = s->st;
    xg_use_set_keys(s, k & 1);
    const int b0 = s->me_bands;
    const int cand[6] = { b0, b0 / 2, 2 * b0, 3 * b0, 4 * b0, 6 * b0 };
    cudaEvent_t e0, e1;
    if (xg_cuda_check(cudaEventCreate(&e0), "tune event") || xg_cuda_check(cudaEventCreate(&e1), "tune event")) return XIN_GPU_ERR_CUDA;
    float best_ms = 0, first_ms = 0;
    int best_b = b0, tried[6], ntried = 0;
    for (int i = 0; i < 6; i++) {
        if (cand[i] < 1 || !xg_me_geometry(s, cand[i])) continue;
        bool seen = false;                       /* a geometry once */
        for (int j = 0; j < ntried; j++) seen |= tried[j] == s->me_bands;
        if (seen) continue;
        tried[ntried++] = s->me_bands;
        float t = 0;
        for (int rep = 0; rep < 4; rep++) {      /* one warm-up, three timed */
            if (rep == 1) cudaEventRecord(e0, st);
            xg_enqueue_me_tiles(s, cur, ref, s->keys, dpp, st);
        }
        cudaEventRecord(e1, st);
        if (xg_cuda_check(cudaEventSynchronize(e1), "tune search")) { cudaEventDestroy(e0); cudaEventDestroy(e1); return XIN_GPU_ERR_CUDA; }
        cudaEventElapsedTime(&t, e0, e1);
        t /= 3;
        s->tune_bands[ntried - 1] = s->me_bands;
        s->tune_ms[ntried - 1] = t;
        s->tune_n = ntried;
        if (i == 0) first_ms = t;
        if (i == 0 || t < best_ms) { best_ms = t; best_b = s->me_bands; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    xg_me_geometry(s, best_b);
    /* the geometry is baked into the captured graphs: capture them again */
    for (auto &g : s->graphs) cudaGraphExecDestroy(g.second.first);
    s->graphs.clear();
    if (bands) *bands = s->me_bands;
    if (ms) { ms[0] = first_ms; ms[1] = best_ms; }
    return xg_cuda_check(cudaGetLastError(), "tune search");
}

extern "C" int xin_gpu_stream_tune_tails(xin_gpu_stream *s, int32_t cpb[2], float ms[6])
{
    xin_gpu_clear_error();
    if (!s) { xg_set_error(XIN_GPU_ERR_ARG, "stream_tune_tails: null stream"); return XIN_GPU_ERR_ARG; }
    const xin_gpu_stream_cfg &c = s->cfg;
    if (c.refs == 2 || s->nsub < 2 || s->nsub != s->ndone) {
        xg_set_error(XIN_GPU_ERR_STATE, "stream_tune_tails: needs one reference, two pictures submitted and none in flight");
        return XIN_GPU_ERR_STATE;
    }
    /* the last picture's tails again (against its list-0 reference, the previous
     * picture): they rewrite that picture's device results with the same values */
    const int ns = s->nslots, k = s->nsub - 1, set = k & 1, cur = k % ns, ref = (k + ns - 1) % ns;
    const XgPicParams *dpp = s->set[set].dpp;
    cudaStream_t st = s->st;
    xg_use_set_keys(s, set);
    const int opt[3] = { 2, 4, 8 };
    cudaEvent_t e0, e1;
    if (xg_cuda_check(cudaEventCreate(&e0), "tune event") || xg_cuda_check(cudaEventCreate(&e1), "tune event")) return XIN_GPU_ERR_CUDA;
    for (int j = 0; j < 2; j++) {                     /* the 16 x 16 and the 8 x 8 level */
        const int L = j ? 3 : 2;
        for (int o = 0; o < 3; o++)
            if (ms) ms[3 * j + o] = 0;
        if (!s->lev_on[L]) continue;
        int li = 0;
        for (int l = 0; l < L; l++) li += s->lev_on[l] ? 1 : 0;
        const XgTailParams tp = xg_tail_params(s, set, cur, ref, ref, L, li);
        const int n = s->lev_cx[L] * s->lev_cy[L];
        float best = 0;
        for (int o = 0; o < 3; o++) {
            for (int rep = 0; rep < 4; rep++) {          /* one warm-up, three timed */
                if (rep == 1) cudaEventRecord(e0, st);
                if (j) xg_launch_small_tail<8>(opt[o], tp, dpp, n, st, s->prio_hi);
                else xg_launch_small_tail<16>(opt[o], tp, dpp, n, st, s->prio_hi);
            }
            cudaEventRecord(e1, st);
            if (xg_cuda_check(cudaEventSynchronize(e1), "tune tails")) { cudaEventDestroy(e0); cudaEventDestroy(e1); return XIN_GPU_ERR_CUDA; }
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            t /= 3;
            if (ms) ms[3 * j + o] = t;
            if (o == 0 || t < best) { best = t; s->tail_cpb[j] = opt[o]; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    /* the launch shapes are baked into the captured graphs: capture them again */
    for (auto &g : s->graphs) cudaGraphExecDestroy(g.second.first);
    s->graphs.clear();
    if (cpb) { cpb[0] = s->tail_cpb[0]; cpb[1] = s->tail_cpb[1]; }
    return xg_cuda_check(cudaGetLastError(), "tune tails");
}

extern "C" int xin_gpu_stream_tune_table(const xin_gpu_stream *s, int32_t *n, int32_t bands[6], float ms[6])
{
    if (!s || !n) return XIN_GPU_ERR_ARG;
    *n = s->tune_n;
    for (int i = 0; i < s->tune_n; i++) {
        if (bands) bands[i] = s->tune_bands[i];
        if (ms) ms[i] = s->tune_ms[i];
    }
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_stream_stage_ms(const xin_gpu_stream *s, float ms[4])
{
    if (!s || !ms) return XIN_GPU_ERR_ARG;
    if (s->ndone < 2) return XIN_GPU_ERR_STATE;
    const xin_gpu_stream::Set &t = s->set[(s->ndone - 1) & 1];   /* the last collected picture */
    for (int i = 0; i < 4; i++) {
        ms[i] = 0;
        if (cudaEventElapsedTime(&ms[i], t.evs[i], t.evs[i + 1]) != cudaSuccess) { cudaGetLastError(); return XIN_GPU_ERR_STATE; }
    }
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_stream_device_results(const xin_gpu_stream *s, void **cu, void *q[3], void *rec[3])
{
    if (!s) return XIN_GPU_ERR_ARG;
    const xin_gpu_stream::Set &t = s->set[(s->ndone - 1) & 1];   /* the last collected picture */
    if (cu) *cu = t.dres;
    for (int p = 0; p < 3; p++) {
        if (q) q[p] = t.dq[p];
        if (rec) rec[p] = t.drec[p];
    }
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_measure_sad_peak(double *absdiff_per_s)
{
    xin_gpu_clear_error();
    if (!absdiff_per_s) return XIN_GPU_ERR_ARG;
    XgThread *t = xg_thread();
    if (!t) return XIN_GPU_ERR_CUDA;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 16, threads = 256, iters = 4096;
    uint32_t *in = (uint32_t *)xg_dalloc(t, 4096), *out = (uint32_t *)xg_dalloc(t, (size_t)blocks * threads * 4);
    if (!in || !out) return XIN_GPU_ERR_NOMEM;
    cudaMemsetAsync(in, 0x5a, 4096, t->stream);
    cudaEvent_t a, b;
    cudaEventCreate(&a); cudaEventCreate(&b);
    /* both packed forms: vabsdiff4 + dp4a, and vabsdiff4 with add-reduction (the
     * form the search kernel issues); the faster one is the ceiling */
    double best = 0;      /* absolute differences per second */
    for (int form = 0; form < 2; form++)
        for (int rep = 0; rep < 4; rep++) {
            cudaEventRecord(a, t->stream);
            int per = 0;  /* absolute differences per thread and loop trip */
            if (XG_BITDEPTH != 8) { k_sad_peak10<<<blocks, threads, 0, t->stream>>>(in, out, iters); per = 64 * 2; }
            else if (form == 0) { k_sad_peak<<<blocks, threads, 0, t->stream>>>(in, out, iters); per = 8 * 4; }
            else { k_sad_peak_add<<<blocks, threads, 0, t->stream>>>(in, out, iters / 8); per = 64 * 4 / 8; }
            cudaEventRecord(b, t->stream);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            double r = (double)blocks * threads * iters * per / (ms * 1e-3);
            if (rep && r > best) best = r;
        }
    xg_count_launch(8);
    cudaEventDestroy(a); cudaEventDestroy(b);
    if (xg_cuda_check(cudaGetLastError(), "sad peak")) return XIN_GPU_ERR_CUDA;
    *absdiff_per_s = best;
    return XIN_GPU_OK;
}
