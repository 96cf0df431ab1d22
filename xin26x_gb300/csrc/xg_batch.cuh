/*
 * xg_batch.cuh -- cross-stream batches: pictures of several streams of one shape
 * through one launch per stage (slot fill, quarter-pel planes, integer search,
 * each level's tails) instead of one graph per picture.  The server forms a
 * batch from the pictures waiting when it launches.  Streams of the plain form
 * take part: exhaustive search, one reference, DCT2 with TU = CU, host
 * pictures.  Each picture keeps its stream's slots, picture set and results, so
 * its results equal those of the same picture submitted alone, and it is
 * collected with xin_gpu_frame_wait on its own stream.
 */

/* the CUDA streams and events one batch runs on */
struct XgBatchLane {
    cudaStream_t st, aux[XG_NLEV - 1], auxq;
    cudaEvent_t ev_fork, ev_join[XG_NLEV - 1], ev_qfork, ev_qjoin;
    int busy;              /* pictures of the lane's batch not yet collected */
};

static void xg_lane_close(XgBatchLane &ln)
{
    if (ln.st) cudaStreamDestroy(ln.st);
    if (ln.auxq) cudaStreamDestroy(ln.auxq);
    for (int i = 0; i < XG_NLEV - 1; i++) {
        if (ln.aux[i]) cudaStreamDestroy(ln.aux[i]);
        if (ln.ev_join[i]) cudaEventDestroy(ln.ev_join[i]);
    }
    if (ln.ev_fork) cudaEventDestroy(ln.ev_fork);
    if (ln.ev_qfork) cudaEventDestroy(ln.ev_qfork);
    if (ln.ev_qjoin) cudaEventDestroy(ln.ev_qjoin);
    memset(&ln, 0, sizeof ln);
}

static int xg_lane_open(XgBatchLane &ln)
{
    memset(&ln, 0, sizeof ln);
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);     /* lo: the least urgent */
    cudaError_t e = cudaStreamCreateWithFlags(&ln.st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&ln.auxq, cudaStreamNonBlocking, lo);
    for (int i = 0; i < XG_NLEV - 1 && e == cudaSuccess; i++) {
        e = cudaStreamCreateWithFlags(&ln.aux[i], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ln.ev_join[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ln.ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ln.ev_qfork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ln.ev_qjoin, cudaEventDisableTiming);
    static std::once_flag attr_once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(attr_once, [] {
        attr_err = cudaFuncSetAttribute(k_me_tiles_batch<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, XG_ME_SMEM_MAX);
#if XG_BITDEPTH == 10
        if (attr_err == cudaSuccess)
            attr_err = cudaFuncSetAttribute(k_me_tiles_batch<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, XG_ME_SMEM_MAX);
#endif
    });
    if (e == cudaSuccess) e = attr_err;
    if (xg_cuda_check(e, "batch lane")) { xg_lane_close(ln); return XIN_GPU_ERR_CUDA; }
    return XIN_GPU_OK;
}

/* a stream whose next picture may join a batch: the plain form with host
 * pictures, its first picture (the first reference) submitted, none in flight */
static bool xg_batchable(const xin_gpu_stream *s)
{
    const xin_gpu_stream_cfg &c = s->cfg;
    return c.search_mode == 0 && c.tu_mode == 0 && c.refs <= 1 && !c.device_io && s->nsub > 0 && s->nsub == s->ndone;
}

/* streams whose pictures take identical launches: grids, shared memory, band
 * geometry of the search, fill mode and wait bound */
static bool xg_batch_compatible(const xin_gpu_stream *a, const xin_gpu_stream *b)
{
    const xin_gpu_stream_cfg &x = a->cfg, &y = b->cfg;
    if (x.width != y.width || x.height != y.height || x.ctu_size != y.ctu_size || x.search_range != y.search_range)
        return false;
    if (a->sbd != b->sbd || a->widen != b->widen || a->pad != b->pad || a->wait_tries != b->wait_tries) return false;
    for (int L = 0; L < XG_NLEV; L++)
        if (a->lev_on[L] != b->lev_on[L]) return false;
    return a->me_bands == b->me_bands && a->me_band_rows == b->me_band_rows && a->me_band_rows_alloc == b->me_band_rows_alloc &&
           a->me_row_words == b->me_row_words && a->me_nb == b->me_nb && a->me_smem == b->me_smem;
}

/* pictures of s's shape one batch takes: as many as keep the integer search's
 * grid (one CTA per SM: 64 x 64 tiles x bands) within two waves of the SMs.  A
 * batch completes its pictures together, so a picture whose search already
 * fills the GPU gains nothing from sharing launches and waits for the others. */
static int xg_batch_fill_limit(const xin_gpu_stream *s, int sms)
{
    const int ctas = ((s->cfg.width + 63) / 64) * ((s->cfg.height + 63) / 64) * (s->me_bands > 0 ? s->me_bands : 1);
    const int n = 2 * sms / (ctas > 0 ? ctas : 1);
    return n < 1 ? 1 : n > XG_BATCH_MAX ? XG_BATCH_MAX : n;
}

/* the next picture of each of n distinct, batchable, mutually compatible
 * streams ss[i] (picture pics[i], coefficient planes into q_dst[i] when that is
 * set), in one batch on lane ln */
static int xg_batch_submit(xin_gpu_stream *const *ss, const xin_gpu_picture *const *pics, xg_coef *const *const *q_dst, int n,
                           XgBatchLane &ln)
{
    xin_gpu_clear_error();
    (void)cudaGetLastError();
    if (!ss || !pics || n < 1 || n > XG_BATCH_MAX) {
        xg_set_error(XIN_GPU_ERR_ARG, "batch_submit: 1..%d pictures", XG_BATCH_MAX);
        return XIN_GPU_ERR_ARG;
    }
    for (int i = 0; i < n; i++) {
        if (!ss[i] || !pics[i]) { xg_set_error(XIN_GPU_ERR_ARG, "batch_submit: null argument"); return XIN_GPU_ERR_ARG; }
        bool dup = false;
        for (int j = 0; j < i; j++) dup |= ss[j] == ss[i];
        if (dup || !xg_batchable(ss[i]) || !xg_batch_compatible(ss[0], ss[i])) {
            xg_set_error(XIN_GPU_ERR_STATE, "batch_submit: streams must be distinct, compatible, of the plain form and idle");
            return XIN_GPU_ERR_STATE;
        }
    }
    XgSubmitPlan plan[XG_BATCH_MAX];
    for (int i = 0; i < n; i++)
        if (int e = xg_frame_prepare(ss[i], pics[i], -1, -1, plan[i])) return e;
    for (int i = 0; i < n; i++) {
        int *rd = ss[i]->set[plan[i].set].rd;
        rd[0] = plan[i].cur; rd[1] = plan[i].l0; rd[2] = plan[i].l1;
    }
    xin_gpu_stream *s0 = ss[0];
    const xin_gpu_stream_cfg &c = s0->cfg;
    cudaStream_t st = ln.st;
    /* each picture after its stream's previous picture (its planes, search and
     * tails), then its parameters and samples */
    for (int i = 0; i < n; i++) {
        xin_gpu_stream *s = ss[i];
        xin_gpu_stream::Set &t = s->set[plan[i].set];
        cudaStreamWaitEvent(st, s->set[1 - plan[i].set].ev_main, 0);
        cudaEventRecord(t.ev0, st);
        cudaMemcpyAsync(t.dpp, t.h_pp, sizeof(XgPicParams), cudaMemcpyHostToDevice, st);
        for (int p = 0; p < 3; p++) {
            const XgPlane &pl = s->slot[plan[i].cur][p];
            if (s->widen)
                cudaMemcpyAsync(t.d_in8[p], t.h_in[p], (size_t)pl.w * pl.h, cudaMemcpyHostToDevice, st);
            else
                cudaMemcpy2DAsync(pl.data, (size_t)pl.pitch * sizeof(xg_pix), t.h_in[p], (size_t)pl.w * sizeof(xg_pix),
                                  (size_t)pl.w * sizeof(xg_pix), pl.h, cudaMemcpyHostToDevice, st);
        }
    }
    for (int i = 0; i < n; i++) cudaEventRecord(ss[i]->set[plan[i].set].evs[0], st);
    /* slot fill: copy-in (8-bit samples << 2) and edge replication */
    {
        XgFillBatch fb;
        memset(&fb, 0, sizeof fb);
        fb.mode = s0->widen ? XG_FILL_STAGED8 : XG_FILL_IN_PLACE;
        for (int i = 0; i < n; i++) {
            xin_gpu_stream::Set &t = ss[i]->set[plan[i].set];
            for (int p = 0; p < 3; p++) { fb.pl[i][p] = ss[i]->slot[plan[i].cur][p]; fb.s8[i][p] = t.d_in8[p]; }
            fb.pp[i] = t.dpp;
        }
        const XgPlane &ly = s0->slot[plan[0].cur][0];
        dim3 grd(((ly.w + 2 * ly.pad + 7) / 8 + 127) / 128, ly.h + 2 * ly.pad, 3 * n);
        k_fill_slot_batch<<<grd, 128, 0, st>>>(fb);
    }
    for (int i = 0; i < n; i++) cudaEventRecord(ss[i]->set[plan[i].set].evs[1], st);
    /* the new pictures' quarter-pel planes (the next pictures' references) on the
     * low-priority stream beside the search */
    cudaEventRecord(ln.ev_qfork, st);
    cudaStreamWaitEvent(ln.auxq, ln.ev_qfork, 0);
    {
        XgQpelBatch qb;
        memset(&qb, 0, sizeof qb);
        qb.wait_tries = s0->wait_tries;
        for (int i = 0; i < n; i++) {
            xin_gpu_stream *s = ss[i];
            qb.tm[i] = s->tm_qp[plan[i].cur];
            qb.ref[i] = s->slot[plan[i].cur][0];
            qb.qp[i] = s->qpel[plan[i].cur];
            qb.status[i] = &s->set[plan[i].set].dpp->status;
        }
        dim3 grd((c.width + 2 * s0->pad - 8 + XG_QP_TW - 1) / XG_QP_TW, (c.height + 2 * s0->pad - 8 + XG_QP_TH - 1) / XG_QP_TH, n);
        k_qpel_planes_batch<<<grd, 256, 0, ln.auxq>>>(qb);
    }
    for (int i = 0; i < n; i++) cudaEventRecord(ss[i]->set[plan[i].set].ev_ref, ln.auxq);
    cudaEventRecord(ln.ev_qjoin, ln.auxq);
    /* the integer search against each stream's previous picture */
    {
        XgMeBatch mb;
        memset(&mb, 0, sizeof mb);
        mb.bands = s0->me_bands;
        for (int i = 0; i < n; i++) {
            xin_gpu_stream *s = ss[i];
            xg_use_set_keys(s, plan[i].set);
            cudaMemsetAsync(s->keys, 0xff, sizeof(unsigned long long) * s->ncus, st);
            mb.p[i] = xg_me_params(s, plan[i].cur, plan[i].l0, s->keys);
            mb.pp[i] = s->set[plan[i].set].dpp;
        }
        dim3 grd((c.width + 63) / 64, (c.height + 63) / 64, s0->me_bands * n);
#if XG_BITDEPTH == 10
        if (s0->sbd == 10) k_me_tiles_batch<10><<<grd, XG_ME_THREADS, s0->me_smem, st>>>(mb);
        else
#endif
            k_me_tiles_batch<8><<<grd, XG_ME_THREADS, s0->me_smem, st>>>(mb);
    }
    for (int i = 0; i < n; i++) cudaEventRecord(ss[i]->set[plan[i].set].evs[2], st);
    /* the levels' tails, forked onto the lane's auxiliary streams */
    cudaEventRecord(ln.ev_fork, st);
    int li = 0, nfork = 0, nl = 3;
    for (int L = 0; L < XG_NLEV; L++) {
        if (!s0->lev_on[L]) continue;
        cudaStream_t ls = st;
        if (li > 0) {
            ls = ln.aux[li - 1];
            cudaStreamWaitEvent(ls, ln.ev_fork, 0);
            nfork = li;
        }
        XgTailBatch tb;
        memset(&tb, 0, sizeof tb);
        for (int i = 0; i < n; i++) {
            xg_use_set_keys(ss[i], plan[i].set);
            tb.p[i] = xg_tail_params(ss[i], plan[i].set, plan[i].cur, plan[i].l0, plan[i].l1, L, li);
            tb.pp[i] = ss[i]->set[plan[i].set].dpp;
        }
        const int ncu = s0->lev_cx[L] * s0->lev_cy[L];
        if (ncu > 0) {
            switch (XG_LEVEL_SIZE[L]) {
            case 64: k_cu_tail_batch<64, 128, 1><<<dim3(ncu, n), 128, xg_tail_smem<64, 128, 1>(), ls>>>(tb, ncu); break;
            case 32: k_cu_tail_batch<32, 128, 1><<<dim3(ncu, n), 128, xg_tail_smem<32, 128, 1>(), ls>>>(tb, ncu); break;
            case 16:
                k_cu_tail_batch<16, 32, 4><<<dim3((ncu + 3) / 4, n), 128, xg_tail_smem<16, 32, 4>(), ls>>>(tb, ncu);
                break;
            case 8:
                k_cu_tail_batch<8, 32, 4><<<dim3((ncu + 3) / 4, n), 128, xg_tail_smem<8, 32, 4>(), ls>>>(tb, ncu);
                break;
            default: break;     /* the 128 level needs the search by levels: no plain stream has it */
            }
            nl++;
        }
        li++;
    }
    for (int i = 0; i < nfork; i++) {
        cudaEventRecord(ln.ev_join[i], ln.aux[i]);
        cudaStreamWaitEvent(st, ln.ev_join[i], 0);
    }
    cudaStreamWaitEvent(st, ln.ev_qjoin, 0);
    /* per picture: done with its planes, search and tails; then its result copies */
    for (int i = 0; i < n; i++) {
        xin_gpu_stream::Set &t = ss[i]->set[plan[i].set];
        cudaEventRecord(t.ev_main, st);
        cudaEventRecord(t.evs[3], st);
    }
    for (int i = 0; i < n; i++) {
        xin_gpu_stream::Set &t = ss[i]->set[plan[i].set];
        for (int p = 0; p < 3; p++) t.q_dst[p] = q_dst && q_dst[i] ? q_dst[i][p] : nullptr;
        xg_enqueue_result_copies(ss[i], t, true, st);
    }
    xg_count_launch((uint64_t)nl);
    if (xg_cuda_check(cudaGetLastError(), "batch_submit")) return XIN_GPU_ERR_CUDA;
    for (int i = 0; i < n; i++) ss[i]->nsub++;
    return XIN_GPU_OK;
}
