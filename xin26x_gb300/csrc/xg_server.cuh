/*
 * xg_server.cuh -- many encoder streams served by one GPU (xin_gpu_server_*).
 *
 * The reference encodes one sequence per encoder instance and runs its pixel
 * kernels on the calling worker thread.  Serving many live sequences from one
 * GPU needs what the reference does not have: admission (a stream is admitted
 * only if its device memory fits the budget and, optionally, if the luma
 * throughput already promised plus its own stays under a sustained budget),
 * per-stream ordering (a picture uses the previous picture of its stream as the
 * reference, so one stream runs one picture at a time), and continuous batching
 * across streams: one scheduler thread keeps up to max_inflight pictures of
 * different streams running at once and starts the oldest waiting picture as
 * soon as a slot frees.  A picture runs on its stream's own CUDA streams and
 * graph, or -- streams of the plain form and one shape, several pictures
 * waiting -- in a cross-stream batch (xg_batch.cuh) with the other waiting
 * pictures of that shape, one launch per stage for all of them.
 *
 * Each stream's device state is private to it, so a stream's results do not
 * depend on which other streams share the GPU.
 */
#include <algorithm>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

/* device and pinned-host bytes that xin_gpu_stream_open allocates for cfg
 * (the same arithmetic as the allocation sequence there) */
static int xg_stream_bytes(const xin_gpu_stream_cfg *c, uint64_t *dev, uint64_t *host)
{
    if (c->width < 16 || c->height < 16 || (c->width & 1) || (c->height & 1) || c->width > 8192 || c->height > 8192 ||
        (c->ctu_size != 64 && c->ctu_size != 128) || c->search_range < 1 || c->search_range > 256 ||
        !(c->level_mask & (8u | 16u | 32u | 64u | 128u)) || (c->level_mask & ~(8u | 16u | 32u | 64u | 128u)) ||
        ((c->level_mask & 128u) && (c->ctu_size != 128 || c->search_mode != 1 || c->tu_mode != 0)) ||
        !xg_input_depth_ok(*c) || (c->search_mode != 0 && c->search_mode != 1) ||
        (c->tu_mode != 0 && c->tu_mode != 1) || c->refs < 0 || c->refs > 2 ||
        (c->refs == 2 && (c->level_mask & 128u)) || c->dpb < 0 || c->dpb > XG_MAX_DPB || (c->dpb && c->dpb < (c->refs == 2 ? 3 : 2)))
        return XIN_GPU_ERR_ARG;
    const bool widen = XG_BITDEPTH == 10 && c->input_bitdepth == 8;
    const uint64_t in_es = widen ? 1 : sizeof(xg_pix);
    int pad = c->ctu_size + 16 > c->search_range + 72 ? c->ctu_size + 16 : c->search_range + 72;
    pad = (pad + 31) & ~31;
    uint64_t pitch = ((c->width + 2 * pad) + 127) & ~127, rows = c->height + 2 * pad;
    uint64_t cpitch = ((c->width / 2 + pad) + 127) & ~127, crows = c->height / 2 + pad;
    uint64_t ysz = pitch * rows * sizeof(xg_pix), csz = cpitch * crows * sizeof(xg_pix);
    uint64_t lq = (uint64_t)c->width * c->height, lc = lq / 4;
    int nlev = 0;
    uint64_t ncus = 0;
    for (int L = 0; L < XG_NLEV; L++)
        if (c->level_mask & (uint32_t)XG_LEVEL_SIZE[L]) {
            nlev++;
            ncus += (uint64_t)(c->width / XG_LEVEL_SIZE[L]) * (c->height / XG_LEVEL_SIZE[L]);
        }
    /* the picture slots (two; three with two references; dpb when set) with their quarter-pel planes,
     * the search keys, and two picture sets (results, parameters, pinned staging) */
    const uint64_t nslots = c->dpb ? c->dpb : (c->refs == 2 ? 3 : 2);
    uint64_t d = nslots * (ysz + 2 * csz) + nslots * 16 * ysz + 2 * 8 * (ncus ? ncus : 1) +
                 2 * (sizeof(xin_gpu_cu_result) * ncus + sizeof(XgPicParams) + (lq + 2 * lc) * nlev * (sizeof(xg_coef) + sizeof(xg_pix)));
    if (c->refs == 2) d += 2 * 8 * (ncus ? ncus : 1) + 2 * sizeof(xin_gpu_cu_bi) * ncus;   /* list 1's keys, bi records */
    if (widen && !c->device_io) d += 2 * (lq + 2 * lc);     /* 8-bit device staging per set */
    if (c->tu_mode == 1) {                                  /* the preset-4 TU stage */
        d += 2 * xg_tu_bytes(c) + 2 * sizeof(xin_gpu_cu_mts) * ncus;   /* a TU state per picture set */
    }
    if (c->search_mode == 1)                                /* 1/2 and 1/4 resolution luma of every slot */
        for (int l = 0; l < 2; l++)
            d += nslots * ((((uint64_t)(c->width + 2 * pad) >> (l + 1)) + 127) & ~127ull) * ((uint64_t)(c->height + 2 * pad) >> (l + 1)) *
                 sizeof(xg_pix);
    uint64_t h = sizeof(XgPicParams) + sizeof(int32_t) + sizeof(xin_gpu_cu_result) * ncus;
    if (c->tu_mode == 1 && !c->device_io) h += sizeof(xin_gpu_cu_mts) * ncus;
    if (c->refs == 2 && !c->device_io) h += sizeof(xin_gpu_cu_bi) * ncus;
    if (!c->device_io) {
        h += (lq + 2 * lc) * in_es;
        if (c->out_flags & XIN_GPU_OUT_Q) h += (lq + 2 * lc) * nlev * sizeof(xg_coef);
        if (c->out_flags & XIN_GPU_OUT_REC) h += (lq + 2 * lc) * nlev * sizeof(xg_pix);
    }
    h *= 2;
    if (dev) *dev = d;
    if (host) *host = h;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_stream_footprint(const xin_gpu_stream_cfg *cfg, uint64_t *device_bytes, uint64_t *host_bytes)
{
    xin_gpu_clear_error();
    if (!cfg) { xg_set_error(XIN_GPU_ERR_ARG, "stream_footprint: null cfg"); return XIN_GPU_ERR_ARG; }
    int st = xg_stream_bytes(cfg, device_bytes, host_bytes);
    if (st) xg_set_error(st, "stream_footprint: unsupported configuration");
    return st;
}

static double xg_now_ms()
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct XgSrvPic {
    uint32_t index;
    uint64_t tag;
    xin_gpu_cu_result *cu_out;
    xg_coef *q_out[3];            /* caller buffers of the coefficient planes (XIN_GPU_OUT_Q streams), or none */
    int32_t qp, uv_qp;
    uint32_t lambda;
    double t_submit, t_launch;
    std::vector<uint8_t> pix;     /* Y, U, V packed (stride = width), input samples */
};

struct XgSrvStream {
    int32_t id;
    xin_gpu_stream *s;
    xin_gpu_stream_cfg cfg;
    uint64_t dev_bytes;
    double mpix;                  /* luma Mpixel/s promised at admission */
    std::deque<XgSrvPic *> queue;
    XgSrvPic *running;
    bool leaving, failed;
    uint32_t next_index;
    uint32_t max_queue;
    int lane;                     /* batch lane of the running picture, or -1 (its own streams) */
    std::vector<XgSrvPic *> spare;
};

struct xin_gpu_server {
    xin_gpu_server_cfg cfg;
    int device;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_left;
    std::thread worker;
    bool stop;
    std::map<int32_t, XgSrvStream *> streams;
    std::deque<xin_gpu_server_done> done;
    uint64_t hbm_budget, hbm_used;
    double mpix_used;
    int32_t next_id;
    int running;
    uint64_t completed, launched, batches, batched_pictures;
    int sms;                          /* SMs of the device (batch sizes) */
    std::vector<XgBatchLane> lanes;   /* cross-stream batches in flight: one lane each */
};

static void xg_srv_release(XgSrvStream *t, XgSrvPic *p)
{
    if (t->spare.size() < 4) t->spare.push_back(p);
    else delete p;
}

static void xg_srv_finish(xin_gpu_server *v, XgSrvStream *t, xin_gpu_server_done &d)
{
    /* called with the lock held, after the picture's results were collected */
    XgSrvPic *p = t->running;
    t->running = nullptr;
    v->running--;
    if (t->lane >= 0) {
        v->lanes[t->lane].busy--;
        t->lane = -1;
    }
    v->completed++;
    xg_srv_release(t, p);
    v->done.push_back(d);
    v->cv_done.notify_all();
}

/* the library picture of a queued server picture (its packed planes) */
static void xg_srv_picture(const XgSrvStream *t, const XgSrvPic *p, xin_gpu_picture *pic)
{
    memset(pic, 0, sizeof *pic);
    const int w = t->cfg.width, h = t->cfg.height;
    const size_t es = xg_in_es(t->cfg);
    pic->plane[0] = (const XG_PIXEL *)p->pix.data();
    pic->plane[1] = (const XG_PIXEL *)(p->pix.data() + (size_t)w * h * es);
    pic->plane[2] = (const XG_PIXEL *)(p->pix.data() + ((size_t)w * h + (size_t)(w / 2) * (h / 2)) * es);
    pic->stride[0] = w; pic->stride[1] = pic->stride[2] = w / 2;
    pic->qp = p->qp; pic->uv_qp = p->uv_qp; pic->sad_lambda = p->lambda;
}

/* scheduler thread: collect finished pictures, close drained streams, start
 * the oldest waiting pictures.  The lock guards the stream table and queues;
 * the CUDA work of a stream (submit, result copies, close) is done by this
 * thread alone, outside the lock. */
static void xg_srv_loop(xin_gpu_server *v)
{
    cudaSetDevice(v->device);
    std::unique_lock<std::mutex> lk(v->mu);
    std::vector<std::pair<XgSrvStream *, cudaError_t>> fin;
    std::vector<XgSrvStream *> drained;
    for (;;) {
        bool progress = false;
        /* completions */
        fin.clear();
        for (auto &kv : v->streams) {
            XgSrvStream *t = kv.second;
            if (!t->running) continue;
            cudaError_t e = cudaEventQuery(xg_stream_last_event(t->s));
            if (e != cudaErrorNotReady) fin.emplace_back(t, e);
        }
        if (!fin.empty()) {
            lk.unlock();
            std::vector<xin_gpu_server_done> ds(fin.size());
            for (size_t i = 0; i < fin.size(); i++) {
                XgSrvStream *t = fin[i].first;
                XgSrvPic *p = t->running;
                xin_gpu_server_done &d = ds[i];
                memset(&d, 0, sizeof d);
                d.stream_id = t->id;
                d.frame_index = p->index;
                d.user_tag = p->tag;
                if (fin[i].second != cudaSuccess) {
                    cudaGetLastError();
                    d.status = XIN_GPU_ERR_CUDA;
                } else {
                    xin_gpu_results r;
                    memset(&r, 0, sizeof r);
                    r.cu = p->cu_out;
                    for (int k = 0; k < 3; k++) r.q[k] = p->q_out[k];   /* already in place: no copy */
                    d.status = xin_gpu_frame_wait(t->s, &r, 0);
                    d.has_results = p->index > 0 && d.status == XIN_GPU_OK;
                    d.gpu_ms = r.gpu_ms;
                }
                d.queue_ms = p->t_launch - p->t_submit;
                d.latency_ms = xg_now_ms() - p->t_submit;
            }
            lk.lock();
            for (size_t i = 0; i < fin.size(); i++) {
                if (ds[i].status) fin[i].first->failed = true;
                xg_srv_finish(v, fin[i].first, ds[i]);
            }
            progress = true;
        }
        /* streams that left and drained */
        drained.clear();
        for (auto it = v->streams.begin(); it != v->streams.end();) {
            XgSrvStream *t = it->second;
            if (t->leaving && !t->running && t->queue.empty()) {
                drained.push_back(t);
                it = v->streams.erase(it);
            } else {
                ++it;
            }
        }
        if (!drained.empty()) {
            lk.unlock();
            for (XgSrvStream *t : drained) xin_gpu_stream_close(t->s);
            lk.lock();
            for (XgSrvStream *t : drained) {
                v->hbm_used -= t->dev_bytes;
                v->mpix_used -= t->mpix;
                for (XgSrvPic *p : t->spare) delete p;
                delete t;
            }
            v->cv_left.notify_all();
            progress = true;
        }
        /* launches, oldest submission first; the oldest picture of a plain stream
         * takes the oldest waiting pictures of compatible streams into its batch */
        bool held = false;
        while (v->running < (int)v->cfg.max_inflight) {
            XgSrvStream *best = nullptr;
            for (auto &kv : v->streams) {
                XgSrvStream *t = kv.second;
                if (t->running || t->queue.empty()) continue;
                if (!best || t->queue.front()->t_submit < best->queue.front()->t_submit) best = t;
            }
            if (!best) break;
            XgSrvStream *mem[XG_BATCH_MAX];
            int nb = 1, lane = -1;
            mem[0] = best;
            if (v->cfg.batch_max > 1 && !best->failed && xg_batchable(best->s)) {
                for (size_t i = 0; i < v->lanes.size() && lane < 0; i++)
                    if (!v->lanes[i].busy) lane = (int)i;
                const int cap = std::min(std::min((int)v->cfg.batch_max, (int)v->cfg.max_inflight - v->running),
                                         xg_batch_fill_limit(best->s, v->sms));
                while (lane >= 0 && nb < cap) {
                    XgSrvStream *nx = nullptr;
                    for (auto &kv : v->streams) {
                        XgSrvStream *t = kv.second;
                        if (t->running || t->queue.empty() || t->failed) continue;
                        bool in = false;
                        for (int j = 0; j < nb; j++) in |= mem[j] == t;
                        if (in || !xg_batchable(t->s) || !xg_batch_compatible(best->s, t->s)) continue;
                        if (!nx || t->queue.front()->t_submit < nx->queue.front()->t_submit) nx = t;
                    }
                    if (!nx) break;
                    mem[nb++] = nx;
                }
                /* hold an incomplete batch open while its oldest picture is younger
                 * than the window */
                if (lane >= 0 && nb < cap && v->cfg.batch_window_us > 0 &&
                    xg_now_ms() - best->queue.front()->t_submit < v->cfg.batch_window_us * 1e-3) {
                    held = true;
                    break;
                }
            }
            if (nb > 1) {
                XgSrvPic *ps[XG_BATCH_MAX];
                xin_gpu_picture pics[XG_BATCH_MAX];
                const xin_gpu_picture *pp[XG_BATCH_MAX];
                xg_coef *const *qd[XG_BATCH_MAX];
                xin_gpu_stream *ss[XG_BATCH_MAX];
                const double now = xg_now_ms();
                for (int j = 0; j < nb; j++) {
                    XgSrvStream *t = mem[j];
                    XgSrvPic *q = t->queue.front();
                    t->queue.pop_front();
                    t->running = q;
                    t->lane = lane;
                    v->running++;
                    q->t_launch = now;
                    xg_srv_picture(t, q, &pics[j]);
                    ps[j] = q;
                    pp[j] = &pics[j];
                    qd[j] = q->q_out[0] ? q->q_out : nullptr;
                    ss[j] = t->s;
                }
                v->lanes[lane].busy = nb;
                progress = true;
                lk.unlock();
                int st = xg_batch_submit(ss, pp, qd, nb, v->lanes[lane]);
                lk.lock();
                v->launched += nb;
                if (st) {
                    for (int j = 0; j < nb; j++) {
                        xin_gpu_server_done d;
                        memset(&d, 0, sizeof d);
                        d.stream_id = mem[j]->id; d.frame_index = ps[j]->index; d.user_tag = ps[j]->tag; d.status = st;
                        mem[j]->failed = true;
                        xg_srv_finish(v, mem[j], d);
                    }
                } else {
                    v->batches++;
                    v->batched_pictures += nb;
                }
                continue;
            }
            XgSrvPic *p = best->queue.front();
            best->queue.pop_front();
            progress = true;
            if (best->failed) {
                xin_gpu_server_done d;
                memset(&d, 0, sizeof d);
                d.stream_id = best->id; d.frame_index = p->index; d.user_tag = p->tag; d.status = XIN_GPU_ERR_STATE;
                v->done.push_back(d);
                v->cv_done.notify_all();
                xg_srv_release(best, p);
                continue;
            }
            best->running = p;
            v->running++;
            p->t_launch = xg_now_ms();
            xin_gpu_picture pic;
            xg_srv_picture(best, p, &pic);
            lk.unlock();
            int st = xg_frame_submit(best->s, &pic, -1, -1, p->q_out[0] ? p->q_out : nullptr);
            lk.lock();
            v->launched++;
            if (st) {
                xin_gpu_server_done d;
                memset(&d, 0, sizeof d);
                d.stream_id = best->id; d.frame_index = p->index; d.user_tag = p->tag; d.status = st;
                best->failed = true;
                xg_srv_finish(v, best, d);
            }
        }
        if (v->stop && v->running == 0) {
            bool queued = false;
            for (auto &kv : v->streams) queued |= !kv.second->queue.empty();
            if (!queued && v->streams.empty()) break;
        }
        if (!progress) {
            if (v->running || held) {
                /* pictures on the GPU: poll their events at a short interval */
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                lk.lock();
            } else {
                v->cv_work.wait_for(lk, std::chrono::milliseconds(5));
            }
        }
    }
}

extern "C" int xin_gpu_server_open(const xin_gpu_server_cfg *cfg, xin_gpu_server **out)
{
    xin_gpu_clear_error();
    if (!out) { xg_set_error(XIN_GPU_ERR_ARG, "server_open: null argument"); return XIN_GPU_ERR_ARG; }
    *out = nullptr;
    if (xg_ensure_init()) return XIN_GPU_ERR_CUDA;
    xin_gpu_server *v = new (std::nothrow) xin_gpu_server();
    if (!v) { xg_set_error(XIN_GPU_ERR_NOMEM, "server_open: host allocation"); return XIN_GPU_ERR_NOMEM; }
    if (cfg) v->cfg = *cfg;
    else memset(&v->cfg, 0, sizeof v->cfg);
    if (!v->cfg.max_inflight) v->cfg.max_inflight = 8;
    if (!v->cfg.max_streams) v->cfg.max_streams = 256;
    if (!v->cfg.max_queue) v->cfg.max_queue = 4;
    if (!v->cfg.batch_max || v->cfg.batch_max > XG_BATCH_MAX) v->cfg.batch_max = XG_BATCH_MAX;
    cudaGetDevice(&v->device);
    v->sms = 0;
    cudaDeviceGetAttribute(&v->sms, cudaDevAttrMultiProcessorCount, v->device);
    if (v->cfg.batch_max > 1) {
        /* a batch carries two pictures or more: at most max_inflight / 2 run at once */
        v->lanes.resize(v->cfg.max_inflight / 2 > 0 ? v->cfg.max_inflight / 2 : 1);
        for (size_t i = 0; i < v->lanes.size(); i++)
            if (int e = xg_lane_open(v->lanes[i])) {
                for (size_t j = 0; j < i; j++) xg_lane_close(v->lanes[j]);
                delete v;
                return e;
            }
    }
    v->hbm_budget = v->cfg.hbm_budget;
    if (!v->hbm_budget) {
        size_t fr = 0, tot = 0;
        if (xg_cuda_check(cudaMemGetInfo(&fr, &tot), "server_open")) { delete v; return XIN_GPU_ERR_CUDA; }
        v->hbm_budget = (uint64_t)(fr * 0.9);
    }
    v->worker = std::thread(xg_srv_loop, v);
    *out = v;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_server_join(xin_gpu_server *v, const xin_gpu_stream_cfg *cfg, double fps, int32_t *stream_id)
{
    xin_gpu_clear_error();
    if (!v || !cfg || !stream_id || fps < 0) { xg_set_error(XIN_GPU_ERR_ARG, "server_join: bad argument"); return XIN_GPU_ERR_ARG; }
    if (cfg->device_io) { xg_set_error(XIN_GPU_ERR_ARG, "server_join: served streams take host pictures (device_io = 0)"); return XIN_GPU_ERR_ARG; }
    uint64_t dev = 0;
    if (xg_stream_bytes(cfg, &dev, nullptr)) { xg_set_error(XIN_GPU_ERR_ARG, "server_join: unsupported stream configuration"); return XIN_GPU_ERR_ARG; }
    double mpix = (double)cfg->width * cfg->height * fps / 1e6;
    {
        std::lock_guard<std::mutex> lk(v->mu);
        if (v->stop) { xg_set_error(XIN_GPU_ERR_STATE, "server_join: server is closing"); return XIN_GPU_ERR_STATE; }
        if (v->streams.size() >= v->cfg.max_streams) {
            xg_set_error(XIN_GPU_ERR_ADMIT, "server_join: %u streams already admitted", v->cfg.max_streams);
            return XIN_GPU_ERR_ADMIT;
        }
        if (v->hbm_used + dev > v->hbm_budget) {
            xg_set_error(XIN_GPU_ERR_ADMIT, "server_join: needs %llu device bytes, %llu of %llu in use",
                         (unsigned long long)dev, (unsigned long long)v->hbm_used, (unsigned long long)v->hbm_budget);
            return XIN_GPU_ERR_ADMIT;
        }
        if (v->cfg.mpix_budget > 0 && v->mpix_used + mpix > v->cfg.mpix_budget) {
            xg_set_error(XIN_GPU_ERR_ADMIT, "server_join: %.1f Mpixel/s requested, %.1f of %.1f promised", mpix, v->mpix_used,
                         v->cfg.mpix_budget);
            return XIN_GPU_ERR_ADMIT;
        }
        v->hbm_used += dev;      /* reserved while the stream opens */
        v->mpix_used += mpix;
    }
    xin_gpu_stream_cfg c = *cfg;
    c.out_flags &= XIN_GPU_OUT_Q;   /* served streams return CU records and, when asked, coefficient planes */
    xin_gpu_stream *s = nullptr;
    int st = xin_gpu_stream_open(&c, &s);
    std::lock_guard<std::mutex> lk(v->mu);
    if (st) {
        v->hbm_used -= dev;
        v->mpix_used -= mpix;
        return st;
    }
    XgSrvStream *t = new XgSrvStream();
    t->id = v->next_id++;
    t->s = s;
    t->cfg = c;
    t->dev_bytes = dev;
    t->mpix = mpix;
    t->running = nullptr;
    t->leaving = t->failed = false;
    t->next_index = 0;
    t->max_queue = v->cfg.max_queue;
    t->lane = -1;
    v->streams[t->id] = t;
    *stream_id = t->id;
    return XIN_GPU_OK;
}

static int xg_server_submit(xin_gpu_server *v, int32_t stream_id, const xin_gpu_picture *pic, xin_gpu_cu_result *cu_out,
                            XG_COEFF *const *q_out, uint64_t user_tag);
extern "C" int xin_gpu_server_submit(xin_gpu_server *v, int32_t stream_id, const xin_gpu_picture *pic,
                                     xin_gpu_cu_result *cu_out, uint64_t user_tag)
{
    return xg_server_submit(v, stream_id, pic, cu_out, nullptr, user_tag);
}
extern "C" int xin_gpu_server_submit_planes(xin_gpu_server *v, int32_t stream_id, const xin_gpu_picture *pic,
                                            xin_gpu_cu_result *cu_out, XG_COEFF *const q_out[3], uint64_t user_tag)
{
    if (!q_out || !q_out[0] || !q_out[1] || !q_out[2]) {
        xin_gpu_clear_error();
        xg_set_error(XIN_GPU_ERR_ARG, "server_submit_planes: three plane buffers needed");
        return XIN_GPU_ERR_ARG;
    }
    return xg_server_submit(v, stream_id, pic, cu_out, q_out, user_tag);
}

static int xg_server_submit(xin_gpu_server *v, int32_t stream_id, const xin_gpu_picture *pic, xin_gpu_cu_result *cu_out,
                            XG_COEFF *const *q_out, uint64_t user_tag)
{
    xin_gpu_clear_error();
    if (!v || !pic) { xg_set_error(XIN_GPU_ERR_ARG, "server_submit: null argument"); return XIN_GPU_ERR_ARG; }
    if (pic->qp < 0 || pic->qp > 63 || pic->uv_qp < 0 || pic->uv_qp > 63) {
        xg_set_error(XIN_GPU_ERR_ARG, "server_submit: QP out of range");
        return XIN_GPU_ERR_ARG;
    }
    /* refused here rather than at launch, where the picture may share a batch with
     * other streams' pictures */
    if (pic->sad_lambda > (1u << 20)) { xg_set_error(XIN_GPU_ERR_ARG, "server_submit: sad_lambda above 2^20"); return XIN_GPU_ERR_ARG; }
    XgSrvPic *p = nullptr;
    int w, h;
    size_t es;
    {
        std::lock_guard<std::mutex> lk(v->mu);
        auto it = v->streams.find(stream_id);
        if (it == v->streams.end() || it->second->leaving) {
            xg_set_error(XIN_GPU_ERR_ARG, "server_submit: no stream %d", stream_id);
            return XIN_GPU_ERR_ARG;
        }
        XgSrvStream *t = it->second;
        if (t->failed) { xg_set_error(XIN_GPU_ERR_STATE, "server_submit: stream %d failed", stream_id); return XIN_GPU_ERR_STATE; }
        if (t->queue.size() >= t->max_queue) {
            xg_set_error(XIN_GPU_ERR_STATE, "server_submit: stream %d already has %u pictures waiting", stream_id, t->max_queue);
            return XIN_GPU_ERR_STATE;
        }
        if (t->next_index > 0 && !cu_out) {
            xg_set_error(XIN_GPU_ERR_ARG, "server_submit: cu_out needed (xin_gpu_stream_num_cus records)");
            return XIN_GPU_ERR_ARG;
        }
        if (q_out && !(t->cfg.out_flags & XIN_GPU_OUT_Q)) {
            xg_set_error(XIN_GPU_ERR_ARG, "server_submit_planes: stream %d was joined without XIN_GPU_OUT_Q", stream_id);
            return XIN_GPU_ERR_ARG;
        }
        w = t->cfg.width; h = t->cfg.height;
        es = xg_in_es(t->cfg);
        if (!t->spare.empty()) { p = t->spare.back(); t->spare.pop_back(); }
    }
    for (int k = 0; k < 3; k++)
        if (!pic->plane[k] || pic->stride[k] < (k ? w / 2 : w)) {
            if (p) delete p;
            xg_set_error(XIN_GPU_ERR_ARG, "server_submit: bad plane");
            return XIN_GPU_ERR_ARG;
        }
    if (!p) p = new XgSrvPic();
    /* copy the picture so that the caller's buffers are free on return */
    size_t lq = (size_t)w * h, lc = lq / 4;
    p->pix.resize((lq + 2 * lc) * es);
    for (int y = 0; y < h; y++)
        memcpy(p->pix.data() + (size_t)y * w * es, (const char *)pic->plane[0] + (size_t)y * pic->stride[0] * es, w * es);
    for (int k = 1; k < 3; k++)
        for (int y = 0; y < h / 2; y++)
            memcpy(p->pix.data() + (lq + (k - 1) * lc + (size_t)y * (w / 2)) * es,
                   (const char *)pic->plane[k] + (size_t)y * pic->stride[k] * es, (w / 2) * es);
    p->tag = user_tag;
    p->cu_out = cu_out;
    for (int k = 0; k < 3; k++) p->q_out[k] = q_out ? (xg_coef *)q_out[k] : nullptr;
    p->qp = pic->qp; p->uv_qp = pic->uv_qp; p->lambda = pic->sad_lambda;
    std::lock_guard<std::mutex> lk(v->mu);
    auto it = v->streams.find(stream_id);
    if (it == v->streams.end() || it->second->leaving) {
        delete p;
        xg_set_error(XIN_GPU_ERR_ARG, "server_submit: stream %d left", stream_id);
        return XIN_GPU_ERR_ARG;
    }
    p->index = it->second->next_index++;
    p->t_submit = xg_now_ms();
    it->second->queue.push_back(p);
    v->cv_work.notify_one();
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_server_poll(xin_gpu_server *v, xin_gpu_server_done *out, int32_t max, int32_t timeout_ms, int32_t *n)
{
    xin_gpu_clear_error();
    if (!v || !out || max <= 0 || !n) { xg_set_error(XIN_GPU_ERR_ARG, "server_poll: bad argument"); return XIN_GPU_ERR_ARG; }
    std::unique_lock<std::mutex> lk(v->mu);
    if (v->done.empty() && timeout_ms != 0) {
        if (timeout_ms < 0) v->cv_done.wait(lk, [&] { return !v->done.empty(); });
        else v->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !v->done.empty(); });
    }
    int k = 0;
    while (k < max && !v->done.empty()) { out[k++] = v->done.front(); v->done.pop_front(); }
    *n = k;
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_server_leave(xin_gpu_server *v, int32_t stream_id, int32_t timeout_ms)
{
    xin_gpu_clear_error();
    if (!v) { xg_set_error(XIN_GPU_ERR_ARG, "server_leave: null server"); return XIN_GPU_ERR_ARG; }
    std::unique_lock<std::mutex> lk(v->mu);
    auto it = v->streams.find(stream_id);
    if (it == v->streams.end() || it->second->leaving) {
        xg_set_error(XIN_GPU_ERR_ARG, "server_leave: no stream %d", stream_id);
        return XIN_GPU_ERR_ARG;
    }
    it->second->leaving = true;
    v->cv_work.notify_one();
    auto gone = [&] { return v->streams.find(stream_id) == v->streams.end(); };
    if (timeout_ms < 0) v->cv_left.wait(lk, gone);
    else if (!v->cv_left.wait_for(lk, std::chrono::milliseconds(timeout_ms), gone)) {
        xg_set_error(XIN_GPU_ERR_TIMEOUT, "server_leave: stream %d still draining after %d ms", stream_id, timeout_ms);
        return XIN_GPU_ERR_TIMEOUT;
    }
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_server_get_stats(xin_gpu_server *v, xin_gpu_server_stats *s)
{
    if (!v || !s) return XIN_GPU_ERR_ARG;
    std::lock_guard<std::mutex> lk(v->mu);
    s->streams = (int32_t)v->streams.size();
    s->running = v->running;
    s->hbm_budget = v->hbm_budget;
    s->hbm_used = v->hbm_used;
    s->mpix_used = v->mpix_used;
    s->launched = v->launched;
    s->completed = v->completed;
    s->batches = v->batches;
    s->batched_pictures = v->batched_pictures;
    s->queued = 0;
    for (auto &kv : v->streams) s->queued += (int32_t)kv.second->queue.size();
    return XIN_GPU_OK;
}

extern "C" int xin_gpu_server_close(xin_gpu_server *v)
{
    if (!v) return XIN_GPU_OK;
    {
        std::lock_guard<std::mutex> lk(v->mu);
        v->stop = true;
        for (auto &kv : v->streams) kv.second->leaving = true;
        v->cv_work.notify_one();
    }
    if (v->worker.joinable()) v->worker.join();
    for (auto &kv : v->streams) {
        XgSrvStream *t = kv.second;
        xin_gpu_stream_close(t->s);
        for (XgSrvPic *p : t->queue) delete p;
        for (XgSrvPic *p : t->spare) delete p;
        delete t;
    }
    for (XgBatchLane &ln : v->lanes) xg_lane_close(ln);
    delete v;
    return XIN_GPU_OK;
}
