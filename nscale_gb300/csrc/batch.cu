// batch.cu — many tiles on one GPU: a pool of workers (host threads), each
// owning a context (workspace arena) and a non-blocking CUDA stream.
//
// The reference segments one tile per process and farms tiles to MPI ranks
// (nu-segment.cpp:274-430).  On one GB300 a single tile leaves most SMs idle
// during its latency-bound stages (the watershed's layer-by-layer BFS and
// per-domain floods, the tail of the reconstruction queue), so the pool keeps
// several tiles in flight and lets their stages overlap:
//
//  * nsg_segment_nuclei_batch: every worker takes the next tile from a shared
//    counter over the tiles sorted largest first, so that the batch ends on
//    small tiles;
//  * nsg_server_*: tiles are submitted one at a time into a bounded FIFO and
//    results are polled; the number of workers is what a memory budget admits,
//    either all of one size or split over size classes
//    (nsg_server_create_classes), so that a small tile holds a small
//    workspace; a full queue rejects new tiles (the caller sheds or retries).
//
// Host code only: the device work is the pipeline of pipeline.cu.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "nsg_internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    nsg_tile tile;
    nsg_seg_params prm;
    long long ticket;
    Clock::time_point t_submit;
    int64_t need;  // capacity (pixels) of the smallest worker class that holds the tile
};

struct Worker {
    nsg_context *ctx = nullptr;
    cudaStream_t stream = nullptr;
    std::thread th;
    int max_rows = 0, max_cols = 0;  // the largest tile its context holds
    bool fits(int rows, int cols) const {
        return rows > 0 && cols > 0 && (int64_t)rows * cols <= (int64_t)max_rows * max_cols &&
               (int64_t)(rows + 2) * (cols + 2) <= (int64_t)(max_rows + 2) * (max_cols + 2);
    }
    int64_t capacity() const { return (int64_t)max_rows * max_cols; }
};

// H channel (colour deconvolution with the feature pipeline's stains) and
// the per-nucleus features of a segmented tile, copied to an nsg_alloc'd
// host array.  Scratch: p_u8[0] (H), p_f32[0] (features), and the feature
// pass's own planes; the labels must live elsewhere.
int tile_features(nsg::Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, const int32_t *lab,
                  nsg_tile &t, cudaStream_t s) {
    float q[6];
    if (nsg_stain_matrix(nullptr, nullptr, q) != NSG_SUCCESS) return NSG_ERR_ARG;
    uint8_t *H = c.ws.p_u8[0];
    float *fd = c.ws.p_f32[0];
    NSG_TRY(nsg::color_deconv_dev(c, bgr, stride, rows, cols, q, H, nullptr, s));
    int cnt = 0;
    const int cap = (int)std::min<int64_t>(c.max_pad / NSG_N_FEATURES, 1 << 30);
    NSG_TRY(nsg::nucleus_features_dev(c, lab, H, rows, cols, fd, cap, &cnt, s));
    float *fh = (float *)nsg_alloc(sizeof(float) * NSG_N_FEATURES * (size_t)(cnt > 0 ? cnt : 1));
    if (!fh) return NSG_ERR_OOM;
    if (cnt > 0) {
        cudaError_t e = cudaMemcpyAsync(fh, fd, sizeof(float) * NSG_N_FEATURES * (size_t)cnt, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            nsg_free(fh);
            return NSG_ERR_CUDA;
        }
    }
    t.features = fh;
    return NSG_SUCCESS;
}

// one tile through the pipeline on a worker; outputs are complete on return
void run_tile(nsg_context *ctx, cudaStream_t s, nsg_tile &t, const nsg_seg_params &p, bool host) {
    t.compcount = 0;
    t.bbox = nullptr;
    t.features = nullptr;
    int32_t **bb = t.want_bbox ? &t.bbox : nullptr;
    int st;
    if (!t.want_features) {
        if (host) {
            st = nsg_segment_nuclei_host(ctx, t.bgr, t.rows, t.cols, &p, t.labels, t.mask, &t.compcount, bb, s);
        } else {
            const size_t stride = t.row_stride_bytes ? t.row_stride_bytes : (size_t)t.cols * 3;
            st = nsg_segment_nuclei(ctx, t.bgr, t.rows, t.cols, stride, &p, t.labels, t.mask, &t.compcount, bb, s);
            if (cudaStreamSynchronize(s) != cudaSuccess && st >= 0) st = NSG_ERR_CUDA;
        }
        t.status = st;
        return;
    }
    // with features: the pipeline on device buffers, then the feature pass
    nsg::Ctx &c = ctx->c;
    if (!t.bgr || t.rows <= 0 || t.cols <= 0 || (int64_t)t.rows * t.cols > c.max_px) {
        t.status = t.bgr ? NSG_ERR_ARG : NSG_INVALID_IMAGE;
        return;
    }
    const int64_t n = (int64_t)t.rows * t.cols;
    const uint8_t *bgr = t.bgr;
    int64_t stride = t.row_stride_bytes ? (int64_t)t.row_stride_bytes : (int64_t)t.cols * 3;
    int32_t *lab = host ? (int32_t *)c.ws.i32[5] : (t.labels ? t.labels : c.ws.p_i32[0]);
    uint8_t *msk = t.mask ? (host ? c.ws.p_u8[9] : t.mask) : nullptr;
    if (host) {
        if (cudaMemcpyAsync(c.ws.p_bgr, t.bgr, (size_t)n * 3, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            t.status = NSG_ERR_CUDA;
            return;
        }
        bgr = c.ws.p_bgr;
        stride = (int64_t)t.cols * 3;
    }
    st = nsg::segment_nuclei_dev(c, bgr, stride, t.rows, t.cols, p, lab, msk, &t.compcount, bb, s);
    if (st == NSG_SUCCESS) st = tile_features(c, bgr, stride, t.rows, t.cols, lab, t, s);
    if (st >= 0 && host) {
        if (t.labels) cudaMemcpyAsync(t.labels, lab, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
        if (t.mask) cudaMemcpyAsync(t.mask, msk, (size_t)n, cudaMemcpyDeviceToHost, s);
    }
    if (cudaStreamSynchronize(s) != cudaSuccess && st >= 0) st = NSG_ERR_CUDA;
    t.status = st;
}

}  // namespace

struct nsg_pool {
    int device = 0;
    std::vector<Worker> w;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_res;
    bool quit = false;
    // batch job (published under mu, then read lock-free by the workers)
    nsg_tile *tiles = nullptr;
    int n = 0;
    std::vector<int> order;  // tiles largest first: the batch's tail is a small tile
    nsg_seg_params prm{};
    int flags = 0;
    std::atomic<int> next{0};
    std::atomic<int> first_error{0};
    unsigned long long gen = 0;
    int busy = 0;
    // server queue
    std::deque<Job> q;
    std::deque<nsg_result> done;
    int qcap = 0;
    long long next_ticket = 0;
    int64_t smallest_class = 0;  // capacity (pixels) of the smallest worker class

    // the smallest worker class (capacity in pixels) that holds a rows x cols
    // tile, 0 when none does
    int64_t class_for(int rows, int cols) const {
        int64_t best = 0;
        for (const Worker &o : w)
            if (o.fits(rows, cols) && (best == 0 || o.capacity() < best)) best = o.capacity();
        return best;
    }

    // The server's admission: a worker takes the oldest queued tile of its own
    // size class first (the tiles that need a context of its size), else the
    // oldest queued tile that fits its context at all, so that small tiles do
    // not keep larger ones waiting for the large workers while no worker idles
    // with work it could do.  -1: nothing fits.
    int pick_job(const Worker &me) const {
        int any = -1;
        const int64_t mine = me.capacity();
        for (int i = 0; i < (int)q.size(); ++i) {
            if (q[i].need == mine) return i;
            if (any < 0 && q[i].need <= mine && me.fits(q[i].tile.rows, q[i].tile.cols)) any = i;
        }
        return any;
    }

    void work(int k) {
        cudaSetDevice(device);
        Worker &me = w[k];
        unsigned long long seen = 0;
        for (;;) {
            std::unique_lock<std::mutex> lk(mu);
            int pick = -1;
            cv_work.wait(lk, [&] {
                if (quit || gen != seen) return true;
                pick = pick_job(me);
                return pick >= 0;
            });
            if (quit) return;
            if (gen == seen && pick >= 0) {
                Job j = q[pick];
                q.erase(q.begin() + pick);
                lk.unlock();
                run_tile(me.ctx, me.stream, j.tile, j.prm, true);
                nsg_result r;
                r.ticket = j.ticket;
                r.status = j.tile.status;
                r.compcount = j.tile.compcount;
                r.bbox = j.tile.bbox;
                r.features = j.tile.features;
                r.latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - j.t_submit).count();
                lk.lock();
                done.push_back(r);
                cv_res.notify_all();
                continue;
            }
            seen = gen;
            lk.unlock();
            const bool host = flags & NSG_TILE_HOST;
            for (;;) {
                const int k = next.fetch_add(1);
                if (k >= n) break;
                const int i = order[k];
                run_tile(me.ctx, me.stream, tiles[i], prm, host);
                if (tiles[i].status < NSG_RUNTIME_FAILED) {
                    int zero = 0;
                    first_error.compare_exchange_strong(zero, tiles[i].status);
                }
            }
            lk.lock();
            if (--busy == 0) cv_done.notify_all();
        }
    }
};

struct nsg_server {
    nsg_pool *pool = nullptr;
};

namespace {

void pool_free(nsg_pool *p) {
    {
        std::lock_guard<std::mutex> lk(p->mu);
        p->quit = true;
    }
    p->cv_work.notify_all();
    for (auto &w : p->w)
        if (w.th.joinable()) w.th.join();
    cudaSetDevice(p->device);
    for (auto &w : p->w) {
        if (w.stream) cudaStreamDestroy(w.stream);
        if (w.ctx) nsg_context_destroy(w.ctx);
    }
    delete p;
}

}  // namespace

extern "C" {

size_t nsg_pool_context_bytes(int max_rows, int max_cols) {
    if (max_rows <= 0 || max_cols <= 0) return 0;
    return nsg::context_bytes_for(max_rows, max_cols);
}

}  // extern "C"

namespace {

// a pool whose worker k holds tiles up to dims[2k] x dims[2k+1]
int pool_create_dims(nsg_pool **out, const std::vector<int> &dims, int device) {
    const int workers = (int)dims.size() / 2;
    if (!out || workers <= 0 || workers > 256) return NSG_ERR_ARG;
    for (int v : dims)
        if (v <= 0) return NSG_ERR_ARG;
    *out = nullptr;
    nsg_pool *p = new (std::nothrow) nsg_pool();
    if (!p) return NSG_ERR_OOM;
    p->device = device;
    p->w.resize(workers);
    if (cudaSetDevice(device) != cudaSuccess) {
        delete p;
        return NSG_ERR_CUDA;
    }
    p->smallest_class = 0;
    for (int k = 0; k < workers; ++k) {
        Worker &w = p->w[k];
        w.max_rows = dims[2 * k];
        w.max_cols = dims[2 * k + 1];
        if (p->smallest_class == 0 || w.capacity() < p->smallest_class) p->smallest_class = w.capacity();
        int r = nsg_context_create(&w.ctx, w.max_rows, w.max_cols, device);
        if (r == NSG_SUCCESS && cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking) != cudaSuccess)
            r = NSG_ERR_CUDA;
        if (r != NSG_SUCCESS) {
            pool_free(p);
            return r;
        }
        // with several tiles in flight, each reconstruction runs on a share
        // of the SMs, 2 x SMs / workers, between 4 CTAs and half the SMs: its
        // CTA-time is about the same on fewer CTAs, and the other tiles get
        // the rest (measured on GB300 with 32 workers: 9 CTAs 882 Mpixel/s,
        // 19 815, 38 765)
        if (workers > 1) {
            const int sm = w.ctx->c.sm_count;
            int r = 2 * sm / workers;
            if (r > sm / 2) r = sm / 2;
            if (r < 4) r = 4;
            w.ctx->c.recon_max_ctas = r;
        }
    }
    for (int k = 0; k < workers; ++k) p->w[k].th = std::thread([p, k] { p->work(k); });
    *out = p;
    return NSG_SUCCESS;
}

}  // namespace

extern "C" {

int nsg_pool_create(nsg_pool **out, int max_rows, int max_cols, int workers, int device) {
    if (!out || max_rows <= 0 || max_cols <= 0 || workers <= 0 || workers > 256) return NSG_ERR_ARG;
    std::vector<int> dims;
    for (int k = 0; k < workers; ++k) dims.push_back(max_rows), dims.push_back(max_cols);
    return pool_create_dims(out, dims, device);
}

int nsg_pool_destroy(nsg_pool *p) {
    if (!p) return NSG_ERR_ARG;
    pool_free(p);
    return NSG_SUCCESS;
}

int nsg_pool_workers(const nsg_pool *p) { return p ? (int)p->w.size() : 0; }

int nsg_pool_set_tuning(nsg_pool *p, const nsg_tuning *t) {
    if (!p || !t) return NSG_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->busy) return NSG_ERR_ARG;  // not while a batch runs
    for (auto &w : p->w) {
        const int r = nsg_context_set_tuning(w.ctx, t);
        if (r != NSG_SUCCESS) return r;
    }
    return NSG_SUCCESS;
}

int nsg_pool_set_timing(nsg_pool *p, int on) {
    if (!p) return NSG_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->busy) return NSG_ERR_ARG;
    for (auto &w : p->w) {
        const int r = nsg_context_set_timing(w.ctx, on);
        if (r != NSG_SUCCESS) return r;
    }
    return NSG_SUCCESS;
}

int nsg_pool_stage_times(nsg_pool *p, double *ms_out, int n, long long *calls) {
    if (!p || !ms_out || n < 0) return NSG_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    if (p->busy) return NSG_ERR_ARG;
    for (int i = 0; i < n; ++i) ms_out[i] = 0.0;
    long long total = 0;
    int stages = 0;
    std::vector<double> one(n > 0 ? n : 1);
    for (auto &w : p->w) {
        long long k = 0;
        stages = nsg_context_stage_times(w.ctx, one.data(), n, &k);
        if (stages < 0) return stages;
        for (int i = 0; i < n && i < stages; ++i) ms_out[i] += one[i];
        total += k;
    }
    if (calls) *calls = total;
    return stages;
}

int nsg_segment_nuclei_batch(nsg_pool *p, nsg_tile *tiles, int n, const nsg_seg_params *prm, int flags) {
    if (!p || n < 0 || (n > 0 && !tiles)) return NSG_ERR_ARG;
    if (n == 0) return NSG_SUCCESS;
    std::unique_lock<std::mutex> lk(p->mu);
    if (p->busy) return NSG_ERR_ARG;  // one batch at a time per pool
    p->tiles = tiles;
    p->n = n;
    p->order.resize(n);
    for (int i = 0; i < n; ++i) p->order[i] = i;
    std::stable_sort(p->order.begin(), p->order.end(), [&](int a, int b) {
        return (int64_t)tiles[a].rows * tiles[a].cols > (int64_t)tiles[b].rows * tiles[b].cols;
    });
    if (prm) p->prm = *prm;
    else nsg_default_params(&p->prm);
    p->flags = flags;
    p->next.store(0);
    p->first_error.store(0);
    p->busy = (int)p->w.size();
    ++p->gen;
    p->cv_work.notify_all();
    p->cv_done.wait(lk, [&] { return p->busy == 0; });
    const int e = p->first_error.load();
    return e ? e : NSG_SUCCESS;
}

int nsg_server_create(nsg_server **out, int max_rows, int max_cols, size_t budget, int queue_cap, int device) {
    if (!out || queue_cap <= 0) return NSG_ERR_ARG;
    *out = nullptr;
    const size_t per = nsg_pool_context_bytes(max_rows, max_cols);
    if (per == 0) return NSG_ERR_ARG;
    const size_t admit = budget / per;
    if (admit < 1) return NSG_ERR_OOM;  // the budget does not hold one tile's workspace
    const int workers = (int)std::min<size_t>(admit, 64);
    nsg_server *s = new (std::nothrow) nsg_server();
    if (!s) return NSG_ERR_OOM;
    int r = nsg_pool_create(&s->pool, max_rows, max_cols, workers, device);
    if (r != NSG_SUCCESS) {
        delete s;
        return r;
    }
    s->pool->qcap = queue_cap;
    *out = s;
    return NSG_SUCCESS;
}

int nsg_server_create_classes(nsg_server **out, const int *class_rows, const int *class_cols, const double *weights,
                              int nclasses, size_t budget, int queue_cap, int device) {
    if (!out || !class_rows || !class_cols || nclasses <= 0 || nclasses > 16 || queue_cap <= 0) return NSG_ERR_ARG;
    *out = nullptr;
    // workers per class: budget split in proportion to weight x bytes, i.e.
    // c_k = floor(lambda * w_k) with lambda = budget / sum(w_j * bytes_j);
    // the largest class keeps at least one worker so that every tile that fits
    // some class can be served
    std::vector<size_t> bytes(nclasses);
    double wsum = 0.0;
    int largest = 0;
    for (int k = 0; k < nclasses; ++k) {
        bytes[k] = nsg_pool_context_bytes(class_rows[k], class_cols[k]);
        const double wk = weights ? weights[k] : 1.0;
        if (bytes[k] == 0 || !(wk >= 0.0)) return NSG_ERR_ARG;
        wsum += wk * (double)bytes[k];
        if ((int64_t)class_rows[k] * class_cols[k] > (int64_t)class_rows[largest] * class_cols[largest]) largest = k;
    }
    if (bytes[largest] > budget) return NSG_ERR_OOM;  // not even one context of the largest class
    std::vector<int> count(nclasses, 0);
    size_t used = 0;
    int total = 0;
    if (wsum > 0.0) {
        const double lambda = (double)budget / wsum;
        for (int k = 0; k < nclasses; ++k) {
            count[k] = (int)((weights ? weights[k] : 1.0) * lambda);
            used += (size_t)count[k] * bytes[k];
            total += count[k];
        }
    }
    if (count[largest] == 0) {
        // make room for one large worker by dropping small ones, smallest first
        while (used + bytes[largest] > budget) {
            int victim = -1;
            for (int k = 0; k < nclasses; ++k)
                if (count[k] > 0 && (victim < 0 || bytes[k] < bytes[victim])) victim = k;
            if (victim < 0) break;
            --count[victim];
            used -= bytes[victim];
            --total;
        }
        count[largest] = 1;
        ++total;
    }
    // at most 64 workers (64 streams already share the 32 hardware queues)
    while (total > 64) {
        int k = 0;
        for (int j = 1; j < nclasses; ++j)
            if (count[j] > count[k]) k = j;
        --count[k];
        --total;
    }
    std::vector<int> dims;
    for (int k = 0; k < nclasses; ++k)
        for (int i = 0; i < count[k]; ++i) dims.push_back(class_rows[k]), dims.push_back(class_cols[k]);
    nsg_server *srv = new (std::nothrow) nsg_server();
    if (!srv) return NSG_ERR_OOM;
    const int r = pool_create_dims(&srv->pool, dims, device);
    if (r != NSG_SUCCESS) {
        delete srv;
        return r;
    }
    srv->pool->qcap = queue_cap;
    *out = srv;
    return NSG_SUCCESS;
}

int nsg_server_workers(const nsg_server *s) { return s ? nsg_pool_workers(s->pool) : 0; }

int nsg_server_class_workers(const nsg_server *s, int max_rows, int max_cols) {
    if (!s) return NSG_ERR_ARG;
    int n = 0;
    for (const Worker &w : s->pool->w) n += w.max_rows == max_rows && w.max_cols == max_cols;
    return n;
}

int nsg_server_submit(nsg_server *s, const nsg_tile *tile, const nsg_seg_params *prm, long long *ticket) {
    if (!s || !tile || !tile->bgr) return NSG_ERR_ARG;
    nsg_pool *p = s->pool;
    const int64_t need = p->class_for(tile->rows, tile->cols);
    if (need == 0) return tile->rows > 0 && tile->cols > 0 ? NSG_ERR_OOM : NSG_ERR_ARG;  // no class holds it
    Job j;
    j.tile = *tile;
    if (prm) j.prm = *prm;
    else nsg_default_params(&j.prm);
    j.t_submit = Clock::now();
    j.need = need;
    {
        std::lock_guard<std::mutex> lk(p->mu);
        if ((int)p->q.size() >= p->qcap) return NSG_ERR_QUEUE_FULL;
        j.ticket = p->next_ticket++;
        p->q.push_back(j);
    }
    if (ticket) *ticket = j.ticket;
    p->cv_work.notify_all();  // only a worker whose class holds the tile can take it
    return NSG_SUCCESS;
}

int nsg_server_poll(nsg_server *s, nsg_result *out, int max, int wait_ms) {
    if (!s || !out || max <= 0) return NSG_ERR_ARG;
    nsg_pool *p = s->pool;
    std::unique_lock<std::mutex> lk(p->mu);
    if (p->done.empty() && wait_ms > 0)
        p->cv_res.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !p->done.empty(); });
    int k = 0;
    while (k < max && !p->done.empty()) {
        out[k++] = p->done.front();
        p->done.pop_front();
    }
    return k;
}

int nsg_server_destroy(nsg_server *s) {
    if (!s) return NSG_ERR_ARG;
    pool_free(s->pool);
    delete s;
    return NSG_SUCCESS;
}

}  // extern "C"
