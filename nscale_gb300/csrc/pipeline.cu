// pipeline.cu — nscale::HistologicalEntities::segmentNuclei on the GPU and
// the per-operation C entry points of include/nsg.h.
//
// segmentNuclei follows HistologicalEntities.cpp:473-598 stage by stage
// (plFindNucleusCandidates :115-304, plSeparateNuclei :308-449).  All
// intermediates live in the context's arena; the host only reads back the
// three counts the reference branches on (background ratio, components after
// the first and the last area filter) and the final component count.  The
// background ratio is read right after the front passes, as the reference
// decides it first; the other two are posted and read only where the branch
// is taken, so the stream keeps running meanwhile.
#include <float.h>
#include <limits.h>
#include <string.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int kB = 256;

__global__ void and_u8(uint8_t *__restrict__ io, const uint8_t *__restrict__ m, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        io[i] = io[i] & m[i];
}
__global__ void keep_ge0(const uint8_t *__restrict__ seg_big, const int *__restrict__ wm, uint8_t *__restrict__ out,
                         int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = wm[i] >= 0 ? seg_big[i] : 0;
}
__global__ void fill_i32(int *__restrict__ a, int v, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = v;
}

int blocks(Ctx &c, int64_t n) {
    int64_t g = (n + kB - 1) / kB;
    int64_t cap = (int64_t)c.sm_count * 16;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

// MATLAB strel('disk', 10) as written out at HistologicalEntities.cpp:169-188:
// row r covers columns 9-hw[r] .. 9+hw[r].
void disk19(uint8_t *se) {
    static const int hw[19] = {5, 6, 7, 8, 9, 9, 9, 9, 9, 9, 9, 9, 9, 9, 9, 8, 7, 6, 5};
    for (int r = 0; r < 19; ++r)
        for (int c = 0; c < 19; ++c) se[r * 19 + c] = (c >= 9 - hw[r] && c <= 9 + hw[r]) ? 1 : 0;
}
// getStructuringElement(MORPH_ELLIPSE, Size(3,3)) = 3x3 cross
const uint8_t kCross3[9] = {0, 1, 0, 1, 1, 1, 0, 1, 0};

// The pipeline's three decisions need device counters on the host.  Instead
// of draining the stream at each one, the readback is posted (copy + event)
// and the host keeps enqueuing the next stages, which are harmless on a tile
// that turns out to be background or empty; it waits for the event only
// where a decision must be taken, so the stream rarely runs dry.
int post_counts(Ctx &c, cudaStream_t s) {
    if (!c.ev_counts) NSG_CUDA_TRY(c, cudaEventCreateWithFlags(&c.ev_counts, cudaEventDisableTiming));
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl, c.ws.ctrl, 8 * sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctr64, c.ws.ctr64, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaEventRecord(c.ev_counts, s));
    return NSG_SUCCESS;
}

// wait for the last posted readback and check the device status word
int take_counts(Ctx &c) {
    NSG_CUDA_TRY(c, cudaEventSynchronize(c.ev_counts));
    int st = c.ws.h_ctrl[C_STATUS];
    if (st & DEV_QUEUE_FULL) {
        c.last_error = "device queue overflow";
        return NSG_ERR_QUEUE_FULL;
    }
    if (st & DEV_TIMEOUT) {
        c.last_error = "device wait exceeded its iteration budget";
        return NSG_ERR_TIMEOUT;
    }
    return NSG_SUCCESS;
}

const char *kStageNames[kStages] = {"background", "RBC", "open19", "reconToNuclei", "fillHoles1",
                                   "areaThreshold1", "blobsGt45", "fillHoles2", "openBlobs", "30To1000",
                                   "dilate", "distTransform", "imhmin", "watershed", "20To1000",
                                   "fillHolesLast", "bwlabel2", "bounding_box", "other", "watershed_P1",
                                   "watershed_BFS", "watershed_P3"};

// timer: record the end of `stage` (the segment since the previous mark)
void t_start(Ctx &c, cudaStream_t s) {
    StageTimer &t = c.timer;
    t.nrec = 0;
    if (!t.on) return;
    if (!t.created) {
        for (int i = 0; i < kStages + 2; ++i) cudaEventCreate(&t.ev[i]);
        t.created = true;
    }
    cudaEventRecord(t.ev[0], s);
    t.stage[0] = -1;
    t.nrec = 1;
}
void t_mark(Ctx &c, int stage, cudaStream_t s) {
    StageTimer &t = c.timer;
    if (!t.on || t.nrec == 0 || t.nrec >= kStages + 2) return;
    cudaEventRecord(t.ev[t.nrec], s);
    t.stage[t.nrec] = stage;
    t.nrec++;
}
// after the stream has been synchronised
void t_finish(Ctx &c, cudaStream_t s) {
    StageTimer &t = c.timer;
    if (!t.on || t.nrec < 2) return;
    cudaEventSynchronize(t.ev[t.nrec - 1]);
    for (int i = 1; i < t.nrec; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t.ev[i - 1], t.ev[i]);
        t.acc_ms[t.stage[i]] += ms;
    }
    t.calls++;
    t.nrec = 0;
    (void)s;
}

}  // namespace

void stage_mark(Ctx &c, int stage, cudaStream_t s) { t_mark(c, stage, s); }

int segment_nuclei_dev(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, const nsg_seg_params &p,
                       int32_t *labels_out, uint8_t *mask_out, int *compcount, int32_t **bbox, cudaStream_t s) {
    if (compcount) *compcount = 0;
    if (bbox) *bbox = nullptr;
    if (!bgr) return NSG_INVALID_IMAGE;
    NSG_TRY(check_dims(c, rows, cols));
    if (stride < (int64_t)cols * 3) {
        c.last_error = "row stride smaller than 3*cols";
        return NSG_ERR_ARG;
    }
    NSG_TRY(check_conn(c, p.fillHolesConnectivity));
    NSG_TRY(check_conn(c, p.reconConnectivity));
    NSG_TRY(check_conn(c, p.watershedConnectivity));
    const int64_t n = (int64_t)rows * cols;
    uint8_t **P = c.ws.p_u8;
    int *ctrl = c.ws.ctrl;
    const int g = blocks(c, n);
    auto fail_fill = [&](int status) -> int {
        if (labels_out) {
            fill_i32<<<g, kB, 0, s>>>(labels_out, -1, n);
            NSG_COUNT_LAUNCH();
        }
        if (mask_out) cudaMemsetAsync(mask_out, 0, n, s);
        return status;
    };
    NSG_CUDA_TRY(c, cudaMemsetAsync(ctrl, 0, 8 * sizeof(int), s));
    t_start(c, s);
    struct Fin {
        Ctx &c;
        cudaStream_t s;
        ~Fin() { t_finish(c, s); }
    } fin_timer{c, s};

    // ---- plFindNucleusCandidates --------------------------------------------
    NSG_TRY(front_fused(c, bgr, stride, rows, cols, p.blue, p.green, p.red, p.T1, p.T2, c.ws.ctr64, P[0], P[1], P[2],
                        P[3], ctrl + C_COUNT0, s));
    t_mark(c, 0, s);
    // the background ratio decides before anything expensive runs (HE:123-137):
    // the readback waits only for the two front passes, and a tissue-free tile
    // costs no reconstruction
    NSG_TRY(post_counts(c, s));
    NSG_TRY(take_counts(c));
    {
        float ratio = (float)c.ws.h_ctr64[0] / (float)n;  // HE:125-126
        if (ratio >= 0.99) return fail_fill(NSG_BACKGROUND);
        if (ratio >= 0.9) return fail_fill(NSG_BACKGROUND_LIKELY);
    }
    // rbc = bwselect(bw2, bw1, 8) & imR2B (no seeds -> all zero, HE:73-79)
    NSG_TRY(bwselect_dev(c, P[2], P[1], P[4], rows, cols, 8, s));
    and_u8<<<g, kB, 0, s>>>(P[4], P[3], n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    t_mark(c, 1, s);
    // rc_open = morphOpen(rc, disk19)
    uint8_t se19[361];
    disk19(se19);
    NSG_TRY(morph_u8(c, P[0], P[5], rows, cols, se19, 19, false, s));
    NSG_TRY(morph_u8(c, P[5], P[6], rows, cols, se19, 19, true, s));
    t_mark(c, 2, s);
    // rc_recon = imreconstruct(rc_open, rc, reconConnectivity)
    NSG_TRY(recon_u8(c, P[6], P[0], P[7], rows, cols, p.reconConnectivity, s));
    // diffIm > G1, diffIm > G2
    NSG_TRY(diff_threshold(c, P[0], P[7], rows, cols, p.G1, p.G2, P[5], P[8], s));
    t_mark(c, 3, s);
    // bw1 = imfillHoles(diffIm > G1, fillHolesConnectivity)
    NSG_TRY(fill_holes_dev(c, P[5], P[6], rows, cols, p.fillHolesConnectivity, s));
    t_mark(c, 4, s);
    // bw1_t = bwareaopen2(bw1, minSize, maxSize, 8)
    NSG_TRY(bwareaopen_dev(c, P[6], P[7], rows, cols, p.minSize, p.maxSize, 8, ctrl + C_COUNT1, s));
    t_mark(c, 5, s);
    NSG_TRY(post_counts(c, s));  // candidates left?  decided before the watershed
    // seg_norbc = bwselect(diffIm > G2, bw1_t, 8) & (rbc == 0)
    NSG_TRY(bwselect_dev(c, P[8], P[7], P[5], rows, cols, 8, s));
    NSG_TRY(and_not(c, P[5], P[4], n, s));
    t_mark(c, 6, s);

    // ---- segmentNuclei body -----------------------------------------------------
    NSG_TRY(fill_holes_dev(c, P[5], P[6], rows, cols, 4, s));  // HE:494 (hard-coded 4)
    t_mark(c, 7, s);
    NSG_TRY(morph_u8(c, P[6], P[7], rows, cols, kCross3, 3, false, s));
    NSG_TRY(morph_u8(c, P[7], P[8], rows, cols, kCross3, 3, true, s));  // seg_open
    t_mark(c, 8, s);

    // ---- plSeparateNuclei ---------------------------------------------------------
    NSG_TRY(bwareaopen_dev(c, P[8], P[5], rows, cols, p.minSizePl, INT_MAX, 8, ctrl + C_COUNT2, s));
    t_mark(c, 9, s);
    NSG_TRY(morph_u8(c, P[5], P[6], rows, cols, kCross3, 3, true, s));  // seg_big
    t_mark(c, 10, s);
    NSG_TRY(dist_transform_dev(c, P[6], c.ws.p_f32[0], rows, cols, s));
    t_mark(c, 11, s);
    // distance = -dist inside seg_big, -FLT_MAX outside (HE:366-374); imhmin(distance, 1, 8) (HE:384, hard-coded
    // 8).  imhmin negates, reconstructs and negates back, and watershed2's localMinima negates again: the
    // negations are folded (each is exact), p_f32[1] holds -imhmin(distance), and the watershed below takes its
    // minima as the maxima of that plane.
    NSG_TRY(imhmin_neg_dist_dev(c, c.ws.p_f32[0], P[6], c.ws.p_f32[1], rows, cols, 1.0f, 8, s));
    t_mark(c, 12, s);
    NSG_TRY(take_counts(c));
    if (c.ws.h_ctrl[C_COUNT1] == 0) return fail_fill(NSG_NO_CANDIDATES_LEFT);
    uint8_t *nuclei = (uint8_t *)c.ws.p_i32[0];
    NSG_TRY(mask_copy_bgr(c, bgr, stride, P[6], rows, cols, nuclei, s));
    NSG_TRY(watershed_dev(c, nuclei, c.ws.p_f32[1], c.ws.p_i32[1], rows, cols, p.watershedConnectivity, s, true));
    keep_ge0<<<g, kB, 0, s>>>(P[6], c.ws.p_i32[1], P[7], n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    t_mark(c, 13, s);

    // ---- final area filter, fill, label, boxes ------------------------------------
    NSG_TRY(bwareaopen_dev(c, P[7], P[8], rows, cols, p.minSizeSeg, p.maxSizeSeg, 4, ctrl + C_COUNT3, s));
    t_mark(c, 14, s);
    // the last decision (any nuclei left?) is read together with the box count
    uint8_t *fin = mask_out ? mask_out : P[9];
    NSG_TRY(fill_holes_dev(c, P[8], fin, rows, cols, p.fillHolesConnectivity, s));
    t_mark(c, 15, s);
    int32_t *labels = labels_out ? labels_out : c.ws.p_i32[0];
    NSG_TRY(bwlabel_dev(c, fin, labels, rows, cols, 8, s));
    t_mark(c, 16, s);
    int32_t *d_bbox = c.ws.p_i32[1];
    if (compcount || bbox) {
        NSG_TRY(bbox_dev(c, labels, rows, cols, d_bbox, c.max_pad, ctrl + C_COUNT0, s));
        t_mark(c, 17, s);
    }
    NSG_TRY(post_counts(c, s));
    NSG_TRY(take_counts(c));
    if (c.ws.h_ctrl[C_COUNT3] == 0) return fail_fill(NSG_NO_CANDIDATES_LEFT);
    if (compcount || bbox) {
        int cnt = c.ws.h_ctrl[C_COUNT0];
        if (compcount) *compcount = cnt;
        if (bbox) {
            int32_t *hb = (int32_t *)nsg_alloc(sizeof(int32_t) * 5 * (size_t)(cnt > 0 ? cnt : 1));
            if (!hb) return NSG_ERR_OOM;
            if (cnt > 0) {
                cudaError_t e = cudaMemcpyAsync(hb, d_bbox, sizeof(int32_t) * 5 * (size_t)cnt,
                                                cudaMemcpyDeviceToHost, s);
                if (e == cudaSuccess) e = cudaStreamSynchronize(s);
                if (e != cudaSuccess) {
                    nsg_free(hb);
                    c.last_error = cudaGetErrorString(e);
                    return NSG_ERR_CUDA;
                }
            }
            *bbox = hb;
        }
    }
    return NSG_SUCCESS;
}

}  // namespace nsg

using namespace nsg;

namespace {

inline cudaStream_t S(nsg_stream_t s) { return (cudaStream_t)s; }

// device -> host copy ordered on the caller's stream (never the legacy stream)
cudaError_t copy_to_host(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
    return e == cudaSuccess ? cudaStreamSynchronize(s) : e;
}

// Every per-operation entry point resets the device status word, enqueues
// its kernels and synchronises the stream, returning the device status: the
// reference's calls return finished results, and spinning kernels report
// their bounded waits through that word.
template <typename F>
int run_op(nsg_context *h, nsg_stream_t s, F &&f) {
    if (!h) return NSG_ERR_ARG;
    Ctx &c = h->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return NSG_ERR_CUDA;
    NSG_TRY(reset_status(c, S(s)));
    NSG_TRY(f(c));
    return sync_status(c, S(s));
}

}  // namespace

extern "C" {

int nsg_get_background(nsg_context *h, const uint8_t *bgr, int rows, int cols, int blue, int green, int red,
                       uint8_t *mask_out, int64_t *count_out, nsg_stream_t s) {
    int r = run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!bgr) return NSG_ERR_ARG;
        return background_count(c, bgr, (int64_t)cols * 3, rows, cols, blue, green, red, mask_out, c.ws.ctr64, S(s));
    });
    if (r == NSG_SUCCESS && count_out) {
        if (copy_to_host(count_out, h->c.ws.ctr64, sizeof(int64_t), S(s)) != cudaSuccess) return NSG_ERR_CUDA;
    }
    return r;
}

int nsg_get_rbc(nsg_context *h, const uint8_t *bgr, int rows, int cols, double T1, double T2, uint8_t *rbc_out,
                nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!bgr || !rbc_out) return NSG_ERR_ARG;
        uint8_t *rc = c.ws.u8[0], *bw1 = c.ws.u8[1], *bw2 = c.ws.u8[2], *r2b = c.ws.u8[3];
        NSG_TRY(front_rbc(c, bgr, (int64_t)cols * 3, rows, cols, T1, T2, rc, bw1, bw2, r2b, c.ws.ctrl + C_COUNT0,
                          S(s)));
        NSG_TRY(bwselect_dev(c, bw2, bw1, rbc_out, rows, cols, 8, S(s)));
        int64_t n = (int64_t)rows * cols;
        and_u8<<<blocks(c, n), kB, 0, S(s)>>>(rbc_out, r2b, n);
        NSG_COUNT_LAUNCH();
        NSG_LAUNCH_CHECK(c);
        return NSG_SUCCESS;
    });
}

int nsg_invert_u8(nsg_context *h, const uint8_t *in, uint8_t *out, int64_t n, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        if (!in || !out || n < 0) return NSG_ERR_ARG;
        return invert_dev<uint8_t>(c, in, out, n, S(s));
    });
}

int nsg_invert_i32(nsg_context *h, const int32_t *in, int32_t *out, int64_t n, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        if (!in || !out || n < 0) return NSG_ERR_ARG;
        return invert_dev<int32_t>(c, in, out, n, S(s));
    });
}

int nsg_invert_f32(nsg_context *h, const float *in, float *out, int64_t n, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        if (!in || !out || n < 0) return NSG_ERR_ARG;
        return invert_dev<float>(c, in, out, n, S(s));
    });
}

int nsg_morph_erode_u8(nsg_context *h, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se, int k,
                       nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!in || !out) return NSG_ERR_ARG;
        return morph_u8(c, in, out, rows, cols, se, k, false, S(s));
    });
}

int nsg_morph_dilate_u8(nsg_context *h, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se, int k,
                        nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!in || !out) return NSG_ERR_ARG;
        return morph_u8(c, in, out, rows, cols, se, k, true, S(s));
    });
}

int nsg_morph_open_u8(nsg_context *h, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se, int k,
                      nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!in || !out) return NSG_ERR_ARG;
        NSG_TRY(morph_u8(c, in, c.ws.u8[0], rows, cols, se, k, false, S(s)));
        return morph_u8(c, c.ws.u8[0], out, rows, cols, se, k, true, S(s));
    });
}

int nsg_imreconstruct_u8(nsg_context *h, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows, int cols,
                         int conn, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        if (!marker || !mask || !out) return NSG_ERR_ARG;
        return recon_u8(c, marker, mask, out, rows, cols, conn, S(s));
    });
}

int nsg_imreconstruct_f32(nsg_context *h, const float *marker, const float *mask, float *out, int rows, int cols,
                          int conn, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        if (!marker || !mask || !out) return NSG_ERR_ARG;
        return recon_f32(c, marker, mask, out, rows, cols, conn, S(s));
    });
}

int nsg_imreconstruct_binary_u8(nsg_context *h, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows,
                                int cols, int conn, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!marker || !mask || !out) return NSG_ERR_ARG;
        return recon_binary_dev(c, marker, mask, out, rows, cols, conn, S(s));
    });
}

int nsg_imfill_holes_u8(nsg_context *h, const uint8_t *img, uint8_t *out, int rows, int cols, int conn,
                        nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!img || !out) return NSG_ERR_ARG;
        return fill_holes_dev(c, img, out, rows, cols, conn, S(s));
    });
}

int nsg_bwselect_u8(nsg_context *h, const uint8_t *bw, const uint8_t *seeds, uint8_t *out, int rows, int cols,
                    int conn, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!bw || !seeds || !out) return NSG_ERR_ARG;
        return bwselect_dev(c, bw, seeds, out, rows, cols, conn, S(s));
    });
}

int nsg_bwlabel(nsg_context *h, const uint8_t *img, int32_t *labels_out, int rows, int cols, int conn,
                nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!img || !labels_out) return NSG_ERR_ARG;
        return bwlabel_dev(c, img, labels_out, rows, cols, conn, S(s));
    });
}

int nsg_bwareaopen(nsg_context *h, const uint8_t *img, uint8_t *out, int rows, int cols, int min_size, int max_size,
                   int conn, int *count_out, nsg_stream_t s) {
    int r = run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!img || !out) return NSG_ERR_ARG;
        return bwareaopen_dev(c, img, out, rows, cols, min_size, max_size, conn, c.ws.ctrl + C_COUNT1, S(s));
    });
    if (r == NSG_SUCCESS && count_out) {
        if (copy_to_host(count_out, h->c.ws.ctrl + C_COUNT1, sizeof(int), S(s)) != cudaSuccess) return NSG_ERR_CUDA;
    }
    return r;
}

int nsg_dist_transform(nsg_context *h, const uint8_t *mask, float *dist_out, int rows, int cols, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!mask || !dist_out) return NSG_ERR_ARG;
        return dist_transform_dev(c, mask, dist_out, rows, cols, S(s));
    });
}

int nsg_imhmin_f32(nsg_context *h, const float *img, float *out, int rows, int cols, float hval, int conn,
                   nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!img || !out) return NSG_ERR_ARG;
        return imhmin_dev(c, img, out, rows, cols, hval, conn, S(s));
    });
}

int nsg_local_maxima_f32(nsg_context *h, const float *img, uint8_t *out, int rows, int cols, int conn,
                         nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!img || !out) return NSG_ERR_ARG;
        return local_extrema_dev(c, img, out, rows, cols, conn, false, S(s));
    });
}

int nsg_local_minima_f32(nsg_context *h, const float *img, uint8_t *out, int rows, int cols, int conn,
                         nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!img || !out) return NSG_ERR_ARG;
        return local_extrema_dev(c, img, out, rows, cols, conn, true, S(s));
    });
}

int nsg_watershed(nsg_context *h, const uint8_t *bgr, const float *img, int32_t *labels_out, int rows, int cols,
                  int conn, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!bgr || !img || !labels_out) return NSG_ERR_ARG;
        return watershed_dev(c, bgr, img, labels_out, rows, cols, conn, S(s));
    });
}

int nsg_watershed_serial(nsg_context *h, const uint8_t *bgr, const float *img, int32_t *labels_out, int rows,
                         int cols, int conn, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        NSG_TRY(check_conn(c, conn));
        if (!bgr || !img || !labels_out) return NSG_ERR_ARG;
        return watershed_serial_dev(c, bgr, img, labels_out, rows, cols, conn, S(s));
    });
}

int nsg_watershed_diagnostics(nsg_context *h, int *out16, nsg_stream_t s) {
    if (!h || !out16) return NSG_ERR_ARG;
    return watershed_diag(h->c, out16, S(s));
}

int nsg_stain_matrix(const double *M9, const uint8_t *b3, float *Q6) {
    if (!Q6) return NSG_ERR_ARG;
    static const double kM[9] = {0.650, 0.072, 0, 0.704, 0.990, 0, 0.286, 0.105, 0};  // nu-features.cpp:691-692
    static const uint8_t kB[3] = {1, 1, 0};
    double q[6];
    if (stain_matrix(M9 ? M9 : kM, b3 ? b3 : kB, q) != 2) return NSG_ERR_ARG;
    for (int i = 0; i < 6; ++i) Q6[i] = (float)q[i];
    return NSG_SUCCESS;
}

int nsg_color_deconv(nsg_context *h, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                     const float *Q6, uint8_t *H, uint8_t *E, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        const int64_t stride = row_stride_bytes ? (int64_t)row_stride_bytes : (int64_t)cols * 3;
        if (!bgr || !Q6 || stride < (int64_t)cols * 3) return NSG_ERR_ARG;
        return color_deconv_dev(c, bgr, stride, rows, cols, Q6, H, E, S(s));
    });
}

int nsg_gradient_u8(nsg_context *h, const uint8_t *in, uint8_t *out, int rows, int cols, nsg_stream_t s) {
    return run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!in || !out) return NSG_ERR_ARG;
        return gradient_dev(c, in, out, rows, cols, S(s));
    });
}

int nsg_nucleus_features(nsg_context *h, const int32_t *labels, const uint8_t *gray, int rows, int cols,
                         float *features, int capacity, int *count, nsg_stream_t s) {
    int cnt = 0;
    int r = run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!labels || !gray || (!features && capacity > 0) || capacity < 0) return NSG_ERR_ARG;
        return nucleus_features_dev(c, labels, gray, rows, cols, features, capacity, &cnt, S(s));
    });
    if (count) *count = cnt;
    return r;
}

int nsg_bounding_box(nsg_context *h, const int32_t *labels, int rows, int cols, int32_t *bbox_out, int capacity,
                     int *compcount, nsg_stream_t s) {
    int r = run_op(h, s, [&](Ctx &c) {
        NSG_TRY(check_dims(c, rows, cols));
        if (!labels) return NSG_ERR_ARG;
        return bbox_dev(c, labels, rows, cols, c.ws.p_i32[1], c.max_pad, c.ws.ctrl + C_COUNT0, S(s));
    });
    if (r != NSG_SUCCESS) return r;
    Ctx &c = h->c;
    int cnt = 0;
    if (copy_to_host(&cnt, c.ws.ctrl + C_COUNT0, sizeof(int), S(s)) != cudaSuccess) return NSG_ERR_CUDA;
    if (compcount) *compcount = cnt;
    if (bbox_out) {
        if (cnt > capacity) {
            c.last_error = "bbox capacity too small";
            return NSG_ERR_ARG;
        }
        if (cnt > 0 && copy_to_host(bbox_out, c.ws.p_i32[1], sizeof(int32_t) * 5 * (size_t)cnt, S(s)) != cudaSuccess)
            return NSG_ERR_CUDA;
    }
    return NSG_SUCCESS;
}

int nsg_context_set_timing(nsg_context *h, int on) {
    if (!h) return NSG_ERR_ARG;
    h->c.timer.on = on != 0;
    for (int i = 0; i < kStages; ++i) h->c.timer.acc_ms[i] = 0.0;
    h->c.timer.calls = 0;
    return NSG_SUCCESS;
}

int nsg_context_stage_times(nsg_context *h, double *ms_out, int n, long long *calls) {
    if (!h || !ms_out) return NSG_ERR_ARG;
    int m = n < kStages ? n : kStages;
    for (int i = 0; i < m; ++i) ms_out[i] = h->c.timer.acc_ms[i];
    if (calls) *calls = h->c.timer.calls;
    return kStages;
}

const char *nsg_stage_name(int i) { return (i >= 0 && i < kStages) ? kStageNames[i] : ""; }

int nsg_segment_nuclei(nsg_context *h, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                       const nsg_seg_params *p, int32_t *labels_out, uint8_t *mask_out, int *compcount,
                       int32_t **bbox, nsg_stream_t s) {
    if (!h) return NSG_ERR_ARG;
    Ctx &c = h->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return NSG_ERR_CUDA;
    nsg_seg_params prm;
    if (p) prm = *p;
    else nsg_default_params(&prm);
    int64_t stride = row_stride_bytes ? (int64_t)row_stride_bytes : (int64_t)cols * 3;
    int r = segment_nuclei_dev(c, bgr, stride, rows, cols, prm, labels_out, mask_out, compcount, bbox, S(s));
    if (r >= 0 && r != NSG_SUCCESS) {
        // early-exit statuses: the fills were enqueued; make them visible
        if (cudaStreamSynchronize(S(s)) != cudaSuccess) return NSG_ERR_CUDA;
    }
    return r;
}

int nsg_segment_nuclei_host(nsg_context *h, const uint8_t *bgr_host, int rows, int cols, const nsg_seg_params *p,
                            int32_t *labels_host, uint8_t *mask_host, int *compcount, int32_t **bbox,
                            nsg_stream_t s) {
    if (!h) return NSG_ERR_ARG;
    Ctx &c = h->c;
    if (!bgr_host) return NSG_INVALID_IMAGE;
    NSG_TRY(check_dims(c, rows, cols));
    if (cudaSetDevice(c.device) != cudaSuccess) return NSG_ERR_CUDA;
    const int64_t n = (int64_t)rows * cols;
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.p_bgr, bgr_host, (size_t)n * 3, cudaMemcpyHostToDevice, S(s)));
    nsg_seg_params prm;
    if (p) prm = *p;
    else nsg_default_params(&prm);
    // device outputs: labels in i32 scratch that the pipeline does not use at
    // the end, mask in the last pipeline byte slot
    int32_t *dl = labels_host ? (int32_t *)c.ws.i32[5] : nullptr;
    uint8_t *dm = mask_host ? c.ws.p_u8[9] : nullptr;
    int r = segment_nuclei_dev(c, c.ws.p_bgr, (int64_t)cols * 3, rows, cols, prm, dl, dm, compcount, bbox, S(s));
    if (r < 0) return r;
    if (labels_host) NSG_CUDA_TRY(c, cudaMemcpyAsync(labels_host, dl, (size_t)n * 4, cudaMemcpyDeviceToHost, S(s)));
    if (mask_host) NSG_CUDA_TRY(c, cudaMemcpyAsync(mask_host, dm, (size_t)n, cudaMemcpyDeviceToHost, S(s)));
    NSG_CUDA_TRY(c, cudaStreamSynchronize(S(s)));
    return r;
}

}  // extern "C"
