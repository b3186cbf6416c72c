// nsg_internal.cuh — shared declarations of libnsg (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <string>

#include "../../include/nsg.h"

namespace nsg {

// Number of kernels this library has launched (process-wide, monotone).
extern std::atomic<long long> g_kernel_launches;
#define NSG_COUNT_LAUNCH() (::nsg::g_kernel_launches.fetch_add(1, std::memory_order_relaxed))

// Device status word bits reported by persistent / spinning kernels.
enum DeviceStatus : int {
    DEV_OK = 0,
    DEV_TIMEOUT = 1,
    DEV_QUEUE_FULL = 2,
};

constexpr int kMaxSE = 31;

// Per-context workspace.  Slots are carved out of one allocation at create
// time; every entry point works inside them.
struct Workspace {
    // op scratch (usable by any single op; ops do not nest except through the
    // explicit internal functions below, which document what they use)
    int32_t *i32[6] = {};  // (rows+2)*(cols+2) int32 each
    float *f32[3] = {};    // (rows+2)*(cols+2) float each
    uint8_t *u8[4] = {};   // (rows+2)*(cols+2) bytes each
    // pipeline intermediates (segmentNuclei only)
    uint8_t *p_u8[10] = {};
    float *p_f32[2] = {};
    int32_t *p_i32[2] = {};
    uint8_t *p_bgr = nullptr;  // dense copy of a strided / host input tile (3 * max_px)
    // small control area
    int *ctrl = nullptr;       // kCtrlInts ints
    int *h_ctrl = nullptr;     // pinned host mirror
    int64_t *ctr64 = nullptr;  // device 64-bit counters
    int64_t *h_ctr64 = nullptr;
    int32_t *scan_tmp = nullptr;  // block sums for scans
    // watershed workspace (carved per call by watershed_dev)
    char *wsb = nullptr;
    size_t wsb_bytes = 0;
};

constexpr int kCtrlInts = 4096;
// ctrl layout
enum Ctrl : int {
    C_STATUS = 0,    // DeviceStatus bits
    C_COUNT0 = 1,    // generic counters
    C_COUNT1 = 2,
    C_COUNT2 = 3,
    C_COUNT3 = 4,
    C_QHEAD = 8,     // work queue head / tail / pending
    C_QTAIL = 9,
    C_QPEND = 10,
    C_FLAG0 = 16,
    C_FLAG1 = 17,
    C_RSTATS = 20,   // grey reconstruction: tile passes, sweeps, pixels changed by whole-image sweeps, lines scanned
    C_WS = 64,       // watershed control block (64 ints)
    C_QSLOTS = 1024, // 3072 ints: generic small arrays
};

// Per-stage CUDA-event timing of segmentNuclei (the GPU analogue of the
// reference's SimpleCSVLogger::logTimeSinceLastLog stage names).  Stages
// 19-21 split the watershed: flood domains + P1, P2 + the BFS, P3 (the
// "watershed" stage keeps the rest of it).
constexpr int kStages = 22;
constexpr int kStageWsP1 = 19, kStageWsBfs = 20, kStageWsP3 = 21;
struct StageTimer {
    bool on = false;
    bool created = false;
    cudaEvent_t ev[kStages + 2];
    int stage[kStages + 2];
    int nrec = 0;
    double acc_ms[kStages] = {};
    long long calls = 0;
};

struct Ctx {
    int device = 0;
    StageTimer timer;
    int max_rows = 0, max_cols = 0;
    int64_t max_px = 0, max_pad = 0;
    void *arena = nullptr;
    size_t arena_bytes = 0;
    Workspace ws;
    int sm_count = 0;
    long long spin_budget = 1ll << 26;
    cudaEvent_t ev_counts = nullptr;  // marks a posted readback of the device counters
    int recon_max_ctas = 0;           // cap on the reconstruction's persistent grid (0: one CTA per SM)
    int bfs_max_cluster = 0;          // largest BFS thread-block cluster tried (0: 16)
    int recon_wl_phases = -1;         // scan-to-queue switchover of the reconstruction (-1: default)
    std::string last_error;
};

}  // namespace nsg

struct nsg_context {
    nsg::Ctx c;
};

namespace nsg {
void stage_mark(Ctx &c, int stage, cudaStream_t s);  // end of `stage` when timing is on
int stain_matrix(const double *M9, const uint8_t *b3, double *Q6);
int color_deconv_dev(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, const float *Q6, uint8_t *H,
                     uint8_t *E, cudaStream_t s);
int gradient_dev(Ctx &c, const uint8_t *in, uint8_t *out, int rows, int cols, cudaStream_t s);
int nucleus_features_dev(Ctx &c, const int32_t *labels, const uint8_t *gray, int rows, int cols, float *out,
                         int capacity, int *count, cudaStream_t s);
// device bytes of a context for images up to max_rows x max_cols
size_t context_bytes_for(int max_rows, int max_cols);
int segment_nuclei_dev(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, const nsg_seg_params &p,
                       int32_t *labels_out, uint8_t *mask_out, int *compcount, int32_t **bbox, cudaStream_t s);
}  // namespace nsg

namespace nsg {

#define NSG_CUDA_TRY(ctx, expr)                                                               \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            (ctx).last_error = std::string(#expr) + ": " + cudaGetErrorString(e_);            \
            return NSG_ERR_CUDA;                                                              \
        }                                                                                     \
    } while (0)

#define NSG_LAUNCH_CHECK(ctx)                                                                 \
    do {                                                                                      \
        cudaError_t e_ = cudaGetLastError();                                                  \
        if (e_ != cudaSuccess) {                                                              \
            (ctx).last_error = std::string("launch: ") + cudaGetErrorString(e_);              \
            return NSG_ERR_CUDA;                                                              \
        }                                                                                     \
    } while (0)

#define NSG_TRY(expr)            \
    do {                         \
        int r_ = (expr);         \
        if (r_ != NSG_SUCCESS) { \
            return r_;           \
        }                        \
    } while (0)

inline int check_dims(Ctx &c, int rows, int cols) {
    if (rows <= 0 || cols <= 0) {
        c.last_error = "rows and cols must be positive";
        return NSG_ERR_ARG;
    }
    if ((int64_t)rows * cols > c.max_px) {
        c.last_error = "image larger than the context";
        return NSG_ERR_OOM;
    }
    if ((int64_t)(rows + 2) * (cols + 2) > c.max_pad) {
        c.last_error = "image larger than the context (padded)";
        return NSG_ERR_OOM;
    }
    return NSG_SUCCESS;
}
inline int check_conn(Ctx &c, int conn) {
    if (conn != 4 && conn != 8) {
        c.last_error = "connectivity must be 4 or 8";
        return NSG_ERR_ARG;
    }
    return NSG_SUCCESS;
}

inline int grid_for(int64_t n, int block, int max_blocks = 1 << 20) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (int)g;
}

// Reads the device status word (synchronises the stream).
int sync_status(Ctx &c, cudaStream_t s);
int reset_status(Ctx &c, cudaStream_t s);

// ---- internal ops (device pointers; scratch slots named in each) ----------
// pixel.cu
int front_rbc(Ctx &c, const uint8_t *bgr, int64_t row_stride, int rows, int cols, double T1, double T2,
              uint8_t *rc, uint8_t *bw1, uint8_t *bw2, uint8_t *r2b, int *d_bw1_count, cudaStream_t s);
int background_count(Ctx &c, const uint8_t *bgr, int64_t row_stride, int rows, int cols, int blue, int green,
                     int red, uint8_t *mask, int64_t *d_count, cudaStream_t s);
int front_fused(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, int blue, int green, int red,
                double T1, double T2, int64_t *d_bg_count, uint8_t *rc, uint8_t *bw1, uint8_t *bw2, uint8_t *r2b,
                int *d_bw1_count, cudaStream_t s);
int diff_threshold(Ctx &c, const uint8_t *rc, const uint8_t *rc_recon, int rows, int cols, int G1, int G2,
                   uint8_t *bw_g1, uint8_t *bw_g2, cudaStream_t s);
int and_not(Ctx &c, uint8_t *inout, const uint8_t *notmask, int64_t n, cudaStream_t s);
int mask_copy_bgr(Ctx &c, const uint8_t *bgr, int64_t row_stride, const uint8_t *mask, int rows, int cols,
                  uint8_t *out, cudaStream_t s);
int invert_u8_dev(Ctx &c, const uint8_t *in, uint8_t *out, int64_t n, cudaStream_t s);
template <typename T>
int invert_dev(Ctx &c, const T *in, T *out, int64_t n, cudaStream_t s);  // uint8_t, int32_t, float
// morph.cu
int morph_u8(Ctx &c, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se_host, int k,
             bool is_max, cudaStream_t s);
// recon.cu (uses i32[5] for the tile queue)
int recon_u8(Ctx &c, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows, int cols, int conn,
             cudaStream_t s);
// preinit: `out` already holds a marker that is <= mask at every pixel
// (min(marker, mask) is then the marker itself and its pass is skipped)
int recon_f32(Ctx &c, const float *marker, const float *mask, float *out, int rows, int cols, int conn,
              cudaStream_t s, bool preinit = false);
// ccl.cu (uses i32[0..1] unless an output array doubles as the parent array)
enum CclMode { CCL_EQUAL = 0, CCL_NONZERO = 1, CCL_NOT255 = 2 };
int ccl_u8(Ctx &c, const uint8_t *img, int32_t *parent, int rows, int cols, int conn, int mode, cudaStream_t s,
           int *zero_at_roots = nullptr, bool flatten = true);
int ccl_f32_masked(Ctx &c, const float *val, const uint8_t *valid, int32_t *parent, int rows, int cols, int conn,
                   cudaStream_t s);
int bwareaopen_dev(Ctx &c, const uint8_t *img, uint8_t *out, int rows, int cols, int min_size, int max_size,
                   int conn, int *d_count, cudaStream_t s);
int bwselect_dev(Ctx &c, const uint8_t *bw, const uint8_t *seeds, uint8_t *out, int rows, int cols, int conn,
                 cudaStream_t s);
int recon_binary_dev(Ctx &c, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows, int cols,
                     int conn, cudaStream_t s);
int fill_holes_dev(Ctx &c, const uint8_t *img, uint8_t *out, int rows, int cols, int conn, cudaStream_t s);
int bwlabel_dev(Ctx &c, const uint8_t *img, int32_t *labels, int rows, int cols, int conn, cudaStream_t s);
int bbox_dev(Ctx &c, const int32_t *labels, int rows, int cols, int32_t *d_bbox, int64_t cap_ints, int *d_count,
             cudaStream_t s);
int exclusive_scan_i32(Ctx &c, const int32_t *in, int32_t *out, int64_t n, int32_t *d_total, cudaStream_t s,
                       const int32_t *d_len = nullptr);
// edt.cu (uses i32[2])
int dist_transform_dev(Ctx &c, const uint8_t *mask, float *dist, int rows, int cols, cudaStream_t s);
// minima.cu (uses f32[0..2], i32[0..1], u8[0])
int imhmin_dev(Ctx &c, const float *img, float *out, int rows, int cols, float h, int conn, cudaStream_t s);
int imhmin_neg_dist_dev(Ctx &c, const float *dist, const uint8_t *seg, float *out, int rows, int cols, float h,
                        int conn, cudaStream_t s);
int local_extrema_dev(Ctx &c, const float *img, uint8_t *out, int rows, int cols, int conn, bool minima,
                      cudaStream_t s);
// watershed.cu (uses i32[2..4], u8[0..2])
// img_negated: `img` holds the negation of watershed2's image (its minima
// are then the maxima of `img`)
int watershed_dev(Ctx &c, const uint8_t *bgr, const float *img, int32_t *out, int rows, int cols, int conn,
                  cudaStream_t s, bool img_negated = false);
// watershed_pws.cu: domain-parallel exact Meyer flooding of a padded marker
// image (markers > 0, unknown 0, negative reset to 0) with packed BGR colours.
// Writes the flooded labels into outp (padded); falls back to the serial
// flood on the device when its exactness conditions do not hold.
size_t pws_workspace_bytes(int64_t npad);
int pws_flood(Ctx &c, const int *mk, const uint32_t *col, int *outp, int H, int W, cudaStream_t s);
int ws_flood_serial_launch(Ctx &c, const int *mk, const uint32_t *col, int *outp, int H, int W, bool conditional,
                           cudaStream_t s);
int watershed_serial_dev(Ctx &c, const uint8_t *bgr, const float *img, int32_t *out, int rows, int cols, int conn,
                         cudaStream_t s);
int watershed_diag(Ctx &c, int *out16, cudaStream_t s);

}  // namespace nsg
