/*
 * nsg.h — C ABI of libnsg.so, the GB300-native (sm_103a) implementation of
 * nscale's nuclei-segmentation hot path.
 *
 * Every entry point replaces one reference interface (cited per function;
 * paths relative to the nscale tree).  All image arguments are DEVICE
 * pointers to dense row-major arrays (row stride == cols elements) unless a
 * function says otherwise; sizes are plain ints; no C++ type crosses the ABI.
 * Work is enqueued on the caller's CUDA stream (`stream` is a cudaStream_t,
 * NULL = legacy default stream).  Functions that return a count to the host
 * synchronise that stream, as the reference returns those counts by value.
 *
 * Status codes: the pipeline returns the reference's own values
 * (HistologicalEntities.h:34-40); library failures are negative NSG_ERR_*.
 * No C++ exception crosses the ABI.
 *
 * Threading: a context (workspace arena) may be used by one host thread at a
 * time; independent contexts are independent.
 */
#ifndef NSG_H
#define NSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status values of nscale::HistologicalEntities (HistologicalEntities.h:34-40) */
#define NSG_SUCCESS 0
#define NSG_BACKGROUND 1
#define NSG_BACKGROUND_LIKELY 2
#define NSG_NO_CANDIDATES_LEFT 3
#define NSG_CONTINUE 4
#define NSG_INVALID_IMAGE (-1)
#define NSG_RUNTIME_FAILED (-2)
/* library errors */
#define NSG_ERR_ARG (-10)        /* bad argument (size, connectivity, NULL pointer) */
#define NSG_ERR_OOM (-11)        /* device allocation failed / image larger than the context */
#define NSG_ERR_TIMEOUT (-12)    /* a device-side wait exceeded its iteration budget */
#define NSG_ERR_QUEUE_FULL (-13) /* a device queue overflowed its capacity */
#define NSG_ERR_CUDA (-14)       /* a CUDA runtime call failed */
#define NSG_ERR_UNSUPPORTED (-15)

typedef struct nsg_context nsg_context;
typedef void *nsg_stream_t; /* cudaStream_t */

/* Parameters of segmentNuclei, same order, meaning and defaults as
 * HistologicalEntities.h:52-54 (the logger is replaced by the per-stage
 * timers, nsg_context_set_timing; there is no intermediate-result handler). */
typedef struct nsg_seg_params {
    int blue, green, red;       /* 220 220 220 */
    double T1, T2;              /* 5.0 4.0 */
    int G1;                     /* 80 */
    int minSize, maxSize;       /* 11 1000 */
    int G2;                     /* 45 */
    int minSizePl;              /* 30 */
    int minSizeSeg, maxSizeSeg; /* 21 1000 */
    int fillHolesConnectivity;  /* 4 */
    int reconConnectivity;      /* 8 */
    int watershedConnectivity;  /* 8 */
} nsg_seg_params;

int nsg_version(void);
void nsg_default_params(nsg_seg_params *p);
const char *nsg_status_string(int status);

/* Workspace arena for images up to max_rows x max_cols on `device`.  All
 * scratch memory the library needs is allocated here, once; no call below
 * allocates device memory. */
int nsg_context_create(nsg_context **ctx, int max_rows, int max_cols, int device);
int nsg_context_destroy(nsg_context *ctx);
const char *nsg_context_last_error(const nsg_context *ctx);
size_t nsg_context_bytes(const nsg_context *ctx);
/* Device-wait budget (iterations) of every bounded device loop: the
 * persistent kernels' queue waits and the union-find's find steps and hooking
 * retries (per union).  A loop that runs out sets the device status word and
 * the call returns NSG_ERR_TIMEOUT; tests set it low to exercise that.  0
 * restores the default (2^26). */
int nsg_context_set_spin_budget(nsg_context *ctx, long long iterations);
/* Launch-shape tuning (no counterpart in the reference, whose kernels have
 * fixed shapes): results do not depend on it.  recon_max_ctas caps the
 * grey reconstruction's persistent grid (0 = one CTA per SM);
 * bfs_max_cluster is the largest thread-block cluster the watershed BFS
 * tries (1-16, 0 = 16); recon_wl_phases is the reconstruction's switchover
 * from scans to its in-tile pixel queue: 0 = row / column phase pairs until
 * a tile is stable, k = 1..8 = k phase pairs, then the pixel worklist
 * (-1 = the library default).  nscale_gb300.autotune measures and picks
 * them. */
typedef struct nsg_tuning {
    int recon_max_ctas;
    int bfs_max_cluster;
    int recon_wl_phases;
} nsg_tuning;
int nsg_context_set_tuning(nsg_context *ctx, const nsg_tuning *t);

/* ---- PixelOperations / HistologicalEntities helpers ---------------------- */
/* HistologicalEntities::getBackground (HistologicalEntities.cpp:93-109):
 * mask = (B > blue) & (G > green) & (R > red); *count = countNonZero. */
int nsg_get_background(nsg_context *ctx, const uint8_t *bgr, int rows, int cols, int blue, int green, int red,
                       uint8_t *mask_out /* nullable */, int64_t *count_out /* host, nullable */,
                       nsg_stream_t stream);
/* HistologicalEntities::getRBC (HistologicalEntities.cpp:33-81), FP32 as the
 * CPU reference computes it. */
int nsg_get_rbc(nsg_context *ctx, const uint8_t *bgr, int rows, int cols, double T1, double T2, uint8_t *rbc_out,
                nsg_stream_t stream);
/* PixelOperations::invert<T> (PixelOperations.cpp:22-43) over n elements:
 * uint8 255 - x; int32 ~x + 1 (two's-complement negation, wrapping at
 * INT_MIN); float32 -x as the reference's scaled copy x * -1 + 0 (+0 stays
 * +0).  In-place (in == out) is allowed. */
int nsg_invert_u8(nsg_context *ctx, const uint8_t *in, uint8_t *out, int64_t n, nsg_stream_t stream);
int nsg_invert_i32(nsg_context *ctx, const int32_t *in, int32_t *out, int64_t n, nsg_stream_t stream);
int nsg_invert_f32(nsg_context *ctx, const float *in, float *out, int64_t n, nsg_stream_t stream);

/* ---- MorphologicOperations ------------------------------------------------ */
/* cv::erode / cv::dilate with a k x k structuring element given in HOST
 * memory (k odd, <= 31); out-of-image samples are neutral (255 for erode, 0
 * for dilate), as morphOpen pads them (MorphologicOperations.cpp:3849-3882). */
int nsg_morph_erode_u8(nsg_context *ctx, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se,
                       int k, nsg_stream_t stream);
int nsg_morph_dilate_u8(nsg_context *ctx, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se,
                        int k, nsg_stream_t stream);
/* nscale::morphOpen<unsigned char> (MorphologicOperations.cpp:3849-3882). */
int nsg_morph_open_u8(nsg_context *ctx, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se, int k,
                      nsg_stream_t stream);

/* nscale::imreconstruct<T>(seeds, image, conn) (MorphologicOperations.cpp:1731-1903). */
int nsg_imreconstruct_u8(nsg_context *ctx, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows,
                         int cols, int conn, nsg_stream_t stream);
int nsg_imreconstruct_f32(nsg_context *ctx, const float *marker, const float *mask, float *out, int rows, int cols,
                          int conn, nsg_stream_t stream);
/* nscale::imreconstructBinary<unsigned char> (MorphologicOperations.cpp:2769-2909). */
int nsg_imreconstruct_binary_u8(nsg_context *ctx, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows,
                                int cols, int conn, nsg_stream_t stream);
/* nscale::imfillHoles<unsigned char>(img, binary=true, conn) (MorphologicOperations.cpp:2940-3006). */
int nsg_imfill_holes_u8(nsg_context *ctx, const uint8_t *img, uint8_t *out, int rows, int cols, int conn,
                        nsg_stream_t stream);
/* No counterpart in the reference.  The same hole filling as
 * nsg_imfill_holes_u8 for callers that cannot allocate device memory and so
 * cannot create an nsg_context (an embedding application that owns the device
 * allocator, or code that must not allocate once it is set up).  It calls no
 * cudaMalloc, cudaFree or allocating library routine; its work planes live in
 * one static device array of NSG_NOALLOC_MAX_PIXELS * 8 bytes (32 MiB) that
 * every GPU loading the library holds until the process exits.
 *  - rows * cols above NSG_NOALLOC_MAX_PIXELS returns NSG_ERR_OOM; bad
 *    pointers, sizes or connectivity return NSG_ERR_ARG.
 *  - The first call on each device looks up the array's device address (with
 *    that device current); make that first call before any stream capture.
 *  - The call enqueues its work on `stream`, then reads its device status
 *    word back into host stack memory and waits for the stream, so `out` is
 *    complete on return.  NSG_ERR_TIMEOUT means the union-find ran out of
 *    its step budget (NSG_SPIN_BUDGET in the environment, read at each call;
 *    default 2^26) and `out` must not be used.
 *  - All calls share the one array, so calls whose work overlaps on the GPU
 *    (other streams, other host threads) race: order them on one stream or
 *    synchronise between them. */
#define NSG_NOALLOC_MAX_PIXELS (4194304) /* e.g. 2048 x 2048 */
int nsg_imfill_holes_u8_noalloc(const uint8_t *img, uint8_t *out, int rows, int cols, int conn,
                                nsg_stream_t stream);
/* nscale::bwselect<unsigned char>(bw, seeds, conn) (MorphologicOperations.cpp:3010-3031). */
int nsg_bwselect_u8(nsg_context *ctx, const uint8_t *bw, const uint8_t *seeds, uint8_t *out, int rows, int cols,
                    int conn, nsg_stream_t stream);
/* nscale::bwlabel2(img, conn, relab) (MorphologicOperations.cpp:3092-3117 over
 * ConnComponents::label, ConnComponents.cpp:52-86): int32 labels, background
 * -1, label = minimum raster index of the component. */
int nsg_bwlabel(nsg_context *ctx, const uint8_t *img, int32_t *labels_out, int rows, int cols, int conn,
                nsg_stream_t stream);
/* nscale::bwareaopen2(img, false, true, min, max, conn, count)
 * (MorphologicOperations.cpp:3281-3314, ConnComponents.cpp:205-239): keeps
 * components with min <= area < max; *count_out (host) = kept components. */
int nsg_bwareaopen(nsg_context *ctx, const uint8_t *img, uint8_t *out, int rows, int cols, int min_size,
                   int max_size, int conn, int *count_out, nsg_stream_t stream);
/* cv::distanceTransform(mask, dist, CV_DIST_L2, CV_DIST_MASK_PRECISE) as
 * called at HistologicalEntities.cpp:359: exact Euclidean distance to the
 * nearest zero pixel, float32. */
int nsg_dist_transform(nsg_context *ctx, const uint8_t *mask, float *dist_out, int rows, int cols,
                       nsg_stream_t stream);
/* nscale::imhmin<float>(img, h, conn) (MorphologicOperations.cpp:3343-3364). */
int nsg_imhmin_f32(nsg_context *ctx, const float *img, float *out, int rows, int cols, float h, int conn,
                   nsg_stream_t stream);
/* nscale::localMaxima<float> / localMinima<float>
 * (MorphologicOperations.cpp:3764-3845): uint8 255 at regional extrema. */
int nsg_local_maxima_f32(nsg_context *ctx, const float *img, uint8_t *out, int rows, int cols, int conn,
                         nsg_stream_t stream);
int nsg_local_minima_f32(nsg_context *ctx, const float *img, uint8_t *out, int rows, int cols, int conn,
                         nsg_stream_t stream);
/* nscale::watershed2(origImage, image, conn) (MorphologicOperations.cpp:3717-3760):
 * minima labelling, OpenCV Meyer flooding with the reference's flooding
 * order, border fix (NeighborOperations.cpp:18-44).  int32 output, -1 on
 * watershed lines. */
int nsg_watershed(nsg_context *ctx, const uint8_t *bgr, const float *img, int32_t *labels_out, int rows, int cols,
                  int conn, nsg_stream_t stream);
/* The same watershed2 with the flood run by the reference's serial queue
 * discipline on one GPU thread (no counterpart of its own in the reference:
 * it is the verified fallback of nsg_watershed, exposed for cross-checks). */
int nsg_watershed_serial(nsg_context *ctx, const uint8_t *bgr, const float *img, int32_t *labels_out, int rows,
                         int cols, int conn, nsg_stream_t stream);
/* Diagnostics of the last nsg_watershed / segmentNuclei flood (16 ints):
 * [0] fallback code (0 = domain-parallel path taken), [1] flood domains,
 * [2] background entries recorded, [6] level of the first background pop,
 * [9] 1 if a background flood event happened, [11] BFS layers; and of the
 * last grey reconstruction: [12] tile passes, [13] in-tile row+column
 * sweeps, [15] tile lines (rows + columns) scanned; [14] CTAs in the BFS
 * cluster. */
int nsg_watershed_diagnostics(nsg_context *ctx, int *out16, nsg_stream_t stream);
/* ConnComponents::boundingBox (ConnComponents.cpp:241-284) on a -1-background
 * label image: writes compcount entries of (label, minx, maxx, miny, maxy) as
 * five consecutive int32 arrays into HOST memory `bbox_out` (capacity
 * 5*capacity ints); labels in increasing order (= first raster appearance). */
int nsg_bounding_box(nsg_context *ctx, const int32_t *labels, int rows, int cols, int32_t *bbox_out, int capacity,
                     int *compcount, nsg_stream_t stream);

/* ---- PixelOperations colour deconvolution (features input) ---------------- */
/* PixelOperations::ComputeInverseStainMatrix (PixelOperations.cpp:94-156):
 * the rows of inv(normalised M) selected by b, as float, row-major 2 x 3
 * (columns R, G, B).  M is 3 x 3 row-major (rows R, G, B; columns stains);
 * NULL M / b = the feature pipeline's stains (nu-features.cpp:691-692).
 * Host only. */
int nsg_stain_matrix(const double *M9, const uint8_t *b3, float *Q6);
/* PixelOperations::ColorDeconv(image, Q, lut, H, E, BGR2RGB = true)
 * (PixelOperations.cpp:170-274) with ComputeLookupTable's optical-density
 * table (:158-168): uint8 hematoxylin H and eosin E (either nullable).  Q6 is
 * host memory (nsg_stain_matrix's output). */
int nsg_color_deconv(nsg_context *ctx, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                     const float *Q6, uint8_t *H, uint8_t *E, nsg_stream_t stream);

/* ---- colour normalisation (before segmentation) --------------------------- */
/* nscale::Normalization::targetParameters (Normalization.cpp:520-577): the
 * mean and std of the lab channels of the pixels its Fisher discriminant
 * calls foreground (HOST float[3] outputs).  Synchronises the stream. */
int nsg_color_target_parameters(nsg_context *ctx, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                                float *mean3, float *std3, nsg_stream_t stream);
/* nscale::Normalization::normalization(originalI, targetMean, targetStd)
 * (Normalization.cpp:487-517): foreground pixels moved in lab space from
 * their own mean / std to the target's (HOST float[3] inputs, e.g. from
 * nsg_color_target_parameters on a target tile), every pixel back to BGR;
 * out_bgr is a DEVICE rows x cols x 3 uint8 buffer (dense).  FP32 as the
 * reference; an output level may differ by one from a CPU evaluation where a
 * value sits on a rounding boundary (log10f / powf last bits).  Synchronises
 * the stream. */
int nsg_color_normalization(nsg_context *ctx, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                            const float *target_mean3, const float *target_std3, uint8_t *out_bgr,
                            nsg_stream_t stream);

/* ---- per-nucleus features (the serving output) ---------------------------- */
/* Operators::gradient (Operators.cpp:568-640): |grad| of a uint8 image,
 * central differences with one-sided ones at the edges, rounded to uint8. */
int nsg_gradient_u8(nsg_context *ctx, const uint8_t *in, uint8_t *out, int rows, int cols, nsg_stream_t stream);
/* For every component of a -1-background label image (bounding-box order =
 * increasing label), NSG_N_FEATURES floats into DEVICE `features`:
 * area (ObjFeatures::area, ObjFeatures.cpp:15-43), perimeter
 * (ObjFeatures::perimeter, :143-270), mean and std of `gray` and mean of its
 * gradient (intensityFeatures / gradientFeatures, :342-418, histogram
 * statistics of Operators.cpp:281-313).  `gray` is normally the H channel of
 * nsg_color_deconv.  *count (host) receives the number of components;
 * NSG_ERR_ARG when it exceeds `capacity`. */
#define NSG_N_FEATURES 5
int nsg_nucleus_features(nsg_context *ctx, const int32_t *labels, const uint8_t *gray, int rows, int cols,
                         float *features, int capacity, int *count, nsg_stream_t stream);

/* ---- HistologicalEntities::segmentNuclei ----------------------------------- */
/* segmentNuclei(img, output, compcount, bbox, params...) (HistologicalEntities.cpp:473-598)
 * and the mask-only overload (HistologicalEntities.cpp:600-664).
 *  bgr:          DEVICE pointer, BGR interleaved uint8, row stride in bytes.
 *  labels_out:   DEVICE int32 rows*cols (nullable): -1 background, label = min raster index.
 *  mask_out:     DEVICE uint8 rows*cols (nullable): the filled final mask (255/0).
 *  compcount:    HOST (nullable): number of components.
 *  bbox:         HOST (nullable): *bbox receives an nsg_alloc'd int32[5*compcount]
 *                (label, minx, maxx, miny, maxy arrays); free with nsg_free.
 * Returns NSG_SUCCESS, NSG_BACKGROUND, NSG_BACKGROUND_LIKELY,
 * NSG_NO_CANDIDATES_LEFT, NSG_INVALID_IMAGE or an NSG_ERR_* code.  On a non-
 * SUCCESS status, labels_out is filled with -1 and mask_out with 0. */
int nsg_segment_nuclei(nsg_context *ctx, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                       const nsg_seg_params *p, int32_t *labels_out, uint8_t *mask_out, int *compcount,
                       int32_t **bbox, nsg_stream_t stream);
/* Same pipeline from HOST memory: copies the tile in, runs, copies labels
 * (and mask) back to HOST buffers (either nullable). */
int nsg_segment_nuclei_host(nsg_context *ctx, const uint8_t *bgr_host, int rows, int cols, const nsg_seg_params *p,
                            int32_t *labels_host, uint8_t *mask_host, int *compcount, int32_t **bbox,
                            nsg_stream_t stream);

/* ---- many tiles: the batched form and the in-process server ---------------- */
/* The reference farms tiles to processes, one segmentNuclei call each
 * (nu-segment.cpp:274-430, one tile per MPI rank at a time).  Here one
 * process keeps several tiles in flight on one GPU: a pool of workers, each a
 * host thread with its own context (workspace arena) and CUDA stream, so that
 * the latency-bound stages of one tile overlap the others. */
typedef struct nsg_tile {
    const uint8_t *bgr;      /* BGR interleaved uint8 (device, or host with NSG_TILE_HOST) */
    int rows, cols;
    size_t row_stride_bytes; /* device tiles only; 0 = 3 * cols (host tiles are dense) */
    int32_t *labels;         /* nullable output (same memory kind as bgr) */
    uint8_t *mask;           /* nullable output (same memory kind as bgr) */
    int want_bbox;           /* 1: fill bbox (nsg_alloc'd, free with nsg_free) */
    int want_features;       /* 1: per-nucleus features of the H channel (nsg_nucleus_features) */
    /* results */
    int status;              /* segmentNuclei status or NSG_ERR_* */
    int compcount;
    int32_t *bbox;
    float *features;         /* compcount x NSG_N_FEATURES, nsg_alloc'd (free with nsg_free), or NULL */
} nsg_tile;
#define NSG_TILE_HOST 1 /* flag: bgr / labels / mask are host pointers */

typedef struct nsg_pool nsg_pool;
/* `workers` tiles in flight (contexts sized for max_rows x max_cols; 32 is
 * the measured best for 4096 x 4096 tiles on GB300).  Each worker has its own
 * CUDA stream: set CUDA_DEVICE_MAX_CONNECTIONS=32 before the process creates
 * its CUDA context, or streams share hardware queues and tiles wait on each
 * other's kernels.  With several workers, each reconstruction runs on
 * 2 x SMs / workers CTAs (nsg_pool_set_tuning overrides). */
int nsg_pool_create(nsg_pool **pool, int max_rows, int max_cols, int workers, int device);
int nsg_pool_destroy(nsg_pool *pool);
int nsg_pool_workers(const nsg_pool *pool);
/* the same tuning on every worker's context (between batches); a pool's
 * default caps each reconstruction at half the SMs */
int nsg_pool_set_tuning(nsg_pool *pool, const nsg_tuning *t);
/* segmentNuclei on every tile of `tiles` (any order, all workers); returns
 * when all are done.  Per-tile statuses land in tiles[i].status; the return
 * value is NSG_SUCCESS or the first NSG_ERR_* a tile produced.  p NULL =
 * defaults (HistologicalEntities.h:52-54). */
int nsg_segment_nuclei_batch(nsg_pool *pool, nsg_tile *tiles, int n, const nsg_seg_params *p, int flags);

/* In-process server (serving form): tiles are submitted one at a time (host
 * memory), processed FIFO by the pool's workers, and collected with poll.
 * The number of workers is what the memory budget admits (one context of
 * nsg_pool_context_bytes each); submit returns NSG_ERR_QUEUE_FULL while
 * `queue_cap` tiles are waiting.  The caller keeps a submitted tile's buffers
 * alive until its result has been polled. */
typedef struct nsg_server nsg_server;
typedef struct nsg_result {
    long long ticket;
    int status, compcount;
    int32_t *bbox;           /* when the tile asked for it: nsg_alloc'd, free with nsg_free */
    float *features;         /* when the tile asked for it: compcount x NSG_N_FEATURES, nsg_alloc'd */
    double latency_ms;       /* submit -> result ready */
} nsg_result;
size_t nsg_pool_context_bytes(int max_rows, int max_cols);
int nsg_server_create(nsg_server **srv, int max_rows, int max_cols, size_t memory_budget_bytes, int queue_cap,
                      int device);
/* The same server with workers in size classes: class k holds tiles up to
 * class_rows[k] x class_cols[k] (one context of nsg_pool_context_bytes each).
 * The budget is split in proportion to weights[k] x bytes[k] (NULL = equal
 * weights), at least one worker of the largest class, at most 64 workers.
 * A submitted tile may run on any worker whose context holds it; a worker
 * takes the oldest waiting tile of its own class first, else the oldest one
 * it can hold.  Submit returns NSG_ERR_OOM for a tile no class holds and
 * NSG_ERR_QUEUE_FULL while queue_cap tiles wait (the caller's shedding
 * point).  No counterpart in the reference, which farms one tile per MPI
 * process (nu-segment.cpp:274-430). */
int nsg_server_create_classes(nsg_server **srv, const int *class_rows, const int *class_cols, const double *weights,
                              int nclasses, size_t memory_budget_bytes, int queue_cap, int device);
int nsg_server_workers(const nsg_server *srv);
/* workers whose context is exactly max_rows x max_cols */
int nsg_server_class_workers(const nsg_server *srv, int max_rows, int max_cols);
/* `tile` is copied (its pointers are not); *ticket identifies the result */
int nsg_server_submit(nsg_server *srv, const nsg_tile *tile, const nsg_seg_params *p, long long *ticket);
/* up to max finished results, waiting up to wait_ms for the first; returns
 * how many were written */
int nsg_server_poll(nsg_server *srv, nsg_result *out, int max, int wait_ms);
int nsg_server_destroy(nsg_server *srv);

/* Per-stage CUDA-event timing of segmentNuclei, in place of the reference's
 * SimpleCSVLogger::logTimeSinceLastLog (UtilsLogger.h:85-183; stage names as
 * HistologicalEntities.cpp logs them).  Enabling resets the accumulators;
 * nsg_context_stage_times copies up to n accumulated milliseconds and returns
 * the number of stages; nsg_stage_name gives stage i's name.  Stages 19-21
 * (watershed_P1, watershed_BFS, watershed_P3) split the watershed's flood;
 * "watershed" keeps the rest of that stage. */
int nsg_context_set_timing(nsg_context *ctx, int on);
int nsg_context_stage_times(nsg_context *ctx, double *ms_out, int n, long long *calls);
/* The same for every worker of a pool (summed over workers; calls = tiles
 * timed).  In the batched form a stage's time includes the waits for SMs
 * that the other tiles in flight hold.  Not while a batch runs. */
int nsg_pool_set_timing(nsg_pool *pool, int on);
int nsg_pool_stage_times(nsg_pool *pool, double *ms_out, int n, long long *calls);
const char *nsg_stage_name(int i);

/* Number of CUDA kernels this library has launched in this process. */
long long nsg_kernel_launches(void);

void *nsg_alloc(size_t bytes);
void nsg_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
