/*
 * nsg_oracle.h — CPU restatement of nscale's segmentNuclei path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle that the CUDA path is
 * compared against; it is never linked into, called by, or shipped with the
 * product library (libnsg.so).  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.
 *
 * Every function cites the reference file:line it restates.  Paths are relative
 * to the nscale project root (SBU-BMI/nscale).
 *
 * Parity pins:
 *   - CCL / area threshold / bounding box are pinned against the reference's own
 *     src/segment/ConnComponents.cpp, compiled from source by oracle/Makefile into
 *     oracle/_ref/ (see tests/golden/make_golden.py).
 *   - The OpenCV 2.4.9 calls on the path (erode/dilate, distanceTransform,
 *     floodFill, watershed) cannot be run here (OpenCV is absent); they are
 *     restated from OpenCV's documented/published algorithms.  For those stages
 *     parity is UNPINNED against a real OpenCV build.
 */
#ifndef NSG_ORACLE_H
#define NSG_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field order and defaults as nscale::HistologicalEntities::segmentNuclei
 * (src/segment/HistologicalEntities.h:52-54). */
typedef struct orc_params {
    int blue, green, red;          /* 220 220 220 */
    double T1, T2;                 /* 5.0 4.0 */
    int G1;                        /* 80 */
    int minSize, maxSize;          /* 11 1000 */
    int G2;                        /* 45 */
    int minSizePl;                 /* 30 */
    int minSizeSeg, maxSizeSeg;    /* 21 1000 */
    int fillHolesConnectivity;     /* 4 */
    int reconConnectivity;         /* 8 */
    int watershedConnectivity;     /* 8 */
} orc_params;

/* Optional intermediate outputs (NULL = not wanted).  Stage ids follow the
 * reference's saveIntermediate() ids in HistologicalEntities.cpp. */
typedef struct orc_dump {
    uint8_t *rbc;            /* 2  */
    uint8_t *rc_open;        /* 3  */
    uint8_t *rc_recon;       /* 4  */
    uint8_t *diffIm;         /* 5  */
    uint8_t *bw1;            /* 7  */
    uint8_t *bw1_t;          /* 8  */
    uint8_t *seg_norbc;      /* 11 */
    uint8_t *seg_nohole;     /* 12 */
    uint8_t *seg_open;       /* 13 */
    uint8_t *seg_big;        /* 15 */
    float   *dist;           /* 16 (positive distances) */
    float   *distance2;      /* 18 */
    uint8_t *minima;
    int32_t *minima_labels;
    int32_t *watermask;      /* 20 */
    uint8_t *seg_nonoverlap; /* 21 */
    uint8_t *seg;            /* 23 */
    uint8_t *final_mask;
    double   stage_seconds[24];
    int      bg_count;
    int      compcount_first; /* kept components after bwareaopen #1 */
    int      compcount_seg;   /* kept components after bwareaopen #3 */
} orc_dump;

/* status codes: HistologicalEntities.h:34-40 */
#define ORC_SUCCESS 0
#define ORC_BACKGROUND 1
#define ORC_BACKGROUND_LIKELY 2
#define ORC_NO_CANDIDATES_LEFT 3
#define ORC_CONTINUE 4
#define ORC_INVALID_IMAGE (-1)

void orc_default_params(orc_params *p);

int64_t orc_get_background(const uint8_t *bgr, int rows, int cols, int blue, int green, int red, uint8_t *out);
void orc_get_rbc(const uint8_t *bgr, int rows, int cols, double T1, double T2, uint8_t *rbc);
void orc_get_rbc_f64(const uint8_t *bgr, int rows, int cols, double T1, double T2, uint8_t *rbc);
void orc_invert_u8(const uint8_t *in, int64_t n, uint8_t *out);

void orc_erode_u8(const uint8_t *in, int rows, int cols, const uint8_t *se, int k, uint8_t *out);
void orc_dilate_u8(const uint8_t *in, int rows, int cols, const uint8_t *se, int k, uint8_t *out);
void orc_morph_open_u8(const uint8_t *in, int rows, int cols, const uint8_t *se, int k, uint8_t *out);
const uint8_t *orc_disk19(void);
const uint8_t *orc_cross3(void);

void orc_imreconstruct_u8(const uint8_t *marker, const uint8_t *mask, int rows, int cols, int conn, uint8_t *out);
void orc_imreconstruct_f32(const float *marker, const float *mask, int rows, int cols, int conn, float *out);
void orc_imreconstruct_binary_u8(const uint8_t *marker, const uint8_t *mask, int rows, int cols, int conn, uint8_t *out);
void orc_imfill_holes_u8(const uint8_t *img, int rows, int cols, int conn, uint8_t *out);
void orc_bwselect_u8(const uint8_t *bw, const uint8_t *seeds, int rows, int cols, int conn, uint8_t *out);

void orc_cc_label(const uint8_t *img, int w, int h, int32_t *label, int bgval, int conn);
int orc_cc_area_threshold_labeled(const int32_t *label, int w, int h, int32_t *out, int bgval, int lower, int upper);
void orc_bwlabel2(const uint8_t *img, int rows, int cols, int conn, int32_t *out);
int orc_bwareaopen2(const uint8_t *img, int rows, int cols, int minSize, int maxSize, int conn, uint8_t *out);

void orc_dist_transform(const uint8_t *mask, int rows, int cols, float *out);
void orc_imhmin_f32(const float *img, int rows, int cols, float h, int conn, float *out);
void orc_local_maxima_f32(const float *img, int rows, int cols, int conn, uint8_t *out);
void orc_local_minima_f32(const float *img, int rows, int cols, int conn, uint8_t *out);

void orc_cv_watershed(const uint8_t *bgr, int32_t *markers, int rows, int cols);
void orc_border_fix_i32(const int32_t *in, int rows, int cols, int32_t bg, int32_t *out);
void orc_watershed2(const uint8_t *bgr, const float *img, int rows, int cols, int conn, int32_t *out,
                    int32_t *labels_out);

int orc_bounding_box(const int32_t *labels, int w, int h, int32_t *bbox_out);
int orc_bounding_box_refbug(const int32_t *labels, int w, int h, int bgval, int32_t *bbox_out);

/* Colour deconvolution (PixelOperations.cpp:94-274), not part of segmentNuclei;
 * the per-nucleus features of the serving configuration read its H channel. */
int orc_stain_matrix(const double *M9, const uint8_t *b3, double *Q6);  /* rows of inv(normalised M) picked by b */
void orc_color_lut(float *lut256);
void orc_color_deconv(const uint8_t *bgr, int rows, int cols, const float *Q6, const float *lut256, uint8_t *H,
                      uint8_t *E);
void orc_color_deconv_f64(const uint8_t *bgr, int rows, int cols, const double *Q6, uint8_t *H, uint8_t *E);

/* Colour normalisation (src/normalization/Normalization.cpp): foreground
 * lab statistics, targetParameters (mean, std of the foreground's lab
 * channels) and normalization (Reinhard transfer to meanT / stdT). */
void orc_norm_stats(const uint8_t *bgr, int rows, int cols, double *count, double *sum3, double *sq3);
void orc_target_parameters(const uint8_t *bgr, int rows, int cols, float *mean3, float *std3);
void orc_normalization(const uint8_t *bgr, int rows, int cols, const float *meanT, const float *stdT,
                       uint8_t *out);

/* Per-nucleus features of the serving output (src/features): gradient
 * magnitude image (Operators.cpp:568-640) and, per label in bounding-box
 * order, {area, perimeter, mean H, std H, mean gradient of H} as float. */
void orc_gradient_u8(const uint8_t *in, int rows, int cols, uint8_t *out);
int orc_nucleus_features(const int32_t *labels, const uint8_t *gray, int rows, int cols, float *feat5);

int orc_segment_nuclei(const uint8_t *bgr, int rows, int cols, const orc_params *p,
                       int32_t *labels_out, uint8_t *mask_out, int *compcount, int32_t *bbox_out,
                       orc_dump *dump);

#ifdef __cplusplus
}
#endif
#endif
