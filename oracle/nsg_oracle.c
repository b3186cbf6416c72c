/*
 * nsg_oracle.c — CPU restatement of nscale's segmentNuclei hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Never linked into the product.
 * Single-threaded, plain C11, written to follow the reference's sequential
 * algorithms step by step so that it can serve as the parity oracle.
 *
 * Citations: HE = src/segment/HistologicalEntities.cpp,
 *            MO = src/segment/MorphologicOperations.cpp,
 *            CC = src/segment/ConnComponents.cpp,
 *            PO = src/segment/PixelOperations.cpp,
 *            NO = src/segment/NeighborOperations.cpp.
 * OpenCV 2.4.9 calls (not in the nscale tree) are restated from OpenCV's
 * published algorithms and marked "OpenCV" below.
 */
#include "nsg_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define WSHED (-1)
#define IN_QUEUE (-2)

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) abort();
    return p;
}
static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) abort();
    return p;
}

/* std::max / std::min exactly as libstdc++ writes them (matters only for the
 * sign of floating-point zeros). */
#define SMAX(a, b) (((a) < (b)) ? (b) : (a))
#define SMIN(a, b) (((b) < (a)) ? (b) : (a))

/* ---------------------------------------------------------------- FIFO --- */
typedef struct {
    int32_t *buf;
    size_t cap, head, n;
} ififo;

static void ff_init(ififo *q, size_t cap) {
    q->cap = cap < 1024 ? 1024 : cap;
    q->buf = (int32_t *)xmalloc(q->cap * sizeof(int32_t));
    q->head = q->n = 0;
}
static void ff_free(ififo *q) { free(q->buf); }
static void ff_push(ififo *q, int32_t v) {
    if (q->n == q->cap) {
        size_t ncap = q->cap * 2;
        int32_t *nb = (int32_t *)xmalloc(ncap * sizeof(int32_t));
        for (size_t i = 0; i < q->n; ++i) nb[i] = q->buf[(q->head + i) % q->cap];
        free(q->buf);
        q->buf = nb;
        q->cap = ncap;
        q->head = 0;
    }
    q->buf[(q->head + q->n) % q->cap] = v;
    q->n++;
}
static int32_t ff_pop(ififo *q) {
    int32_t v = q->buf[q->head];
    q->head = (q->head + 1) % q->cap;
    q->n--;
    return v;
}

/* ------------------------------------------------------------- params --- */
void orc_default_params(orc_params *p) {
    /* HistologicalEntities.h:53 */
    p->blue = p->green = p->red = 220;
    p->T1 = 5.0;
    p->T2 = 4.0;
    p->G1 = 80;
    p->minSize = 11;
    p->maxSize = 1000;
    p->G2 = 45;
    p->minSizePl = 30;
    p->minSizeSeg = 21;
    p->maxSizeSeg = 1000;
    p->fillHolesConnectivity = 4;
    p->reconConnectivity = 8;
    p->watershedConnectivity = 8;
}

/* ---------------------------------------------------------- pixel ops --- */
/* HE:93-109: (B > blue) & (G > green) & (R > red), strict. */
int64_t orc_get_background(const uint8_t *bgr, int rows, int cols, int blue, int green, int red, uint8_t *out) {
    int64_t n = (int64_t)rows * cols, cnt = 0;
    for (int64_t i = 0; i < n; ++i) {
        const uint8_t *p = bgr + 3 * i;
        uint8_t v = (p[0] > blue && p[1] > green && p[2] > red) ? 255 : 0;
        if (out) out[i] = v;
        cnt += v != 0;
    }
    return cnt;
}

/* HE:33-81.  bd = B + FLT_EPSILON, gd = G + FLT_EPSILON, rd = R (float32,
 * convertTo with float scale/shift); imR2G = rd/gd; imR2B = (rd/bd) > 1;
 * bw1 = imR2G > T1; bw2 = imR2G > T2 (the double thresholds are converted to
 * float as OpenCV's compare() does for a CV_32F array);
 * rbc = any(bw1) ? bwselect(bw2, bw1, 8) & imR2B : 0. */
void orc_get_rbc(const uint8_t *bgr, int rows, int cols, double T1, double T2, uint8_t *rbc) {
    int64_t n = (int64_t)rows * cols;
    uint8_t *bw1 = (uint8_t *)xmalloc(n), *bw2 = (uint8_t *)xmalloc(n), *r2b = (uint8_t *)xmalloc(n);
    const float t1 = (float)T1, t2 = (float)T2;
    int64_t any = 0;
    for (int64_t i = 0; i < n; ++i) {
        volatile float bd = (float)bgr[3 * i + 0] + FLT_EPSILON;
        volatile float gd = (float)bgr[3 * i + 1] + FLT_EPSILON;
        float rd = (float)bgr[3 * i + 2];
        volatile float r2g = rd / gd;
        volatile float rb = rd / bd;
        bw1[i] = r2g > t1 ? 255 : 0;
        bw2[i] = r2g > t2 ? 255 : 0;
        r2b[i] = rb > 1.0f ? 255 : 0;
        any += bw1[i] != 0;
    }
    if (any > 0) {
        orc_bwselect_u8(bw2, bw1, rows, cols, 8, rbc);
        for (int64_t i = 0; i < n; ++i) rbc[i] &= r2b[i];
    } else {
        memset(rbc, 0, (size_t)n);
    }
    free(bw1);
    free(bw2);
    free(r2b);
}

/* FP64 variant (the GPU reference's choice, HistologicalEntitiesGPU.cpp:100-110):
 * used only to count threshold flips against the FP32 path. */
void orc_get_rbc_f64(const uint8_t *bgr, int rows, int cols, double T1, double T2, uint8_t *rbc) {
    int64_t n = (int64_t)rows * cols;
    uint8_t *bw1 = (uint8_t *)xmalloc(n), *bw2 = (uint8_t *)xmalloc(n), *r2b = (uint8_t *)xmalloc(n);
    int64_t any = 0;
    for (int64_t i = 0; i < n; ++i) {
        double bd = (double)bgr[3 * i + 0] + DBL_EPSILON;
        double gd = (double)bgr[3 * i + 1] + DBL_EPSILON;
        double rd = (double)bgr[3 * i + 2];
        double r2g = rd / gd;
        bw1[i] = r2g > T1 ? 255 : 0;
        bw2[i] = r2g > T2 ? 255 : 0;
        r2b[i] = (rd / bd) > 1.0 ? 255 : 0;
        any += bw1[i] != 0;
    }
    if (any > 0) {
        orc_bwselect_u8(bw2, bw1, rows, cols, 8, rbc);
        for (int64_t i = 0; i < n; ++i) rbc[i] &= r2b[i];
    } else {
        memset(rbc, 0, (size_t)n);
    }
    free(bw1);
    free(bw2);
    free(r2b);
}

/* PO:22-43, unsigned branch: 255 - x. */
void orc_invert_u8(const uint8_t *in, int64_t n, uint8_t *out) {
    for (int64_t i = 0; i < n; ++i) out[i] = (uint8_t)(255 - in[i]);
}

/* ---------------------------------------------------- erode / dilate --- */
/* 19x19 MATLAB disk, HE:169-188 (the structuring-element table must be the
 * same to give the same opening; it is a fixed mask, restated by its chord
 * half-widths: rows 0..18 cover |dx| <= hw[row]). */
static const int disk19_hw[19] = {5, 6, 7, 8, 9, 9, 9, 9, 9, 9, 9, 9, 9, 9, 9, 8, 7, 6, 5};
static uint8_t disk19_tab[361];
static const uint8_t cross3_tab[9] = {0, 1, 0, 1, 1, 1, 0, 1, 0};

const uint8_t *orc_disk19(void) {
    for (int r = 0; r < 19; ++r)
        for (int c = 0; c < 19; ++c) disk19_tab[r * 19 + c] = (abs(c - 9) <= disk19_hw[r]) ? 1 : 0;
    return disk19_tab;
}
/* getStructuringElement(MORPH_ELLIPSE, Size(3,3)) is the 3x3 cross (HE:498). */
const uint8_t *orc_cross3(void) { return cross3_tab; }

/* OpenCV cv::erode / cv::dilate: dst(y,x) = min/max over the kernel support of
 * src(y+dy, x+dx), anchor at the centre.  Out-of-image samples are neutral
 * (the reference pads erode input with 255 and dilate input with 0,
 * MO:3861/3869; HE:330 uses the default border, which is also neutral). */
static void morph_u8(const uint8_t *in, int rows, int cols, const uint8_t *se, int k, uint8_t *out, int is_max) {
    int r = k / 2;
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x) {
            int v = is_max ? 0 : 255;
            for (int dy = -r; dy <= r; ++dy) {
                int yy = y + dy;
                if (yy < 0 || yy >= rows) continue;
                for (int dx = -r; dx <= r; ++dx) {
                    if (!se[(dy + r) * k + (dx + r)]) continue;
                    int xx = x + dx;
                    if (xx < 0 || xx >= cols) continue;
                    int s = in[(int64_t)yy * cols + xx];
                    if (is_max) {
                        if (s > v) v = s;
                    } else {
                        if (s < v) v = s;
                    }
                }
            }
            out[(int64_t)y * cols + x] = (uint8_t)v;
        }
}
void orc_erode_u8(const uint8_t *in, int rows, int cols, const uint8_t *se, int k, uint8_t *out) {
    morph_u8(in, rows, cols, se, k, out, 0);
}
void orc_dilate_u8(const uint8_t *in, int rows, int cols, const uint8_t *se, int k, uint8_t *out) {
    morph_u8(in, rows, cols, se, k, out, 1);
}
/* MO:3849-3882: erode with outside = 255, crop, dilate with outside = 0. */
void orc_morph_open_u8(const uint8_t *in, int rows, int cols, const uint8_t *se, int k, uint8_t *out) {
    uint8_t *tmp = (uint8_t *)xmalloc((size_t)rows * cols);
    morph_u8(in, rows, cols, se, k, tmp, 0);
    morph_u8(tmp, rows, cols, se, k, out, 1);
    free(tmp);
}

/* ------------------------------------------- grey reconstruction (MO) --- */
/* MO:1731-1903 (Vincent's hybrid algorithm): pad marker and mask with one
 * pixel of 0, raster scan, anti-raster scan with seed capture, FIFO
 * propagation (MO:431-441).  Instantiated for uint8 and float. */
#define DEFINE_RECON(NAME, T)                                                                            \
    void NAME(const T *marker, const T *mask, int rows, int cols, int conn, T *out) {                   \
        int W = cols + 2, H = rows + 2;                                                                 \
        T *o = (T *)xcalloc((size_t)W * H, sizeof(T));                                                  \
        T *in = (T *)xcalloc((size_t)W * H, sizeof(T));                                                 \
        for (int y = 0; y < rows; ++y) {                                                                \
            memcpy(o + (int64_t)(y + 1) * W + 1, marker + (int64_t)y * cols, sizeof(T) * cols);         \
            memcpy(in + (int64_t)(y + 1) * W + 1, mask + (int64_t)y * cols, sizeof(T) * cols);          \
        }                                                                                               \
        int maxx = W - 1, maxy = H - 1;                                                                 \
        T pval, preval;                                                                                 \
        for (int y = 1; y < maxy; ++y) {                                                                \
            T *oP = o + (int64_t)y * W, *oM = o + (int64_t)(y - 1) * W, *iP = in + (int64_t)y * W;        \
            preval = oP[0];                                                                             \
            for (int x = 1; x < maxx; ++x) {                                                            \
                pval = oP[x];                                                                           \
                pval = SMAX(pval, SMAX(preval, oM[x]));                                                 \
                if (conn == 8) pval = SMAX(pval, SMAX(oM[x + 1], oM[x - 1]));                           \
                preval = SMIN(pval, iP[x]);                                                             \
                oP[x] = preval;                                                                         \
            }                                                                                           \
        }                                                                                               \
        ififo q;                                                                                        \
        ff_init(&q, (size_t)W * 4);                                                                     \
        for (int y = maxy - 1; y > 0; --y) {                                                            \
            T *oP = o + (int64_t)y * W, *oPl = o + (int64_t)(y + 1) * W;                                 \
            T *iP = in + (int64_t)y * W, *iPl = in + (int64_t)(y + 1) * W;                               \
            preval = oP[maxx];                                                                          \
            for (int x = maxx - 1; x > 0; --x) {                                                        \
                pval = oP[x];                                                                           \
                pval = SMAX(pval, SMAX(preval, oPl[x]));                                                \
                if (conn == 8) pval = SMAX(pval, SMAX(oPl[x + 1], oPl[x - 1]));                         \
                preval = SMIN(pval, iP[x]);                                                             \
                oP[x] = preval;                                                                         \
                pval = oP[x];                                                                           \
                if ((oP[x + 1] < SMIN(pval, iP[x + 1])) || (oPl[x] < SMIN(pval, iPl[x]))) {             \
                    ff_push(&q, y * W + x);                                                             \
                    continue;                                                                           \
                }                                                                                       \
                if (conn == 8) {                                                                        \
                    if ((oPl[x + 1] < SMIN(pval, iPl[x + 1])) || (oPl[x - 1] < SMIN(pval, iPl[x - 1]))) { \
                        ff_push(&q, y * W + x);                                                         \
                        continue;                                                                       \
                    }                                                                                   \
                }                                                                                       \
            }                                                                                           \
        }                                                                                               \
        static const int dx8[8] = {0, 0, -1, 1, -1, 1, -1, 1};                                          \
        static const int dy8[8] = {-1, 1, 0, 0, -1, -1, 1, 1};                                          \
        while (q.n) {                                                                                   \
            int32_t p = ff_pop(&q);                                                                     \
            int x = p % W, y = p / W;                                                                   \
            pval = o[p];                                                                                \
            int nn = conn == 8 ? 8 : 4;                                                                 \
            for (int k = 0; k < nn; ++k) {                                                              \
                int xx = x + dx8[k], yy = y + dy8[k];                                                   \
                if (xx < 0 || xx > maxx || yy < 0 || yy > maxy) continue;                               \
                int64_t qi = (int64_t)yy * W + xx;                                                      \
                T qval = o[qi], ival = in[qi];                                                          \
                if ((qval < pval) && (ival != qval)) {                                                  \
                    o[qi] = SMIN(pval, ival);                                                           \
                    ff_push(&q, (int32_t)qi);                                                           \
                }                                                                                       \
            }                                                                                           \
        }                                                                                               \
        ff_free(&q);                                                                                    \
        for (int y = 0; y < rows; ++y)                                                                  \
            memcpy(out + (int64_t)y * cols, o + (int64_t)(y + 1) * W + 1, sizeof(T) * cols);            \
        free(o);                                                                                        \
        free(in);                                                                                       \
    }

DEFINE_RECON(orc_imreconstruct_u8, uint8_t)
DEFINE_RECON(orc_imreconstruct_f32, float)

/* MO:2769-2909: binary reconstruction.  Padding 0; seeds are contour pixels
 * (marker != 0, mask != 0, some neighbour of the marker is 0); FIFO
 * propagation sets reached mask pixels to 255 (MO:2746-2753). */
void orc_imreconstruct_binary_u8(const uint8_t *marker, const uint8_t *mask, int rows, int cols, int conn, uint8_t *out) {
    int W = cols + 2, H = rows + 2;
    uint8_t *o = (uint8_t *)xcalloc((size_t)W * H, 1);
    uint8_t *in = (uint8_t *)xcalloc((size_t)W * H, 1);
    for (int y = 0; y < rows; ++y) {
        memcpy(o + (int64_t)(y + 1) * W + 1, marker + (int64_t)y * cols, cols);
        memcpy(in + (int64_t)(y + 1) * W + 1, mask + (int64_t)y * cols, cols);
    }
    int maxx = W - 1, maxy = H - 1;
    ififo q;
    ff_init(&q, (size_t)W * 4);
    for (int y = 1; y < maxy; ++y) {
        uint8_t *oP = o + (int64_t)y * W, *oPl = o + (int64_t)(y + 1) * W, *oM = o + (int64_t)(y - 1) * W;
        uint8_t *iP = in + (int64_t)y * W;
        for (int x = 1; x < maxx; ++x) {
            if (oP[x] != 0 && iP[x] != 0) {
                if (oM[x] == 0 || oPl[x] == 0 || oP[x + 1] == 0 || oP[x - 1] == 0) {
                    ff_push(&q, y * W + x);
                    continue;
                }
                if (conn == 8) {
                    if (oM[x - 1] == 0 || oM[x + 1] == 0 || oPl[x - 1] == 0 || oPl[x + 1] == 0) {
                        ff_push(&q, y * W + x);
                        continue;
                    }
                }
            }
        }
    }
    static const int dx8[8] = {0, 0, -1, 1, -1, 1, -1, 1};
    static const int dy8[8] = {-1, 1, 0, 0, -1, -1, 1, 1};
    while (q.n) {
        int32_t p = ff_pop(&q);
        int x = p % W, y = p / W;
        int nn = conn == 8 ? 8 : 4;
        for (int k = 0; k < nn; ++k) {
            int xx = x + dx8[k], yy = y + dy8[k];
            if (xx < 0 || xx > maxx || yy < 0 || yy > maxy) continue;
            int64_t qi = (int64_t)yy * W + xx;
            if (o[qi] == 0 && in[qi] != 0) {
                o[qi] = 255;
                ff_push(&q, (int32_t)qi);
            }
        }
    }
    ff_free(&q);
    for (int y = 0; y < rows; ++y) memcpy(out + (int64_t)y * cols, o + (int64_t)(y + 1) * W + 1, cols);
    free(o);
    free(in);
}

/* MO:2940-3006 with binary = true: pad the image with mn = 0; marker = mn
 * inside, mx = 255 on the border; mask = invert(padded image);
 * recon = imreconstructBinary(marker, mask, conn); output = invert(recon),
 * cropped. */
void orc_imfill_holes_u8(const uint8_t *img, int rows, int cols, int conn, uint8_t *out) {
    int W = cols + 2, H = rows + 2;
    uint8_t *mask = (uint8_t *)xmalloc((size_t)W * H);
    uint8_t *marker = (uint8_t *)xmalloc((size_t)W * H);
    uint8_t *rec = (uint8_t *)xmalloc((size_t)W * H);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int inner = (y > 0 && y < H - 1 && x > 0 && x < W - 1);
            uint8_t v = inner ? img[(int64_t)(y - 1) * cols + (x - 1)] : 0;
            mask[(int64_t)y * W + x] = (uint8_t)(255 - v);
            marker[(int64_t)y * W + x] = inner ? 0 : 255;
        }
    orc_imreconstruct_binary_u8(marker, mask, H, W, conn, rec);
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x)
            out[(int64_t)y * cols + x] = (uint8_t)(255 - rec[(int64_t)(y + 1) * W + (x + 1)]);
    free(mask);
    free(marker);
    free(rec);
}

/* MO:3010-3031: marker = bw where seeds != 0; recon binary under bw; & bw. */
void orc_bwselect_u8(const uint8_t *bw, const uint8_t *seeds, int rows, int cols, int conn, uint8_t *out) {
    int64_t n = (int64_t)rows * cols;
    uint8_t *marker = (uint8_t *)xmalloc(n);
    for (int64_t i = 0; i < n; ++i) marker[i] = seeds[i] ? bw[i] : 0;
    orc_imreconstruct_binary_u8(marker, bw, rows, cols, conn, out);
    for (int64_t i = 0; i < n; ++i) out[i] &= bw[i];
    free(marker);
}

/* ------------------------------------------------ union-find CCL (CC) --- */
static int32_t uf_find(int32_t *label, int32_t x) {
    int32_t r = x;
    while (label[r] != r) r = label[r];
    while (label[x] != r) {
        int32_t nx = label[x];
        label[x] = r;
        x = nx;
    }
    return r;
}
/* CC:34-43: link the larger root under the smaller, so roots are the minimum
 * raster index of their component. */
static void uf_merge(int32_t *label, int32_t x, int32_t y) {
    x = uf_find(label, x);
    y = uf_find(label, y);
    if (x < y)
        label[y] = x;
    else if (x > y)
        label[x] = y;
}

/* CC:52-86: equal-valued non-zero neighbours (left, up, and for 8-conn up-left
 * and up-right) are merged; background gets bgval; final flatten (CC:137-147). */
void orc_cc_label(const uint8_t *img, int w, int h, int32_t *label, int bgval, int conn) {
    int64_t length = (int64_t)w * h;
    for (int64_t i = 0; i < length; ++i) label[i] = (int32_t)i;
    int64_t i = -1;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            ++i;
            uint8_t p = img[i];
            if (p == 0) {
                label[i] = bgval;
            } else {
                int64_t imw = i - w;
                if (x > 0 && p == img[i - 1]) uf_merge(label, (int32_t)i, (int32_t)(i - 1));
                if (y > 0 && p == img[imw]) uf_merge(label, (int32_t)i, (int32_t)imw);
                if (conn == 8) {
                    if (y > 0 && x > 0 && p == img[imw - 1]) uf_merge(label, (int32_t)i, (int32_t)(imw - 1));
                    if (y > 0 && x < w - 1 && p == img[imw + 1]) uf_merge(label, (int32_t)i, (int32_t)(imw + 1));
                }
            }
        }
    for (int64_t j = 0; j < length; ++j) {
        if (label[j] == bgval) continue;
        /* all non-background chains end at a root (label[r] == r) */
        label[j] = uf_find(label, (int32_t)j);
    }
}

/* CC:205-239: areas of labels, keep lower <= area < upper, count kept. */
int orc_cc_area_threshold_labeled(const int32_t *label, int w, int h, int32_t *out, int bgval, int lower, int upper) {
    int64_t length = (int64_t)w * h;
    int32_t *area = (int32_t *)xcalloc((size_t)length, sizeof(int32_t));
    for (int64_t i = 0; i < length; ++i)
        if (label[i] != bgval) area[label[i]]++;
    int j = 0;
    for (int64_t i = 0; i < length; ++i)
        if (area[i] > 0 && area[i] >= lower && area[i] < upper) ++j;
    for (int64_t i = 0; i < length; ++i) {
        int32_t l = label[i];
        out[i] = (l != bgval && area[l] >= lower && area[l] < upper) ? l : bgval;
    }
    free(area);
    return j;
}

/* MO:3092-3117 (relabel disabled): int32 labels, background -1, label = min
 * raster index of the component. */
void orc_bwlabel2(const uint8_t *img, int rows, int cols, int conn, int32_t *out) {
    orc_cc_label(img, cols, rows, out, -1, conn);
}

/* MO:3281-3314 with labeled = false, flatten = true. */
int orc_bwareaopen2(const uint8_t *img, int rows, int cols, int minSize, int maxSize, int conn, uint8_t *out) {
    int64_t n = (int64_t)rows * cols;
    int32_t *lab = (int32_t *)xmalloc(n * sizeof(int32_t));
    int32_t *lab2 = (int32_t *)xmalloc(n * sizeof(int32_t));
    orc_cc_label(img, cols, rows, lab, -1, conn);
    int count = orc_cc_area_threshold_labeled(lab, cols, rows, lab2, -1, minSize, maxSize);
    for (int64_t i = 0; i < n; ++i) out[i] = lab2[i] > -1 ? 255 : 0;
    free(lab);
    free(lab2);
    return count;
}

/* ---------------------------------------------- distance transform --- */
/* OpenCV cv::distanceTransform(src, dst, CV_DIST_L2, CV_DIST_MASK_PRECISE):
 * exact Euclidean distance of every pixel to the nearest zero pixel, as
 * float32 = sqrtf(float(d^2)) (OpenCV's trueDistTrans: column pass, then the
 * Felzenszwalb lower envelope per row, then sqrt of the float sum).
 * Out-of-image pixels are not zeros.  When the image has no zero pixel at all
 * OpenCV returns sqrt(1e15f) everywhere; this restatement does the same.
 * The lower envelope here uses exact integer arithmetic; OpenCV's float
 * envelope gives the same d^2 whenever distances stay well below ~2000 px. */
void orc_dist_transform(const uint8_t *mask, int rows, int cols, float *out) {
    const int64_t INF = (int64_t)1 << 60;
    int64_t n = (int64_t)rows * cols;
    int64_t *g = (int64_t *)xmalloc(n * sizeof(int64_t));
    int anyzero = 0;
    for (int x = 0; x < cols; ++x) {
        int64_t d = INF;
        for (int y = 0; y < rows; ++y) {
            if (mask[(int64_t)y * cols + x] == 0) d = 0, anyzero = 1;
            else if (d != INF) d++;
            g[(int64_t)y * cols + x] = d;
        }
        d = INF;
        for (int y = rows - 1; y >= 0; --y) {
            if (mask[(int64_t)y * cols + x] == 0) d = 0;
            else if (d != INF) d++;
            if (d < g[(int64_t)y * cols + x]) g[(int64_t)y * cols + x] = d;
        }
    }
    if (!anyzero) {
        float v = sqrtf(1e15f);
        for (int64_t i = 0; i < n; ++i) out[i] = v;
        free(g);
        return;
    }
    int *v = (int *)xmalloc(sizeof(int) * (cols + 1));
    int64_t *f = (int64_t *)xmalloc(sizeof(int64_t) * (cols + 1));
    for (int y = 0; y < rows; ++y) {
        int64_t *gr = g + (int64_t)y * cols;
        /* candidate parabolas: columns with a finite column distance */
        int k = -1;
        for (int q = 0; q < cols; ++q) {
            if (gr[q] == INF) continue;
            int64_t fq = gr[q] * gr[q];
            while (k >= 0) {
                /* remove v[k] if it is never strictly needed: the intersection of
                 * q with v[k] is at or before the intersection of v[k] with v[k-1] */
                if (k == 0) break;
                int p = v[k], pp = v[k - 1];
                int64_t fp = f[k], fpp = f[k - 1];
                /* s(q,p) = ((fq+q^2)-(fp+p^2)) / (2(q-p)); s(p,pp) likewise */
                __int128 lhs = (__int128)((fq + (int64_t)q * q) - (fp + (int64_t)p * p)) * (2 * (int64_t)(p - pp));
                __int128 rhs = (__int128)((fp + (int64_t)p * p) - (fpp + (int64_t)pp * pp)) * (2 * (int64_t)(q - p));
                if (lhs <= rhs) --k;
                else break;
            }
            ++k;
            v[k] = q;
            f[k] = fq;
        }
        /* evaluate: the envelope is a sequence of parabolas ordered by x;
         * walk it while the next parabola gives a value <= the current one */
        int j = 0;
        for (int q = 0; q < cols; ++q) {
            while (j < k) {
                int64_t a = f[j] + (int64_t)(q - v[j]) * (q - v[j]);
                int64_t b = f[j + 1] + (int64_t)(q - v[j + 1]) * (q - v[j + 1]);
                if (b <= a) ++j;
                else break;
            }
            int64_t d2 = f[j] + (int64_t)(q - v[j]) * (q - v[j]);
            out[(int64_t)y * cols + q] = sqrtf((float)d2);
        }
    }
    free(v);
    free(f);
    free(g);
}

/* ------------------------------------------------------ imhmin (MO) --- */
/* MO:3343-3364: mask = invert(img) (float: -x, PO:40); marker = mask - h
 * (float arithmetic, OpenCV converts the scalar to the array depth);
 * out = invert(imreconstruct(marker, mask, conn)). */
void orc_imhmin_f32(const float *img, int rows, int cols, float h, int conn, float *out) {
    int64_t n = (int64_t)rows * cols;
    float *mask = (float *)xmalloc(n * sizeof(float)), *marker = (float *)xmalloc(n * sizeof(float));
    for (int64_t i = 0; i < n; ++i) {
        mask[i] = -img[i];
        volatile float t = mask[i] + (-h);
        marker[i] = t;
    }
    orc_imreconstruct_f32(marker, mask, rows, cols, conn, out);
    for (int64_t i = 0; i < n; ++i) out[i] = -out[i];
    free(mask);
    free(marker);
}

/* ------------------------------------------- local maxima / minima --- */
/* MO:3764-3836.  candidates = (img-1) < recon(img-1, img, conn) marks
 * NON-maxima (255); the rest (0) are candidate maxima.  A candidate pixel with
 * a strictly greater neighbour (4-neighbours, plus diagonals for conn 8;
 * out-of-image = -FLT_MAX) triggers OpenCV cv::floodFill with MASK_ONLY |
 * FIXED_RANGE, zero tolerance and the given connectivity: every candidate
 * pixel conn-connected to it with exactly the same value is marked.  The
 * result is the set of candidate pixels never marked. */
void orc_local_maxima_f32(const float *img, int rows, int cols, int conn, uint8_t *out) {
    int64_t n = (int64_t)rows * cols;
    float *marker = (float *)xmalloc(n * sizeof(float)), *rec = (float *)xmalloc(n * sizeof(float));
    for (int64_t i = 0; i < n; ++i) {
        volatile float t = img[i] + (-1.0f);
        marker[i] = t;
    }
    orc_imreconstruct_f32(marker, img, rows, cols, conn, rec);
    int W = cols + 2, H = rows + 2;
    uint8_t *m = (uint8_t *)xmalloc((size_t)W * H);
    float *in = (float *)xmalloc((size_t)W * H * sizeof(float));
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int inner = (y > 0 && y < H - 1 && x > 0 && x < W - 1);
            int64_t s = (int64_t)(y - 1) * cols + (x - 1);
            m[(int64_t)y * W + x] = inner ? ((marker[s] < rec[s]) ? 255 : 0) : 255;
            in[(int64_t)y * W + x] = inner ? img[s] : -FLT_MAX;
        }
    free(marker);
    free(rec);
    ififo q;
    ff_init(&q, 4096);
    static const int dx8[8] = {-1, 1, 0, 0, -1, 1, -1, 1};
    static const int dy8[8] = {0, 0, -1, 1, -1, -1, 1, 1};
    int nn = conn == 8 ? 8 : 4;
    for (int y = 1; y < H - 1; ++y)
        for (int x = 1; x < W - 1; ++x) {
            int64_t p = (int64_t)y * W + x;
            if (m[p] > 0) continue;
            float val = in[p];
            int greater = 0;
            for (int k = 0; k < nn; ++k)
                if (val < in[p + dy8[k] * W + dx8[k]]) greater = 1;
            if (!greater) continue;
            /* flood: zero-tolerance fixed range against the seed value */
            m[p] = 1;
            ff_push(&q, (int32_t)p);
            while (q.n) {
                int32_t c = ff_pop(&q);
                for (int k = 0; k < nn; ++k) {
                    int64_t d = c + dy8[k] * W + dx8[k];
                    if (m[d] == 0 && in[d] == val) {
                        m[d] = 1;
                        ff_push(&q, (int32_t)d);
                    }
                }
            }
        }
    ff_free(&q);
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x)
            out[(int64_t)y * cols + x] = m[(int64_t)(y + 1) * W + (x + 1)] == 0 ? 255 : 0;
    free(m);
    free(in);
}

/* MO:3839-3845: localMaxima(invert(img)). */
void orc_local_minima_f32(const float *img, int rows, int cols, int conn, uint8_t *out) {
    int64_t n = (int64_t)rows * cols;
    float *c = (float *)xmalloc(n * sizeof(float));
    for (int64_t i = 0; i < n; ++i) c[i] = -img[i];
    orc_local_maxima_f32(c, rows, cols, conn, out);
    free(c);
}

/* ---------------------------------------------------------- watershed --- */
/* OpenCV 2.4.9 cv::watershed (Meyer flooding), restated from OpenCV's
 * published algorithm: 256 FIFO queues keyed by the colour difference
 * max(|dB|,|dG|,|dR|); the one-pixel image border is set to -1; negative
 * markers are reset to 0 (unknown); unknown pixels 4-adjacent to a marker > 0
 * are queued at the minimum difference to those markers, in raster order;
 * then the lowest non-empty queue is popped repeatedly: a pixel takes the
 * label of its labelled 4-neighbours, or -1 if they disagree, and (unless -1)
 * queues its unknown 4-neighbours (left, right, up, down) at their colour
 * difference, lowering the active queue if needed.  rows/cols include the
 * border; `markers` is updated in place. */
static inline int cdiff(const uint8_t *a, const uint8_t *b) {
    int db = abs((int)a[0] - (int)b[0]);
    int dg = abs((int)a[1] - (int)b[1]);
    int dr = abs((int)a[2] - (int)b[2]);
    int d = db > dg ? db : dg;
    return d > dr ? d : dr;
}

void orc_cv_watershed(const uint8_t *img, int32_t *mask, int rows, int cols) {
    const int NQ = 256;
    int64_t n = (int64_t)rows * cols;
    int32_t *next = (int32_t *)xmalloc(n * sizeof(int32_t));
    int32_t qh[256], qt[256];
    for (int i = 0; i < NQ; ++i) qh[i] = qt[i] = -1;
#define WS_PUSH(idx, ofs)                                \
    do {                                                 \
        int32_t o_ = (int32_t)(ofs);                     \
        next[o_] = -1;                                   \
        if (qt[idx] < 0) qh[idx] = o_;                   \
        else next[qt[idx]] = o_;                         \
        qt[idx] = o_;                                    \
    } while (0)
    int ms = cols;
    for (int j = 0; j < cols; ++j) mask[j] = mask[j + (int64_t)ms * (rows - 1)] = WSHED;
    for (int i = 1; i < rows - 1; ++i) {
        int32_t *row = mask + (int64_t)i * ms;
        const uint8_t *irow = img + (int64_t)i * cols * 3;
        row[0] = row[cols - 1] = WSHED;
        for (int j = 1; j < cols - 1; ++j) {
            int32_t *m = row + j;
            if (m[0] < 0) m[0] = 0;
            if (m[0] == 0 && (m[-1] > 0 || m[1] > 0 || m[-ms] > 0 || m[ms] > 0)) {
                const uint8_t *ptr = irow + j * 3;
                int idx = 256, t;
                if (m[-1] > 0) idx = cdiff(ptr, ptr - 3);
                if (m[1] > 0) {
                    t = cdiff(ptr, ptr + 3);
                    idx = idx < t ? idx : t;
                }
                if (m[-ms] > 0) {
                    t = cdiff(ptr, ptr - 3 * cols);
                    idx = idx < t ? idx : t;
                }
                if (m[ms] > 0) {
                    t = cdiff(ptr, ptr + 3 * cols);
                    idx = idx < t ? idx : t;
                }
                WS_PUSH(idx, (int64_t)i * ms + j);
                m[0] = IN_QUEUE;
            }
        }
    }
    int active = 0;
    while (active < NQ && qh[active] < 0) ++active;
    if (active == NQ) {
        free(next);
        return;
    }
    for (;;) {
        if (qh[active] < 0) {
            int i;
            for (i = active + 1; i < NQ; ++i)
                if (qh[i] >= 0) break;
            if (i == NQ) break;
            active = i;
        }
        int32_t mofs = qh[active];
        qh[active] = next[mofs];
        if (qh[active] < 0) qt[active] = -1;
        int32_t *m = mask + mofs;
        const uint8_t *ptr = img + (int64_t)mofs * 3;
        int lab = 0, t;
        t = m[-1];
        if (t > 0) lab = t;
        t = m[1];
        if (t > 0) {
            if (lab == 0) lab = t;
            else if (t != lab) lab = WSHED;
        }
        t = m[-ms];
        if (t > 0) {
            if (lab == 0) lab = t;
            else if (t != lab) lab = WSHED;
        }
        t = m[ms];
        if (t > 0) {
            if (lab == 0) lab = t;
            else if (t != lab) lab = WSHED;
        }
        m[0] = lab;
        if (lab == WSHED) continue;
        if (m[-1] == 0) {
            t = cdiff(ptr, ptr - 3);
            WS_PUSH(t, mofs - 1);
            active = active < t ? active : t;
            m[-1] = IN_QUEUE;
        }
        if (m[1] == 0) {
            t = cdiff(ptr, ptr + 3);
            WS_PUSH(t, mofs + 1);
            active = active < t ? active : t;
            m[1] = IN_QUEUE;
        }
        if (m[-ms] == 0) {
            t = cdiff(ptr, ptr - 3 * cols);
            WS_PUSH(t, mofs - ms);
            active = active < t ? active : t;
            m[-ms] = IN_QUEUE;
        }
        if (m[ms] == 0) {
            t = cdiff(ptr, ptr + 3 * cols);
            WS_PUSH(t, mofs + ms);
            active = active < t ? active : t;
            m[ms] = IN_QUEUE;
        }
    }
#undef WS_PUSH
    free(next);
}

/* NO:18-44: on a padded image, for y >= 1 and 1 <= x < cols-1:
 * p becomes bg when up == bg, p != bg and ((up-left != bg && left == bg) ||
 * (up-right != bg && right == bg)).  Row 0 and the first/last column are not
 * written by the reference (they are cropped away); here they copy the input. */
void orc_border_fix_i32(const int32_t *in, int rows, int cols, int32_t bg, int32_t *out) {
    memcpy(out, in, sizeof(int32_t) * (size_t)rows * cols);
    for (int y = 1; y < rows; ++y) {
        const int32_t *p = in + (int64_t)y * cols, *pm = in + (int64_t)(y - 1) * cols;
        int32_t *r = out + (int64_t)y * cols;
        for (int x = 1; x < cols - 1; ++x) {
            if (pm[x] == bg && p[x] != bg &&
                ((pm[x - 1] != bg && p[x - 1] == bg) || (pm[x + 1] != bg && p[x + 1] == bg)))
                r[x] = bg;
            else
                r[x] = p[x];
        }
    }
}

/* MO:3717-3760: minima = localMinima(img, conn); labels = bwlabel2(minima,
 * conn); pad labels with 0 and the colour image with 0; cv::watershed;
 * border fix with bg -1; crop. */
void orc_watershed2(const uint8_t *bgr, const float *img, int rows, int cols, int conn, int32_t *out,
                    int32_t *labels_out) {
    int64_t n = (int64_t)rows * cols;
    uint8_t *minima = (uint8_t *)xmalloc(n);
    orc_local_minima_f32(img, rows, cols, conn, minima);
    int32_t *labels = (int32_t *)xmalloc(n * sizeof(int32_t));
    orc_bwlabel2(minima, rows, cols, conn, labels);
    if (labels_out) memcpy(labels_out, labels, n * sizeof(int32_t));
    int W = cols + 2, H = rows + 2;
    int32_t *t = (int32_t *)xcalloc((size_t)W * H, sizeof(int32_t));
    uint8_t *in = (uint8_t *)xcalloc((size_t)W * H * 3, 1);
    for (int y = 0; y < rows; ++y) {
        memcpy(t + (int64_t)(y + 1) * W + 1, labels + (int64_t)y * cols, sizeof(int32_t) * cols);
        memcpy(in + ((int64_t)(y + 1) * W + 1) * 3, bgr + (int64_t)y * cols * 3, (size_t)cols * 3);
    }
    orc_cv_watershed(in, t, H, W);
    int32_t *fixed = (int32_t *)xmalloc((size_t)W * H * sizeof(int32_t));
    orc_border_fix_i32(t, H, W, -1, fixed);
    for (int y = 0; y < rows; ++y)
        memcpy(out + (int64_t)y * cols, fixed + (int64_t)(y + 1) * W + 1, sizeof(int32_t) * cols);
    free(minima);
    free(labels);
    free(t);
    free(in);
    free(fixed);
}

/* ------------------------------------------------------ bounding box --- */
/* CC:241-284 with the background value the label image actually uses (-1):
 * per label, in first-appearance raster order (= increasing label for
 * min-raster-index labels): label, minx, maxx, miny, maxy, written as five
 * consecutive arrays of compcount ints. */
int orc_bounding_box(const int32_t *labels, int w, int h, int32_t *bbox_out) {
    int64_t n = (int64_t)w * h;
    int32_t *slot = (int32_t *)xmalloc(n * sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) slot[i] = -1;
    int j = 0;
    int32_t *lab = (int32_t *)xmalloc(n * sizeof(int32_t));
    int32_t *mnx = (int32_t *)xmalloc(n * sizeof(int32_t)), *mxx = (int32_t *)xmalloc(n * sizeof(int32_t));
    int32_t *mny = (int32_t *)xmalloc(n * sizeof(int32_t)), *mxy = (int32_t *)xmalloc(n * sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) {
        int32_t l = labels[i];
        if (l < 0) continue;
        int x = (int)(i % w), y = (int)(i / w);
        if (slot[l] < 0) {
            slot[l] = j;
            lab[j] = l;
            mnx[j] = mxx[j] = x;
            mny[j] = mxy[j] = y;
            ++j;
        } else {
            int s = slot[l];
            if (x < mnx[s]) mnx[s] = x;
            if (x > mxx[s]) mxx[s] = x;
            if (y < mny[s]) mny[s] = y;
            if (y > mxy[s]) mxy[s] = y;
        }
    }
    if (bbox_out) {
        memcpy(bbox_out, lab, j * sizeof(int32_t));
        memcpy(bbox_out + j, mnx, j * sizeof(int32_t));
        memcpy(bbox_out + 2 * j, mxx, j * sizeof(int32_t));
        memcpy(bbox_out + 3 * j, mny, j * sizeof(int32_t));
        memcpy(bbox_out + 4 * j, mxy, j * sizeof(int32_t));
    }
    free(slot);
    free(lab);
    free(mnx);
    free(mxx);
    free(mny);
    free(mxy);
    return j;
}

/* CC:241-284 exactly as HE:591 calls it (bgval = 0 on a -1 background): the
 * scan stops at the first -1 pixel (CC:252), so compcount is usually 0.
 * Kept only to report the deviation. */
int orc_bounding_box_refbug(const int32_t *labels, int w, int h, int bgval, int32_t *bbox_out) {
    int64_t n = (int64_t)w * h;
    int32_t *tmp = (int32_t *)xmalloc(n * sizeof(int32_t));
    int64_t stop = n;
    for (int64_t i = 0; i < n; ++i) {
        if (labels[i] == bgval) {
            tmp[i] = -1;
            continue;
        }
        if (labels[i] == -1 || labels[i] == 0) {
            stop = i;
            break;
        }
        tmp[i] = labels[i];
    }
    for (int64_t i = stop; i < n; ++i) tmp[i] = -1;
    int c = orc_bounding_box(tmp, w, h, bbox_out);
    free(tmp);
    return c;
}

/* ------------------------------------------------------ segmentNuclei --- */
#define TIC(k) double t_##k = now_s()
#define TOC(k, id) if (dump) dump->stage_seconds[id] += now_s() - t_##k
#define DUMP(field, src, nbytes) if (dump && dump->field) memcpy(dump->field, src, nbytes)

/* HE:473-598 (plFindNucleusCandidates HE:115-304, plSeparateNuclei HE:308-449). */
int orc_segment_nuclei(const uint8_t *bgr, int rows, int cols, const orc_params *pin,
                       int32_t *labels_out, uint8_t *mask_out, int *compcount, int32_t *bbox_out,
                       orc_dump *dump) {
    orc_params p;
    if (pin) p = *pin;
    else orc_default_params(&p);
    if (compcount) *compcount = 0;
    if (!bgr || rows <= 0 || cols <= 0) return ORC_INVALID_IMAGE;
    int64_t n = (int64_t)rows * cols;
    int status = ORC_SUCCESS;
    uint8_t *R = (uint8_t *)xmalloc(n), *rc = (uint8_t *)xmalloc(n), *rc_open = (uint8_t *)xmalloc(n);
    uint8_t *rc_recon = (uint8_t *)xmalloc(n), *diff = (uint8_t *)xmalloc(n), *tmp = (uint8_t *)xmalloc(n);
    uint8_t *bw1 = (uint8_t *)xmalloc(n), *bw1_t = (uint8_t *)xmalloc(n), *rbc = (uint8_t *)xmalloc(n);
    uint8_t *seg_norbc = (uint8_t *)xmalloc(n), *seg_nohole = (uint8_t *)xmalloc(n);
    uint8_t *seg_open = (uint8_t *)xmalloc(n), *seg_big_t = (uint8_t *)xmalloc(n);
    uint8_t *seg_big = (uint8_t *)xmalloc(n), *nuclei = (uint8_t *)xmalloc(n * 3);
    uint8_t *seg_nonoverlap = (uint8_t *)xmalloc(n), *seg = (uint8_t *)xmalloc(n), *fin = (uint8_t *)xmalloc(n);
    float *dist = (float *)xmalloc(n * sizeof(float)), *distance = (float *)xmalloc(n * sizeof(float));
    float *distance2 = (float *)xmalloc(n * sizeof(float));
    int32_t *watermask = (int32_t *)xmalloc(n * sizeof(int32_t));
    int32_t *labels = labels_out ? labels_out : (int32_t *)xmalloc(n * sizeof(int32_t));
    int cc;

    /* ---- plFindNucleusCandidates ---- */
    TIC(bg);
    int64_t bgArea = orc_get_background(bgr, rows, cols, p.blue, p.green, p.red, NULL);
    float ratio = (float)bgArea / (float)n;
    TOC(bg, 1);
    if (dump) dump->bg_count = (int)bgArea;
    if (ratio >= 0.99) { status = ORC_BACKGROUND; goto done; }
    if (ratio >= 0.9) { status = ORC_BACKGROUND_LIKELY; goto done; }

    TIC(rbc);
    orc_get_rbc(bgr, rows, cols, p.T1, p.T2, rbc);
    TOC(rbc, 2);
    DUMP(rbc, rbc, n);

    for (int64_t i = 0; i < n; ++i) R[i] = bgr[3 * i + 2];
    orc_invert_u8(R, n, rc);
    TIC(open);
    orc_morph_open_u8(rc, rows, cols, orc_disk19(), 19, rc_open);
    TOC(open, 3);
    DUMP(rc_open, rc_open, n);
    TIC(recon);
    orc_imreconstruct_u8(rc_open, rc, rows, cols, p.reconConnectivity, rc_recon);
    TOC(recon, 4);
    DUMP(rc_recon, rc_recon, n);
    for (int64_t i = 0; i < n; ++i) diff[i] = rc[i] > rc_recon[i] ? (uint8_t)(rc[i] - rc_recon[i]) : 0;
    DUMP(diffIm, diff, n);
    for (int64_t i = 0; i < n; ++i) tmp[i] = diff[i] > p.G1 ? 255 : 0;
    TIC(fill1);
    orc_imfill_holes_u8(tmp, rows, cols, p.fillHolesConnectivity, bw1);
    TOC(fill1, 7);
    DUMP(bw1, bw1, n);
    TIC(ao1);
    cc = orc_bwareaopen2(bw1, rows, cols, p.minSize, p.maxSize, 8, bw1_t);
    TOC(ao1, 8);
    DUMP(bw1_t, bw1_t, n);
    if (dump) dump->compcount_first = cc;
    if (cc == 0) { status = ORC_NO_CANDIDATES_LEFT; goto done; }
    for (int64_t i = 0; i < n; ++i) tmp[i] = diff[i] > p.G2 ? 255 : 0;
    TIC(sel);
    orc_bwselect_u8(tmp, bw1_t, rows, cols, 8, seg_norbc);
    for (int64_t i = 0; i < n; ++i) seg_norbc[i] = (rbc[i] == 0) ? seg_norbc[i] : 0;
    TOC(sel, 11);
    DUMP(seg_norbc, seg_norbc, n);

    /* ---- segmentNuclei body ---- */
    TIC(fill2);
    orc_imfill_holes_u8(seg_norbc, rows, cols, 4, seg_nohole);
    TOC(fill2, 12);
    DUMP(seg_nohole, seg_nohole, n);
    TIC(open3);
    orc_morph_open_u8(seg_nohole, rows, cols, orc_cross3(), 3, seg_open);
    TOC(open3, 13);
    DUMP(seg_open, seg_open, n);

    /* ---- plSeparateNuclei ---- */
    TIC(ao2);
    orc_bwareaopen2(seg_open, rows, cols, p.minSizePl, INT_MAX, 8, seg_big_t);
    TOC(ao2, 14);
    TIC(dil);
    orc_dilate_u8(seg_big_t, rows, cols, orc_cross3(), 3, seg_big);
    TOC(dil, 15);
    DUMP(seg_big, seg_big, n);
    TIC(edt);
    orc_dist_transform(seg_big, rows, cols, dist);
    for (int64_t i = 0; i < n; ++i) distance[i] = seg_big[i] ? -dist[i] : -FLT_MAX;
    TOC(edt, 16);
    DUMP(dist, dist, n * sizeof(float));
    TIC(hmin);
    orc_imhmin_f32(distance, rows, cols, 1.0f, 8, distance2);
    TOC(hmin, 18);
    DUMP(distance2, distance2, n * sizeof(float));
    for (int64_t i = 0; i < n; ++i) {
        int on = seg_big[i] != 0;
        nuclei[3 * i + 0] = on ? bgr[3 * i + 0] : 0;
        nuclei[3 * i + 1] = on ? bgr[3 * i + 1] : 0;
        nuclei[3 * i + 2] = on ? bgr[3 * i + 2] : 0;
    }
    TIC(ws);
    orc_watershed2(nuclei, distance2, rows, cols, p.watershedConnectivity, watermask,
                   dump ? dump->minima_labels : NULL);
    TOC(ws, 20);
    if (dump && dump->minima) orc_local_minima_f32(distance2, rows, cols, p.watershedConnectivity, dump->minima);
    DUMP(watermask, watermask, n * sizeof(int32_t));
    for (int64_t i = 0; i < n; ++i) seg_nonoverlap[i] = watermask[i] >= 0 ? seg_big[i] : 0;
    DUMP(seg_nonoverlap, seg_nonoverlap, n);

    TIC(ao3);
    cc = orc_bwareaopen2(seg_nonoverlap, rows, cols, p.minSizeSeg, p.maxSizeSeg, 4, seg);
    TOC(ao3, 21);
    if (dump) dump->compcount_seg = cc;
    DUMP(seg, seg, n);
    if (cc == 0) { status = ORC_NO_CANDIDATES_LEFT; goto done; }
    TIC(fill3);
    orc_imfill_holes_u8(seg, rows, cols, p.fillHolesConnectivity, fin);
    TOC(fill3, 22);
    DUMP(final_mask, fin, n);
    if (mask_out) memcpy(mask_out, fin, n);
    TIC(lab);
    orc_bwlabel2(fin, rows, cols, 8, labels);
    TOC(lab, 23);
    {
        int c = orc_bounding_box(labels, cols, rows, bbox_out);
        if (compcount) *compcount = c;
    }
    status = ORC_SUCCESS;
done:
    free(R); free(rc); free(rc_open); free(rc_recon); free(diff); free(tmp);
    free(bw1); free(bw1_t); free(rbc); free(seg_norbc); free(seg_nohole); free(seg_open);
    free(seg_big_t); free(seg_big); free(nuclei); free(seg_nonoverlap); free(seg); free(fin);
    free(dist); free(distance); free(distance2); free(watermask);
    if (!labels_out) free(labels);
    return status;
}

/* ------------------------------------------------------------------------- */
/* Colour deconvolution, PixelOperations.cpp:94-274.                         */
/* ------------------------------------------------------------------------- */

/* PixelOperations::ComputeInverseStainMatrix (PixelOperations.cpp:94-156):
 * normalise each stain column of M (3x3, row-major) to unit length; if the
 * last column is zero, fill it row by row with sqrt(1 - |row|^2) (0 when the
 * row norm exceeds 1) and normalise it; invert; keep the rows i with
 * b[i] == 1.  Q6 receives up to two rows of 3 (the reference drops the first
 * row of its gathered matrix, which is a placeholder).  Returns the number of
 * rows kept.  The inverse is Gaussian elimination with partial pivoting, the
 * method OpenCV's Mat::inv (DECOMP_LU) uses. */
int orc_stain_matrix(const double *M9, const uint8_t *b3, double *Q6) {
    double N[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) N[r][c] = M9[r * 3 + c];
    for (int c = 0; c < 3; ++c) {
        double nrm = sqrt(N[0][c] * N[0][c] + N[1][c] * N[1][c] + N[2][c] * N[2][c]);
        if (nrm > 0)
            for (int r = 0; r < 3; ++r) N[r][c] /= nrm;
    }
    double last = sqrt(N[0][2] * N[0][2] + N[1][2] * N[1][2] + N[2][2] * N[2][2]);
    if (last == 0) {
        for (int r = 0; r < 3; ++r) {
            double nrm = sqrt(N[r][0] * N[r][0] + N[r][1] * N[r][1] + N[r][2] * N[r][2]);
            N[r][2] = nrm > 1 ? 0 : sqrt(1 - nrm * nrm);
        }
        double n2 = sqrt(N[0][2] * N[0][2] + N[1][2] * N[1][2] + N[2][2] * N[2][2]);
        if (n2 == 0) return 0;
        for (int r = 0; r < 3; ++r) N[r][2] /= n2;
    }
    /* [N | I] -> [I | inv(N)] */
    double A[3][6];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 6; ++c) A[r][c] = c < 3 ? N[r][c] : (c - 3 == r ? 1.0 : 0.0);
    for (int k = 0; k < 3; ++k) {
        int piv = k;
        for (int r = k + 1; r < 3; ++r)
            if (fabs(A[r][k]) > fabs(A[piv][k])) piv = r;
        if (A[piv][k] == 0) return 0;
        if (piv != k)
            for (int c = 0; c < 6; ++c) {
                double t = A[k][c];
                A[k][c] = A[piv][c];
                A[piv][c] = t;
            }
        double d = A[k][k];
        for (int c = 0; c < 6; ++c) A[k][c] /= d;
        for (int r = 0; r < 3; ++r) {
            if (r == k) continue;
            double f = A[r][k];
            for (int c = 0; c < 6; ++c) A[r][c] -= f * A[k][c];
        }
    }
    int kept = 0;
    for (int i = 0; i < 3 && kept < 2; ++i)
        if (b3[i] == 1) {
            for (int c = 0; c < 3; ++c) Q6[kept * 3 + c] = A[i][3 + c];
            ++kept;
        }
    return kept;
}

/* PixelOperations::ComputeLookupTable (PixelOperations.cpp:158-168):
 * k = (float)(-255/ln 255); lut[i] = (float)(k * ln(i + 1) + 255) in double. */
void orc_color_lut(float *lut) {
    const float k = (float)(-255.0 / log(255.0));
    for (int i = 0; i < 256; ++i) lut[i] = (float)((double)k * log((double)(float)i + 1.0) + 255.0);
}

static uint8_t sat_round_u8(float v) { /* saturate_cast<uchar>(float): round half to even, clamp */
    long r = lrintf(v);
    return (uint8_t)(r < 0 ? 0 : (r > 255 ? 255 : r));
}

/* PixelOperations::ColorDeconv(image, Q, lut, H, E, BGR2RGB = true)
 * (PixelOperations.cpp:170-274): dn = lut[BGR]; cn = dn * flip(Q^T) (the
 * float matrix product, whose 32-bit products OpenCV 2.4 sums in double:
 * restated, unpinned), i.e. cn_j = dn_B * Q[j][B] + dn_G * Q[j][G] +
 * dn_R * Q[j][R] in that order; out = saturate_u8(expf((cn - 255) *
 * (float)(-ln 255 / 255))). */
void orc_color_deconv(const uint8_t *bgr, int rows, int cols, const float *Q6, const float *lut, uint8_t *H,
                      uint8_t *E) {
    const float c = (float)(-log(255.0) / 255.0);
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = 0; i < n; ++i) {
        const float db = lut[bgr[3 * i]], dg = lut[bgr[3 * i + 1]], dr = lut[bgr[3 * i + 2]];
        for (int j = 0; j < 2; ++j) {
            double acc = (double)db * (double)Q6[j * 3 + 2];
            acc += (double)dg * (double)Q6[j * 3 + 1];
            acc += (double)dr * (double)Q6[j * 3 + 0];
            const float cn = (float)acc;
            const float v = expf((cn - 255.0f) * c);
            (j == 0 ? H : E)[i] = sat_round_u8(v);
        }
    }
}

/* the same in double throughout (the reference's GPU path computes in FP64):
 * the FP oracle for flip counts */
void orc_color_deconv_f64(const uint8_t *bgr, int rows, int cols, const double *Q6, uint8_t *H, uint8_t *E) {
    const double k = -255.0 / log(255.0), c = -log(255.0) / 255.0;
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = 0; i < n; ++i) {
        const double db = k * log(bgr[3 * i] + 1.0) + 255.0, dg = k * log(bgr[3 * i + 1] + 1.0) + 255.0,
                     dr = k * log(bgr[3 * i + 2] + 1.0) + 255.0;
        for (int j = 0; j < 2; ++j) {
            const double cn = db * Q6[j * 3 + 2] + dg * Q6[j * 3 + 1] + dr * Q6[j * 3 + 0];
            double v = exp((cn - 255.0) * c);
            v = v < 0 ? 0 : (v > 255 ? 255 : v);
            (j == 0 ? H : E)[i] = (uint8_t)lrint(v);
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Colour normalisation (src/normalization/Normalization.cpp): Reinhard     */
/* colour transfer in lab space of the foreground found by a Fisher          */
/* discriminant.  The arithmetic follows the reference's order and widths:   */
/* float where it computes on float Mats, double where it uses double        */
/* literals or accumulators.  Restated, unpinned (OpenCV's MatExpr            */
/* evaluation is part of it).                                                 */
/* ------------------------------------------------------------------------- */

/* discriminant coefficients M (Normalization.cpp:504-505, 555-556) */
static const float kNormM[8] = {-0.154f, 0.035f, 0.549f, -45.718f, -0.057f, -0.817f, 1.170f, -49.887f};

/* segFG (Normalization.cpp:19-55): d_k = M(k,0) R + M(k,1) G + M(k,2) B +
 * M(k,3) evaluated as OpenCV 2.4 evaluates the MatExpr: addWeighted of the
 * first two products, then addWeighted of that and the third with the
 * constant as gamma, each computed in double and stored as float;
 * foreground = d1 < d2. */
static int norm_fg(const uint8_t *px) {
    const float bd = (float)px[0], gd = (float)px[1], rd = (float)px[2];
    float d[2];
    for (int k = 0; k < 2; ++k) {
        const float *m = kNormM + 4 * k;
        const float t = (float)((double)rd * (double)m[0] + (double)gd * (double)m[1] + 0.0);
        d[k] = (float)((double)t * 1.0 + (double)bd * (double)m[2] + (double)m[3]);
    }
    return d[0] < d[1];
}

/* bgr2Lab (Normalization.cpp:64-149) of one pixel of I / 255 (convertTo,
 * then the Mat divided by 255: a float scale by (float)(1 / 255.0)) */
static void norm_lab(const uint8_t *px, float lab[3]) {
    const float s = (float)(1.0 / 255.0);
    const float b = (float)px[0] * s, g = (float)px[1] * s, r = (float)px[2] * s;
    const float L = (float)(0.3811 * r + 0.5783 * g + 0.0402 * b);
    const float M = (float)(0.1967 * r + 0.7244 * g + 0.0782 * b);
    const float S = (float)(0.0241 * r + 0.1288 * g + 0.8444 * b);
    const float l = log10f(L), m = log10f(M), sl = log10f(S);
    const float i3 = 1 / sqrtf(3.0f), i6 = 1 / sqrtf(6.0f), i2 = 1 / sqrtf(2.0f);
    /* Matrix2 = diag(1/sqrt3, 1/sqrt6, 1/sqrt2) * [1 1 1; 1 1 -2; 1 -1 0] */
    lab[0] = l * i3 + m * i3 + sl * i3;
    lab[1] = l * i6 + m * i6 + sl * (-2.0f * i6);
    lab[2] = l * i2 + m * (-i2) + sl * 0.0f;
}

static int norm_rndint(float n) { /* Normalization.cpp:153-162 */
    int ret = (int)floor(n);
    float t = n - (float)floor(n);
    if (t >= 0.5) ret = (int)floor(n) + 1;
    return ret;
}

/* lab2BGR (Normalization.cpp:166-292) of one pixel */
static void norm_bgr(const float lab[3], uint8_t *out) {
    const float i3 = 1 / sqrtf(3.0f), i6 = 1 / sqrtf(6.0f), i2 = 1 / sqrtf(2.0f);
    /* Matrix1 = [1 1 1; 1 1 -1; 1 -2 0] * diag(1/sqrt3, 1/sqrt6, 1/sqrt2) */
    const float l = lab[0], a = lab[1], b = lab[2];
    float lms[3];
    lms[0] = l * i3 + a * i6 + b * i2;
    lms[1] = l * i3 + a * i6 + b * (-i2);
    lms[2] = l * i3 + a * (-2.0f * i6) + b * 0.0f;
    for (int c = 0; c < 3; ++c) {
        float x = powf(10.0f, lms[c]);
        if (!(x <= DBL_MAX && x >= -DBL_MAX)) x = 0.0f; /* -Inf / NaN -> 0 */
        lms[c] = x;
    }
    static const float M2[9] = {4.4687f, -3.5887f, 0.1196f, -1.2197f, 2.3831f, -0.1626f, 0.0585f, -0.2611f, 1.2057f};
    const float L = lms[0], M = lms[1], S = lms[2];
    const float bf = L * M2[6] + M * M2[7] + S * M2[8];
    const float gf = L * M2[3] + M * M2[4] + S * M2[5];
    const float rf = L * M2[0] + M * M2[1] + S * M2[2];
    const float v[3] = {bf, gf, rf};
    for (int c = 0; c < 3; ++c) {
        float sc = (float)(v[c] * 255.0);
        if (sc < 0.0) sc = 0.0f;
        if (sc > 255.0) sc = 255.0f;
        out[c] = (uint8_t)norm_rndint(sc);
    }
}

/* the foreground's lab statistics (TransferI / targetParameters,
 * Normalization.cpp:296-350, 520-577): over foreground pixels whose
 * L * a * b product (float) is positive, sum and sum of squares (the square
 * in float, the sums in double), mean = sum / n, std = sqrt(sq / n - mean^2) */
void orc_norm_stats(const uint8_t *bgr, int rows, int cols, double *count, double *sum3, double *sq3) {
    const int64_t n = (int64_t)rows * cols;
    double c = 0.0, s[3] = {0, 0, 0}, q[3] = {0, 0, 0};
    for (int ch = 0; ch < 3; ++ch) { /* the reference sums channel by channel */
        for (int64_t i = 0; i < n; ++i) {
            const uint8_t *px = bgr + 3 * i;
            if (!norm_fg(px)) continue;
            float lab[3];
            norm_lab(px, lab);
            if (!((lab[0] * lab[1]) * lab[2] > 0)) continue;
            s[ch] += lab[ch];
            q[ch] += lab[ch] * lab[ch];
            if (ch == 0) c += 1.0;
        }
    }
    *count = c;
    for (int k = 0; k < 3; ++k) sum3[k] = s[k], sq3[k] = q[k];
}

/* Normalization::targetParameters (Normalization.cpp:520-577) */
void orc_target_parameters(const uint8_t *bgr, int rows, int cols, float *mean3, float *std3) {
    double c, s[3], q[3];
    orc_norm_stats(bgr, rows, cols, &c, s, q);
    for (int k = 0; k < 3; ++k) {
        const double mean = s[k] / c;
        const double var = q[k] / c - mean * mean;
        mean3[k] = (float)mean;
        std3[k] = (float)sqrt(var);
    }
}

/* Normalization::normalization (Normalization.cpp:487-517): foreground lab
 * values mapped by (v - mean) * (stdT / std) + meanT (float), background lab
 * kept, every pixel back through lab2BGR. */
void orc_normalization(const uint8_t *bgr, int rows, int cols, const float *meanT, const float *stdT,
                       uint8_t *out) {
    float meanL[3], stdL[3];
    orc_target_parameters(bgr, rows, cols, meanL, stdL);
    float ratio[3];
    for (int k = 0; k < 3; ++k) ratio[k] = stdT[k] / stdL[k];
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = 0; i < n; ++i) {
        const uint8_t *px = bgr + 3 * i;
        float lab[3];
        norm_lab(px, lab);
        if (norm_fg(px))
            for (int k = 0; k < 3; ++k) lab[k] = (lab[k] - meanL[k]) * ratio[k] + meanT[k];
        norm_bgr(lab, out + 3 * i);
    }
}

/* ------------------------------------------------------------------------- */
/* Per-nucleus features (src/features/ObjFeatures.cpp, Operators.cpp).       */
/* ------------------------------------------------------------------------- */

/* rndint (Operators.cpp:554-564): floor, plus one when the fraction >= 0.5 */
static int feat_rndint(float n) {
    int ret = (int)floorf(n);
    float t = n - floorf(n);
    if (t >= 0.5f) ret = (int)floorf(n) + 1;
    return ret;
}

/* Operators::gradient (Operators.cpp:568-640): correlation with
 * [-0.5, 0, 0.5] along x and along y (cvFilter2D, replicated border), the
 * first and last column (row) doubled, magnitude sqrt(dx^2 + dy^2) in float,
 * then rndint and clamp to uint8. */
void orc_gradient_u8(const uint8_t *in, int rows, int cols, uint8_t *out) {
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x) {
            const int xl = x > 0 ? x - 1 : 0, xr = x + 1 < cols ? x + 1 : cols - 1;
            const int yu = y > 0 ? y - 1 : 0, yd = y + 1 < rows ? y + 1 : rows - 1;
            float dx = -0.5f * (float)in[(int64_t)y * cols + xl] + 0.5f * (float)in[(int64_t)y * cols + xr];
            float dy = -0.5f * (float)in[(int64_t)yu * cols + x] + 0.5f * (float)in[(int64_t)yd * cols + x];
            if (x == 0 || x == cols - 1) dx *= 2;
            if (y == 0 || y == rows - 1) dy *= 2;
            float acc = 0.0f;
            acc += dx * dx;
            acc += dy * dy;
            const float m = sqrtf(acc);
            out[(int64_t)y * cols + x] = m < 0.0f ? 0 : (m > 255.0f ? 255 : (uint8_t)feat_rndint(m));
        }
}

/* Operators::calcMeanFromHistogram / calcStdFromHistogram (Operators.cpp:281-313) */
static double feat_mean(const int *h) {
    double m = 0.0;
    int n = 0;
    for (int i = 0; i < 256; ++i) {
        m += h[i] * i;
        n += h[i];
    }
    return n == 0 ? 0.0 : m / n;
}
static double feat_std(const int *h) {
    double sum = 0.0, n = 0;
    for (int i = 0; i < 256; ++i) {
        sum += i * h[i];
        n += h[i];
    }
    const double mean = sum / n;
    double sq = 0.0;
    for (int i = 0; i < 256; ++i) {
        const double d = i - mean;
        sq += d * d * h[i];
    }
    return sqrt(sq / n);
}

/* For every component of a -1-background label image, in bounding-box order
 * (increasing label): ObjFeatures::area (ObjFeatures.cpp:15-43),
 * ObjFeatures::perimeter (:143-270, marching squares over the box and its
 * one-pixel ring, summed in the reference's order), and the histogram mean /
 * std of `gray` (intensityFeatures, :342-375) and the histogram mean of its
 * gradient (gradientFeatures, :377-418).  feat5 receives 5 floats per
 * component; returns the component count. */
int orc_nucleus_features(const int32_t *labels, const uint8_t *gray, int rows, int cols, float *feat5) {
    const int64_t n = (int64_t)rows * cols;
    int32_t *bb = (int32_t *)malloc(sizeof(int32_t) * 5 * (size_t)(n > 0 ? n : 1));
    const int cnt = orc_bounding_box(labels, cols, rows, bb);
    uint8_t *grad = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
    orc_gradient_u8(gray, rows, cols, grad);
    static const double lut[16] = {0.0,          0.70710678118, 0.70710678118, 1.0,
                                   0.70710678118, 1.41421356237, 1.0,           0.70710678118,
                                   0.70710678118, 1.0,           1.41421356237, 0.70710678118,
                                   1.0,           0.70710678118, 0.70710678118, 0.0};
    int hg[256], hd[256];
    for (int i = 0; i < cnt; ++i) {
        /* the five arrays of the box buffer: label, minx, maxx, miny, maxy */
        const int L = bb[i], x0 = bb[cnt + i], x1 = bb[2 * cnt + i], y0 = bb[3 * cnt + i], y1 = bb[4 * cnt + i];
#define LB(yy, xx) (labels[(int64_t)(yy) * cols + (xx)] == L)
        int area = 0;
        memset(hg, 0, sizeof hg);
        memset(hd, 0, sizeof hd);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x)
                if (LB(y, x)) {
                    ++area;
                    ++hg[gray[(int64_t)y * cols + x]];
                    ++hd[grad[(int64_t)y * cols + x]];
                }
        double per = 0.0;
        for (int y = y0; y < y1; ++y)
            for (int x = x0; x < x1; ++x) {
                int m = LB(y, x);
                m = (m << 1) | LB(y, x + 1);
                m = (m << 1) | LB(y + 1, x + 1);
                m = (m << 1) | LB(y + 1, x);
                per += lut[m];
            }
        for (int x = x0; x < x1; ++x) {
            int m = LB(y1, x);
            m = ((m << 1) | LB(y1, x + 1)) << 2;
            per += lut[m];
            m = LB(y0, x + 1);
            m = (m << 1) | LB(y0, x);
            per += lut[m];
        }
        for (int y = y0; y < y1; ++y) {
            int m = LB(y, x0);
            m = ((m << 1) | LB(y + 1, x0)) << 1;
            per += lut[m];
            m = LB(y, x1) << 2;
            m = (m << 1) | LB(y + 1, x1);
            per += lut[m];
        }
        per += lut[LB(y0, x0) << 1];
        per += lut[LB(y0, x1)];
        per += lut[LB(y1, x1) << 3];
        per += lut[LB(y1, x0) << 2];
#undef LB
        float *f = feat5 + 5 * (int64_t)i;
        f[0] = (float)area;
        f[1] = (float)per;
        f[2] = (float)feat_mean(hg);
        f[3] = (float)feat_std(hg);
        f[4] = (float)feat_mean(hd);
    }
    free(grad);
    free(bb);
    return cnt;
}
