// minima.cu — h-minima transform and regional extrema on float32 images.
//
//  * imhmin<float>(img, h, conn)      MorphologicOperations.cpp:3343-3364:
//        invert, marker = mask - h (float), reconstruct, invert back.
//  * localMaxima<float>(img, conn)    MorphologicOperations.cpp:3764-3836 and
//    localMinima<float>               MorphologicOperations.cpp:3839-3845:
//        candidates = !((img-1) < recon(img-1, img, conn));
//        the reference then flood-fills (cv::floodFill, zero tolerance,
//        conn-connected) every equal-valued candidate plateau that contains a
//        pixel with a strictly greater neighbour.  That set does not depend on
//        the scan order, so it is computed as: label equal-valued candidate
//        plateaus (union-find), flag a plateau when any of its pixels has a
//        strictly greater conn-neighbour (out-of-image = -FLT_MAX, never
//        greater), keep the unflagged candidates.
#include <float.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int kB = 256;

// img may be the caller's output plane too (in-place imhmin): each thread
// reads its pixel before writing it, so no __restrict__ on img / marker
__global__ void hmin_prep(const float *img, float h, float *__restrict__ mask, float *marker, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float m = -img[i];
        mask[i] = m;
        marker[i] = __fadd_rn(m, -h);
    }
}
// the segmentation's imhmin input built from the distance transform: the
// pipeline's distance is -dist inside seg_big and -FLT_MAX outside
// (HistologicalEntities.cpp:366-374) and imhmin negates it again, so the
// reconstruction's mask is dist / FLT_MAX directly (negation is exact)
__global__ void hmin_prep_dist(const float *__restrict__ dist, const uint8_t *__restrict__ seg, float h,
                               float *__restrict__ mask, float *__restrict__ marker, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float m = seg[i] ? dist[i] : FLT_MAX;
        mask[i] = m;
        marker[i] = __fadd_rn(m, -h);
    }
}
// maxima: the candidates' marker c - 1, the image itself serving as c
__global__ void ext_marker(const float *__restrict__ c, float *__restrict__ marker, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        marker[i] = __fadd_rn(c[i], -1.0f);
}
__global__ void negate(float *__restrict__ a, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        a[i] = -a[i];
}
// c = the image (negated for minima); marker = c - 1, written straight into
// the reconstruction's output (it is <= c everywhere, so it is already
// min(marker, c)); ext_cand recomputes the same marker value from c
__global__ void ext_prep(const float *__restrict__ img, bool neg, float *__restrict__ c, float *__restrict__ marker,
                         int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float v = neg ? -img[i] : img[i];
        c[i] = v;
        marker[i] = __fadd_rn(v, -1.0f);
    }
}
__global__ void ext_cand(const float *__restrict__ c, const float *__restrict__ rec, uint8_t *__restrict__ cand,
                         int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        cand[i] = (__fadd_rn(c[i], -1.0f) < rec[i]) ? 0 : 1;
}
__global__ void ext_zero_roots(const int *__restrict__ lab, int *__restrict__ flag, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (lab[i] == (int)i) flag[i] = 0;
}
__global__ void ext_flag(const float *__restrict__ c, const int *__restrict__ lab, int *__restrict__ flag, int rows,
                         int cols, int conn) {
    int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int l = lab[i];
        if (l < 0) continue;
        int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        float v = c[i];
        bool g = false;
        if (y > 0 && v < c[i - cols]) g = true;
        if (y < rows - 1 && v < c[i + cols]) g = true;
        if (x > 0 && v < c[i - 1]) g = true;
        if (x < cols - 1 && v < c[i + 1]) g = true;
        if (conn == 8) {
            if (y > 0 && x > 0 && v < c[i - cols - 1]) g = true;
            if (y > 0 && x < cols - 1 && v < c[i - cols + 1]) g = true;
            if (y < rows - 1 && x > 0 && v < c[i + cols - 1]) g = true;
            if (y < rows - 1 && x < cols - 1 && v < c[i + cols + 1]) g = true;
        }
        if (g && !__ldcg(flag + l)) flag[l] = 1;
    }
}
__global__ void ext_out(const int *__restrict__ lab, const int *__restrict__ flag, uint8_t *__restrict__ out,
                        int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int l = lab[i];
        out[i] = (l >= 0 && !flag[l]) ? 255 : 0;
    }
}

int blocks(Ctx &c, int64_t n) {
    int64_t g = (n + kB - 1) / kB;
    int64_t cap = (int64_t)c.sm_count * 16;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

// scratch: f32[0..1], recon's i32[5]
int imhmin_dev(Ctx &c, const float *img, float *out, int rows, int cols, float h, int conn, cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    // h >= 0: the marker (mask - h <= mask) goes straight into the
    // reconstruction's output, which is then already min(marker, mask)
    const bool direct = h >= 0.0f;
    float *mask = c.ws.f32[0], *marker = direct ? out : c.ws.f32[1];
    hmin_prep<<<blocks(c, n), kB, 0, s>>>(img, h, mask, marker, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_TRY(recon_f32(c, marker, mask, out, rows, cols, conn, s, direct));
    negate<<<blocks(c, n), kB, 0, s>>>(out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// The pipeline's imhmin, kept negated: out = -imhmin(distance, h, conn) where
// distance = -dist inside seg and -FLT_MAX outside.  imhmin negates its
// input, reconstructs and negates back, and watershed2's localMinima negates
// the result once more; here the negations fold away (each is exact), the
// reconstruction's output is returned as it is, and the watershed takes its
// minima as the maxima of this plane.  scratch: f32[0], recon's i32[5]
int imhmin_neg_dist_dev(Ctx &c, const float *dist, const uint8_t *seg, float *out, int rows, int cols, float h,
                        int conn, cudaStream_t s) {
    if (!(h >= 0.0f)) return NSG_ERR_ARG;  // the marker must stay <= the mask
    int64_t n = (int64_t)rows * cols;
    float *mask = c.ws.f32[0];
    hmin_prep_dist<<<blocks(c, n), kB, 0, s>>>(dist, seg, h, mask, out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return recon_f32(c, out, mask, out, rows, cols, conn, s, true);
}

// scratch: f32[0] (minima) and f32[2], u8[0], i32[0..1], recon's i32[5]
int local_extrema_dev(Ctx &c, const float *img, uint8_t *out, int rows, int cols, int conn, bool minima,
                      cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    float *rec = c.ws.f32[2];
    uint8_t *cand = c.ws.u8[0];
    int *lab = c.ws.i32[0], *flag = c.ws.i32[1];
    int g = blocks(c, n);
    // c = the image for maxima (read in place), its negation for minima
    const float *cim = img;
    if (minima) {
        ext_prep<<<g, kB, 0, s>>>(img, true, c.ws.f32[0], rec, n);
        cim = c.ws.f32[0];
    } else {
        ext_marker<<<g, kB, 0, s>>>(img, rec, n);
    }
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_TRY(recon_f32(c, rec, cim, rec, rows, cols, conn, s, true));
    ext_cand<<<g, kB, 0, s>>>(cim, rec, cand, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_TRY(ccl_f32_masked(c, cim, cand, lab, rows, cols, conn, s));
    ext_zero_roots<<<g, kB, 0, s>>>(lab, flag, n);
    NSG_COUNT_LAUNCH();
    ext_flag<<<g, kB, 0, s>>>(cim, lab, flag, rows, cols, conn);
    NSG_COUNT_LAUNCH();
    ext_out<<<g, kB, 0, s>>>(lab, flag, out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

}  // namespace nsg
