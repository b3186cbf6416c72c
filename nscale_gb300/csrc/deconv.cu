// deconv.cu — colour deconvolution into hematoxylin and eosin channels
// (nscale::PixelOperations::ComputeInverseStainMatrix / ComputeLookupTable /
// ColorDeconv, PixelOperations.cpp:94-274).  Not part of segmentNuclei; the
// per-nucleus features of the serving configuration read its H channel.
//
// Host: the 2 x 3 inverse stain matrix and the 256-entry optical-density
// table are computed in double, as the reference computes them.  Device: one
// pass, 3 B read and 2 B written per pixel; the 3-term product of each output
// channel is summed in double in B, G, R order with each product rounded (as
// OpenCV's 32-bit matrix product sums it), then expf and round-half-even
// saturation to uint8.
#include <math.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

struct DeconvConst {
    float lut[256];
    float q[6];  // rows H, E; columns R, G, B
    float c;     // (float)(-ln 255 / 255)
};

__device__ __forceinline__ uint8_t sat_rn_u8(float v) {
    int r = __float2int_rn(v);
    return (uint8_t)(r < 0 ? 0 : (r > 255 ? 255 : r));
}

__device__ __forceinline__ float dot_bgr(double db, double dg, double dr, const float *q) {
    // no fused multiply-add: each product rounds before the sum
    return (float)__dadd_rn(__dadd_rn(__dmul_rn(db, (double)q[2]), __dmul_rn(dg, (double)q[1])),
                            __dmul_rn(dr, (double)q[0]));
}

__global__ void deconv_kernel(const uint8_t *__restrict__ bgr, int64_t stride, int rows, int cols, DeconvConst k,
                              uint8_t *__restrict__ H, uint8_t *__restrict__ E) {
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        const uint8_t *p = bgr + (int64_t)y * stride + 3 * x;
        const double db = k.lut[p[0]], dg = k.lut[p[1]], dr = k.lut[p[2]];
        if (H) H[i] = sat_rn_u8(expf((dot_bgr(db, dg, dr, k.q) - 255.0f) * k.c));
        if (E) E[i] = sat_rn_u8(expf((dot_bgr(db, dg, dr, k.q + 3) - 255.0f) * k.c));
    }
}

}  // namespace

// PixelOperations::ComputeInverseStainMatrix (PixelOperations.cpp:94-156):
// normalised stain columns, a completed third column when it is zero, the
// inverse by Gaussian elimination with partial pivoting (Mat::inv with
// DECOMP_LU), the first two rows selected by b.  Returns the rows kept.
int stain_matrix(const double *M9, const uint8_t *b3, double *Q6) {
    double N[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) N[r][c] = M9[r * 3 + c];
    for (int c = 0; c < 3; ++c) {
        const double nrm = sqrt(N[0][c] * N[0][c] + N[1][c] * N[1][c] + N[2][c] * N[2][c]);
        if (nrm > 0)
            for (int r = 0; r < 3; ++r) N[r][c] /= nrm;
    }
    if (sqrt(N[0][2] * N[0][2] + N[1][2] * N[1][2] + N[2][2] * N[2][2]) == 0) {
        for (int r = 0; r < 3; ++r) {
            const double nrm = sqrt(N[r][0] * N[r][0] + N[r][1] * N[r][1] + N[r][2] * N[r][2]);
            N[r][2] = nrm > 1 ? 0 : sqrt(1 - nrm * nrm);
        }
        const double n2 = sqrt(N[0][2] * N[0][2] + N[1][2] * N[1][2] + N[2][2] * N[2][2]);
        if (n2 == 0) return 0;
        for (int r = 0; r < 3; ++r) N[r][2] /= n2;
    }
    double A[3][6];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 6; ++c) A[r][c] = c < 3 ? N[r][c] : (c - 3 == r ? 1.0 : 0.0);
    for (int k = 0; k < 3; ++k) {
        int piv = k;
        for (int r = k + 1; r < 3; ++r)
            if (fabs(A[r][k]) > fabs(A[piv][k])) piv = r;
        if (A[piv][k] == 0) return 0;  // singular
        if (piv != k)
            for (int c = 0; c < 6; ++c) {
                const double t = A[k][c];
                A[k][c] = A[piv][c];
                A[piv][c] = t;
            }
        const double d = A[k][k];
        for (int c = 0; c < 6; ++c) A[k][c] /= d;
        for (int r = 0; r < 3; ++r) {
            if (r == k) continue;
            const double f = A[r][k];
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

int color_deconv_dev(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, const float *Q6, uint8_t *H,
                     uint8_t *E, cudaStream_t s) {
    DeconvConst k;
    const float kk = (float)(-255.0 / log(255.0));  // PixelOperations.cpp:161-166
    for (int i = 0; i < 256; ++i) k.lut[i] = (float)((double)kk * log((double)(float)i + 1.0) + 255.0);
    for (int i = 0; i < 6; ++i) k.q[i] = Q6[i];
    k.c = (float)(-log(255.0) / 255.0);  // PixelOperations.cpp:238
    const int64_t n = (int64_t)rows * cols;
    int64_t g = (n + 255) / 256;
    if (g > (int64_t)c.sm_count * 16) g = (int64_t)c.sm_count * 16;
    deconv_kernel<<<(int)(g < 1 ? 1 : g), 256, 0, s>>>(bgr, stride, rows, cols, k, H, E);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

}  // namespace nsg
