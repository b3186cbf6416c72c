// normalize.cu — colour normalisation before segmentation
// (nscale::Normalization, src/normalization/Normalization.cpp, called by the
// reference's test driver before segmentNuclei, nu-segmentTest.cpp:200).
//
// Reinhard colour transfer: pixels that a Fisher discriminant calls
// foreground (segFG, Normalization.cpp:19-55) are taken to lab space
// (bgr2Lab, :64-149), shifted and scaled channel by channel from their own
// mean / std to the target's (TransferI, :296-350), and every pixel goes back
// through lab2BGR (:166-292).  targetParameters (:520-577) is the statistics
// step alone.  Two fused pointwise passes over the BGR tile:
//   1. norm_stats: discriminant, lab, and the foreground's count, sums and
//      sums of squares (double, block-reduced, one atomic per block);
//   2. norm_apply: discriminant and lab again, the transfer for foreground
//      pixels, lab2BGR, uint8 BGR out.
// The arithmetic follows the reference's order and widths (float where it
// computes on float matrices, double for its double literals and sums;
// separate roundings: no fused multiply-add); log10f and powf are CUDA's,
// so an output level can differ by one where a value sits on a rounding
// boundary (the tests bound and count those).
#include <float.h>
#include <math.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int kB = 256;

__constant__ float kM[8] = {-0.154f, 0.035f, 0.549f, -45.718f, -0.057f, -0.817f, 1.170f, -49.887f};

__device__ __forceinline__ bool seg_fg(float bd, float gd, float rd) {
    float d[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const float *m = kM + 4 * k;
        const float t = (float)__dadd_rn(__dmul_rn((double)rd, (double)m[0]), __dmul_rn((double)gd, (double)m[1]));
        d[k] = (float)__dadd_rn(__dadd_rn((double)t, __dmul_rn((double)bd, (double)m[2])), (double)m[3]);
    }
    return d[0] < d[1];
}

struct Consts {
    float i3, i6, i2;
};
__device__ __forceinline__ Consts consts() {
    return Consts{__fdiv_rn(1.0f, sqrtf(3.0f)), __fdiv_rn(1.0f, sqrtf(6.0f)), __fdiv_rn(1.0f, sqrtf(2.0f))};
}

// a + b + c in float, left to right, each product rounded
__device__ __forceinline__ float dot3(float x, float a, float y, float b, float z, float c) {
    return __fadd_rn(__fadd_rn(__fmul_rn(x, a), __fmul_rn(y, b)), __fmul_rn(z, c));
}

__device__ __forceinline__ void to_lab(float B, float G, float R, const Consts &k, float lab[3]) {
    const float s = (float)(1.0 / 255.0);
    const float b = __fmul_rn(B, s), g = __fmul_rn(G, s), r = __fmul_rn(R, s);
    const double rd = r, gd = g, bd = b;
    const float L = (float)__dadd_rn(__dadd_rn(__dmul_rn(0.3811, rd), __dmul_rn(0.5783, gd)), __dmul_rn(0.0402, bd));
    const float M = (float)__dadd_rn(__dadd_rn(__dmul_rn(0.1967, rd), __dmul_rn(0.7244, gd)), __dmul_rn(0.0782, bd));
    const float S = (float)__dadd_rn(__dadd_rn(__dmul_rn(0.0241, rd), __dmul_rn(0.1288, gd)), __dmul_rn(0.8444, bd));
    const float l = log10f(L), m = log10f(M), sl = log10f(S);
    lab[0] = dot3(l, k.i3, m, k.i3, sl, k.i3);
    lab[1] = dot3(l, k.i6, m, k.i6, sl, -2.0f * k.i6);
    lab[2] = dot3(l, k.i2, m, -k.i2, sl, 0.0f);
}

__device__ __forceinline__ int rndint(float n) {
    const float f = floorf(n);
    int ret = (int)f;
    if (__fsub_rn(n, f) >= 0.5f) ret = (int)f + 1;
    return ret;
}

__device__ __forceinline__ void to_bgr(const float lab[3], const Consts &k, uint8_t *out) {
    float lms[3];
    lms[0] = dot3(lab[0], k.i3, lab[1], k.i6, lab[2], k.i2);
    lms[1] = dot3(lab[0], k.i3, lab[1], k.i6, lab[2], -k.i2);
    lms[2] = dot3(lab[0], k.i3, lab[1], -2.0f * k.i6, lab[2], 0.0f);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float x = powf(10.0f, lms[c]);
        if (!(x <= FLT_MAX && x >= -FLT_MAX)) x = 0.0f;  // -Inf / NaN -> 0
        lms[c] = x;
    }
    const float bf = dot3(lms[0], 0.0585f, lms[1], -0.2611f, lms[2], 1.2057f);
    const float gf = dot3(lms[0], -1.2197f, lms[1], 2.3831f, lms[2], -0.1626f);
    const float rf = dot3(lms[0], 4.4687f, lms[1], -3.5887f, lms[2], 0.1196f);
    const float v[3] = {bf, gf, rf};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        float sc = (float)__dmul_rn((double)v[c], 255.0);
        if (sc < 0.0f) sc = 0.0f;
        if (sc > 255.0f) sc = 255.0f;
        out[c] = (uint8_t)rndint(sc);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// acc[0] count, [1..3] sums, [4..6] sums of squares (double)
__global__ void __launch_bounds__(kB) norm_stats(const uint8_t *__restrict__ bgr, int64_t stride, int rows, int cols,
                                                 double *acc) {
    const Consts k = consts();
    double v[7] = {0, 0, 0, 0, 0, 0, 0};
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        const uint8_t *px = bgr + y * stride + 3 * x;
        const float B = px[0], G = px[1], R = px[2];
        if (!seg_fg(B, G, R)) continue;
        float lab[3];
        to_lab(B, G, R, k, lab);
        if (!(__fmul_rn(__fmul_rn(lab[0], lab[1]), lab[2]) > 0.0f)) continue;
        v[0] += 1.0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            v[1 + c] += (double)lab[c];
            v[4 + c] += (double)__fmul_rn(lab[c], lab[c]);
        }
    }
    __shared__ double part[kB / 32][7];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < 7; ++j) {
        const double w = warp_sum(v[j]);
        if (lane == 0) part[warp][j] = w;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        double t = 0;
        for (int w = 0; w < kB / 32; ++w) t += part[w][threadIdx.x];
        if (t != 0.0) atomicAdd(acc + threadIdx.x, t);
    }
}

// coef[0..2] own mean, [3..5] stdT / std, [6..8] target mean
__global__ void __launch_bounds__(kB) norm_apply(const uint8_t *__restrict__ bgr, int64_t stride, int rows, int cols,
                                                 const float *__restrict__ coef, uint8_t *__restrict__ out,
                                                 int64_t ostride) {
    const Consts k = consts();
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        const uint8_t *px = bgr + y * stride + 3 * x;
        const float B = px[0], G = px[1], R = px[2];
        float lab[3];
        to_lab(B, G, R, k, lab);
        if (seg_fg(B, G, R)) {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                lab[c] = __fadd_rn(__fmul_rn(__fsub_rn(lab[c], coef[c]), coef[3 + c]), coef[6 + c]);
        }
        uint8_t o[3];
        to_bgr(lab, k, o);
        uint8_t *q = out + y * ostride + 3 * x;
        q[0] = o[0];
        q[1] = o[1];
        q[2] = o[2];
    }
}

int blocks(Ctx &c, int64_t n) {
    int64_t g = (n + kB - 1) / kB;
    int64_t cap = (int64_t)c.sm_count * 8;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

// foreground lab mean / std (as floats, the reference's meanLAB / stdLAB);
// synchronises the stream
int norm_params(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, float *mean3, float *std3,
                cudaStream_t s) {
    double *acc = reinterpret_cast<double *>(c.ws.ctr64 + 16);
    NSG_CUDA_TRY(c, cudaMemsetAsync(acc, 0, 7 * sizeof(double), s));
    norm_stats<<<blocks(c, (int64_t)rows * cols), kB, 0, s>>>(bgr, stride, rows, cols, acc);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    double h[7];
    NSG_CUDA_TRY(c, cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaStreamSynchronize(s));
    for (int k = 0; k < 3; ++k) {
        const double mean = h[1 + k] / h[0];
        const double var = h[4 + k] / h[0] - mean * mean;
        mean3[k] = (float)mean;
        std3[k] = (float)sqrt(var);
    }
    return NSG_SUCCESS;
}

}  // namespace

}  // namespace nsg

using namespace nsg;

extern "C" {

int nsg_color_target_parameters(nsg_context *h, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                                float *mean3, float *std3, nsg_stream_t stream) {
    if (!h || !bgr || !mean3 || !std3) return NSG_ERR_ARG;
    Ctx &c = h->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return NSG_ERR_CUDA;
    NSG_TRY(check_dims(c, rows, cols));
    const int64_t stride = row_stride_bytes ? (int64_t)row_stride_bytes : (int64_t)cols * 3;
    if (stride < (int64_t)cols * 3) return NSG_ERR_ARG;
    return norm_params(c, bgr, stride, rows, cols, mean3, std3, (cudaStream_t)stream);
}

int nsg_color_normalization(nsg_context *h, const uint8_t *bgr, int rows, int cols, size_t row_stride_bytes,
                            const float *target_mean3, const float *target_std3, uint8_t *out_bgr,
                            nsg_stream_t stream) {
    if (!h || !bgr || !target_mean3 || !target_std3 || !out_bgr) return NSG_ERR_ARG;
    Ctx &c = h->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return NSG_ERR_CUDA;
    NSG_TRY(check_dims(c, rows, cols));
    const int64_t stride = row_stride_bytes ? (int64_t)row_stride_bytes : (int64_t)cols * 3;
    if (stride < (int64_t)cols * 3) return NSG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    float mean[3], sd[3];
    NSG_TRY(norm_params(c, bgr, stride, rows, cols, mean, sd, s));
    float coef[9];
    for (int k = 0; k < 3; ++k) {
        coef[k] = mean[k];
        coef[3 + k] = target_std3[k] / sd[k];  // float / float, as the reference's stdT / stdLAB
        coef[6 + k] = target_mean3[k];
    }
    float *d_coef = reinterpret_cast<float *>(c.ws.ctr64 + 32);
    NSG_CUDA_TRY(c, cudaMemcpyAsync(d_coef, coef, sizeof(coef), cudaMemcpyHostToDevice, s));
    norm_apply<<<blocks(c, (int64_t)rows * cols), kB, 0, s>>>(bgr, stride, rows, cols, d_coef, out_bgr,
                                                               (int64_t)cols * 3);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_CUDA_TRY(c, cudaStreamSynchronize(s));  // coef lives on this call's stack
    return NSG_SUCCESS;
}

}  // extern "C"
