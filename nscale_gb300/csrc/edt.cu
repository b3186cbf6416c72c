// edt.cu — exact Euclidean distance transform
// (cv::distanceTransform(seg_big, dist, CV_DIST_L2, CV_DIST_MASK_PRECISE),
// HistologicalEntities.cpp:359).
//
// OpenCV's precise L2 transform is separable: the distance to the nearest
// zero along each column, then the lower envelope of parabolas along each row,
// then sqrt of the float sum (out-of-image pixels are not zeros; an image with
// no zero at all gives sqrt(1e15f) everywhere).  Here:
//   pass 1  one thread per column, down and up sweeps -> column distance g
//           (coalesced across a warp: 32 neighbouring columns per row);
//   pass 2  per pixel, d^2 = min_x' g(x')^2 + (x-x')^2 searched outward from
//           x and stopped as soon as (x-x')^2 alone exceeds the best value,
//           so the work is proportional to the distance itself;
//   out     sqrtf((float)d^2), correctly rounded like the CPU's sqrt.
#include <limits.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int kInf = 1 << 29;

__global__ void edt_cols(const uint8_t *__restrict__ m, int *__restrict__ g, int rows, int cols, int *anyzero) {
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= cols) return;
    int d = kInf;
    bool z = false;
    for (int y = 0; y < rows; ++y) {
        int64_t i = (int64_t)y * cols + x;
        if (m[i] == 0) {
            d = 0;
            z = true;
        } else if (d != kInf) {
            d++;
        }
        g[i] = d;
    }
    d = kInf;
    for (int y = rows - 1; y >= 0; --y) {
        int64_t i = (int64_t)y * cols + x;
        if (m[i] == 0) d = 0;
        else if (d != kInf) d++;
        if (d < g[i]) g[i] = d;
    }
    if (z) atomicOr(anyzero, 1);
}

__global__ void edt_rows(const int *__restrict__ g, float *__restrict__ out, int rows, int cols,
                         const int *__restrict__ anyzero) {
    int64_t n = (int64_t)rows * cols;
    const bool az = *anyzero != 0;
    const float none = sqrtf(1e15f);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (!az) {
            out[i] = none;
            continue;
        }
        int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        const int *gr = g + (int64_t)y * cols;
        long long best = LLONG_MAX;
        int g0 = gr[x];
        if (g0 != kInf) best = (long long)g0 * g0;
        for (int k = 1; (long long)k * k < best; ++k) {
            bool l = x - k >= 0, r = x + k < cols;
            if (!l && !r) break;
            long long kk = (long long)k * k;
            if (l) {
                int gv = gr[x - k];
                if (gv != kInf) {
                    long long v = (long long)gv * gv + kk;
                    if (v < best) best = v;
                }
            }
            if (r) {
                int gv = gr[x + k];
                if (gv != kInf) {
                    long long v = (long long)gv * gv + kk;
                    if (v < best) best = v;
                }
            }
        }
        out[i] = __fsqrt_rn((float)best);
    }
}

}  // namespace

// scratch: i32[2] (column distances)
int dist_transform_dev(Ctx &c, const uint8_t *mask, float *dist, int rows, int cols, cudaStream_t s) {
    int *g = c.ws.i32[2];
    int *anyz = c.ws.ctrl + C_FLAG0;
    NSG_CUDA_TRY(c, cudaMemsetAsync(anyz, 0, sizeof(int), s));
    edt_cols<<<(cols + 127) / 128, 128, 0, s>>>(mask, g, rows, cols, anyz);
    NSG_COUNT_LAUNCH();
    int64_t n = (int64_t)rows * cols;
    int64_t gb = (n + 255) / 256;
    if (gb > (int64_t)c.sm_count * 16) gb = (int64_t)c.sm_count * 16;
    edt_rows<<<(int)gb, 256, 0, s>>>(g, dist, rows, cols, anyz);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

}  // namespace nsg
