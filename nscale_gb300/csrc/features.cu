// features.cu — per-nucleus features of the serving output, from the label
// image and a grey channel (normally the hematoxylin channel of deconv.cu):
//
//  * gradient magnitude (Operators::gradient, Operators.cpp:568-640);
//  * area (ObjFeatures::area, ObjFeatures.cpp:15-43);
//  * perimeter (ObjFeatures::perimeter, ObjFeatures.cpp:143-270): marching
//    squares over every 2 x 2 cell that touches the component;
//  * mean / std of the grey channel and mean of its gradient, from 256-bin
//    histograms (intensityFeatures / gradientFeatures, ObjFeatures.cpp:342-418;
//    Operators.cpp:281-313).
//
// Components are numbered in bounding-box order (increasing label = first
// raster appearance) by a scan of the root flags.  Histograms and the three
// perimeter cell classes are integer counts gathered with atomics, so they are
// exact; the finishing pass per component sums them in the reference's order
// without fused multiply-adds.
#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int kB = 256;

__device__ __forceinline__ int rndint_u8(float n) {  // Operators.cpp:554-564, then clamped
    if (n < 0.0f) return 0;
    if (n > 255.0f) return 255;
    const float f = floorf(n);
    return (int)f + (n - f >= 0.5f ? 1 : 0);
}

__global__ void gradient_kernel(const uint8_t *__restrict__ in, int rows, int cols, uint8_t *__restrict__ out) {
    const int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        const int xl = x > 0 ? x - 1 : 0, xr = x + 1 < cols ? x + 1 : cols - 1;
        const int yu = y > 0 ? y - 1 : 0, yd = y + 1 < rows ? y + 1 : rows - 1;
        // halves of integers: every step below is exact in float
        float dx = -0.5f * (float)in[(int64_t)y * cols + xl] + 0.5f * (float)in[(int64_t)y * cols + xr];
        float dy = -0.5f * (float)in[(int64_t)yu * cols + x] + 0.5f * (float)in[(int64_t)yd * cols + x];
        if (x == 0 || x == cols - 1) dx *= 2.0f;
        if (y == 0 || y == rows - 1) dy *= 2.0f;
        const float m = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
        out[i] = (uint8_t)rndint_u8(m);
    }
}

__global__ void root_index_flags(const int32_t *__restrict__ lab, int32_t *__restrict__ f, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        f[i] = lab[i] == (int32_t)i ? 1 : 0;
}

// per-pixel histograms of the grey channel and of its gradient
__global__ void feat_hist(const int32_t *__restrict__ lab, const int32_t *__restrict__ pos,
                          const uint8_t *__restrict__ gray, const uint8_t *__restrict__ grad, int64_t n, int cnt,
                          int *__restrict__ hg, int *__restrict__ hd) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int l = lab[i];
        if (l < 0) continue;
        const int k = pos[l];
        if (k >= cnt) continue;
        atomicAdd(hg + (int64_t)k * 256 + gray[i], 1);
        atomicAdd(hd + (int64_t)k * 256 + grad[i], 1);
    }
}

// marching-squares cells (x, y) for x in [-1, cols-1], y in [-1, rows-1]:
// corners (x,y) (x+1,y) (x+1,y+1) (x,y+1) give mask bits 3, 2, 1, 0; outside
// the image is background.  Class 1 (one or three corners): 1/sqrt(2);
// class 2 (two adjacent): 1; class 3 (two diagonal): sqrt(2).
__device__ __forceinline__ int cell_class(int m) {
    switch (m) {
        case 3: case 6: case 9: case 12: return 2;
        case 5: case 10: return 3;
        case 0: case 15: return 0;
        default: return 1;
    }
}

__global__ void feat_perimeter(const int32_t *__restrict__ lab, const int32_t *__restrict__ pos, int rows, int cols,
                               int cnt, int *__restrict__ pc) {
    const int64_t nc = (int64_t)(rows + 1) * (cols + 1);
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(c / (cols + 1)) - 1, x = (int)(c - (int64_t)(y + 1) * (cols + 1)) - 1;
        int v[4];  // bits 3, 2, 1, 0
        v[0] = (y >= 0 && x >= 0) ? lab[(int64_t)y * cols + x] : -1;
        v[1] = (y >= 0 && x + 1 < cols) ? lab[(int64_t)y * cols + x + 1] : -1;
        v[2] = (y + 1 < rows && x + 1 < cols) ? lab[(int64_t)(y + 1) * cols + x + 1] : -1;
        v[3] = (y + 1 < rows && x >= 0) ? lab[(int64_t)(y + 1) * cols + x] : -1;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int L = v[j];
            if (L < 0) continue;
            bool seen = false;
            for (int t = 0; t < j; ++t) seen |= v[t] == L;
            if (seen) continue;  // each label of the cell once
            const int m = ((v[0] == L) << 3) | ((v[1] == L) << 2) | ((v[2] == L) << 1) | (v[3] == L);
            const int cls = cell_class(m);
            const int k = pos[L];
            if (cls && k < cnt) atomicAdd(pc + (int64_t)k * 3 + (cls - 1), 1);
        }
    }
}

__device__ double hist_mean(const int *h) {  // Operators.cpp:281-292
    double m = 0.0;
    int n = 0;
    for (int i = 0; i < 256; ++i) {
        m = __dadd_rn(m, (double)(h[i] * i));
        n += h[i];
    }
    return n == 0 ? 0.0 : __ddiv_rn(m, (double)n);
}
__device__ double hist_std(const int *h) {  // Operators.cpp:296-313
    double sum = 0.0, n = 0.0;
    for (int i = 0; i < 256; ++i) {
        sum = __dadd_rn(sum, (double)(i * h[i]));
        n = __dadd_rn(n, (double)h[i]);
    }
    const double mean = __ddiv_rn(sum, n);
    double sq = 0.0;
    for (int i = 0; i < 256; ++i) {
        const double d = __dsub_rn((double)i, mean);
        sq = __dadd_rn(sq, __dmul_rn(__dmul_rn(d, d), (double)h[i]));
    }
    return __dsqrt_rn(__ddiv_rn(sq, n));
}

__global__ void feat_finish(const int *__restrict__ hg, const int *__restrict__ hd, const int *__restrict__ pc,
                            int cnt, float *__restrict__ out) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
        const int *g = hg + (int64_t)k * 256;
        int area = 0;
        for (int i = 0; i < 256; ++i) area += g[i];
        const int *p = pc + (int64_t)k * 3;
        const double per = __dadd_rn(__dadd_rn(__dmul_rn((double)p[0], 0.70710678118), (double)p[1]),
                                     __dmul_rn((double)p[2], 1.41421356237));
        float *f = out + (int64_t)k * 5;
        f[0] = (float)area;
        f[1] = (float)per;
        f[2] = (float)hist_mean(g);
        f[3] = (float)hist_std(g);
        f[4] = (float)hist_mean(hd + (int64_t)k * 256);
    }
}

int grid_for(Ctx &c, int64_t n) {
    int64_t g = (n + kB - 1) / kB;
    const int64_t cap = (int64_t)c.sm_count * 16;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

int gradient_dev(Ctx &c, const uint8_t *in, uint8_t *out, int rows, int cols, cudaStream_t s) {
    gradient_kernel<<<grid_for(c, (int64_t)rows * cols), kB, 0, s>>>(in, rows, cols, out);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// scratch: i32[0] root flags -> component index, i32[1] grey histograms,
// i32[2] gradient histograms, i32[3] perimeter classes, u8[0] gradient image.
// The component count is read back to size the passes (it is returned).
int nucleus_features_dev(Ctx &c, const int32_t *labels, const uint8_t *gray, int rows, int cols, float *out,
                         int capacity, int *count, cudaStream_t s) {
    const int64_t n = (int64_t)rows * cols;
    int32_t *pos = c.ws.i32[0];
    int *hg = c.ws.i32[1], *hd = c.ws.i32[2], *pc = c.ws.i32[3];
    uint8_t *grad = c.ws.u8[0];
    int32_t *d_cnt = c.ws.ctrl + C_COUNT0;
    root_index_flags<<<grid_for(c, n), kB, 0, s>>>(labels, pos, n);
    NSG_COUNT_LAUNCH();
    NSG_TRY(exclusive_scan_i32(c, pos, pos, n, d_cnt, s));
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl + C_COUNT0, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaStreamSynchronize(s));
    const int cnt = c.ws.h_ctrl[C_COUNT0];
    *count = cnt;
    if (cnt > capacity || (int64_t)cnt * 256 > c.max_pad) {
        c.last_error = "more components than the output (or the workspace) holds";
        return NSG_ERR_ARG;
    }
    if (cnt == 0) return NSG_SUCCESS;
    NSG_TRY(gradient_dev(c, gray, grad, rows, cols, s));
    NSG_CUDA_TRY(c, cudaMemsetAsync(hg, 0, sizeof(int) * 256 * (size_t)cnt, s));
    NSG_CUDA_TRY(c, cudaMemsetAsync(hd, 0, sizeof(int) * 256 * (size_t)cnt, s));
    NSG_CUDA_TRY(c, cudaMemsetAsync(pc, 0, sizeof(int) * 3 * (size_t)cnt, s));
    feat_hist<<<grid_for(c, n), kB, 0, s>>>(labels, pos, gray, grad, n, cnt, hg, hd);
    NSG_COUNT_LAUNCH();
    feat_perimeter<<<grid_for(c, (int64_t)(rows + 1) * (cols + 1)), kB, 0, s>>>(labels, pos, rows, cols, cnt, pc);
    NSG_COUNT_LAUNCH();
    feat_finish<<<grid_for(c, cnt), kB, 0, s>>>(hg, hd, pc, cnt, out);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

}  // namespace nsg
