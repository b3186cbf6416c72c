// pixel.cu — the elementwise stages of segmentNuclei, fused where the
// reference runs them back to back.
//
//  * background test + count       HistologicalEntities.cpp:93-109, 123-137
//  * RBC ratio masks, red invert   HistologicalEntities.cpp:54-71, 158
//  * diffIm thresholds             HistologicalEntities.cpp:211, 227, 279
//  * masks / negated distances     HistologicalEntities.cpp:295, 366-374, 407
#include <float.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void warp_add_u64(unsigned long long *dst, unsigned v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, (unsigned long long)v);
}

// 16 pixels per thread along a row: 48 contiguous bytes of BGR.
template <int PX>
__global__ void background_kernel(const uint8_t *__restrict__ bgr, int64_t stride, int rows, int cols, int blue,
                                  int green, int red, uint8_t *__restrict__ mask,
                                  unsigned long long *__restrict__ count) {
    int64_t chunks_per_row = (cols + PX - 1) / PX;
    int64_t total = chunks_per_row * rows;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t - threadIdx.x < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        unsigned cnt = 0;
        if (t < total) {
            int y = (int)(t / chunks_per_row);
            int x0 = (int)(t - (int64_t)y * chunks_per_row) * PX;
            const uint8_t *row = bgr + (int64_t)y * stride;
#pragma unroll
            for (int k = 0; k < PX; ++k) {
                int x = x0 + k;
                if (x < cols) {
                    const uint8_t *p = row + 3 * x;
                    bool on = p[0] > blue && p[1] > green && p[2] > red;
                    cnt += on;
                    if (mask) mask[(int64_t)y * cols + x] = on ? 255 : 0;
                }
            }
        }
        warp_add_u64(count, cnt);
    }
}

// getRBC's float32 ratios and the red-channel complement in one pass.
__global__ void front_rbc_kernel(const uint8_t *__restrict__ bgr, int64_t stride, int rows, int cols, float t1,
                                 float t2, uint8_t *__restrict__ rc, uint8_t *__restrict__ bw1,
                                 uint8_t *__restrict__ bw2, uint8_t *__restrict__ r2b, int *__restrict__ bw1_count) {
    int64_t n = (int64_t)rows * cols;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = i0 + threadIdx.x;
        unsigned on1 = 0;
        if (i < n) {
            int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
            const uint8_t *p = bgr + (int64_t)y * stride + 3 * x;
            uint8_t B = p[0], G = p[1], R = p[2];
            // convertTo(CV_32F, 1.0, FLT_EPSILON) on B and G, plain convert on R
            float bd = __fadd_rn((float)B, FLT_EPSILON);
            float gd = __fadd_rn((float)G, FLT_EPSILON);
            float rd = (float)R;
            float r2g = __fdiv_rn(rd, gd);
            float rb = __fdiv_rn(rd, bd);
            on1 = r2g > t1;
            bw1[i] = on1 ? 255 : 0;
            bw2[i] = r2g > t2 ? 255 : 0;
            r2b[i] = rb > 1.0f ? 255 : 0;
            rc[i] = (uint8_t)(255 - R);
        }
        unsigned b = __ballot_sync(0xffffffffu, on1);
        if ((threadIdx.x & 31) == 0 && b) atomicAdd(bw1_count, __popc(b));
    }
}

// The front of segmentNuclei in one pass over the tile, 16 pixels per thread
// with 128-bit accesses: three 16-byte loads of BGR, the background test
// (HE:93-109, counted), getRBC's float32 ratios (HE:54-71) and the red
// complement (HE:158) for the 16 pixels, four 16-byte stores.  Consecutive
// threads take consecutive 16-pixel chunks of a row.  Needs cols % 16 == 0 and
// a 16-byte aligned tile, row stride and outputs (front_fused checks).
union V16 {
    uint4 u;
    uint8_t b[16];
};
__device__ __forceinline__ void front_px(uint8_t B, uint8_t G, uint8_t R, int blue, int green, int red, float t1,
                                         float t2, unsigned &bg, uint8_t &rc, uint8_t &b1, uint8_t &b2,
                                         uint8_t &r2b) {
    bg += (B > blue && G > green && R > red) ? 1u : 0u;
    const float bd = __fadd_rn((float)B, FLT_EPSILON);
    const float gd = __fadd_rn((float)G, FLT_EPSILON);
    const float rd = (float)R;
    const float r2g = __fdiv_rn(rd, gd), rb = __fdiv_rn(rd, bd);
    b1 = r2g > t1 ? 255 : 0;
    b2 = r2g > t2 ? 255 : 0;
    r2b = rb > 1.0f ? 255 : 0;
    rc = (uint8_t)(255 - R);
}
__global__ void __launch_bounds__(256) front16_kernel(const uint8_t *__restrict__ bgr, int64_t stride, int rows,
                                                      int cols, int blue, int green, int red, float t1, float t2,
                                                      uint8_t *__restrict__ rc, uint8_t *__restrict__ bw1,
                                                      uint8_t *__restrict__ bw2, uint8_t *__restrict__ r2b,
                                                      unsigned long long *__restrict__ bg_count,
                                                      int *__restrict__ bw1_count) {
    const int64_t cpr = cols / 16, total = cpr * rows;
    for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x; t0 < total; t0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = t0 + threadIdx.x;
        unsigned bg = 0, n1 = 0;
        if (t < total) {
            const int y = (int)(t / cpr);
            const int x0 = (int)(t - (int64_t)y * cpr) * 16;
            const uint4 *src = reinterpret_cast<const uint4 *>(bgr + (int64_t)y * stride + 3 * x0);
            V16 in[3];
            in[0].u = __ldg(src);
            in[1].u = __ldg(src + 1);
            in[2].u = __ldg(src + 2);
            V16 o_rc, o_b1, o_b2, o_rb;
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const int j = 3 * k;
                const uint8_t B = in[j >> 4].b[j & 15], G = in[(j + 1) >> 4].b[(j + 1) & 15],
                              R = in[(j + 2) >> 4].b[(j + 2) & 15];
                front_px(B, G, R, blue, green, red, t1, t2, bg, o_rc.b[k], o_b1.b[k], o_b2.b[k], o_rb.b[k]);
                n1 += o_b1.b[k] ? 1u : 0u;
            }
            const int64_t o = (int64_t)y * cols + x0;
            *reinterpret_cast<uint4 *>(rc + o) = o_rc.u;
            *reinterpret_cast<uint4 *>(bw1 + o) = o_b1.u;
            *reinterpret_cast<uint4 *>(bw2 + o) = o_b2.u;
            *reinterpret_cast<uint4 *>(r2b + o) = o_rb.u;
        }
        warp_add_u64(bg_count, bg);
        for (int off = 16; off > 0; off >>= 1) n1 += __shfl_down_sync(0xffffffffu, n1, off);
        if ((threadIdx.x & 31) == 0 && n1) atomicAdd(bw1_count, (int)n1);
    }
}

__global__ void diff_threshold_kernel(const uint8_t *__restrict__ rc, const uint8_t *__restrict__ rec, int64_t n,
                                      int g1, int g2, uint8_t *__restrict__ o1, uint8_t *__restrict__ o2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int a = rc[i], b = rec[i];
        int d = a > b ? a - b : 0;  // saturating u8 subtraction (HE:211)
        if (o1) o1[i] = d > g1 ? 255 : 0;
        if (o2) o2[i] = d > g2 ? 255 : 0;
    }
}

__global__ void and_not_kernel(uint8_t *__restrict__ io, const uint8_t *__restrict__ nm, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (nm[i]) io[i] = 0;
}

__global__ void mask_copy_bgr_kernel(const uint8_t *__restrict__ bgr, int64_t stride, const uint8_t *__restrict__ m,
                                     int rows, int cols, uint8_t *__restrict__ out) {
    int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        const uint8_t *p = bgr + (int64_t)y * stride + 3 * x;
        bool on = m[i] != 0;
        out[3 * i + 0] = on ? p[0] : 0;
        out[3 * i + 1] = on ? p[1] : 0;
        out[3 * i + 2] = on ? p[2] : 0;
    }
}

// PixelOperations::invert<T> (PixelOperations.cpp:22-43): unsigned
// max - x, signed ~x + 1 (two's-complement negation, wrapping), float -x as
// the reference's scaled copy x * -1 + 0 (so +0 stays +0)
__device__ __forceinline__ uint8_t inv1(uint8_t v) { return (uint8_t)(255 - v); }
__device__ __forceinline__ int32_t inv1(int32_t v) { return (int32_t)(~(uint32_t)v + 1u); }
__device__ __forceinline__ float inv1(float v) { return __fadd_rn(__fmul_rn(v, -1.0f), 0.0f); }

// 16 bytes per thread and step when both arrays are 16-byte aligned (the
// grid strides over 16-byte words, consecutive lanes on consecutive words),
// the remainder one element per thread
template <typename T>
__global__ void invert_kernel(const T *__restrict__ in, T *__restrict__ out, int64_t n, int vec) {
    constexpr int K = 16 / sizeof(T);
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
    int64_t done = 0;
    if (vec) {
        const int64_t nw = n / K;
        const uint4 *src = reinterpret_cast<const uint4 *>(in);
        uint4 *dst = reinterpret_cast<uint4 *>(out);
        for (int64_t w = tid; w < nw; w += nth) {
            union {
                uint4 u;
                T e[K];
            } a;
            a.u = __ldg(src + w);
#pragma unroll
            for (int k = 0; k < K; ++k) a.e[k] = inv1(a.e[k]);
            dst[w] = a.u;
        }
        done = nw * K;
    }
    for (int64_t i = done + tid; i < n; i += nth) out[i] = inv1(in[i]);
}

}  // namespace

static int blocks_for(Ctx &c, int64_t n) {
    int64_t want = (n + kBlock - 1) / kBlock;
    int64_t cap = (int64_t)c.sm_count * 16;
    return (int)(want < cap ? (want < 1 ? 1 : want) : cap);
}

int background_count(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, int blue, int green, int red,
                     uint8_t *mask, int64_t *d_count, cudaStream_t s) {
    NSG_CUDA_TRY(c, cudaMemsetAsync(d_count, 0, sizeof(int64_t), s));
    int64_t chunks = (int64_t)((cols + 15) / 16) * rows;
    background_kernel<16><<<blocks_for(c, chunks), kBlock, 0, s>>>(bgr, stride, rows, cols, blue, green, red, mask,
                                                                   (unsigned long long *)d_count);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

int front_rbc(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, double T1, double T2, uint8_t *rc,
              uint8_t *bw1, uint8_t *bw2, uint8_t *r2b, int *d_bw1_count, cudaStream_t s) {
    NSG_CUDA_TRY(c, cudaMemsetAsync(d_bw1_count, 0, sizeof(int), s));
    int64_t n = (int64_t)rows * cols;
    front_rbc_kernel<<<blocks_for(c, n), kBlock, 0, s>>>(bgr, stride, rows, cols, (float)T1, (float)T2, rc, bw1, bw2,
                                                         r2b, d_bw1_count);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// background count and the RBC front in one 128-bit pass where the layout
// allows it, else the two scalar passes
int front_fused(Ctx &c, const uint8_t *bgr, int64_t stride, int rows, int cols, int blue, int green, int red,
                double T1, double T2, int64_t *d_bg_count, uint8_t *rc, uint8_t *bw1, uint8_t *bw2, uint8_t *r2b,
                int *d_bw1_count, cudaStream_t s) {
    const auto a16 = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    if (cols % 16 == 0 && stride % 16 == 0 && a16(bgr) && a16(rc) && a16(bw1) && a16(bw2) && a16(r2b)) {
        NSG_CUDA_TRY(c, cudaMemsetAsync(d_bg_count, 0, sizeof(int64_t), s));
        NSG_CUDA_TRY(c, cudaMemsetAsync(d_bw1_count, 0, sizeof(int), s));
        const int64_t chunks = (int64_t)(cols / 16) * rows;
        front16_kernel<<<blocks_for(c, chunks), kBlock, 0, s>>>(bgr, stride, rows, cols, blue, green, red, (float)T1,
                                                                (float)T2, rc, bw1, bw2, r2b,
                                                                (unsigned long long *)d_bg_count, d_bw1_count);
        NSG_COUNT_LAUNCH();
        NSG_LAUNCH_CHECK(c);
        return NSG_SUCCESS;
    }
    NSG_TRY(background_count(c, bgr, stride, rows, cols, blue, green, red, nullptr, d_bg_count, s));
    return front_rbc(c, bgr, stride, rows, cols, T1, T2, rc, bw1, bw2, r2b, d_bw1_count, s);
}

int diff_threshold(Ctx &c, const uint8_t *rc, const uint8_t *rec, int rows, int cols, int G1, int G2, uint8_t *o1,
                   uint8_t *o2, cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    diff_threshold_kernel<<<blocks_for(c, n), kBlock, 0, s>>>(rc, rec, n, G1, G2, o1, o2);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

int and_not(Ctx &c, uint8_t *io, const uint8_t *nm, int64_t n, cudaStream_t s) {
    and_not_kernel<<<blocks_for(c, n), kBlock, 0, s>>>(io, nm, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

int mask_copy_bgr(Ctx &c, const uint8_t *bgr, int64_t stride, const uint8_t *m, int rows, int cols, uint8_t *out,
                  cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    mask_copy_bgr_kernel<<<blocks_for(c, n), kBlock, 0, s>>>(bgr, stride, m, rows, cols, out);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

template <typename T>
int invert_dev(Ctx &c, const T *in, T *out, int64_t n, cudaStream_t s) {
    const int vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
    const int64_t work = vec ? (n * (int64_t)sizeof(T) + 15) / 16 : n;
    invert_kernel<T><<<blocks_for(c, work), kBlock, 0, s>>>(in, out, n, vec);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}
template int invert_dev<uint8_t>(Ctx &, const uint8_t *, uint8_t *, int64_t, cudaStream_t);
template int invert_dev<int32_t>(Ctx &, const int32_t *, int32_t *, int64_t, cudaStream_t);
template int invert_dev<float>(Ctx &, const float *, float *, int64_t, cudaStream_t);

int invert_u8_dev(Ctx &c, const uint8_t *in, uint8_t *out, int64_t n, cudaStream_t s) {
    return invert_dev<uint8_t>(c, in, out, n, s);
}

}  // namespace nsg
