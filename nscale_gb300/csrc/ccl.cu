// ccl.cu — union-find connected components and everything built on them:
//
//  * bwlabel2 / ConnComponents::label        (MorphologicOperations.cpp:3092-3117,
//                                             ConnComponents.cpp:52-86)
//  * bwareaopen2 / areaThresholdLabeled       (MorphologicOperations.cpp:3281-3314,
//                                             ConnComponents.cpp:205-239)
//  * imreconstructBinary / bwselect / imfillHoles (binary)
//                                            (MorphologicOperations.cpp:2769-3031)
//  * ConnComponents::boundingBox              (ConnComponents.cpp:241-284)
//
// Labels follow the reference exactly: the root of every component is its
// minimum raster index (the reference's merge() links the larger root under
// the smaller, ConnComponents.cpp:34-43).  Here every pixel unions with its
// already-visited neighbours (left, up, up-left, up-right) concurrently;
// union hooks the larger root under the smaller with atomicMin and retries
// when it lost a race, and find() halves paths.  Because hooking always goes
// to a smaller index, the minimum index of a component is the only node that
// can never be hooked, so the final roots are the reference's labels.
//
// Binary reconstruction has a unique answer — the mask components (under the
// given connectivity) that contain a marker pixel — so imreconstructBinary,
// bwselect and imfillHoles are all "label the mask, flag the components that
// touch a seed (or the image border), select".
#include <limits.h>
#include <stdlib.h>

#include <mutex>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int kB = 256;

// Bounded union: every find step and every lost hooking race counts against
// `budget`; when it runs out the union is abandoned, DEV_TIMEOUT is set in
// the device status word and the host call returns NSG_ERR_TIMEOUT (the
// labels are then incomplete, never silently returned as correct).
struct UfGuard {
    long long budget;
    int *status;
};

__device__ __forceinline__ int find_root_counted(int *parent, int x, long long &steps) {
    for (;;) {
        int p = __ldcg(parent + x);
        if (p == x) return x;
        int gp = __ldcg(parent + p);
        if (gp != p) parent[x] = gp;  // path halving (benign race: ancestors only)
        x = p;
        ++steps;
    }
}

__device__ __forceinline__ void unite(int *parent, int a, int b, const UfGuard &g) {
    long long steps = 0;
    for (;;) {
        a = find_root_counted(parent, a, steps);
        b = find_root_counted(parent, b, steps);
        if (a == b) return;
        if (steps >= g.budget) {
            atomicOr(g.status, DEV_TIMEOUT);
            return;
        }
        if (a < b) {
            int t = a;
            a = b;
            b = t;
        }
        int old = atomicMin(parent + a, b);
        if (old == a) return;
        a = old;
        ++steps;
    }
}

// Final pass: every pixel points at its root.  The find here must not
// compress paths: a compressing find could overwrite another pixel's final
// root with an intermediate ancestor after that pixel was written.
__global__ void ccl_flatten(int *parent, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int x = __ldcg(parent + i);
        if (x < 0) continue;
        for (;;) {
            int p = __ldcg(parent + x);
            if (p == x) break;
            x = p;
        }
        parent[i] = x;
    }
}

// The root of pixel i in a forest that was not flattened (-1 background).
// After ccl_local every pixel points at its tile-local root and ccl_border
// only hooks roots under smaller roots (or halves paths to ancestors), so
// the chain is short and strictly decreasing.  With `write_back` the pixel's
// link is replaced by its root when they differ: only final roots are
// written, so another thread walking a chain through this pixel meets either
// the old ancestor or the root, never a wrong node.  This is the flatten pass
// folded into the first consumer of the labels.
__device__ __forceinline__ int ccl_root(int *parent, int64_t i, bool write_back) {
    const int x0 = __ldcg(parent + i);
    if (x0 < 0) return x0;
    int x = x0;
    for (;;) {
        const int p = __ldcg(parent + x);
        if (p == x) break;
        x = p;
    }
    if (write_back && x != x0) parent[i] = x;
    return x;
}

// ---- block-local union-find ------------------------------------------------
// A 32x32 tile is labelled in shared memory (union by atomicMin on local
// indices, so local roots are the tile's minimum raster index of each piece,
// which is also the minimum global index); then only pixel pairs that cross a
// tile border are united in global memory.
constexpr int LT = 32;

struct PredU8 {
    const uint8_t *img;
    int mode;
    __device__ __forceinline__ bool fg(int64_t i) const {
        uint8_t v = img[i];
        return mode == CCL_NOT255 ? v != 255 : v != 0;
    }
    __device__ __forceinline__ bool joins(int64_t i, int64_t j) const {
        uint8_t a = img[i], b = img[j];
        if (mode == CCL_EQUAL) return a == b && a != 0;
        if (mode == CCL_NONZERO) return a != 0 && b != 0;
        return a != 255 && b != 255;
    }
};
struct PredF32 {
    const float *val;
    const uint8_t *valid;
    __device__ __forceinline__ bool fg(int64_t i) const { return valid[i] != 0; }
    __device__ __forceinline__ bool joins(int64_t i, int64_t j) const {
        return valid[i] && valid[j] && val[i] == val[j];
    }
};

__device__ __forceinline__ int lfind(int *l, int x) {
    int p = l[x];
    while (p != x) {
        int gp = l[p];
        l[x] = gp;  // halving in shared memory
        x = p;
        p = gp;
    }
    return x;
}
__device__ __forceinline__ void lunite(int *l, int a, int b) {
    for (;;) {
        a = lfind(l, a);
        b = lfind(l, b);
        if (a == b) return;
        if (a < b) {
            int t = a;
            a = b;
            b = t;
        }
        int old = atomicMin(l + a, b);
        if (old == a) return;
        a = old;
    }
}

// zero_at_roots (nullable): a per-pixel int plane whose entry at every local
// root is set to 0 (the component flags or areas the consumers accumulate at
// roots; every final root is a local root, so none is missed)
template <typename Pred>
__global__ void __launch_bounds__(256) ccl_local(Pred pr, int *__restrict__ parent, int rows, int cols, int conn,
                                                 int *__restrict__ zero_at_roots) {
    __shared__ int l[LT * LT];
    const int x0 = blockIdx.x * LT, y0 = blockIdx.y * LT;
    const int tx = threadIdx.x & 31, tyb = threadIdx.x >> 5;  // 8 row groups
    // init
    for (int ty = tyb; ty < LT; ty += 8) {
        int y = y0 + ty, x = x0 + tx, li = ty * LT + tx;
        bool f = (y < rows && x < cols) && pr.fg((int64_t)y * cols + x);
        l[li] = f ? li : -1;
    }
    __syncthreads();
    for (int ty = tyb; ty < LT; ty += 8) {
        int y = y0 + ty, x = x0 + tx, li = ty * LT + tx;
        if (l[li] < 0) continue;
        int64_t i = (int64_t)y * cols + x;
        if (tx > 0 && pr.joins(i, i - 1)) lunite(l, li, li - 1);
        if (ty > 0) {
            int64_t u = i - cols;
            if (pr.joins(i, u)) lunite(l, li, li - LT);
            if (conn == 8) {
                if (tx > 0 && pr.joins(i, u - 1)) lunite(l, li, li - LT - 1);
                if (tx < LT - 1 && x < cols - 1 && pr.joins(i, u + 1)) lunite(l, li, li - LT + 1);
            }
        }
    }
    __syncthreads();
    for (int ty = tyb; ty < LT; ty += 8) {
        int y = y0 + ty, x = x0 + tx, li = ty * LT + tx;
        if (y >= rows || x >= cols) continue;
        int r = l[li];
        if (r >= 0) {
            while (l[r] != r) r = l[r];
            if (zero_at_roots && r == li) zero_at_roots[(int64_t)y * cols + x] = 0;
            r = (y0 + r / LT) * cols + (x0 + r % LT);
        }
        parent[(int64_t)y * cols + x] = r;
    }
}

// unions of neighbour pairs that cross a tile border (backward neighbours:
// left, up, up-left, up-right, the pairs ConnComponents::label visits).
// One block per 32x32 tile, one thread per pixel that can have such a pair:
// the tile's top row (32), its left and right columns below it (31 + 31).
// Union-find hooks the larger root under the smaller, so the final roots do
// not depend on the order of the unions.
constexpr int kBorderPx = LT + 2 * (LT - 1);  // 94
template <typename Pred>
__global__ void __launch_bounds__(128) ccl_border(Pred pr, int *parent, int rows, int cols, int conn, UfGuard ug) {
    const int t = threadIdx.x;
    if (t >= kBorderPx) return;
    int bx, by;
    if (t < LT) {
        bx = t;
        by = 0;
    } else if (t < 2 * LT - 1) {
        bx = 0;
        by = t - (LT - 1);
    } else {
        bx = LT - 1;
        by = t - (2 * LT - 2);
    }
    const int x = blockIdx.x * LT + bx, y = blockIdx.y * LT + by;
    if (x >= cols || y >= rows) return;
    const int64_t i = (int64_t)y * cols + x;
    if (!pr.fg(i)) return;
    if (x > 0 && bx == 0 && pr.joins(i, i - 1)) unite(parent, (int)i, (int)(i - 1), ug);
    if (y > 0) {
        const int64_t u = i - cols;
        if (by == 0 && pr.joins(i, u)) unite(parent, (int)i, (int)u, ug);
        if (conn == 8) {
            if (x > 0 && (bx == 0 || by == 0) && pr.joins(i, u - 1)) unite(parent, (int)i, (int)(u - 1), ug);
            if (x < cols - 1 && (bx == LT - 1 || by == 0) && pr.joins(i, u + 1))
                unite(parent, (int)i, (int)(u + 1), ug);
        }
    }
}

// the first consumer of an unflattened forest: flattens it as it counts
__global__ void area_count(int *lab, int *__restrict__ area, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int l = ccl_root(lab, i, true);
        // warp-aggregate pixels of the same component
        unsigned act = __activemask();
        unsigned same = __match_any_sync(act, l);
        int leader = __ffs(same) - 1;
        if (l >= 0 && (threadIdx.x & 31) == leader) atomicAdd(area + l, __popc(same));
    }
}

__global__ void area_select(const int *__restrict__ lab, const int *__restrict__ area, int64_t n, int lower,
                            int upper, uint8_t *__restrict__ out, int *__restrict__ count) {
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = i0 + threadIdx.x;
        bool root_kept = false;
        if (i < n) {
            int l = lab[i];
            bool keep = false;
            if (l >= 0) {
                int a = area[l];
                keep = a >= lower && a < upper;
                root_kept = keep && l == (int)i;
            }
            out[i] = keep ? 255 : 0;
        }
        unsigned b = __ballot_sync(0xffffffffu, root_kept);
        if ((threadIdx.x & 31) == 0 && b) atomicAdd(count, __popc(b));
    }
}

// flag[root] |= seed present in the component; the first consumer of an
// unflattened forest, so it flattens it on the way
__global__ void flag_seeds(int *lab, const uint8_t *__restrict__ seed, const uint8_t *__restrict__ mask,
                           int *__restrict__ flag, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int l = ccl_root(lab, i, true);
        if (l >= 0 && seed[i] && mask[i] && !__ldcg(flag + l)) flag[l] = 1;
    }
}
// reads an unflattened forest (roots found, nothing written back)
__global__ void flag_border(int *lab, int *__restrict__ flag, int rows, int cols) {
    int64_t nb = 2 * (int64_t)cols + 2 * (int64_t)rows;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += (int64_t)gridDim.x * blockDim.x) {
        int64_t i;
        if (k < cols) i = k;
        else if (k < 2 * cols) i = (int64_t)(rows - 1) * cols + (k - cols);
        else if (k < 2 * cols + rows) i = (int64_t)(k - 2 * cols) * cols;
        else i = (int64_t)(k - 2 * cols - rows) * cols + (cols - 1);
        int l = ccl_root(lab, i, false);
        if (l >= 0) flag[l] = 1;
    }
}
// imreconstructBinary: marker pixels keep their value, reached mask pixels 255
__global__ void select_recon(const int *__restrict__ lab, const int *__restrict__ flag,
                             const uint8_t *__restrict__ marker, const uint8_t *__restrict__ mask,
                             uint8_t *__restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint8_t mk = marker[i];
        int l = lab[i];
        out[i] = mk ? mk : ((mask[i] && l >= 0 && flag[l]) ? 255 : 0);
    }
}
// bwselect: bw value on selected components
__global__ void select_bw(const int *__restrict__ lab, const int *__restrict__ flag, const uint8_t *__restrict__ bw,
                          uint8_t *__restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int l = lab[i];
        out[i] = (l >= 0 && flag[l]) ? bw[i] : 0;
    }
}
// imfillHoles: pixels reached from the border through (img != 255) become 0,
// everything else 255 (reads an unflattened forest: the last consumer)
__global__ void select_fill(int *lab, const int *__restrict__ flag, uint8_t *__restrict__ out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int l = ccl_root(lab, i, false);
        out[i] = (l >= 0 && flag[l]) ? 0 : 255;
    }
}

// ---- bounding boxes --------------------------------------------------------
__global__ void bbox_init(int *mnx, int *mxx, int *mny, int *mxy, const int *__restrict__ lab, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (lab[i] == (int)i) {
            mnx[i] = INT_MAX;
            mxx[i] = -1;
            mny[i] = INT_MAX;
            mxy[i] = -1;
        }
    }
}
__global__ void bbox_accum(const int *__restrict__ lab, int rows, int cols, int *mnx, int *mxx, int *mny, int *mxy) {
    int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int l = lab[i];
        if (l < 0) continue;
        int y = (int)(i / cols), x = (int)(i - (int64_t)y * cols);
        atomicMin(mnx + l, x);
        atomicMax(mxx + l, x);
        atomicMin(mny + l, y);
        atomicMax(mxy + l, y);
    }
}
__global__ void root_flags(const int *__restrict__ lab, int *__restrict__ f, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        f[i] = lab[i] == (int)i ? 1 : 0;
}
__global__ void bbox_write(const int *__restrict__ lab, const int *__restrict__ pos, int64_t n,
                           const int *__restrict__ total, const int *mnx, const int *mxx, const int *mny,
                           const int *mxy, int *__restrict__ out, int64_t cap_ints, int *status) {
    int cnt = *total;
    if ((int64_t)cnt * 5 > cap_ints) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(status, DEV_QUEUE_FULL);
        return;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (lab[i] != (int)i) continue;
        int k = pos[i];
        out[k] = (int)i;
        out[cnt + k] = mnx[i];
        out[2 * cnt + k] = mxx[i];
        out[3 * cnt + k] = mny[i];
        out[4 * cnt + k] = mxy[i];
    }
}

// ---- exclusive scan (three passes) ------------------------------------------
constexpr int kScanThreads = 1024, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

__device__ int block_exclusive_scan(int v, int *sh, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        int z = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, z, d);
            if (lane >= d) z += y;
        }
        sh[lane] = z - w;
        if (lane == 31) sh[32] = z;
    }
    __syncthreads();
    int r = sh[warp] + x - v;
    if (total) *total = sh[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_tiles(const int *__restrict__ in, int *__restrict__ out,
                                                           int64_t n, int *__restrict__ block_sums,
                                                           const int *__restrict__ d_len) {
    __shared__ int sh[33];
    if (d_len && *d_len < n) n = *d_len;
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    int tot;
    int pre = block_exclusive_scan(s, sh, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = pre;
        pre += v[k];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}
__global__ void __launch_bounds__(kScanThreads) scan_sums(int *sums, int nb, int *total) {
    __shared__ int sh[33];
    int carry = 0;
    for (int base = 0; base < nb; base += kScanThreads) {
        int i = base + threadIdx.x;
        int v = i < nb ? sums[i] : 0;
        int tot;
        int pre = block_exclusive_scan(v, sh, &tot);
        if (i < nb) sums[i] = pre + carry;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}
__global__ void scan_add(int *out, int64_t n, const int *__restrict__ sums, const int *__restrict__ d_len) {
    if (d_len && *d_len < n) n = *d_len;
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int add = sums[blockIdx.x];
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

int blocks(Ctx &c, int64_t n) {
    int64_t g = (n + kB - 1) / kB;
    int64_t cap = (int64_t)c.sm_count * 16;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

// d_len (nullable, device): scan only the first *d_len entries (at most n)
int exclusive_scan_i32(Ctx &c, const int32_t *in, int32_t *out, int64_t n, int32_t *d_total, cudaStream_t s,
                       const int32_t *d_len) {
    int nb = (int)((n + kScanTile - 1) / kScanTile);
    if (nb < 1) nb = 1;
    scan_tiles<<<nb, kScanThreads, 0, s>>>(in, out, n, c.ws.scan_tmp, d_len);
    NSG_COUNT_LAUNCH();
    scan_sums<<<1, kScanThreads, 0, s>>>(c.ws.scan_tmp, nb, d_total);
    NSG_COUNT_LAUNCH();
    scan_add<<<nb, 256, 0, s>>>(out, n, c.ws.scan_tmp, d_len);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// zero_at_roots (nullable): a per-pixel int plane cleared at every component
// root.  flatten = false leaves the forest unflattened: the caller's first
// consumer finds roots itself (ccl_root) and writes them back.
int ccl_u8(Ctx &c, const uint8_t *img, int32_t *parent, int rows, int cols, int conn, int mode, cudaStream_t s,
           int *zero_at_roots, bool flatten) {
    int64_t n = (int64_t)rows * cols;
    PredU8 pr{img, mode};
    dim3 grid((cols + LT - 1) / LT, (rows + LT - 1) / LT);
    ccl_local<PredU8><<<grid, 256, 0, s>>>(pr, parent, rows, cols, conn, zero_at_roots);
    NSG_COUNT_LAUNCH();
    ccl_border<PredU8><<<grid, 128, 0, s>>>(pr, parent, rows, cols, conn, UfGuard{c.spin_budget, c.ws.ctrl + C_STATUS});
    NSG_COUNT_LAUNCH();
    if (flatten) {
        ccl_flatten<<<blocks(c, n), kB, 0, s>>>(parent, n);
        NSG_COUNT_LAUNCH();
    }
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

int ccl_f32_masked(Ctx &c, const float *val, const uint8_t *valid, int32_t *parent, int rows, int cols, int conn,
                   cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    PredF32 pr{val, valid};
    dim3 grid((cols + LT - 1) / LT, (rows + LT - 1) / LT);
    ccl_local<PredF32><<<grid, 256, 0, s>>>(pr, parent, rows, cols, conn, nullptr);
    NSG_COUNT_LAUNCH();
    ccl_border<PredF32><<<grid, 128, 0, s>>>(pr, parent, rows, cols, conn, UfGuard{c.spin_budget, c.ws.ctrl + C_STATUS});
    NSG_COUNT_LAUNCH();
    ccl_flatten<<<blocks(c, n), kB, 0, s>>>(parent, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// scratch: i32[0] (labels), i32[1] (areas)
int bwareaopen_dev(Ctx &c, const uint8_t *img, uint8_t *out, int rows, int cols, int min_size, int max_size,
                   int conn, int *d_count, cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    int *lab = c.ws.i32[0], *area = c.ws.i32[1];
    // areas cleared at the roots by the labelling; area_count flattens the forest
    NSG_TRY(ccl_u8(c, img, lab, rows, cols, conn, CCL_EQUAL, s, area, false));
    NSG_CUDA_TRY(c, cudaMemsetAsync(d_count, 0, sizeof(int), s));
    int g = blocks(c, n);
    area_count<<<g, kB, 0, s>>>(lab, area, n);
    NSG_COUNT_LAUNCH();
    area_select<<<g, kB, 0, s>>>(lab, area, n, min_size, max_size, out, d_count);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// scratch: i32[0] (labels), i32[1] (flags)
int recon_binary_dev(Ctx &c, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows, int cols, int conn,
                     cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    int *lab = c.ws.i32[0], *flag = c.ws.i32[1];
    NSG_TRY(ccl_u8(c, mask, lab, rows, cols, conn, CCL_NONZERO, s, flag, false));
    int g = blocks(c, n);
    flag_seeds<<<g, kB, 0, s>>>(lab, marker, mask, flag, n);
    NSG_COUNT_LAUNCH();
    select_recon<<<g, kB, 0, s>>>(lab, flag, marker, mask, out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

int bwselect_dev(Ctx &c, const uint8_t *bw, const uint8_t *seeds, uint8_t *out, int rows, int cols, int conn,
                 cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    int *lab = c.ws.i32[0], *flag = c.ws.i32[1];
    NSG_TRY(ccl_u8(c, bw, lab, rows, cols, conn, CCL_NONZERO, s, flag, false));
    int g = blocks(c, n);
    flag_seeds<<<g, kB, 0, s>>>(lab, seeds, bw, flag, n);
    NSG_COUNT_LAUNCH();
    select_bw<<<g, kB, 0, s>>>(lab, flag, bw, out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

int fill_holes_dev(Ctx &c, const uint8_t *img, uint8_t *out, int rows, int cols, int conn, cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    int *lab = c.ws.i32[0], *flag = c.ws.i32[1];
    NSG_TRY(ccl_u8(c, img, lab, rows, cols, conn, CCL_NOT255, s, flag, false));
    int g = blocks(c, n);
    flag_border<<<blocks(c, 2 * (int64_t)rows + 2 * cols), kB, 0, s>>>(lab, flag, rows, cols);
    NSG_COUNT_LAUNCH();
    select_fill<<<g, kB, 0, s>>>(lab, flag, out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

int bwlabel_dev(Ctx &c, const uint8_t *img, int32_t *labels, int rows, int cols, int conn, cudaStream_t s) {
    return ccl_u8(c, img, labels, rows, cols, conn, CCL_EQUAL, s);
}

// scratch: i32[0..4]; d_bbox holds cap_ints ints (5 per component)
int bbox_dev(Ctx &c, const int32_t *labels, int rows, int cols, int32_t *d_bbox, int64_t cap_ints, int *d_count,
             cudaStream_t s) {
    int64_t n = (int64_t)rows * cols;
    int *mnx = c.ws.i32[0], *mxx = c.ws.i32[1], *mny = c.ws.i32[2], *mxy = c.ws.i32[3], *pos = c.ws.i32[4];
    int g = blocks(c, n);
    bbox_init<<<g, kB, 0, s>>>(mnx, mxx, mny, mxy, labels, n);
    NSG_COUNT_LAUNCH();
    bbox_accum<<<g, kB, 0, s>>>(labels, rows, cols, mnx, mxx, mny, mxy);
    NSG_COUNT_LAUNCH();
    root_flags<<<g, kB, 0, s>>>(labels, pos, n);
    NSG_COUNT_LAUNCH();
    NSG_TRY(exclusive_scan_i32(c, pos, pos, n, d_count, s));
    bbox_write<<<g, kB, 0, s>>>(labels, pos, n, d_count, mnx, mxx, mny, mxy, d_bbox, cap_ints,
                                c.ws.ctrl + C_STATUS);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// ---- imfillHoles with no allocation at all ----------------------------------
// Some callers cannot create an nsg_context: code that runs where allocating
// device memory is not allowed (a host that hands the library a memory budget
// it has already spent, a plugin sandbox whose device allocator is owned by
// the embedding application, or a process that must not allocate after its
// set-up phase).  For them nsg_imfill_holes_u8_noalloc takes its two int32
// work planes (component labels and per-component border flags) from one
// file-scope device array instead of the context arena.  The array is part
// of this library's device image: every GPU that loads the library holds it
// (NSG_NOALLOC_MAX_PIXELS * 8 bytes) until the process exits.  A second
// file-scope word is the call's device status word: the union-find's bounded
// retries report through it, and the call reads it back before returning.
namespace {

__device__ __align__(256) int g_noalloc_scratch[2 * (int64_t)NSG_NOALLOC_MAX_PIXELS];
__device__ int g_noalloc_status;

struct NoAllocScratch {
    int *base = nullptr;    // device address of g_noalloc_scratch on this device
    int *status = nullptr;  // device address of g_noalloc_status on this device
    int sm_count = 0;
};
constexpr int kNoAllocDevices = 64;
std::mutex g_noalloc_mu;
NoAllocScratch g_noalloc[kNoAllocDevices];

// Set-up, once per device and with that device current: the symbol name is
// only a host-side handle, so the device address comes from the runtime.
int noalloc_scratch(NoAllocScratch *out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return NSG_ERR_CUDA;
    }
    if (dev < 0 || dev >= kNoAllocDevices) return NSG_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocScratch &e = g_noalloc[dev];
    if (!e.base) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return NSG_ERR_CUDA;
        }
        void *ps = nullptr;
        if (cudaGetSymbolAddress(&ps, g_noalloc_status) != cudaSuccess || !ps) {
            cudaGetLastError();
            return NSG_ERR_CUDA;
        }
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
            cudaGetLastError();
            return NSG_ERR_CUDA;
        }
        e.sm_count = sms;
        e.status = static_cast<int *>(ps);
        e.base = static_cast<int *>(p);
    }
    *out = e;
    return NSG_SUCCESS;
}

// union-find step budget of the no-allocation entry (it has no context to
// carry one): NSG_SPIN_BUDGET in the environment, read at each call, else
// the context default
long long noalloc_spin_budget() {
    const char *e = getenv("NSG_SPIN_BUDGET");
    if (e) {
        const long long v = atoll(e);
        if (v > 0) return v;
    }
    return 1ll << 26;
}

int noalloc_blocks(int sm_count, int64_t n) {
    int64_t g = (n + kB - 1) / kB;
    int64_t cap = (int64_t)sm_count * 16;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

}  // namespace nsg

extern "C" int nsg_imfill_holes_u8_noalloc(const uint8_t *img, uint8_t *out, int rows, int cols, int conn,
                                           nsg_stream_t stream) {
    using namespace nsg;
    if (!img || !out || rows <= 0 || cols <= 0 || (conn != 4 && conn != 8)) return NSG_ERR_ARG;
    const int64_t n = (int64_t)rows * cols;
    if (n > (int64_t)NSG_NOALLOC_MAX_PIXELS) return NSG_ERR_OOM;
    NoAllocScratch sc;
    int st = noalloc_scratch(&sc);
    if (st != NSG_SUCCESS) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Every call overwrites the labels of all rows*cols pixels and clears the
    // flag of every component root before setting any, so nothing the
    // previous call left in the array is read.
    int *lab = sc.base, *flag = sc.base + (int64_t)NSG_NOALLOC_MAX_PIXELS;
    PredU8 pr{img, CCL_NOT255};
    const int g = noalloc_blocks(sc.sm_count, n);
    dim3 grid((cols + LT - 1) / LT, (rows + LT - 1) / LT);
    if (cudaMemsetAsync(sc.status, 0, sizeof(int), s) != cudaSuccess) {
        cudaGetLastError();
        return NSG_ERR_CUDA;
    }
    ccl_local<PredU8><<<grid, 256, 0, s>>>(pr, lab, rows, cols, conn, flag);
    NSG_COUNT_LAUNCH();
    ccl_border<PredU8><<<grid, 128, 0, s>>>(pr, lab, rows, cols, conn, UfGuard{noalloc_spin_budget(), sc.status});
    NSG_COUNT_LAUNCH();
    flag_border<<<noalloc_blocks(sc.sm_count, 2 * (int64_t)rows + 2 * cols), kB, 0, s>>>(lab, flag, rows, cols);
    NSG_COUNT_LAUNCH();
    select_fill<<<g, kB, 0, s>>>(lab, flag, out, n);
    NSG_COUNT_LAUNCH();
    if (cudaGetLastError() != cudaSuccess) return NSG_ERR_CUDA;
    // the status word into host stack memory (no pinned buffer: nothing is
    // allocated); this waits for the stream, so `out` is complete on return
    int dev_status = 0;
    if (cudaMemcpyAsync(&dev_status, sc.status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return NSG_ERR_CUDA;
    }
    if (dev_status & DEV_TIMEOUT) return NSG_ERR_TIMEOUT;
    return NSG_SUCCESS;
}
