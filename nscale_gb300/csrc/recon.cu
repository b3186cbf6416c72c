// recon.cu — morphological reconstruction by dilation, uint8 and float32
// (nscale::imreconstruct<T>, MorphologicOperations.cpp:1731-1903).
//
// The reference runs Vincent's hybrid algorithm: a raster and an anti-raster
// scan, then a FIFO wavefront.  Its result is the unique least fixed point
//     out = max(min(marker, mask), min(max over conn-neighbours of out, mask))
// on the image padded with a one-pixel ring of value 0 (marker and mask),
// so any propagation order reproduces it exactly; that is what this kernel
// does, GB300-style:
//
//  * the image is cut into 64-wide tiles; ONE WARP owns a tile at a time and
//    keeps it (plus a one-pixel halo) in shared memory;
//  * inside the tile the warp runs the reference's raster / anti-raster
//    scans row by row: the vertical step is elementwise, the horizontal
//    dependence  out[x] = min(max(v[x], out[x-1]), mask[x])  is a prefix
//    composition of clamp functions, evaluated with warp shuffles (a scan of
//    (lo, hi) pairs), so a whole row propagates in log2(32) steps;
//  * scans repeat until the tile is stable; changed tile edges re-queue the
//    neighbouring tiles;
//  * tiles circulate through a device-resident work queue inside ONE
//    persistent kernel (the queue wavefront): no host round trip until the
//    whole image has converged.  A per-tile state machine (idle / queued /
//    processing / processing+requeue) guarantees one warp per tile, and one
//    `outstanding` counter detects global termination.  Every wait is
//    bounded by the context's spin budget and reports NSG_ERR_TIMEOUT.
#include <float.h>
#include <math.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int TW = 64;  // tile width (2 pixels per lane)

// std::max / std::min as the reference writes them
template <typename T>
__device__ __forceinline__ T smax(T a, T b) {
    return (a < b) ? b : a;
}
template <typename T>
__device__ __forceinline__ T smin(T a, T b) {
    return (b < a) ? b : a;
}
template <typename T>
__device__ __forceinline__ T clampv(T x, T lo, T hi) {
    return smin(smax(x, lo), hi);
}

template <typename T>
__device__ __forceinline__ T shfl_up(T v, int d) {
    return __shfl_up_sync(0xffffffffu, v, d);
}
template <>
__device__ __forceinline__ uint8_t shfl_up<uint8_t>(uint8_t v, int d) {
    return (uint8_t)__shfl_up_sync(0xffffffffu, (int)v, d);
}
template <typename T>
__device__ __forceinline__ T shfl_down(T v, int d) {
    return __shfl_down_sync(0xffffffffu, v, d);
}
template <>
__device__ __forceinline__ uint8_t shfl_down<uint8_t>(uint8_t v, int d) {
    return (uint8_t)__shfl_down_sync(0xffffffffu, (int)v, d);
}

template <typename T>
__device__ __forceinline__ T ldcg(const T *p) {
    return __ldcg(p);
}
template <>
__device__ __forceinline__ uint8_t ldcg<uint8_t>(const uint8_t *p) {
    return (uint8_t)__ldcg((const unsigned char *)p);
}

__global__ void init_min_u8(const uint8_t *__restrict__ a, const uint8_t *__restrict__ b, uint8_t *__restrict__ o,
                            int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint8_t x = a[i], y = b[i];
        o[i] = (y < x) ? y : x;
    }
}
__global__ void init_min_f32(const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ o,
                             int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float x = a[i], y = b[i];
        o[i] = (y < x) ? y : x;
    }
}

__global__ void init_queue(int *state, int *queue, int qcap, int ntiles, int *ctrl) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < qcap; i += gridDim.x * blockDim.x) {
        queue[i] = i < ntiles ? i + 1 : 0;
        if (i < ntiles) state[i] = 1;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctrl[C_QHEAD] = 0;
        ctrl[C_QTAIL] = ntiles;
        ctrl[C_QPEND] = ntiles;
        ctrl[C_RSTATS] = 0;
        ctrl[C_RSTATS + 1] = 0;
    }
}

struct Queue {
    int *state;
    int *queue;
    int qcap;
    int *head, *tail, *outstanding, *status;
    int *stats;  // [0] tile passes, [1] row+column sweeps (recon_cta)
    long long budget;
};

// lane 0 only
__device__ int q_pop(Queue &q) {
    long long spins = 0;
    for (;;) {
        int h = *(volatile int *)q.head;
        int tl = *(volatile int *)q.tail;
        if (h < tl) {
            if (atomicCAS(q.head, h, h + 1) == h) {
                int slot = h % q.qcap;
                int v;
                long long k = 0;
                while ((v = atomicExch(&q.queue[slot], 0)) == 0) {
                    if (++k > q.budget) {
                        atomicOr(q.status, DEV_TIMEOUT);
                        return -2;
                    }
                    __nanosleep(32);
                }
                int t = v - 1;
                atomicExch(&q.state[t], 2);
                __threadfence();
                return t;
            }
            continue;
        }
        if (atomicAdd(q.outstanding, 0) == 0) return -1;
        if (*(volatile int *)q.status & DEV_TIMEOUT) return -2;
        if (++spins > q.budget) {
            atomicOr(q.status, DEV_TIMEOUT);
            return -2;
        }
        __nanosleep(64);
    }
}

// lane 0 only: give tile `t` pending work
__device__ void q_push(Queue &q, int t) {
    for (int guard = 0; guard < 1 << 20; ++guard) {
        int s = *(volatile int *)&q.state[t];
        if (s == 1 || s == 3) return;
        if (s == 0) {
            if (atomicCAS(&q.state[t], 0, 1) == 0) {
                atomicAdd(q.outstanding, 1);
                int slot = atomicAdd(q.tail, 1) % q.qcap;
                atomicExch(&q.queue[slot], t + 1);
                return;
            }
        } else if (s == 2) {
            if (atomicCAS(&q.state[t], 2, 3) == 2) {
                atomicAdd(q.outstanding, 1);
                return;
            }
        }
    }
    atomicOr(q.status, DEV_TIMEOUT);
}

// lane 0 only: returns 1 when the tile must be processed again
__device__ int q_finish(Queue &q, int t) {
    int old = atomicCAS(&q.state[t], 2, 0);
    if (old == 2) {
        atomicSub(q.outstanding, 1);
        return 0;
    }
    // old == 3: another tile changed our halo while we worked
    atomicExch(&q.state[t], 2);
    atomicSub(q.outstanding, 1);
    return 1;
}

template <typename T, int TH>
__device__ void process_tile(const T *__restrict__ mask, T *out, int rows, int cols, bool conn8, int tx, int ty,
                             T *o, T *m, unsigned &edges) {
    const int lane = threadIdx.x & 31;
    const int OW = TW + 2;
    const int y0 = ty * TH, x0 = tx * TW;
    // load tile + halo (ring outside the image = 0)
    for (int i = lane; i < (TH + 2) * OW; i += 32) {
        int r = i / OW, cc = i - r * OW;
        int y = y0 - 1 + r, x = x0 - 1 + cc;
        o[i] = (y >= 0 && y < rows && x >= 0 && x < cols) ? ldcg(out + (int64_t)y * cols + x) : (T)0;
    }
    for (int i = lane; i < TH * TW; i += 32) {
        int r = i / TW, cc = i - r * TW;
        int y = y0 + r, x = x0 + cc;
        m[i] = (y < rows && x < cols) ? __ldg(mask + (int64_t)y * cols + x) : (T)0;
    }
    __syncwarp();
    const int xa = 2 * lane, xb = 2 * lane + 1;
    const bool ina = (x0 + xa) < cols, inb = (x0 + xb) < cols;
    unsigned my_edges = 0;
    bool any = true;
    for (int it = 0; any && it < 4096; ++it) {
        any = false;
        // forward (raster) scan
        for (int r = 0; r < TH; ++r) {
            const bool rowin = (y0 + r) < rows;
            T *orow = o + (r + 1) * OW + 1;
            const T *up = orow - OW;
            T ca = orow[xa], cb = orow[xb];
            T wa = smax(ca, up[xa]), wb = smax(cb, up[xb]);
            if (conn8) {
                wa = smax(wa, smax(up[xa - 1], up[xa + 1]));
                wb = smax(wb, smax(up[xb - 1], up[xb + 1]));
            }
            T ma = m[r * TW + xa], mb = m[r * TW + xb];
            T loa, hia, lob, hib;
            if (rowin && ina) { loa = smin(wa, ma); hia = ma; } else { loa = (T)0; hia = (T)0; }
            if (rowin && inb) { lob = smin(wb, mb); hib = mb; } else { lob = (T)0; hib = (T)0; }
            // lane function F = f_b o f_a
            T lo = clampv(loa, lob, hib), hi = clampv(hia, lob, hib);
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                T pl = shfl_up(lo, d), ph = shfl_up(hi, d);
                if (lane >= d) {
                    T nl = clampv(pl, lo, hi), nh = clampv(ph, lo, hi);
                    lo = nl;
                    hi = nh;
                }
            }
            T el = shfl_up(lo, 1), eh = shfl_up(hi, 1);
            T left = orow[-1];
            T in = lane == 0 ? left : clampv(left, el, eh);
            T na = clampv(in, loa, hia);
            T nb = clampv(na, lob, hib);
            if (rowin && ina && !(na == ca)) {
                orow[xa] = na;
                any = true;
                if (r == 0) my_edges |= 1u;
                if (r == TH - 1) my_edges |= 2u;
                if (xa == 0) my_edges |= 4u;
            }
            if (rowin && inb && !(nb == cb)) {
                orow[xb] = nb;
                any = true;
                if (r == 0) my_edges |= 1u;
                if (r == TH - 1) my_edges |= 2u;
                if (xb == TW - 1) my_edges |= 8u;
            }
            __syncwarp();
        }
        // backward (anti-raster) scan
        for (int r = TH - 1; r >= 0; --r) {
            const bool rowin = (y0 + r) < rows;
            T *orow = o + (r + 1) * OW + 1;
            const T *dn = orow + OW;
            T ca = orow[xa], cb = orow[xb];
            T wa = smax(ca, dn[xa]), wb = smax(cb, dn[xb]);
            if (conn8) {
                wa = smax(wa, smax(dn[xa - 1], dn[xa + 1]));
                wb = smax(wb, smax(dn[xb - 1], dn[xb + 1]));
            }
            T ma = m[r * TW + xa], mb = m[r * TW + xb];
            T loa, hia, lob, hib;
            if (rowin && ina) { loa = smin(wa, ma); hia = ma; } else { loa = (T)0; hia = (T)0; }
            if (rowin && inb) { lob = smin(wb, mb); hib = mb; } else { lob = (T)0; hib = (T)0; }
            // right-to-left: lane function F = f_a o f_b
            T lo = clampv(lob, loa, hia), hi = clampv(hib, loa, hia);
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                T pl = shfl_down(lo, d), ph = shfl_down(hi, d);
                if (lane + d < 32) {
                    T nl = clampv(pl, lo, hi), nh = clampv(ph, lo, hi);
                    lo = nl;
                    hi = nh;
                }
            }
            T el = shfl_down(lo, 1), eh = shfl_down(hi, 1);
            T right = orow[TW];
            T in = lane == 31 ? right : clampv(right, el, eh);
            T nb = clampv(in, lob, hib);
            T na = clampv(nb, loa, hia);
            if (rowin && inb && !(nb == cb)) {
                orow[xb] = nb;
                any = true;
                if (r == 0) my_edges |= 1u;
                if (r == TH - 1) my_edges |= 2u;
                if (xb == TW - 1) my_edges |= 8u;
            }
            if (rowin && ina && !(na == ca)) {
                orow[xa] = na;
                any = true;
                if (r == 0) my_edges |= 1u;
                if (r == TH - 1) my_edges |= 2u;
                if (xa == 0) my_edges |= 4u;
            }
            __syncwarp();
        }
        any = __any_sync(0xffffffffu, any);
    }
    // edge changes (bits 0-3) and "not yet stable" (bit 4: re-queue self)
    if (any) my_edges |= 16u;
    edges = __reduce_or_sync(0xffffffffu, my_edges);
    // write back
    for (int i = lane; i < TH * TW; i += 32) {
        int r = i / TW, cc = i - r * TW;
        int y = y0 + r, x = x0 + cc;
        if (y < rows && x < cols) out[(int64_t)y * cols + x] = o[(r + 1) * OW + cc + 1];
    }
    __threadfence();
    __syncwarp();
}

template <typename T, int TH, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) recon_persistent(const T *__restrict__ mask, T *out, int rows, int cols,
                                                              int conn, int tiles_x, int tiles_y, Queue q) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int per_warp = (TH + 2) * (TW + 2) + TH * TW;
    T *o = reinterpret_cast<T *>(sm_raw) + warp * per_warp;
    T *m = o + (TH + 2) * (TW + 2);
    const bool conn8 = conn == 8;
    for (;;) {
        int t = 0;
        if (lane == 0) t = q_pop(q);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t < 0) break;
        __threadfence();
        int again;
        do {
            int tx = t % tiles_x, ty = t / tiles_x;
            unsigned edges = 0;
            process_tile<T, TH>(mask, out, rows, cols, conn8, tx, ty, o, m, edges);
            if (lane == 0 && edges) {
                // corner pixels changed?  (tracked through the edge bits: a
                // change on two perpendicular edges may involve a corner, so
                // diagonal tiles are re-queued conservatively)
                if (edges & 16u) q_push(q, t);
                if (edges & 1u && ty > 0) q_push(q, t - tiles_x);
                if (edges & 2u && ty + 1 < tiles_y) q_push(q, t + tiles_x);
                if (edges & 4u && tx > 0) q_push(q, t - 1);
                if (edges & 8u && tx + 1 < tiles_x) q_push(q, t + 1);
                if (conn8) {
                    if ((edges & 5u) == 5u && ty > 0 && tx > 0) q_push(q, t - tiles_x - 1);
                    if ((edges & 9u) == 9u && ty > 0 && tx + 1 < tiles_x) q_push(q, t - tiles_x + 1);
                    if ((edges & 6u) == 6u && ty + 1 < tiles_y && tx > 0) q_push(q, t + tiles_x - 1);
                    if ((edges & 10u) == 10u && ty + 1 < tiles_y && tx + 1 < tiles_x) q_push(q, t + tiles_x + 1);
                }
            }
            again = 0;
            if (lane == 0) again = q_finish(q, t);
            again = __shfl_sync(0xffffffffu, again, 0);
            if (again) __threadfence();
        } while (again);
    }
}

// ---------------------------------------------------------------------------
// CTA-per-tile variant: one CTA (8 warps) owns a TW x TH tile.  Row phases
// scan every row of the tile in parallel (one warp per row at a time, PX
// pixels per lane, clamp-function prefix scans left->right then right->left,
// vertical and diagonal neighbours taken from the current tile); column
// phases do the same down and up the columns.  Phases alternate until a
// whole phase pair changes nothing: then every pixel satisfies the 8- (or 4-)
// neighbour fixed-point equation inside the tile.  Concurrent reads of rows
// other warps are updating are benign: values only grow and stay below the
// fixed point.
template <typename T>
__device__ __forceinline__ T ident_lo();
template <>
__device__ __forceinline__ uint8_t ident_lo<uint8_t>() { return 0; }
template <>
__device__ __forceinline__ float ident_lo<float>() { return -INFINITY; }
template <typename T>
__device__ __forceinline__ T ident_hi();
template <>
__device__ __forceinline__ uint8_t ident_hi<uint8_t>() { return 255; }
template <>
__device__ __forceinline__ float ident_hi<float>() { return INFINITY; }

template <typename T, int TW, int TH, int P>
struct TileSmem {
    static constexpr int OW = P;  // row pitch of the halo tile (elements)
    T o[(TH + 2) * P];
    T m[TH * TW];
    T eN[TW], eS[TW], eW[TH], eE[TH];          // the tile's edge values when it was loaded
    T mN[TW + 2], mS[TW + 2], mW[TH], mE[TH];  // the mask just outside the tile (neighbours' pixels)
    int edges;
    int changed;
    int tile;
    int again;
    int sweeps;
};

// One line (row or column) of N = 32 * K pixels: forward then backward
// clamp scans.  get(i) / put(i, v) address pixel i of the line (i = lane*K+k),
// `lo`/`hi` are the per-pixel clamp bounds after the cross-line step, `first`
// and `last` the values just outside the line.
template <typename T, int K>
__device__ __forceinline__ void line_scan(T (&lo)[K], T (&hi)[K], T first, T last, T (&res)[K]) {
    const int lane = threadIdx.x & 31;
    // forward: F = f_{K-1} o ... o f_0
    T FL = lo[0], FH = hi[0];
#pragma unroll
    for (int k = 1; k < K; ++k) {
        T nl = clampv(FL, lo[k], hi[k]), nh = clampv(FH, lo[k], hi[k]);
        FL = nl;
        FH = nh;
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T pl = shfl_up(FL, d), ph = shfl_up(FH, d);
        if (lane >= d) {
            T nl = clampv(pl, FL, FH), nh = clampv(ph, FL, FH);
            FL = nl;
            FH = nh;
        }
    }
    T el = shfl_up(FL, 1), eh = shfl_up(FH, 1);
    T y = lane == 0 ? first : clampv(first, el, eh);
    T v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        y = clampv(y, lo[k], hi[k]);
        v[k] = y;
    }
    // backward on the forward result: g_k(y) = clamp(y, v_k, hi_k)
    T BL = v[K - 1], BH = hi[K - 1];
    if (hi[K - 1] == (T)0 && lo[K - 1] == (T)0) BL = (T)0;
#pragma unroll
    for (int k = K - 2; k >= 0; --k) {
        T l2 = (hi[k] == (T)0 && lo[k] == (T)0) ? (T)0 : v[k];
        T nl = clampv(BL, l2, hi[k]), nh = clampv(BH, l2, hi[k]);
        BL = nl;
        BH = nh;
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T pl = shfl_down(BL, d), ph = shfl_down(BH, d);
        if (lane + d < 32) {
            T nl = clampv(pl, BL, BH), nh = clampv(ph, BL, BH);
            BL = nl;
            BH = nh;
        }
    }
    el = shfl_down(BL, 1);
    eh = shfl_down(BH, 1);
    y = lane == 31 ? last : clampv(last, el, eh);
#pragma unroll
    for (int k = K - 1; k >= 0; --k) {
        T l2 = (hi[k] == (T)0 && lo[k] == (T)0) ? (T)0 : v[k];
        y = clampv(y, l2, hi[k]);
        res[k] = y;
    }
}

template <typename T, int TW, int TH, int P>
__device__ void cta_process_tile(const T *__restrict__ mask, T *out, int rows, int cols, bool conn8, int tx, int ty,
                                 TileSmem<T, TW, TH, P> &sm) {
    constexpr int NW = 8;
    constexpr int KX = TW / 32, KY = TH / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int y0 = ty * TH, x0 = tx * TW;
    T *o = sm.o;
    // load tile + halo (image ring = 0) and the mask
    for (int i = threadIdx.x; i < (TH + 2) * (TW + 2); i += NW * 32) {
        int r = i / (TW + 2), cc = i - r * (TW + 2);
        int y = y0 - 1 + r, x = x0 - 1 + cc;
        o[r * P + cc] = (y >= 0 && y < rows && x >= 0 && x < cols) ? ldcg(out + (int64_t)y * cols + x) : (T)0;
    }
    for (int i = threadIdx.x; i < TH * TW; i += NW * 32) {
        int r = i / TW, cc = i - r * TW;
        int y = y0 + r, x = x0 + cc;
        sm.m[i] = (y < rows && x < cols) ? __ldg(mask + (int64_t)y * cols + x) : (T)0;
    }
    if (threadIdx.x == 0) {
        sm.edges = 0;
        sm.sweeps = 0;
    }
    auto mask_at = [&](int y, int x) -> T {
        return (y >= 0 && y < rows && x >= 0 && x < cols) ? __ldg(mask + (int64_t)y * cols + x) : (T)0;
    };
    for (int i = threadIdx.x; i < TW + 2; i += NW * 32) {
        sm.mN[i] = mask_at(y0 - 1, x0 - 1 + i);
        sm.mS[i] = mask_at(y0 + TH, x0 - 1 + i);
    }
    for (int i = threadIdx.x; i < TH; i += NW * 32) {
        sm.mW[i] = mask_at(y0 + i, x0 - 1);
        sm.mE[i] = mask_at(y0 + i, x0 + TW);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TW; i += NW * 32) {
        sm.eN[i] = o[P + i + 1];
        sm.eS[i] = o[TH * P + i + 1];
    }
    for (int i = threadIdx.x; i < TH; i += NW * 32) {
        sm.eW[i] = o[(i + 1) * P + 1];
        sm.eE[i] = o[(i + 1) * P + TW];
    }
    unsigned my_edges = 0;
    bool anych = false;
    const int vr = rows - y0, vc = cols - x0;  // valid extent of this tile
    for (int it = 0; it < 1024; ++it) {
        bool ch = false;
        // ---- row phase
        for (int r = warp; r < TH; r += NW) {
            T *row = o + (r + 1) * P + 1;
            const T *up = row - P, *dn = row + P;
            T lo[KX], hi[KX], cur[KX], res[KX];
#pragma unroll
            for (int k = 0; k < KX; ++k) {
                int x = lane * KX + k;
                cur[k] = row[x];
                T w = smax(cur[k], smax(up[x], dn[x]));
                if (conn8) w = smax(w, smax(smax(up[x - 1], up[x + 1]), smax(dn[x - 1], dn[x + 1])));
                T mk = sm.m[r * TW + x];
                bool in = r < vr && x < vc;
                lo[k] = in ? smin(w, mk) : (T)0;
                hi[k] = in ? mk : (T)0;
            }
            line_scan<T, KX>(lo, hi, row[-1], row[TW], res);
#pragma unroll
            for (int k = 0; k < KX; ++k) {
                int x = lane * KX + k;
                if (!(res[k] == cur[k])) {
                    row[x] = res[k];
                    ch = true;
                }
            }
        }
        __syncthreads();
        // ---- column phase
        for (int cidx = warp; cidx < TW; cidx += NW) {
            T lo[KY], hi[KY], cur[KY], res[KY];
#pragma unroll
            for (int k = 0; k < KY; ++k) {
                int y = lane * KY + k;
                T *p = o + (y + 1) * P + (cidx + 1);
                cur[k] = p[0];
                T w = smax(cur[k], smax(p[-1], p[1]));
                if (conn8) w = smax(w, smax(smax(p[-P - 1], p[-P + 1]), smax(p[P - 1], p[P + 1])));
                T mk = sm.m[y * TW + cidx];
                bool in = y < vr && cidx < vc;
                lo[k] = in ? smin(w, mk) : (T)0;
                hi[k] = in ? mk : (T)0;
            }
            line_scan<T, KY>(lo, hi, o[cidx + 1], o[(TH + 1) * P + cidx + 1], res);
#pragma unroll
            for (int k = 0; k < KY; ++k) {
                int y = lane * KY + k;
                if (!(res[k] == cur[k])) {
                    o[(y + 1) * P + cidx + 1] = res[k];
                    ch = true;
                }
            }
        }
        const bool any = __syncthreads_or(ch);
        if (threadIdx.x == 0) sm.sweeps = it + 1;
        if (!any) break;
        anych = true;
        if (it == 1023) my_edges |= 16u;  // not stable yet: process again later
    }
    // A neighbour tile needs another pass only if an edge pixel that changed
    // here can raise one of its pixels: new value above that pixel's value
    // (as loaded; it can only have grown since) and that pixel below its mask.
    if (anych) {
        const int c8 = conn8 ? 1 : 0;
        for (int x = threadIdx.x; x < TW; x += NW * 32) {
            T v = o[P + x + 1];
            if (!(v == sm.eN[x]))
                for (int d = -c8; d <= c8; ++d) {
                    int h = x + d;
                    if (h < 0 || h >= TW) continue;
                    T hv = o[h + 1];
                    if (v > hv && sm.mN[h + 1] > hv) my_edges |= 1u;
                }
            v = o[TH * P + x + 1];
            if (!(v == sm.eS[x]))
                for (int d = -c8; d <= c8; ++d) {
                    int h = x + d;
                    if (h < 0 || h >= TW) continue;
                    T hv = o[(TH + 1) * P + h + 1];
                    if (v > hv && sm.mS[h + 1] > hv) my_edges |= 2u;
                }
        }
        for (int y = threadIdx.x; y < TH; y += NW * 32) {
            T v = o[(y + 1) * P + 1];
            if (!(v == sm.eW[y]))
                for (int d = -c8; d <= c8; ++d) {
                    int h = y + d;
                    if (h < 0 || h >= TH) continue;
                    T hv = o[(h + 1) * P];
                    if (v > hv && sm.mW[h] > hv) my_edges |= 4u;
                }
            v = o[(y + 1) * P + TW];
            if (!(v == sm.eE[y]))
                for (int d = -c8; d <= c8; ++d) {
                    int h = y + d;
                    if (h < 0 || h >= TH) continue;
                    T hv = o[(h + 1) * P + TW + 1];
                    if (v > hv && sm.mE[h] > hv) my_edges |= 8u;
                }
        }
        if (c8 && threadIdx.x == 0) {
            T v, hv;
            v = o[P + 1], hv = o[0];
            if (!(v == sm.eN[0]) && v > hv && sm.mN[0] > hv) my_edges |= 32u;  // up-left
            v = o[P + TW], hv = o[TW + 1];
            if (!(v == sm.eN[TW - 1]) && v > hv && sm.mN[TW + 1] > hv) my_edges |= 64u;  // up-right
            v = o[TH * P + 1], hv = o[(TH + 1) * P];
            if (!(v == sm.eS[0]) && v > hv && sm.mS[0] > hv) my_edges |= 128u;  // down-left
            v = o[TH * P + TW], hv = o[(TH + 1) * P + TW + 1];
            if (!(v == sm.eS[TW - 1]) && v > hv && sm.mS[TW + 1] > hv) my_edges |= 256u;  // down-right
        }
    }
    if (my_edges) atomicOr(&sm.edges, (int)my_edges);
    // write back (only a tile that changed)
    if (anych)
        for (int i = threadIdx.x; i < TH * TW; i += NW * 32) {
            int r = i / TW, cc = i - r * TW;
            int y = y0 + r, x = x0 + cc;
            if (y < rows && x < cols) out[(int64_t)y * cols + x] = o[(r + 1) * P + cc + 1];
        }
    __threadfence();
    __syncthreads();
}

template <typename T, int TW, int TH, int P>
__global__ void __launch_bounds__(256) recon_cta(const T *__restrict__ mask, T *out, int rows, int cols, int conn,
                                                 int tiles_x, int tiles_y, Queue q) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    TileSmem<T, TW, TH, P> &sm = *reinterpret_cast<TileSmem<T, TW, TH, P> *>(sm_raw);
    const bool conn8 = conn == 8;
    for (;;) {
        if (threadIdx.x == 0) sm.tile = q_pop(q);
        __syncthreads();
        const int t = sm.tile;
        __syncthreads();
        if (t < 0) break;
        __threadfence();
        for (;;) {
            const int tx = t % tiles_x, ty = t / tiles_x;
            cta_process_tile<T, TW, TH, P>(mask, out, rows, cols, conn8, tx, ty, sm);
            if (threadIdx.x == 0) {
                unsigned edges = (unsigned)sm.edges;
                if (edges & 16u) q_push(q, t);
                if (edges & 1u && ty > 0) q_push(q, t - tiles_x);
                if (edges & 2u && ty + 1 < tiles_y) q_push(q, t + tiles_x);
                if (edges & 4u && tx > 0) q_push(q, t - 1);
                if (edges & 8u && tx + 1 < tiles_x) q_push(q, t + 1);
                if (edges & 32u && ty > 0 && tx > 0) q_push(q, t - tiles_x - 1);
                if (edges & 64u && ty > 0 && tx + 1 < tiles_x) q_push(q, t - tiles_x + 1);
                if (edges & 128u && ty + 1 < tiles_y && tx > 0) q_push(q, t + tiles_x - 1);
                if (edges & 256u && ty + 1 < tiles_y && tx + 1 < tiles_x) q_push(q, t + tiles_x + 1);
                atomicAdd(q.stats, 1);
                atomicAdd(q.stats + 1, sm.sweeps);
                sm.again = q_finish(q, t);
            }
            __syncthreads();
            const int again = sm.again;
            __syncthreads();
            if (!again) break;
            __threadfence();
        }
    }
}

template <typename T, int TW, int TH, int P>
int run_recon_cta(Ctx &c, const T *marker, const T *mask, T *out, int rows, int cols, int conn, cudaStream_t s) {
    NSG_TRY(check_dims(c, rows, cols));
    NSG_TRY(check_conn(c, conn));
    const int64_t n = (int64_t)rows * cols;
    const int tiles_x = (cols + TW - 1) / TW, tiles_y = (rows + TH - 1) / TH;
    const int ntiles = tiles_x * tiles_y;
    const int qcap = 2 * ntiles;
    int *state = c.ws.i32[5];
    int *queue = state + ntiles;
    if ((int64_t)ntiles + qcap > c.max_pad) {
        c.last_error = "tile queue does not fit";
        return NSG_ERR_OOM;
    }
    int blocks = (int)((n + 255) / 256);
    if (blocks > c.sm_count * 16) blocks = c.sm_count * 16;
    if (sizeof(T) == 1)
        init_min_u8<<<blocks, 256, 0, s>>>((const uint8_t *)marker, (const uint8_t *)mask, (uint8_t *)out, n);
    else
        init_min_f32<<<blocks, 256, 0, s>>>((const float *)marker, (const float *)mask, (float *)out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    init_queue<<<(qcap + 255) / 256, 256, 0, s>>>(state, queue, qcap, ntiles, c.ws.ctrl);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    Queue q;
    q.state = state;
    q.queue = queue;
    q.qcap = qcap;
    q.head = c.ws.ctrl + C_QHEAD;
    q.tail = c.ws.ctrl + C_QTAIL;
    q.outstanding = c.ws.ctrl + C_QPEND;
    q.status = c.ws.ctrl + C_STATUS;
    q.budget = c.spin_budget;
    q.stats = c.ws.ctrl + C_RSTATS;
    const size_t smem = sizeof(TileSmem<T, TW, TH, P>);
    auto kfn = recon_cta<T, TW, TH, P>;
    NSG_CUDA_TRY(c, cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    NSG_CUDA_TRY(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 256, smem));
    if (per_sm < 1) per_sm = 1;
    int grid = c.sm_count * per_sm;
    if (grid > ntiles) grid = ntiles;
    kfn<<<grid, 256, smem, s>>>(mask, out, rows, cols, conn, tiles_x, tiles_y, q);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

template <typename T, int TH, int WARPS>
int run_recon(Ctx &c, const T *marker, const T *mask, T *out, int rows, int cols, int conn, cudaStream_t s) {
    NSG_TRY(check_dims(c, rows, cols));
    NSG_TRY(check_conn(c, conn));
    const int64_t n = (int64_t)rows * cols;
    const int tiles_x = (cols + TW - 1) / TW, tiles_y = (rows + TH - 1) / TH;
    const int ntiles = tiles_x * tiles_y;
    const int qcap = 2 * ntiles;
    int *state = c.ws.i32[5];
    int *queue = state + ntiles;
    if ((int64_t)ntiles + qcap > c.max_pad) {
        c.last_error = "tile queue does not fit";
        return NSG_ERR_OOM;
    }
    int blocks = (int)((n + 255) / 256);
    if (blocks > c.sm_count * 16) blocks = c.sm_count * 16;
    if (sizeof(T) == 1)
        init_min_u8<<<blocks, 256, 0, s>>>((const uint8_t *)marker, (const uint8_t *)mask, (uint8_t *)out, n);
    else
        init_min_f32<<<blocks, 256, 0, s>>>((const float *)marker, (const float *)mask, (float *)out, n);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    init_queue<<<(qcap + 255) / 256, 256, 0, s>>>(state, queue, qcap, ntiles, c.ws.ctrl);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    Queue q;
    q.state = state;
    q.queue = queue;
    q.qcap = qcap;
    q.head = c.ws.ctrl + C_QHEAD;
    q.tail = c.ws.ctrl + C_QTAIL;
    q.outstanding = c.ws.ctrl + C_QPEND;
    q.status = c.ws.ctrl + C_STATUS;
    q.budget = c.spin_budget;
    q.stats = c.ws.ctrl + C_RSTATS;
    const size_t smem = (size_t)WARPS * ((TH + 2) * (TW + 2) + TH * TW) * sizeof(T);
    auto kfn = recon_persistent<T, TH, WARPS>;
    NSG_CUDA_TRY(c, cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    NSG_CUDA_TRY(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, WARPS * 32, smem));
    if (per_sm < 1) per_sm = 1;
    int grid = c.sm_count * per_sm;
    int need = (ntiles + WARPS - 1) / WARPS;
    if (grid > need) grid = need;
    kfn<<<grid, WARPS * 32, smem, s>>>(mask, out, rows, cols, conn, tiles_x, tiles_y, q);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

}  // namespace

int recon_u8(Ctx &c, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows, int cols, int conn,
             cudaStream_t s) {
    return run_recon_cta<uint8_t, 128, 128, 132>(c, marker, mask, out, rows, cols, conn, s);
}

int recon_f32(Ctx &c, const float *marker, const float *mask, float *out, int rows, int cols, int conn,
              cudaStream_t s) {
    return run_recon_cta<float, 64, 64, 67>(c, marker, mask, out, rows, cols, conn, s);
}

// the warp-per-tile variant (kept for comparison)
int recon_u8_warp(Ctx &c, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows, int cols, int conn,
                  cudaStream_t s) {
    return run_recon<uint8_t, 64, 4>(c, marker, mask, out, rows, cols, conn, s);
}
int recon_f32_warp(Ctx &c, const float *marker, const float *mask, float *out, int rows, int cols, int conn,
                   cudaStream_t s) {
    return run_recon<float, 32, 4>(c, marker, mask, out, rows, cols, conn, s);
}

}  // namespace nsg
