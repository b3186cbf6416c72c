// recon.cu — morphological reconstruction by dilation, uint8 and float32
// (nscale::imreconstruct<T>, MorphologicOperations.cpp:1731-1903).
//
// The reference runs Vincent's hybrid algorithm: a raster and an anti-raster
// scan, then a FIFO wavefront.  Its result is the unique least fixed point
//     out = max(min(marker, mask), min(max over conn-neighbours of out, mask))
// on the image padded with a one-pixel ring of value 0 (marker and mask),
// so any propagation order reproduces it exactly; this file computes it with
// one persistent kernel:
//
//  * the image is cut into tiles (128 x 128 uint8, 64 x 64 float32); a CTA
//    owns a tile at a time and keeps it, a one-pixel halo and its mask in
//    shared memory;
//  * inside the tile, row phases and column phases alternate.  In a row
//    phase the cross-row step (the neighbours in the rows above and below) is
//    elementwise, and the along-row dependence
//    out[x] = clamp(out[x-1], lo[x], hi[x]) of the raster and anti-raster
//    scans is either run pixel by pixel with one lane per row (uint8, when
//    many rows of a 32-row group are dirty) or evaluated by a whole warp per
//    row as a prefix composition of clamp functions with warp shuffles;
//    column phases do the same down and up the columns;
//  * only dirty lines are scanned: a pixel changed by a row phase dirties its
//    column and the two next to it for the following column phase, and the
//    other way round, so a pass costs what actually propagates;
//  * a tile whose edge changed in a way that can raise a neighbour's pixel
//    queues that neighbour with the neighbour's edge line marked dirty;
//    tiles circulate through a device-resident work queue (idle / queued /
//    processing / processing+requeue per tile) and an `outstanding` counter
//    detects global termination, with no host round trip.  Every wait is
//    bounded by the context's spin budget and reports NSG_ERR_TIMEOUT.
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cuda.h>  // CUtensorMap (the encoder comes from the runtime's driver entry point)

#include <type_traits>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

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

// dirty lines a tile starts a pass with (set by the tiles that notify it)
enum : int { D_N = 1, D_S = 2, D_W = 4, D_E = 8, D_ALL = 16, D_FRESH = 32 };

__global__ void init_queue(int *state, int *queue, int *dirty, int qcap, int ntiles, int *ctrl) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < qcap; i += gridDim.x * blockDim.x) {
        queue[i] = i < ntiles ? i + 1 : 0;
        if (i < ntiles) {
            state[i] = 1;
            dirty[i] = D_ALL;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ctrl[C_QHEAD] = 0;
        ctrl[C_QTAIL] = ntiles;
        ctrl[C_QPEND] = ntiles;
        ctrl[C_RSTATS] = 0;
        ctrl[C_RSTATS + 1] = 0;
        ctrl[C_RSTATS + 3] = 0;
    }
}

// ---- whole-image sweeps ------------------------------------------------------
// One thread per row (per column): the raster scan then the anti-raster scan
// of the reference, restricted to one line, with the cross-line neighbours read
// as they are (other threads may be raising them: values only grow, so any
// value read is a valid lower bound).  Outside the image everything is 0, the
// reference's padding ring.  A few row + column sweeps settle most of an
// image with almost no SM time held; the tile queue finishes the rest.
// plain (L1-cached) loads: a stale value is an older lower bound, still valid
template <typename T>
__device__ __forceinline__ T at0(const T *p, int64_t i, bool ok) {
    return ok ? p[i] : (T)0;
}

template <typename T>
__global__ void sweep_rows(const T *__restrict__ mask, T *out, int rows, int cols, int conn8, int *changed) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= rows) return;
    T *row = out + (int64_t)y * cols;
    const T *mrow = mask + (int64_t)y * cols;
    const bool hu = y > 0, hd = y + 1 < rows;
    const int64_t U = -(int64_t)cols, D = cols;
    int nch = 0;
    T prev = (T)0;
    for (int x = 0; x < cols; ++x) {
        const T cur = row[x];
        T w = smax(cur, smax(at0(row, U + x, hu), at0(row, D + x, hd)));
        if (conn8) {
            const bool l = x > 0, r = x + 1 < cols;
            w = smax(w, smax(smax(at0(row, U + x - 1, hu && l), at0(row, U + x + 1, hu && r)),
                             smax(at0(row, D + x - 1, hd && l), at0(row, D + x + 1, hd && r))));
        }
        const T m = mrow[x];
        const T v = clampv(prev, smin(w, m), m);
        if (!(v == cur)) {
            row[x] = v;
            ++nch;
        }
        prev = v;
    }
    T nxt = (T)0;
    for (int x = cols - 1; x >= 0; --x) {
        const T f = row[x];
        const T v = clampv(nxt, f, mrow[x]);
        if (!(v == f)) {
            row[x] = v;
            ++nch;
        }
        nxt = v;
    }
    if (nch) atomicAdd(changed, nch);
}

// column sweep; when `tdirty` is given, every tile with a changed pixel is
// marked for the tile queue (full pass, unconditional edge checks)
template <typename T>
__global__ void sweep_cols(const T *__restrict__ mask, T *out, int rows, int cols, int conn8, int *changed,
                           int *tdirty, int tw, int th, int tiles_x) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= cols) return;
    const bool hl = x > 0, hr = x + 1 < cols;
    int nch = 0;
    int last_tile = -1;
    T prev = (T)0;
    for (int y = 0; y < rows; ++y) {
        const int64_t i = (int64_t)y * cols + x;
        const T cur = out[i];
        T w = smax(cur, smax(at0(out, i - 1, hl), at0(out, i + 1, hr)));
        if (conn8) {
            const bool u = y > 0, d = y + 1 < rows;
            w = smax(w, smax(smax(at0(out, i - cols - 1, u && hl), at0(out, i - cols + 1, u && hr)),
                             smax(at0(out, i + cols - 1, d && hl), at0(out, i + cols + 1, d && hr))));
        }
        const T m = mask[i];
        const T v = clampv(prev, smin(w, m), m);
        if (!(v == cur)) {
            out[i] = v;
            ++nch;
            if (tdirty) {
                const int t = (y / th) * tiles_x + x / tw;
                if (t != last_tile) tdirty[t] = D_ALL | D_FRESH;
                last_tile = t;
            }
        }
        prev = v;
    }
    T nxt = (T)0;
    for (int y = rows - 1; y >= 0; --y) {
        const int64_t i = (int64_t)y * cols + x;
        const T f = out[i];
        const T v = clampv(nxt, f, mask[i]);
        if (!(v == f)) {
            out[i] = v;
            ++nch;
            if (tdirty) {
                const int t = (y / th) * tiles_x + x / tw;
                if (t != last_tile) tdirty[t] = D_ALL | D_FRESH;
                last_tile = t;
            }
        }
        nxt = v;
    }
    if (nch) atomicAdd(changed, nch);
}

__global__ void zero_ints(int *p, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0;
}

// the tile queue holds exactly the marked tiles (one block, in tile order)
__global__ void __launch_bounds__(1024) queue_marked(int *state, int *queue, const int *dirty, int qcap, int ntiles,
                                                     int *ctrl) {
    __shared__ int wsum[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    for (int i = threadIdx.x; i < qcap; i += blockDim.x) queue[i] = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int t = base + threadIdx.x;
        const bool on = t < ntiles && dirty[t] != 0;
        if (t < ntiles) state[t] = on ? 1 : 0;
        const unsigned b = __ballot_sync(0xffffffffu, on);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        if (lane == 0) wsum[warp] = __popc(b);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = carry;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                const int v = wsum[w];
                wsum[w] = acc;
                acc += v;
            }
            carry = acc;
        }
        __syncthreads();
        if (on) queue[wsum[warp] + __popc(b & ((1u << lane) - 1u))] = t + 1;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ctrl[C_QHEAD] = 0;
        ctrl[C_QTAIL] = carry;
        ctrl[C_QPEND] = carry;
        ctrl[C_RSTATS] = 0;
        ctrl[C_RSTATS + 1] = 0;
        ctrl[C_RSTATS + 3] = 0;
    }
}

struct Queue {
    int *state;
    int *queue;
    int qcap;
    int *head, *tail, *outstanding, *status;
    int *dirty;  // per tile: D_* bits for its next pass
    int *stats;  // [0] tile passes, [1] row+column sweeps
    long long budget;
    int idle_limit;  // empty-queue polls before an idle CTA leaves (0: stay until done)
    int seq_min;     // dirty lines of a 32-line group from which lanes scan one line each
    int wl_phases;   // row + column phase pairs a whole-tile pass runs before the pixel worklist
};

// lane 0 only
// An idle CTA may leave while other CTAs still hold tiles: a CTA that queues
// a tile always comes back here and takes it if nobody else does, so every
// queued tile is processed; leaving early hands the SM to other streams.
__device__ int q_pop(Queue &q) {
    long long spins = 0;
    int idle = 0;
    for (;;) {
        int h = *(volatile int *)q.head;
        int tl = *(volatile int *)q.tail;
        if (h < tl) {
            idle = 0;
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
        if (q.idle_limit > 0 && ++idle > q.idle_limit) return -1;
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

template <typename T, int TW, int TH, int P>
struct TileSmem {
    T o[(TH + 2) * P];                         // the tile and its halo (row pitch P)
    T m[TH * P];                               // the mask (row pitch P: a thread per row reads it without bank conflicts)
    T eN[TW], eS[TW], eW[TH], eE[TH];          // the tile's edge values when it was loaded
    T mN[TW + 2], mS[TW + 2], mW[TH], mE[TH];  // the mask just outside the tile (neighbours' pixels)
    unsigned drow[TH / 32], dcol[TW / 32];     // dirty rows / columns
    int edges, tile, again, sweeps, dirty, lines;
};

// The same tile plus the in-tile pixel worklist (see wl_run): a ring of
// tile-local pixel indices, the set of queued pixels, and the pixels the last
// column phase changed (column-major bits), which seed the worklist.
//
// The ring is a bounded multi-producer / multi-consumer queue with a sequence
// number per slot (the slot of ticket t is t mod kCap): a producer with
// ticket t writes only once the slot's sequence is t, and publishes t + 1; a
// consumer with ticket t reads only once the sequence is t + 1, and frees
// the slot for ticket t + kCap.  A slot word holds the sequence (mod 2^SB) in
// its high bits and the pixel index in its low VB bits.  Tickets count up
// for the CTA's lifetime; since a pixel is queued at most once at a time,
// at most kCap tickets are outstanding, so producers never wait for space.
template <typename T, int TW, int TH, int P>
struct TileWL : TileSmem<T, TW, TH, P> {
    static constexpr int kCap = TW * TH;  // every pixel at most once in the ring
    static constexpr int VB = kCap == 16384 ? 14 : (kCap == 4096 ? 12 : 0);
    static_assert(VB > 0, "tile of 128 x 128 or 64 x 64 pixels");
    static constexpr unsigned kSeqMask = (1u << (32 - VB)) - 1u;
    unsigned ring[kCap];
    unsigned inq[TW * TH / 32];  // row-major pixel bits
    unsigned cbm[TW * TH / 32];  // column-major: bit c * TH + r
    int head, tail, pending, abort, raised;
};

// Whole warp: lane l changed the pixels of its K-pixel slice (l*K .. l*K+K-1)
// given by the bits of `changed`; mark those lines and the lines next to
// them in the N-line dirty set `m` (one shared-memory atomic per word).
template <int K, int N>
__device__ __forceinline__ void mark_dirty(unsigned *m, unsigned changed) {
    constexpr int NWORD = N / 32;
    const int lane = threadIdx.x & 31;
    unsigned w[NWORD];
#pragma unroll
    for (int j = 0; j < NWORD; ++j) {
        const unsigned mine = ((lane * K) >> 5) == j ? changed << ((lane * K) & 31) : 0u;
        w[j] = __reduce_or_sync(0xffffffffu, mine);
    }
#pragma unroll
    for (int j = 0; j < NWORD; ++j) {
        unsigned d = w[j] | (w[j] << 1) | (w[j] >> 1);
        if (j > 0) d |= w[j - 1] >> 31;
        if (j + 1 < NWORD) d |= w[j + 1] << 31;
        if (lane == j && d) atomicOr(&m[j], d);
    }
}

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

// ---- one line per lane ---------------------------------------------------------
// When many lines of a 32-line group are dirty, each lane scans one whole line
// of the group itself: the raster step then the anti-raster step, pixel by
// pixel, with the cross-line neighbours kept in a sliding window.  About a
// quarter of the instructions of the shuffle scan per line; a group with few
// dirty lines keeps the shuffle scan (a lane-per-line pass costs the same
// whether 1 or 32 of its lines are dirty).  uint8 only: a pixel outside the
// image has mask 0, so min/max alone keep it 0.
constexpr int kSeqMinLines = 8;  // default: dirty lines of a group from which lanes scan one line each

// Row r (tile coordinates) of the tile in `o` (pitch P, one-pixel halo), mask
// row `m`.  chg[j] bit k: pixel j * 32 + k changed.
template <int TW, int P>
__device__ __forceinline__ void row_seq(uint8_t *o, const uint8_t *m, int r, bool conn8, unsigned (&chg)[TW / 32]) {
    uint8_t *row = o + (r + 1) * P + 1;
    const uint8_t *up = row - P, *dn = row + P;
    uint8_t prev = row[-1];
    uint8_t ul = up[-1], uc = up[0], dl = dn[-1], dc = dn[0];
#pragma unroll 1
    for (int j = 0; j < TW / 32; ++j) {
        unsigned bits = 0;
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
            const int x = j * 32 + k;
            const uint8_t ur = up[x + 1], dr = dn[x + 1], cur = row[x], mk = m[x];
            uint8_t w8 = smax(cur, smax(uc, dc));
            if (conn8) w8 = smax(w8, smax(smax(ul, ur), smax(dl, dr)));
            const uint8_t v = clampv(prev, smin(w8, mk), mk);
            if (v != cur) {
                row[x] = v;
                bits |= 1u << k;
            }
            prev = v;
            ul = uc;
            uc = ur;
            dl = dc;
            dc = dr;
        }
        chg[j] = bits;
    }
    uint8_t nxt = row[TW];
#pragma unroll 1
    for (int j = TW / 32 - 1; j >= 0; --j) {
        unsigned bits = 0;
#pragma unroll 8
        for (int k = 31; k >= 0; --k) {
            const int x = j * 32 + k;
            const uint8_t f = row[x];
            const uint8_t v = clampv(nxt, f, m[x]);
            if (v != f) {
                row[x] = v;
                bits |= 1u << k;
            }
            nxt = v;
        }
        chg[j] |= bits;
    }
}

// Column c of the tile; chg[j] bit k: pixel of row j * 32 + k changed.
template <int TH, int P>
__device__ __forceinline__ void col_seq(uint8_t *o, const uint8_t *m, int c, bool conn8, unsigned (&chg)[TH / 32]) {
    uint8_t *col = o + P + c + 1;  // pixel (0, c)
    const uint8_t *mc = m + c;
    uint8_t prev = col[-P];
    uint8_t lp = col[-P - 1], rp = col[-P + 1], lc = col[-1], rc = col[1];
#pragma unroll 1
    for (int j = 0; j < TH / 32; ++j) {
        unsigned bits = 0;
#pragma unroll 8
        for (int k = 0; k < 32; ++k) {
            const int y = j * 32 + k;
            uint8_t *px = col + y * P;
            const uint8_t ln = px[P - 1], rn = px[P + 1], cur = px[0], mk = mc[y * P];
            uint8_t w8 = smax(cur, smax(lc, rc));
            if (conn8) w8 = smax(w8, smax(smax(lp, rp), smax(ln, rn)));
            const uint8_t v = clampv(prev, smin(w8, mk), mk);
            if (v != cur) {
                px[0] = v;
                bits |= 1u << k;
            }
            prev = v;
            lp = lc;
            rp = rc;
            lc = ln;
            rc = rn;
        }
        chg[j] = bits;
    }
    uint8_t nxt = col[TH * P];
#pragma unroll 1
    for (int j = TH / 32 - 1; j >= 0; --j) {
        unsigned bits = 0;
#pragma unroll 8
        for (int k = 31; k >= 0; --k) {
            const int y = j * 32 + k;
            uint8_t *px = col + y * P;
            const uint8_t f = px[0];
            const uint8_t v = clampv(nxt, f, mc[y * P]);
            if (v != f) {
                px[0] = v;
                bits |= 1u << k;
            }
            nxt = v;
        }
        chg[j] |= bits;
    }
}

// Whole warp: every lane changed the pixels chg[] of one line; mark the
// perpendicular lines they lie on and the ones beside them in `m` (N lines).
template <int N>
__device__ __forceinline__ void mark_dirty_seq(unsigned *m, const unsigned (&chg)[N / 32]) {
    const int lane = threadIdx.x & 31;
    unsigned w[N / 32];
#pragma unroll
    for (int j = 0; j < N / 32; ++j) w[j] = __reduce_or_sync(0xffffffffu, chg[j]);
#pragma unroll
    for (int j = 0; j < N / 32; ++j) {
        unsigned d = w[j] | (w[j] << 1) | (w[j] >> 1);
        if (j > 0) d |= w[j - 1] >> 31;
        if (j + 1 < N / 32) d |= w[j + 1] << 31;
        if (lane == j && d) atomicOr(&m[j], d);
    }
}


// ---- in-tile pixel worklist --------------------------------------------------
// After one row + column phase pair, what is left to propagate inside a tile
// follows winding single-pixel paths (noisy masks), where further phase
// pairs rescan whole lines for a one-pixel advance.  The rest is therefore
// run as an asynchronous worklist in shared memory: a popped pixel p raises
// every in-tile neighbour q with o[q] < min(o[p], m[q]) to that value and
// queues q unless it is queued already.  Values only grow and every raise
// re-queues, so the worklist ends at the same least fixed point as the scans
// (the result does not depend on the order).  Warps claim up to 32 ring slots
// at a time; `pending` (queued + in progress) reaching 0 ends the tile.  All
// waits are bounded by the spin budget; running out sets DEV_TIMEOUT.

// raise o[idx] to `cand` if it is below; true when this call raised it
__device__ __forceinline__ bool wl_raise(uint8_t *o, int idx, uint8_t cand) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(o + idx);
    unsigned *w = reinterpret_cast<unsigned *>(a & ~(uintptr_t)3);
    const int sh = (int)(a & 3) * 8;
    unsigned old = *reinterpret_cast<volatile unsigned *>(w);
    for (int guard = 0; guard < 4096; ++guard) {
        if (((old >> sh) & 255u) >= cand) return false;
        const unsigned nw = (old & ~(255u << sh)) | ((unsigned)cand << sh);
        const unsigned prev = atomicCAS(w, old, nw);
        if (prev == old) return true;
        old = prev;
    }
    return false;  // unreachable: each failed exchange saw a larger value
}
__device__ __forceinline__ bool wl_raise(float *o, int idx, float cand) {
    int *w = reinterpret_cast<int *>(o + idx);
    int old = *reinterpret_cast<volatile int *>(w);
    for (int guard = 0; guard < (1 << 20); ++guard) {
        if (!(__int_as_float(old) < cand)) return false;
        const int prev = atomicCAS(w, old, __float_as_int(cand));
        if (prev == old) return true;
        old = prev;
    }
    return false;
}

template <typename T>
__device__ __forceinline__ T vld(const T *p) {
    return *reinterpret_cast<const volatile T *>(p);
}

// queue pixel p (tile-local index r * TW + c) if it is not queued already
template <typename WLT>
__device__ __forceinline__ void wl_push(WLT &sm, int p, long long budget, int *status) {
    const unsigned bit = 1u << (p & 31);
    if (atomicOr(&sm.inq[p >> 5], bit) & bit) return;
    atomicAdd(&sm.pending, 1);
    const unsigned t = (unsigned)atomicAdd(&sm.tail, 1);
    volatile unsigned *slot = &sm.ring[t & (WLT::kCap - 1)];
    for (long long k = 0; (*slot >> WLT::VB) != (t & WLT::kSeqMask); ++k) {
        if (k > budget) {  // cannot happen while at most kCap tickets are outstanding
            atomicOr(status, DEV_TIMEOUT);
            atomicExch(&sm.abort, 1);
            return;
        }
    }
    *slot = (((t + 1u) & WLT::kSeqMask) << WLT::VB) | (unsigned)p;
}

// every thread of the CTA; returns when the worklist is empty (or aborted)
template <typename T, int TW, int TH, int P, int NW>
__device__ void wl_run(TileWL<T, TW, TH, P> &sm, bool conn8, long long budget, int *status) {
    using W = TileWL<T, TW, TH, P>;
    static_assert((W::kCap & (W::kCap - 1)) == 0, "ring capacity must be a power of two");
    const int lane = threadIdx.x & 31;
    T *o = sm.o;
    long long spins = 0;
    for (;;) {
        if (vld(&sm.abort)) break;
        int h = 0, n = 0;
        if (lane == 0) {
            const int hh = vld(&sm.head), tt = vld(&sm.tail);
            if (hh < tt) {
                const int want = tt - hh < 32 ? tt - hh : 32;
                if (atomicCAS(&sm.head, hh, hh + want) == hh) h = hh, n = want;
            } else if (vld(&sm.pending) == 0) {
                n = -1;
            }
        }
        n = __shfl_sync(0xffffffffu, n, 0);
        h = __shfl_sync(0xffffffffu, h, 0);
        if (n < 0) break;
        if (n == 0) {
            if (++spins > budget) {
                if (lane == 0) {
                    atomicOr(status, DEV_TIMEOUT);
                    atomicExch(&sm.abort, 1);
                }
                break;
            }
            continue;
        }
        if (lane < n) {
            const unsigned t = (unsigned)(h + lane);
            volatile unsigned *slot = &sm.ring[t & (W::kCap - 1)];
            unsigned word = *slot;
            bool ok = true;
            for (long long k = 0; (word >> W::VB) != ((t + 1u) & W::kSeqMask); word = *slot, ++k) {
                if (k > budget) {
                    atomicOr(status, DEV_TIMEOUT);
                    atomicExch(&sm.abort, 1);
                    ok = false;
                    break;
                }
            }
            if (ok) {
                const int p = (int)(word & ((1u << W::VB) - 1u));
                *slot = ((t + (unsigned)W::kCap) & W::kSeqMask) << W::VB;  // free for ticket t + kCap
                atomicAnd(&sm.inq[p >> 5], ~(1u << (p & 31)));
                __threadfence_block();
                const int r = p / TW, c = p - r * TW;
                const T v = vld(&o[(r + 1) * P + c + 1]);
                bool any = false;
#pragma unroll
                for (int d = 0; d < 8; ++d) {
                    const int dy = d < 3 ? -1 : (d < 5 ? 0 : 1);
                    const int dx = d < 3 ? d - 1 : (d < 5 ? (d == 3 ? -1 : 1) : d - 6);
                    if (!conn8 && dy != 0 && dx != 0) continue;
                    const int rq = r + dy, cq = c + dx;
                    if (rq < 0 || rq >= TH || cq < 0 || cq >= TW) continue;
                    const T mq = sm.m[rq * P + cq];
                    const T cand = smin(v, mq);
                    const int oi = (rq + 1) * P + cq + 1;
                    if (vld(&o[oi]) < cand && wl_raise(o, oi, cand)) {
                        any = true;
                        wl_push(sm, rq * TW + cq, budget, status);
                    }
                }
                if (any) sm.raised = 1;
                atomicSub(&sm.pending, 1);
            }
        }
        __syncwarp();
    }
}

// Seed the worklist from the pixels the last column phase changed (cbm),
// then clear cbm.  Called by every thread; ends with a barrier.
template <typename T, int TW, int TH, int P, int NW>
__device__ void wl_seed_changed(TileWL<T, TW, TH, P> &sm, long long budget, int *status) {
    constexpr int NWORD = TW * TH / 32;
    for (int w = threadIdx.x; w < NWORD; w += NW * 32) {
        unsigned b = sm.cbm[w];
        sm.cbm[w] = 0;
        while (b) {
            const int k = __ffs(b) - 1;
            b &= b - 1;
            const int bit = w * 32 + k;  // column-major: c * TH + r
            const int c = bit / TH, r = bit - c * TH;
            wl_push(sm, r * TW + c, budget, status);
        }
    }
    __syncthreads();
}

// Seed from the halo on the sides in `dirty_in`: an edge pixel below
// min(halo neighbour, its mask) is raised to it and queued.  The worklist
// then carries the change inward.  Ends with a barrier.
template <typename T, int TW, int TH, int P, int NW>
__device__ void wl_seed_halo(TileWL<T, TW, TH, P> &sm, int dirty_in, bool conn8, long long budget, int *status) {
    T *o = sm.o;
    const int c8 = conn8 ? 1 : 0;
    auto pull = [&](int r, int c, int hr, int hc0, int hstep) {
        // pixel (r, c) from the halo pixels hr/hc0 + k * hstep, k = -c8..c8
        const T mq = sm.m[r * P + c];
        T best = (T)0;
        bool have = false;
        for (int k = -c8; k <= c8; ++k) {
            const int yy = hr + (hstep ? 0 : k), xx = hc0 + (hstep ? k : 0);
            const T hv = vld(&o[(yy + 1) * P + xx + 1]);
            const T cand = smin(hv, mq);
            if (!have || best < cand) best = cand, have = true;
        }
        const int oi = (r + 1) * P + c + 1;
        if (vld(&o[oi]) < best && wl_raise(o, oi, best)) {
            sm.raised = 1;
            wl_push(sm, r * TW + c, budget, status);
        }
    };
    if (dirty_in & D_N)
        for (int c = threadIdx.x; c < TW; c += NW * 32) pull(0, c, -1, c, 1);
    if (dirty_in & D_S)
        for (int c = threadIdx.x; c < TW; c += NW * 32) pull(TH - 1, c, TH, c, 1);
    if (dirty_in & D_W)
        for (int r = threadIdx.x; r < TH; r += NW * 32) pull(r, 0, r, -1, 0);
    if (dirty_in & D_E)
        for (int r = threadIdx.x; r < TH; r += NW * 32) pull(r, TW - 1, r, TW, 0);
    __syncthreads();
}


// ---- TMA-fed tile load (uint8, 128 x 128 tiles) -----------------------------
// One elected thread stages the tile's out plane and mask, each with a
// one-pixel ring, into shared memory with two 2-D tensor copies
// (cp.async.bulk.tensor) that complete on one mbarrier; the CTA waits on the
// barrier (bounded) and unpacks the staging boxes into the padded tile
// layout.  The boxes are 160 x 130 bytes starting at (x0 - 16, y0 - 1): the
// innermost start coordinate stays a multiple of 16 bytes (x0 is a multiple
// of 128), and samples outside the image read as 0, which is the
// reconstruction's padding ring and the mask outside the image.  The host
// only enables this when the row pitch and both base addresses are
// multiples of 16 bytes (the tensor-map rules); otherwise the plain loads run.
constexpr int kStW = 160, kStH = 130, kStageBytes = kStW * kStH;
// a tensor copy's shared-memory destination must sit on a 128-byte boundary:
// each staging box starts at one (20800 bytes rounded up to 20864)
constexpr int kStagePitch = (kStageBytes + 127) & ~127;

struct TmaArgs {
    const CUtensorMap *out_map, *mask_map;  // the kernel's __grid_constant__ parameters
    uint8_t *stage;                         // 2 boxes kStagePitch apart, 128-byte aligned
    uint64_t *bar;                          // the copies' mbarrier
    unsigned *phase;                        // its current phase parity
    int on;
};

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes) : "memory");
}
// true when the phase with parity `parity` has completed within `budget` polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, long long budget) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(bar);
    for (long long k = 0; k <= budget; ++k) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void tma_load_2d(uint8_t *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst), b = (unsigned)__cvta_generic_to_shared(bar);
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(d), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(b)
        : "memory");
}

// the tile (ty, tx) and its ring into `o` (pitch P), the mask into `m`, and
// the mask just outside the tile into mN / mS / mW / mE; returns false when
// the copies did not arrive within the budget (DEV_TIMEOUT is then set)
template <int P>
__device__ bool tma_tile_u8(const TmaArgs &ta, int tx, int ty, uint8_t *o, uint8_t *m, uint8_t *mN, uint8_t *mS,
                            uint8_t *mW, uint8_t *mE, long long budget, int *status) {
    constexpr int TW = 128, TH = 128;
    const int x0 = tx * TW, y0 = ty * TH;
    const unsigned parity = *ta.phase;
    if (threadIdx.x == 0) {
        // `out` was last written by generic stores (this CTA's or, before the
        // queue handed the tile over, other CTAs'); the staging area was last
        // read by generic loads: order both before the async-proxy copies
        asm volatile("fence.proxy.async.global;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(ta.bar, 2 * kStageBytes);
        tma_load_2d(ta.stage, ta.out_map, x0 - 16, y0 - 1, ta.bar);
        tma_load_2d(ta.stage + kStagePitch, ta.mask_map, x0 - 16, y0 - 1, ta.bar);
    }
    bool ok = mbar_wait(ta.bar, parity, budget);
    if (!ok) {
        atomicOr(status, DEV_TIMEOUT);
        ok = mbar_wait(ta.bar, parity, budget);  // do not leave copies in flight into this CTA's memory
    }
    __syncthreads();
    if (threadIdx.x == 0) *ta.phase = parity ^ 1u;
    const uint8_t *so = ta.stage, *sk = ta.stage + kStagePitch;
    for (int i = threadIdx.x; i < (TH + 2) * (TW + 2); i += blockDim.x) {
        const int r = i / (TW + 2), c = i - r * (TW + 2);
        o[r * P + c] = so[r * kStW + 15 + c];
    }
    for (int i = threadIdx.x; i < TH * TW; i += blockDim.x) {
        const int r = i / TW, c = i - r * TW;
        m[r * P + c] = sk[(r + 1) * kStW + 16 + c];
    }
    for (int i = threadIdx.x; i < TW + 2; i += blockDim.x) {
        mN[i] = sk[15 + i];
        mS[i] = sk[(TH + 1) * kStW + 15 + i];
    }
    for (int i = threadIdx.x; i < TH; i += blockDim.x) {
        mW[i] = sk[(i + 1) * kStW + 15];
        mE[i] = sk[(i + 1) * kStW + 16 + TW];
    }
    return ok;
}

// One pass over tile (tx, ty): load, alternate row / column phases over the
// dirty lines until nothing changes, report which neighbours must run again,
// write back.
//
// WL: a pass over a whole tile (D_ALL / D_FRESH) runs `wl_phases` row +
// column phase pairs and hands what is still moving to the pixel worklist
// (seeded with the pixels the last column phase changed); a pass for changed
// halo sides skips the phases and seeds the worklist from those sides.
template <typename T, int TW, int TH, int P, int NW, bool HYB, bool WL, typename SM>
__device__ void cta_process_tile(const T *__restrict__ mask, T *out, int rows, int cols, bool conn8, int tx, int ty,
                                 int dirty_in, SM &sm, int seq_min, int wl_phases, long long budget, int *status,
                                 const TmaArgs &ta) {
    static_assert(!HYB || (std::is_same<T, uint8_t>::value && NW == TH / 32 && NW == TW / 32),
                  "lane-per-line scans: uint8, one warp per 32-line group");
    constexpr int NWORD = TW * TH / 32;
    constexpr int KX = TW / 32, KY = TH / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int y0 = ty * TH, x0 = tx * TW;
    T *o = sm.o;
    bool tma_loaded = false;
    if constexpr (std::is_same<T, uint8_t>::value && TW == 128 && TH == 128) {
        if (ta.on) {
            tma_tile_u8<P>(ta, tx, ty, o, sm.m, sm.mN, sm.mS, sm.mW, sm.mE, budget, status);
            tma_loaded = true;
        }
    }
    if (!tma_loaded) {
        // load tile + halo (image ring = 0) and the mask
        for (int i = threadIdx.x; i < (TH + 2) * (TW + 2); i += NW * 32) {
            int r = i / (TW + 2), cc = i - r * (TW + 2);
            int y = y0 - 1 + r, x = x0 - 1 + cc;
            o[r * P + cc] = (y >= 0 && y < rows && x >= 0 && x < cols) ? ldcg(out + (int64_t)y * cols + x) : (T)0;
        }
        for (int i = threadIdx.x; i < TH * TW; i += NW * 32) {
            int r = i / TW, cc = i - r * TW;
            int y = y0 + r, x = x0 + cc;
            sm.m[r * P + cc] = (y < rows && x < cols) ? __ldg(mask + (int64_t)y * cols + x) : (T)0;
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
    }
    const bool all = dirty_in & D_ALL;
    if (threadIdx.x < TH / 32) {
        const int w = threadIdx.x;
        unsigned b = all ? ~0u : 0u;
        if ((dirty_in & D_N) && w == 0) b |= 1u;
        if ((dirty_in & D_S) && w == TH / 32 - 1) b |= 1u << 31;
        sm.drow[w] = b;
    }
    if (threadIdx.x >= 32 && threadIdx.x < 32 + TW / 32) {
        const int w = threadIdx.x - 32;
        unsigned b = all ? ~0u : 0u;
        if ((dirty_in & D_W) && w == 0) b |= 1u;
        if ((dirty_in & D_E) && w == TW / 32 - 1) b |= 1u << 31;
        sm.dcol[w] = b;
    }
    if (threadIdx.x == 0) {
        sm.edges = 0;
        sm.sweeps = 0;
        sm.lines = 0;
        if constexpr (WL) {
            sm.pending = 0;
            sm.abort = 0;
            sm.raised = 0;
        }
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
    const bool phases = !WL || (dirty_in & (D_ALL | D_FRESH));
    const int max_it = WL ? wl_phases : 1024;
    bool need_wl = false;
    for (int it = 0; phases && it < max_it; ++it) {
        if constexpr (WL)
            for (int w = threadIdx.x; w < NWORD; w += NW * 32) sm.cbm[w] = 0;
        // ---- row phase over the dirty rows (round robin over warps)
        unsigned rm[TH / 32];
#pragma unroll
        for (int w = 0; w < TH / 32; ++w) rm[w] = sm.drow[w];
        if (threadIdx.x == 0)
            for (int w = 0; w < TH / 32; ++w) sm.lines += __popc(rm[w]);
        __syncthreads();
        if (threadIdx.x < TH / 32) sm.drow[threadIdx.x] = 0;
        bool chr = false;
        int seq = 0;
#pragma unroll
        for (int w = 0; w < TH / 32; ++w) {
            unsigned bits = rm[w];
            if constexpr (HYB) {
                if (__popc(bits) >= seq_min) {
                    if (warp == w) {
                        unsigned chg[TW / 32] = {};
                        const int r = w * 32 + lane;
                        if ((bits >> lane) & 1u) row_seq<TW, P>(o, sm.m + r * P, r, conn8, chg);
                        unsigned any = 0;
#pragma unroll
                        for (int j = 0; j < TW / 32; ++j) any |= chg[j];
                        if (__any_sync(0xffffffffu, any != 0)) {
                            chr = true;
                            mark_dirty_seq<TW>(sm.dcol, chg);
                        }
                    }
                    continue;
                }
            }
            while (bits) {
                const int r = w * 32 + __ffs(bits) - 1;
                bits &= bits - 1;
                if ((seq++ & (NW - 1)) != warp) continue;
                T *row = o + (r + 1) * P + 1;
                const T *up = row - P, *dn = row + P;
                T lo[KX], hi[KX], cur[KX], res[KX];
#pragma unroll
                for (int k = 0; k < KX; ++k) {
                    int x = lane * KX + k;
                    cur[k] = row[x];
                    T w8 = smax(cur[k], smax(up[x], dn[x]));
                    if (conn8) w8 = smax(w8, smax(smax(up[x - 1], up[x + 1]), smax(dn[x - 1], dn[x + 1])));
                    T mk = sm.m[r * P + x];
                    bool in = r < vr && x < vc;
                    lo[k] = in ? smin(w8, mk) : (T)0;
                    hi[k] = in ? mk : (T)0;
                }
                line_scan<T, KX>(lo, hi, row[-1], row[TW], res);
                unsigned changed = 0;
#pragma unroll
                for (int k = 0; k < KX; ++k) {
                    int x = lane * KX + k;
                    if (!(res[k] == cur[k])) {
                        row[x] = res[k];
                        changed |= 1u << k;
                    }
                }
                if (__any_sync(0xffffffffu, changed != 0)) {
                    chr = true;
                    mark_dirty<KX, TW>(sm.dcol, changed);
                }
            }
        }
        chr = __syncthreads_or(chr);
        // ---- column phase over the dirty columns
        unsigned cm[TW / 32];
#pragma unroll
        for (int w = 0; w < TW / 32; ++w) cm[w] = sm.dcol[w];
        if (threadIdx.x == 0)
            for (int w = 0; w < TW / 32; ++w) sm.lines += __popc(cm[w]);
        __syncthreads();
        if (threadIdx.x < TW / 32) sm.dcol[threadIdx.x] = 0;
        bool chc = false;
        seq = 0;
#pragma unroll
        for (int w = 0; w < TW / 32; ++w) {
            unsigned bits = cm[w];
            if constexpr (HYB) {
                if (__popc(bits) >= seq_min) {
                    if (warp == w) {
                        unsigned chg[TH / 32] = {};
                        if ((bits >> lane) & 1u) col_seq<TH, P>(o, sm.m, w * 32 + lane, conn8, chg);
                        if constexpr (WL) {
#pragma unroll
                            for (int j = 0; j < TH / 32; ++j)
                                if (chg[j]) sm.cbm[(w * 32 + lane) * (TH / 32) + j] = chg[j];
                        }
                        unsigned any = 0;
#pragma unroll
                        for (int j = 0; j < TH / 32; ++j) any |= chg[j];
                        if (__any_sync(0xffffffffu, any != 0)) {
                            chc = true;
                            mark_dirty_seq<TH>(sm.drow, chg);
                        }
                    }
                    continue;
                }
            }
            while (bits) {
                const int cidx = w * 32 + __ffs(bits) - 1;
                bits &= bits - 1;
                if ((seq++ & (NW - 1)) != warp) continue;
                T lo[KY], hi[KY], cur[KY], res[KY];
#pragma unroll
                for (int k = 0; k < KY; ++k) {
                    int y = lane * KY + k;
                    T *p = o + (y + 1) * P + (cidx + 1);
                    cur[k] = p[0];
                    T w8 = smax(cur[k], smax(p[-1], p[1]));
                    if (conn8) w8 = smax(w8, smax(smax(p[-P - 1], p[-P + 1]), smax(p[P - 1], p[P + 1])));
                    T mk = sm.m[y * P + cidx];
                    bool in = y < vr && cidx < vc;
                    lo[k] = in ? smin(w8, mk) : (T)0;
                    hi[k] = in ? mk : (T)0;
                }
                line_scan<T, KY>(lo, hi, o[cidx + 1], o[(TH + 1) * P + cidx + 1], res);
                unsigned changed = 0;
#pragma unroll
                for (int k = 0; k < KY; ++k) {
                    int y = lane * KY + k;
                    if (!(res[k] == cur[k])) {
                        o[(y + 1) * P + cidx + 1] = res[k];
                        changed |= 1u << k;
                    }
                }
                if constexpr (WL) {
                    if (changed)
                        atomicOr(&sm.cbm[cidx * (TH / 32) + ((lane * KY) >> 5)], changed << ((lane * KY) & 31));
                }
                if (__any_sync(0xffffffffu, changed != 0)) {
                    chc = true;
                    mark_dirty<KY, TH>(sm.drow, changed);
                }
            }
        }
        chc = __syncthreads_or(chc);
        if (threadIdx.x == 0) sm.sweeps = it + 1;
        anych = anych || chr || chc;
        if (!chc) break;  // no row is dirty: the tile is stable
        if (it == max_it - 1) {
            if (WL) need_wl = true;  // the worklist finishes the tile
            else my_edges |= 16u;    // not stable yet: process again later
        }
    }
    if constexpr (WL) {
        if (need_wl) wl_seed_changed<T, TW, TH, P, NW>(sm, budget, status);
        else if (!phases) wl_seed_halo<T, TW, TH, P, NW>(sm, dirty_in, conn8, budget, status);
        if (need_wl || !phases) {
            wl_run<T, TW, TH, P, NW>(sm, conn8, budget, status);
            __syncthreads();
            if (sm.raised) anych = true;
        }
    }
    // A neighbour tile needs another pass only if an edge pixel that changed
    // here can raise one of its pixels: new value above that pixel's value
    // (as loaded; it can only have grown since) and that pixel below its mask.
    const bool fresh = dirty_in & D_FRESH;  // the tile changed before this pass: check every edge pixel
    if (anych || fresh) {
        const int c8 = conn8 ? 1 : 0;
        for (int x = threadIdx.x; x < TW; x += NW * 32) {
            T v = o[P + x + 1];
            if (fresh || !(v == sm.eN[x]))
                for (int d = -c8; d <= c8; ++d) {
                    int h = x + d;
                    if (h < 0 || h >= TW) continue;
                    T hv = o[h + 1];
                    if (v > hv && sm.mN[h + 1] > hv) my_edges |= 1u;
                }
            v = o[TH * P + x + 1];
            if (fresh || !(v == sm.eS[x]))
                for (int d = -c8; d <= c8; ++d) {
                    int h = x + d;
                    if (h < 0 || h >= TW) continue;
                    T hv = o[(TH + 1) * P + h + 1];
                    if (v > hv && sm.mS[h + 1] > hv) my_edges |= 2u;
                }
        }
        for (int y = threadIdx.x; y < TH; y += NW * 32) {
            T v = o[(y + 1) * P + 1];
            if (fresh || !(v == sm.eW[y]))
                for (int d = -c8; d <= c8; ++d) {
                    int h = y + d;
                    if (h < 0 || h >= TH) continue;
                    T hv = o[(h + 1) * P];
                    if (v > hv && sm.mW[h] > hv) my_edges |= 4u;
                }
            v = o[(y + 1) * P + TW];
            if (fresh || !(v == sm.eE[y]))
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
            if ((fresh || !(v == sm.eN[0])) && v > hv && sm.mN[0] > hv) my_edges |= 32u;  // up-left
            v = o[P + TW], hv = o[TW + 1];
            if ((fresh || !(v == sm.eN[TW - 1])) && v > hv && sm.mN[TW + 1] > hv) my_edges |= 64u;  // up-right
            v = o[TH * P + 1], hv = o[(TH + 1) * P];
            if ((fresh || !(v == sm.eS[0])) && v > hv && sm.mS[0] > hv) my_edges |= 128u;  // down-left
            v = o[TH * P + TW], hv = o[(TH + 1) * P + TW + 1];
            if ((fresh || !(v == sm.eS[TW - 1])) && v > hv && sm.mS[TW + 1] > hv) my_edges |= 256u;  // down-right
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

// ---- packed uint8 tile pass ---------------------------------------------------
// The uint8 reconstruction keeps its tile twice in shared memory, row-major
// (`o`) and transposed (`oT`), so that both phases are the same "strip" scan:
// a warp takes 4 adjacent lines as one 32-bit word per position and scans
// across the lanes with byte-wise SIMD (__vmaxu4 / __vminu4), 4 lines per
// instruction.  The row phase is a strip scan on oT, the column phase one on
// o; a phase writes the words it changes into its own layout and the changed
// bytes into the other one.  Interior pixel (r, c) of a layout with pitch PL
// sits at byte (r + 1) * PL + 4 + c, so every strip word is 4-byte aligned
// and its halo neighbours are byte 3 of the word before / byte 0 of the word
// after.
template <int TW, int TH>
struct TileU8 {
    static constexpr int P = TW + 8;   // pitch of o: 4 pad bytes, halo at byte 3, TW pixels, halo, pad
    static constexpr int PT = TH + 8;  // pitch of oT
    uint8_t o[(TH + 2) * P];
    uint8_t oT[(TW + 2) * PT];
    uint8_t m[TH * TW];   // mask, row-major
    uint8_t mT[TW * TH];  // mask, transposed
    uint8_t eN[TW], eS[TW], eW[TH], eE[TH];
    uint8_t mN[TW + 2], mS[TW + 2], mW[TH], mE[TH];
    unsigned drow[TH / 32], dcol[TW / 32];
    int edges, tile, again, sweeps, dirty, lines;
};

__device__ __forceinline__ uint32_t clamp4(uint32_t x, uint32_t lo, uint32_t hi) {
    return __vminu4(__vmaxu4(x, lo), hi);
}

// forward then backward clamp scans of K words per lane (4 lines at once)
template <int K>
__device__ __forceinline__ void line_scan_u8x4(const uint32_t (&lo)[K], const uint32_t (&hi)[K], uint32_t first,
                                               uint32_t last, uint32_t (&res)[K]) {
    const int lane = threadIdx.x & 31;
    uint32_t FL = lo[0], FH = hi[0];
#pragma unroll
    for (int k = 1; k < K; ++k) {
        const uint32_t nl = clamp4(FL, lo[k], hi[k]), nh = clamp4(FH, lo[k], hi[k]);
        FL = nl;
        FH = nh;
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t pl = __shfl_up_sync(0xffffffffu, FL, d), ph = __shfl_up_sync(0xffffffffu, FH, d);
        if (lane >= d) {
            const uint32_t nl = clamp4(pl, FL, FH), nh = clamp4(ph, FL, FH);
            FL = nl;
            FH = nh;
        }
    }
    uint32_t el = __shfl_up_sync(0xffffffffu, FL, 1), eh = __shfl_up_sync(0xffffffffu, FH, 1);
    uint32_t y = lane == 0 ? first : clamp4(first, el, eh);
    uint32_t v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        y = clamp4(y, lo[k], hi[k]);
        v[k] = y;
    }
    // backward on the forward result: g_k(y) = clamp(y, v_k, hi_k) (v_k <= hi_k)
    uint32_t BL = v[K - 1], BH = hi[K - 1];
#pragma unroll
    for (int k = K - 2; k >= 0; --k) {
        const uint32_t nl = clamp4(BL, v[k], hi[k]), nh = clamp4(BH, v[k], hi[k]);
        BL = nl;
        BH = nh;
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t pl = __shfl_down_sync(0xffffffffu, BL, d), ph = __shfl_down_sync(0xffffffffu, BH, d);
        if (lane + d < 32) {
            const uint32_t nl = clamp4(pl, BL, BH), nh = clamp4(ph, BL, BH);
            BL = nl;
            BH = nh;
        }
    }
    el = __shfl_down_sync(0xffffffffu, BL, 1);
    eh = __shfl_down_sync(0xffffffffu, BH, 1);
    y = lane == 31 ? last : clamp4(last, el, eh);
#pragma unroll
    for (int k = K - 1; k >= 0; --k) {
        y = clamp4(y, v[k], hi[k]);
        res[k] = y;
    }
}

// One phase on layout L (LEN interior rows, the scan direction; NL interior
// columns, the lines): every dirty strip of 4 columns is scanned down and up.
// Changed words are stored into L, changed bytes into X (the transpose, pitch
// PX), and rows next to a change are marked in `other` (LEN bits).  Returns
// whether this warp changed anything.
template <int LEN, int NL, int PL, int PX, int NW>
__device__ bool strip_phase(uint8_t *L, const uint8_t *__restrict__ M, uint8_t *X, const unsigned (&dirty)[NL / 32],
                            unsigned *other, bool conn8, int &lines) {
    constexpr int K = LEN / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool ch = false;
    int seq = 0;
#pragma unroll
    for (int w = 0; w < NL / 32; ++w) {
#pragma unroll 1
        for (int g = 0; g < 8; ++g) {  // 8 strips of 4 columns per 32-bit dirty word
            if (!((dirty[w] >> (4 * g)) & 15u)) continue;
            if ((seq++ & (NW - 1)) != warp) continue;
            if (lane == 0) ++lines;
            const int s = w * 8 + g;
            const int cb = 4 + 4 * s;
            uint32_t cur[K], h2[K + 2];
#pragma unroll
            for (int t = 0; t < K + 2; ++t) {
                const uint8_t *row = L + (lane * K + t) * PL;  // L-row lane*K - 1 + t
                const uint32_t c = *reinterpret_cast<const uint32_t *>(row + cb);
                const uint32_t l = *reinterpret_cast<const uint32_t *>(row + cb - 4);
                const uint32_t r = *reinterpret_cast<const uint32_t *>(row + cb + 4);
                h2[t] = __vmaxu4(__byte_perm(l, c, 0x6543), __byte_perm(c, r, 0x4321));
                if (t >= 1 && t <= K) cur[t - 1] = c;
            }
            uint32_t lo[K], hi[K], res[K];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t mk = *reinterpret_cast<const uint32_t *>(M + (lane * K + k) * NL + 4 * s);
                uint32_t w8 = __vmaxu4(cur[k], h2[k + 1]);
                if (conn8) w8 = __vmaxu4(w8, __vmaxu4(h2[k], h2[k + 2]));
                lo[k] = __vminu4(w8, mk);
                hi[k] = mk;
            }
            const uint32_t first = *reinterpret_cast<const uint32_t *>(L + cb);
            const uint32_t last = *reinterpret_cast<const uint32_t *>(L + (LEN + 1) * PL + cb);
            line_scan_u8x4<K>(lo, hi, first, last, res);
            unsigned changed = 0;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t diff = res[k] ^ cur[k];
                if (diff) {
                    const int r = lane * K + k;
                    *reinterpret_cast<uint32_t *>(L + (r + 1) * PL + cb) = res[k];
#pragma unroll
                    for (int b = 0; b < 4; ++b)
                        if ((diff >> (8 * b)) & 255u) X[(4 * s + b + 1) * PX + 4 + r] = (uint8_t)(res[k] >> (8 * b));
                    changed |= 1u << k;
                }
            }
            if (__any_sync(0xffffffffu, changed != 0)) {
                ch = true;
                mark_dirty<K, LEN>(other, changed);
            }
        }
    }
    return ch;
}

template <int TW, int TH, int NW>
__device__ void cta_process_tile_u8(const uint8_t *__restrict__ mask, uint8_t *out, int rows, int cols, bool conn8,
                                    int tx, int ty, int dirty_in, TileU8<TW, TH> &sm) {
    constexpr int P = TileU8<TW, TH>::P, PT = TileU8<TW, TH>::PT;
    const int y0 = ty * TH, x0 = tx * TW;
    uint8_t *o = sm.o, *oT = sm.oT;
    auto O = [&](int y, int x) -> uint8_t & { return o[(y + 1) * P + 4 + x]; };  // y in [-1, TH], x in [-1, TW]
    // load tile + halo (image ring = 0) into both layouts, and the mask
    for (int i = threadIdx.x; i < (TH + 2) * (TW + 2); i += NW * 32) {
        const int r = i / (TW + 2) - 1, cc = i - (r + 1) * (TW + 2) - 1;
        const int y = y0 + r, x = x0 + cc;
        const uint8_t v = (y >= 0 && y < rows && x >= 0 && x < cols) ? ldcg(out + (int64_t)y * cols + x) : 0;
        o[(r + 1) * P + 4 + cc] = v;
        oT[(cc + 1) * PT + 4 + r] = v;
    }
    for (int i = threadIdx.x; i < TH * TW; i += NW * 32) {
        const int r = i / TW, cc = i - r * TW;
        const int y = y0 + r, x = x0 + cc;
        const uint8_t v = (y < rows && x < cols) ? __ldg(mask + (int64_t)y * cols + x) : 0;
        sm.m[r * TW + cc] = v;
        sm.mT[cc * TH + r] = v;
    }
    auto mask_at = [&](int y, int x) -> uint8_t {
        return (y >= 0 && y < rows && x >= 0 && x < cols) ? __ldg(mask + (int64_t)y * cols + x) : 0;
    };
    for (int i = threadIdx.x; i < TW + 2; i += NW * 32) {
        sm.mN[i] = mask_at(y0 - 1, x0 - 1 + i);
        sm.mS[i] = mask_at(y0 + TH, x0 - 1 + i);
    }
    for (int i = threadIdx.x; i < TH; i += NW * 32) {
        sm.mW[i] = mask_at(y0 + i, x0 - 1);
        sm.mE[i] = mask_at(y0 + i, x0 + TW);
    }
    const bool all = dirty_in & D_ALL;
    if (threadIdx.x < TH / 32) {
        const int w = threadIdx.x;
        unsigned b = all ? ~0u : 0u;
        if ((dirty_in & D_N) && w == 0) b |= 1u;
        if ((dirty_in & D_S) && w == TH / 32 - 1) b |= 1u << 31;
        sm.drow[w] = b;
    }
    if (threadIdx.x >= 32 && threadIdx.x < 32 + TW / 32) {
        const int w = threadIdx.x - 32;
        unsigned b = all ? ~0u : 0u;
        if ((dirty_in & D_W) && w == 0) b |= 1u;
        if ((dirty_in & D_E) && w == TW / 32 - 1) b |= 1u << 31;
        sm.dcol[w] = b;
    }
    if (threadIdx.x == 0) {
        sm.edges = 0;
        sm.sweeps = 0;
        sm.lines = 0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TW; i += NW * 32) {
        sm.eN[i] = O(0, i);
        sm.eS[i] = O(TH - 1, i);
    }
    for (int i = threadIdx.x; i < TH; i += NW * 32) {
        sm.eW[i] = O(i, 0);
        sm.eE[i] = O(i, TW - 1);
    }
    unsigned my_edges = 0;
    bool anych = false;
    int lines = 0;
    for (int it = 0; it < 1024; ++it) {
        // ---- row phase: strips of 4 rows, scanned along x in the transposed copy
        unsigned rm[TH / 32];
#pragma unroll
        for (int w = 0; w < TH / 32; ++w) rm[w] = sm.drow[w];
        __syncthreads();
        if (threadIdx.x < TH / 32) sm.drow[threadIdx.x] = 0;
        bool chr = strip_phase<TW, TH, PT, P, NW>(oT, sm.mT, o, rm, sm.dcol, conn8, lines);
        chr = __syncthreads_or(chr);
        // ---- column phase: strips of 4 columns, scanned along y in the tile
        unsigned cm[TW / 32];
#pragma unroll
        for (int w = 0; w < TW / 32; ++w) cm[w] = sm.dcol[w];
        __syncthreads();
        if (threadIdx.x < TW / 32) sm.dcol[threadIdx.x] = 0;
        bool chc = strip_phase<TH, TW, P, PT, NW>(o, sm.m, oT, cm, sm.drow, conn8, lines);
        chc = __syncthreads_or(chc);
        if (threadIdx.x == 0) sm.sweeps = it + 1;
        anych = anych || chr || chc;
        if (!chc) break;  // no row is dirty: the tile is stable
        if (it == 1023) my_edges |= 16u;  // not stable yet: process again later
    }
    if ((threadIdx.x & 31) == 0 && lines) atomicAdd(&sm.lines, 4 * lines);
    // notifications, as in the scalar pass
    const bool fresh = dirty_in & D_FRESH;
    if (anych || fresh) {
        const int c8 = conn8 ? 1 : 0;
        for (int x = threadIdx.x; x < TW; x += NW * 32) {
            uint8_t v = O(0, x);
            if (fresh || v != sm.eN[x])
                for (int d = -c8; d <= c8; ++d) {
                    const int h = x + d;
                    if (h < 0 || h >= TW) continue;
                    const uint8_t hv = O(-1, h);
                    if (v > hv && sm.mN[h + 1] > hv) my_edges |= 1u;
                }
            v = O(TH - 1, x);
            if (fresh || v != sm.eS[x])
                for (int d = -c8; d <= c8; ++d) {
                    const int h = x + d;
                    if (h < 0 || h >= TW) continue;
                    const uint8_t hv = O(TH, h);
                    if (v > hv && sm.mS[h + 1] > hv) my_edges |= 2u;
                }
        }
        for (int y = threadIdx.x; y < TH; y += NW * 32) {
            uint8_t v = O(y, 0);
            if (fresh || v != sm.eW[y])
                for (int d = -c8; d <= c8; ++d) {
                    const int h = y + d;
                    if (h < 0 || h >= TH) continue;
                    const uint8_t hv = O(h, -1);
                    if (v > hv && sm.mW[h] > hv) my_edges |= 4u;
                }
            v = O(y, TW - 1);
            if (fresh || v != sm.eE[y])
                for (int d = -c8; d <= c8; ++d) {
                    const int h = y + d;
                    if (h < 0 || h >= TH) continue;
                    const uint8_t hv = O(h, TW);
                    if (v > hv && sm.mE[h] > hv) my_edges |= 8u;
                }
        }
        if (c8 && threadIdx.x == 0) {
            uint8_t v, hv;
            v = O(0, 0), hv = O(-1, -1);
            if ((fresh || v != sm.eN[0]) && v > hv && sm.mN[0] > hv) my_edges |= 32u;
            v = O(0, TW - 1), hv = O(-1, TW);
            if ((fresh || v != sm.eN[TW - 1]) && v > hv && sm.mN[TW + 1] > hv) my_edges |= 64u;
            v = O(TH - 1, 0), hv = O(TH, -1);
            if ((fresh || v != sm.eS[0]) && v > hv && sm.mS[0] > hv) my_edges |= 128u;
            v = O(TH - 1, TW - 1), hv = O(TH, TW);
            if ((fresh || v != sm.eS[TW - 1]) && v > hv && sm.mS[TW + 1] > hv) my_edges |= 256u;
        }
    }
    if (my_edges) atomicOr(&sm.edges, (int)my_edges);
    if (anych)
        for (int i = threadIdx.x; i < TH * TW; i += NW * 32) {
            const int r = i / TW, cc = i - r * TW;
            const int y = y0 + r, x = x0 + cc;
            if (y < rows && x < cols) out[(int64_t)y * cols + x] = O(r, cc);
        }
    __threadfence();
    __syncthreads();
}

// lane 0 only: mark the neighbour's dirty edge, then queue it
__device__ __forceinline__ void notify(Queue &q, int t, int bits) {
    atomicOr(q.dirty + t, bits);
    q_push(q, t);
}

template <typename T, int TW, int TH, int P, int NW, bool PACKED, bool WL = false>
using TileOf = typename std::conditional<
    PACKED, TileU8<TW, TH>,
    typename std::conditional<WL, TileWL<T, TW, TH, P>, TileSmem<T, TW, TH, P>>::type>::type;

// MINB: CTAs per SM the register budget is sized for (8 warps: 4, i.e. at
// most 64 registers a thread, so the reconstructions of several tiles in
// flight can share an SM; 2 is kept as a tuning knob)
// dynamic shared memory of a tile CTA: the tile struct, then (TMA form) the
// two staging boxes, each on a 128-byte boundary (the base address is
// rounded up at run time, hence the 128 bytes of slack), the mbarrier and
// its phase
template <typename Sm>
constexpr size_t tile_smem_bytes(bool tma) {
    return tma ? sizeof(Sm) + 128 + 2 * (size_t)kStagePitch + 16 : sizeof(Sm);
}
template <typename Sm>
__device__ __forceinline__ uint8_t *tma_stage(unsigned char *sm_raw) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(sm_raw + sizeof(Sm));
    return reinterpret_cast<uint8_t *>((a + 127) & ~(uintptr_t)127);
}

template <typename T, int TW, int TH, int P, int NW, bool PACKED, int MINB, bool HYB, bool WL>
__global__ void __launch_bounds__(NW * 32, MINB) recon_cta(const T *__restrict__ mask, T *out, int rows, int cols,
                                                           int conn, int tiles_x, int tiles_y, Queue q,
                                                           const __grid_constant__ CUtensorMap out_map,
                                                           const __grid_constant__ CUtensorMap mask_map, int use_tma) {
    extern __shared__ __align__(128) unsigned char sm_raw[];
    using Sm = TileOf<T, TW, TH, P, NW, PACKED, WL>;
    Sm &sm = *reinterpret_cast<Sm *>(sm_raw);
    const bool conn8 = conn == 8;
    TmaArgs ta{&out_map, &mask_map, nullptr, nullptr, nullptr, 0};
    if (use_tma) {
        ta.stage = tma_stage<Sm>(sm_raw);
        ta.bar = reinterpret_cast<uint64_t *>(ta.stage + 2 * kStagePitch);
        ta.phase = reinterpret_cast<unsigned *>(ta.bar + 1);
        // self-check of the copy rules (destinations on 128-byte boundaries,
        // barrier on 8): the plain loads run when they do not hold
        ta.on = (reinterpret_cast<uintptr_t>(ta.stage) & 127) == 0 &&
                ((reinterpret_cast<uintptr_t>(ta.stage) + kStagePitch) & 127) == 0 &&
                (reinterpret_cast<uintptr_t>(ta.bar) & 7) == 0;
        if (threadIdx.x == 0) {
            mbar_init(ta.bar);
            *ta.phase = 0;
        }
        __syncthreads();
    }
    if constexpr (WL) {
        // the worklist starts empty (slot i free for ticket i) with nothing
        // queued; every tile pass leaves it empty
        for (int i = threadIdx.x; i < Sm::kCap; i += NW * 32) sm.ring[i] = ((unsigned)i & Sm::kSeqMask) << Sm::VB;
        for (int i = threadIdx.x; i < TW * TH / 32; i += NW * 32) sm.inq[i] = sm.cbm[i] = 0;
        if (threadIdx.x == 0) sm.head = sm.tail = 0;
        __syncthreads();
    }
    for (;;) {
        if (threadIdx.x == 0) sm.tile = q_pop(q);
        __syncthreads();
        const int t = sm.tile;
        __syncthreads();
        if (t < 0) break;
        __threadfence();
        for (;;) {
            if (threadIdx.x == 0) sm.dirty = atomicExch(q.dirty + t, 0);
            __syncthreads();
            const int dirty = sm.dirty;
            const int tx = t % tiles_x, ty = t / tiles_x;
            if constexpr (PACKED)
                cta_process_tile_u8<TW, TH, NW>(mask, out, rows, cols, conn8, tx, ty, dirty, sm);
            else
                cta_process_tile<T, TW, TH, P, NW, HYB, WL>(mask, out, rows, cols, conn8, tx, ty, dirty, sm, q.seq_min,
                                                            q.wl_phases, q.budget, q.status, ta);
            if constexpr (WL) {
                // a worklist wait ran out of budget (DEV_TIMEOUT is set): leave;
                // the other CTAs see the status word and leave too
                if (vld(&sm.abort)) return;
            }
            if (threadIdx.x == 0) {
                const unsigned edges = (unsigned)sm.edges;
                // our top edge is the upper tile's bottom halo, and so on
                if (edges & 16u) notify(q, t, D_ALL);
                if (edges & 1u && ty > 0) notify(q, t - tiles_x, D_S);
                if (edges & 2u && ty + 1 < tiles_y) notify(q, t + tiles_x, D_N);
                if (edges & 4u && tx > 0) notify(q, t - 1, D_E);
                if (edges & 8u && tx + 1 < tiles_x) notify(q, t + 1, D_W);
                if (edges & 32u && ty > 0 && tx > 0) notify(q, t - tiles_x - 1, D_S);
                if (edges & 64u && ty > 0 && tx + 1 < tiles_x) notify(q, t - tiles_x + 1, D_S);
                if (edges & 128u && ty + 1 < tiles_y && tx > 0) notify(q, t + tiles_x - 1, D_N);
                if (edges & 256u && ty + 1 < tiles_y && tx + 1 < tiles_x) notify(q, t + tiles_x + 1, D_N);
                atomicAdd(q.stats, 1);
                atomicAdd(q.stats + 1, sm.sweeps);
                atomicAdd(q.stats + 3, sm.lines);
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

// TMA-fed tile loads on (default) or off (tuning knob NSG_RECON_TMA=0)
bool recon_tma() {
    if (const char *e = getenv("NSG_RECON_TMA")) return atoi(e) != 0;
    return true;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// link-time dependency on the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// 2-D uint8 maps of `out` and `mask` (cols x rows, pitch cols) with the
// 160 x 130 staging box; false when the layout does not allow it
bool encode_u8_maps(void *out, const void *mask, int rows, int cols, CUtensorMap *om, CUtensorMap *mm) {
    EncodeTiledFn fn = encode_fn();
    if (!fn || cols % 16 != 0 || (reinterpret_cast<uintptr_t>(out) & 15) || (reinterpret_cast<uintptr_t>(mask) & 15))
        return false;
    const cuuint64_t dim[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t stride[1] = {(cuuint64_t)cols};
    const cuuint32_t box[2] = {(cuuint32_t)kStW, (cuuint32_t)kStH};
    const cuuint32_t estride[2] = {1, 1};
    for (int k = 0; k < 2; ++k) {
        CUtensorMap *m = k ? mm : om;
        void *base = k ? const_cast<void *>(mask) : out;
        if (fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dim, stride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    }
    return true;
}

template <typename T, int TW, int TH, int P, int NW, bool PACKED = false, int MINB = (NW >= 16 && !PACKED) ? 1 : 2,
          bool HYB = false, bool WL = false>
int run_recon_cta(Ctx &c, const T *marker, const T *mask, T *out, int rows, int cols, int conn, cudaStream_t s,
                  bool preinit = false) {
    NSG_TRY(check_dims(c, rows, cols));
    NSG_TRY(check_conn(c, conn));
    const int64_t n = (int64_t)rows * cols;
    const int tiles_x = (cols + TW - 1) / TW, tiles_y = (rows + TH - 1) / TH;
    const int ntiles = tiles_x * tiles_y;
    const int qcap = 2 * ntiles;
    int *state = c.ws.i32[5];
    int *queue = state + ntiles;
    int *dirty = queue + qcap;
    if (2 * (int64_t)ntiles + qcap > c.max_pad) {
        c.last_error = "tile queue does not fit";
        return NSG_ERR_OOM;
    }
    // out = min(marker, mask), unless the caller wrote a marker that is
    // already <= mask everywhere into `out` (preinit): then min() is the
    // marker itself, bit for bit, and the pass is skipped
    if (!preinit) {
        int blocks = (int)((n + 255) / 256);
        if (blocks > c.sm_count * 16) blocks = c.sm_count * 16;
        if (sizeof(T) == 1)
            init_min_u8<<<blocks, 256, 0, s>>>((const uint8_t *)marker, (const uint8_t *)mask, (uint8_t *)out, n);
        else
            init_min_f32<<<blocks, 256, 0, s>>>((const float *)marker, (const float *)mask, (float *)out, n);
        NSG_COUNT_LAUNCH();
        NSG_LAUNCH_CHECK(c);
    }
    // Whole-image row + column sweep pairs before the tile queue.  Off by
    // default: a thread per line walks the line serially, and on the tiles of
    // this pipeline a pair costs more than the tile passes it saves.
    int nsweep = 0;
    if (const char *e = getenv("NSG_RECON_SWEEPS")) nsweep = atoi(e);  // tuning knob (0: tile queue only)
    if (nsweep <= 0) {
        init_queue<<<(qcap + 255) / 256, 256, 0, s>>>(state, queue, dirty, qcap, ntiles, c.ws.ctrl);
        NSG_COUNT_LAUNCH();
    } else {
        int *changed = c.ws.ctrl + C_RSTATS + 2;
        zero_ints<<<(ntiles + 255) / 256, 256, 0, s>>>(dirty, ntiles);
        NSG_COUNT_LAUNCH();
        NSG_CUDA_TRY(c, cudaMemsetAsync(changed, 0, sizeof(int), s));
        const int c8 = conn == 8;
        for (int k = 0; k < nsweep; ++k) {
            sweep_rows<T><<<(rows + 127) / 128, 128, 0, s>>>(mask, out, rows, cols, c8, changed);
            NSG_COUNT_LAUNCH();
            sweep_cols<T><<<(cols + 127) / 128, 128, 0, s>>>(mask, out, rows, cols, c8, changed,
                                                             k + 1 == nsweep ? dirty : nullptr, TW, TH, tiles_x);
            NSG_COUNT_LAUNCH();
        }
        queue_marked<<<1, 1024, 0, s>>>(state, queue, dirty, qcap, ntiles, c.ws.ctrl);
        NSG_COUNT_LAUNCH();
    }
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
    q.dirty = dirty;
    q.idle_limit = 2048;
    if (const char *e = getenv("NSG_RECON_IDLE")) q.idle_limit = atoi(e);  // tuning knob
    q.seq_min = kSeqMinLines;
    if (const char *e = getenv("NSG_RECON_SEQMIN")) q.seq_min = atoi(e);  // tuning knob
    q.wl_phases = c.recon_wl_phases >= 1 ? c.recon_wl_phases : 1;
    if (const char *e = getenv("NSG_RECON_WLPH")) {  // tuning knob: phase pairs before the worklist (1-8)
        const int v = atoi(e);
        if (v >= 1 && v <= 8) q.wl_phases = v;
    }
    q.stats = c.ws.ctrl + C_RSTATS;
    // TMA-fed tile loads (uint8, 128 x 128 lane-per-line form): tensor maps of
    // the output plane and the mask, when their layout meets the tensor-map
    // rules (16-byte aligned bases, row pitch a multiple of 16 bytes)
    CUtensorMap out_map, mask_map;
    memset(&out_map, 0, sizeof(out_map));
    memset(&mask_map, 0, sizeof(mask_map));
    int use_tma = 0;
    if (std::is_same<T, uint8_t>::value && TW == 128 && TH == 128 && !PACKED && recon_tma())
        use_tma = encode_u8_maps(out, mask, rows, cols, &out_map, &mask_map) ? 1 : 0;
    using SmT = TileOf<T, TW, TH, P, NW, PACKED, WL>;
    const size_t smem = tile_smem_bytes<SmT>(use_tma != 0);
    auto kfn = recon_cta<T, TW, TH, P, NW, PACKED, MINB, HYB, WL>;
    // The attribute is per kernel and process-wide, and the tiles of a batch
    // run on several host threads, some with TMA staging and some without:
    // every caller sets the same value (the larger, TMA size), so one
    // thread's setting can never undercut another thread's launch.
    NSG_CUDA_TRY(c, cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tile_smem_bytes<SmT>(true)));
    int per_sm = 0;
    NSG_CUDA_TRY(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, NW * 32, smem));
    // One CTA per SM by default (two for the 4-warp lane-per-line form): the
    // work is CTA-throughput bound and more CTAs per SM mostly take room that
    // concurrent streams' kernels can use (measured on one 4096^2 tile, 4
    // warps: 1 CTA per SM 12.2 ms, 2 9.6 ms, 4 12.5 ms).
    int want = HYB ? 2 : 1;
    if (const char *e = getenv("NSG_RECON_CTAS_PER_SM")) want = atoi(e);  // tuning knob
    if (want >= 1 && want < per_sm) per_sm = want;
    if (per_sm < 1) per_sm = 1;
    int grid = c.sm_count * per_sm;
    // a context that shares the GPU with other tiles in flight (a pool worker)
    // runs its reconstructions on part of the SMs: the queue's CTA-time is
    // about the same on fewer CTAs, and the other tiles get the rest
    if (c.recon_max_ctas > 0 && c.recon_max_ctas < grid) grid = c.recon_max_ctas;
    if (const char *e = getenv("NSG_RECON_MAX_CTAS")) {  // tuning knob: cap on the persistent grid
        const int v = atoi(e);
        if (v >= 1 && v < grid) grid = v;
    }
    if (grid > ntiles) grid = ntiles;
    kfn<<<grid, NW * 32, smem, s>>>(mask, out, rows, cols, conn, tiles_x, tiles_y, q, out_map, mask_map, use_tma);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// warps per tile CTA
int recon_warps() {
    if (const char *e = getenv("NSG_RECON_WARPS")) {  // tuning knob: 8, 16 or 32
        const int v = atoi(e);
        if (v == 8 || v == 16 || v == 32) return v;
    }
    return 8;  // more warps shorten one reconstruction but crowd out concurrent tiles
}

// Tuning knob NSG_RECON_WL=1: the in-tile pixel worklist after NSG_RECON_WLPH
// phase pairs.  Off by default: measured on GB300, one 4096^2 pipeline
// reconstruction 9.6 ms (phases until stable) vs 10.6 / 9.5 / 8.8 ms (worklist
// after 1 / 2 / 3 phase pairs), but the batched form 1018 vs 822 / 868 Mpixel/s
// (1 / 3 phase pairs): the worklist's serial chains hold a CTA (and its larger
// shared-memory footprint) longer than the phase loop does.
bool recon_worklist(const Ctx &c) {
    if (const char *e = getenv("NSG_RECON_WL")) return atoi(e) != 0;
    return c.recon_wl_phases >= 1;  // the context's tuning (nsg_tuning.recon_wl_phases)
}

// register budget of the 8-warp tile CTA: sized for 4 CTAs per SM (default) or 2
int recon_minb() {
    if (const char *e = getenv("NSG_RECON_MINB")) {  // tuning knob: 2 or 4
        if (atoi(e) == 2) return 2;
    }
    return 4;
}

}  // namespace

int recon_u8(Ctx &c, const uint8_t *marker, const uint8_t *mask, uint8_t *out, int rows, int cols, int conn,
             cudaStream_t s) {
    const int nw = recon_warps();
    bool packed = false;  // 4 x uint8 SIMD strips (tuning knob NSG_RECON_PACKED)
    if (const char *e = getenv("NSG_RECON_PACKED")) packed = atoi(e) != 0;
    if (packed) {
        if (nw == 16) return run_recon_cta<uint8_t, 128, 128, 132, 16, true>(c, marker, mask, out, rows, cols, conn, s);
        return run_recon_cta<uint8_t, 128, 128, 132, 8, true>(c, marker, mask, out, rows, cols, conn, s);
    }
    bool hyb = true;  // lane-per-line scans for dense line groups, 4 warps (tuning knob NSG_RECON_HYB=0: shuffle scans only)
    if (const char *e = getenv("NSG_RECON_HYB")) hyb = atoi(e) != 0;
    if (hyb && !getenv("NSG_RECON_WARPS")) {
        if (recon_worklist(c))
            return run_recon_cta<uint8_t, 128, 128, 132, 4, false, 4, true, true>(c, marker, mask, out, rows, cols,
                                                                                  conn, s);
        return run_recon_cta<uint8_t, 128, 128, 132, 4, false, 4, true>(c, marker, mask, out, rows, cols, conn, s);
    }
    if (nw == 8) {
        if (recon_minb() == 2) return run_recon_cta<uint8_t, 128, 128, 132, 8, false, 2>(c, marker, mask, out, rows, cols, conn, s);
        return run_recon_cta<uint8_t, 128, 128, 132, 8, false, 4>(c, marker, mask, out, rows, cols, conn, s);
    }
    if (nw == 32) return run_recon_cta<uint8_t, 128, 128, 132, 32>(c, marker, mask, out, rows, cols, conn, s);
    return run_recon_cta<uint8_t, 128, 128, 132, 16>(c, marker, mask, out, rows, cols, conn, s);
}

int recon_f32(Ctx &c, const float *marker, const float *mask, float *out, int rows, int cols, int conn,
              cudaStream_t s, bool preinit) {
    const int nw = recon_warps();
    if (nw == 8) {
        if (recon_worklist(c) && !getenv("NSG_RECON_WARPS"))
            return run_recon_cta<float, 64, 64, 67, 8, false, 4, false, true>(c, marker, mask, out, rows, cols, conn,
                                                                              s, preinit);
        if (recon_minb() == 2)
            return run_recon_cta<float, 64, 64, 67, 8, false, 2>(c, marker, mask, out, rows, cols, conn, s, preinit);
        return run_recon_cta<float, 64, 64, 67, 8, false, 4>(c, marker, mask, out, rows, cols, conn, s, preinit);
    }
    if (nw == 32) return run_recon_cta<float, 64, 64, 67, 32>(c, marker, mask, out, rows, cols, conn, s, preinit);
    return run_recon_cta<float, 64, 64, 67, 16>(c, marker, mask, out, rows, cols, conn, s, preinit);
}

}  // namespace nsg
