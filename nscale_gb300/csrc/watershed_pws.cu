// watershed_pws.cu — exact, domain-parallel reproduction of OpenCV's Meyer
// flooding order (cv::watershed as nscale::watershed2 calls it,
// MorphologicOperations.cpp:3742-3750).
//
// The sequential algorithm pops the lowest non-empty of 256 FIFO queues; ties
// are FIFO, so the result depends on the global pop order.  Two facts make an
// exact parallel version possible:
//
//  1. Unknown pixels that are not black ("fg") split into DOMAINS — 4-connected
//     components of unknown fg pixels.  Domains never touch each other, so the
//     global pop sequence restricted to one domain equals that domain flooded
//     on its own.  Only black unknown pixels ("U", the zeroed background of the
//     masked colour image, whose label is 0 when it holds pixel 0) couple
//     domains.
//  2. Before the first U pixel is popped (time T_e) every domain is
//     independent, and the global order of any two pops of different domains
//     can be recovered from their own histories: a pop is "top-level" when its
//     level is >= every earlier pop of its domain, otherwise it belongs to the
//     dip of the last top-level pop; top-level pops are globally ordered by
//     (level, push time) and push time is the pop time of the pusher, so
//     comparing two pops walks their pushers' top-level origins (cmp_top).
//
// Phases (all on the device, no host round trip):
//   P0  classify pixels, label domains (union-find), initial queue entries.
//   P1  one thread floods each domain to completion; every push of a U pixel is
//       kept as a "dummy" entry (it has no effect) so that its pop time is known.
//   P2  the true entry of each U pixel is its earliest push; T_e is the
//       earliest true U pop (a tournament with cmp_top); each domain's state at
//       T_e is a prefix of its pop list (binary search with cmp_top).  At T_e
//       the first U pixel e floods, at level 0, every black unknown pixel
//       connected to it (region R) in FIFO BFS order; fg pixels that R touches
//       are queued with R's label at their colour level, in that BFS order —
//       a layer-synchronous BFS in one thread-block cluster computes the exact
//       order.  U pixels queued before T_e ("shells") and black regions R does
//       not reach ("pockets") are attached to the domains they touch; domains
//       that share a shell or a pocket are merged into one flood group.
//   P3  one thread per group brings each member to its T_e state (a group of
//       one domain from P1's records, a larger group by replaying its members),
//       merges the members' pending queues by push time, appends R's pushes and
//       floods the group to completion.
// Whenever an exactness condition fails (the first U pop at level 0, a
// watershed-labelled first U pixel, an unowned active shell, an overflow) a
// device flag makes the serial flood (ws_flood_serial) produce the result.
#include <limits.h>
#include <stdlib.h>

#include <cooperative_groups.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int WSHED = -1;
constexpr int IN_QUEUE = -2;
constexpr int kB = 256;

// pixel flags
constexpr uint8_t F_UNK = 1, F_U = 2, F_INIT = 4, F_FG = 8, F_BORDER = 16;
// state bits at T_e
constexpr uint8_t S_POPPED = 1, S_QUEUED = 2, S_R = 4, S_CERTAIN = 8, S_ACTIVE = 16, S_POCKET = 32;
// rec_meta: level (8) | top << 8 | dir << 9
__device__ __forceinline__ int m_level(int m) { return m & 255; }
__device__ __forceinline__ int m_dir(int m) { return (m >> 9) & 3; }

// control block indices (ctrl + C_WS)
enum {
    W_FALLBACK = 0,
    W_ND,
    W_POOL,  // unused (kept so that the diagnostic indices stay put)
    W_E,
    W_EP,
    W_DOME,
    W_LE,
    W_X,
    W_NCAND,
    W_EVENT,
    W_PEND,
    W_LAYERS,
    W_BFSCTAS,
    W_DTOT,  // dummy slots reserved over all domains
    W_NORD,  // entries of the size-ordered dispatch list (PW::ord)
};

struct PW {
    int H, W, n, pc;  // padded sizes, dummy-pool capacity
    const int *mk;
    const uint32_t *col;
    int *outp;
    int *ctl;  // ctrl + C_WS
    int *status;
    // per pixel
    uint8_t *flags, *initlvl, *st, *fgimg;
    int *domroot, *dom, *lab, *utrue, *inj, *claim, *uown, *proot, *fr0, *fr1, *popl, *isroot, *rank;
    // per entry (n + pc)
    int *next, *rparent, *rlocal, *rorigin, *rmeta;
    // dummy pool
    int *dpix, *ddom, *dseq, *dnextu;
    // per domain
    int *dsize, *doff, *bbx0, *bbx1, *bby0, *bby1, *npop, *cut, *sup, *mcount, *moff, *mfill, *mlist, *icount,
        *ioff, *ifill, *ilist, *cand, *pend, *pend2;
    unsigned long long *dfirst;
    int *grp;  // P3: flood group owning each pixel, -1 none (aliases the BFS frontier, free by then)
    // per domain: dummy slots reserved (distinct U pixels beside it) and where they start;
    // alias the root flags / root ranks, which are free once the domains are numbered
    int *ducnt, *duoff;
    // size-ordered dispatch of the per-domain (P1) and per-group (P3) floods:
    // the ids by decreasing work class, each id's class, 32 class counts + 32 offsets
    int *ord, *okey, *obucket;
};

// A pop's reads, issued together: the four neighbours' flags, markers,
// labels and colours (and, in P3, states and groups) do not depend on one
// another, so one memory round trip serves the pop instead of a chain of
// dependent loads.  Labels are the only ones the flood writes; a pop writes
// its own pixel and the neighbours it queues, each once, after reading them.
struct Nb4 {
    uint8_t f[4];
    int mk[4], lab[4];
    uint32_t col[4];
};
__device__ __forceinline__ void load_nb(const PW &a, const int (&nb)[4], Nb4 &o) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        o.f[k] = __ldg((const unsigned char *)a.flags + nb[k]);
        o.mk[k] = __ldg(a.mk + nb[k]);
        o.lab[k] = a.lab[nb[k]];
        o.col[k] = __ldg(a.col + nb[k]);
    }
}

__device__ __forceinline__ int cdiff(uint32_t a, uint32_t b) {
    int db = abs((int)(a & 255) - (int)(b & 255));
    int dg = abs((int)((a >> 8) & 255) - (int)((b >> 8) & 255));
    int dr = abs((int)((a >> 16) & 255) - (int)((b >> 16) & 255));
    int d = db > dg ? db : dg;
    return d > dr ? d : dr;
}

__device__ __forceinline__ void set_fallback(const PW &a, int code) { atomicCAS(a.ctl + W_FALLBACK, 0, code); }

// ---------------------------------------------------------------- P0 --------
__global__ void k_classify(PW a) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        int y = p / a.W, x = p - y * a.W;
        uint8_t f = 0, il = 0;
        if (y == 0 || y == a.H - 1 || x == 0 || x == a.W - 1) {
            f = F_BORDER;
        } else {
            int m = a.mk[p];
            if (m <= 0) {
                f = F_UNK;
                uint32_t c = a.col[p];
                f |= c == 0 ? F_U : F_FG;
                int idx = 256;
                const int nb[4] = {p - 1, p + 1, p - a.W, p + a.W};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    int q = nb[k];
                    int qy = q / a.W, qx = q - qy * a.W;
                    bool border = qy == 0 || qy == a.H - 1 || qx == 0 || qx == a.W - 1;
                    if (!border && a.mk[q] > 0) {
                        int t = cdiff(c, a.col[q]);
                        idx = t < idx ? t : idx;
                    }
                }
                if (idx < 256) {
                    f |= F_INIT;
                    il = (uint8_t)idx;
                }
            }
        }
        a.flags[p] = f;
        a.initlvl[p] = il;
        a.fgimg[p] = (f & F_FG) ? 1 : 0;
        a.lab[p] = 0;
        a.utrue[p] = -1;
        a.st[p] = 0;
        a.inj[p] = INT_MAX;
        a.claim[p] = INT_MAX;
        a.uown[p] = -1;
        a.rlocal[p] = -1;
        a.rparent[p] = -2;
        // (isroot is written for every pixel by k_roots, after the labelling)
    }
}

// per-domain arrays, once the number of domains is known (only those entries
// are ever read: every consumer indexes them by a domain or group id)
__global__ void k_domain_init(PW a, const int *nd_total) {
    const int nd = *nd_total;
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        a.dsize[d] = 0;
        a.bbx0[d] = INT_MAX;
        a.bby0[d] = INT_MAX;
        a.bbx1[d] = -1;
        a.bby1[d] = -1;
        a.dfirst[d] = ~0ull;
        a.sup[d] = d;
        a.mcount[d] = 0;
        a.mfill[d] = 0;
        a.icount[d] = 0;
        a.ifill[d] = 0;
        a.npop[d] = 0;
        a.cut[d] = 0;
        a.ducnt[d] = 0;
    }
}

__global__ void k_roots(PW a) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x)
        a.isroot[p] = (a.domroot[p] == p) ? 1 : 0;
}

__global__ void k_domains(PW a, const int *nd_total) {
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl[W_ND] = *nd_total;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        int r = a.domroot[p];
        int d = r >= 0 ? a.rank[r] : -1;
        a.dom[p] = d;
        if (d >= 0) {
            int y = p / a.W, x = p - y * a.W;
            atomicAdd(a.dsize + d, 1);
            atomicMin(a.bbx0 + d, x);
            atomicMax(a.bbx1 + d, x);
            atomicMin(a.bby0 + d, y);
            atomicMax(a.bby1 + d, y);
        }
    }
}

// Dummy slots: P1 pushes a U pixel (unknown, black, not queued from the
// start) at most once per domain beside it, so each domain reserves one slot
// per such pixel; P1 then takes slots without a global counter.
__global__ void k_udom_count(PW a) {
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += gridDim.x * blockDim.x) {
        const uint8_t f = a.flags[u];
        if (!(f & F_UNK) || !(f & F_U) || (f & F_INIT)) continue;
        const int nb[4] = {u - 1, u + 1, u - a.W, u + a.W};
        int dk[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            dk[k] = a.dom[nb[k]];
            bool seen = dk[k] < 0;
#pragma unroll
            for (int j = 0; j < k; ++j) seen = seen || dk[j] == dk[k];
            if (!seen) atomicAdd(a.ducnt + dk[k], 1);
        }
    }
}

// the U pixel -> dummies lists (k_true_dummies walks them), from P1's slots
__global__ void k_dummy_lists(PW a) {
    for (int kk = blockIdx.x * blockDim.x + threadIdx.x; kk < a.pc; kk += gridDim.x * blockDim.x) {
        const int q = a.dpix[kk];
        if (q >= 0) a.dnextu[kk] = atomicExch(a.utrue + q, a.n + kk);
    }
}

// ---------------------------------------------------------------- queues ----
// 256 FIFO queues (one per level) as heads and tails of lists linked
// through `next`; the heads and tails live wherever the caller puts them
// (P1: shared memory, P3: local memory)
struct Q {
    int *h, *t;
};
__device__ __forceinline__ void q_init(Q &q) {
    for (int i = 0; i < 256; ++i) q.h[i] = q.t[i] = -1;
}
__device__ __forceinline__ void q_push(Q &q, int *next, int lvl, int e) {
    next[e] = -1;
    if (q.t[lvl] < 0) q.h[lvl] = e;
    else next[q.t[lvl]] = e;
    q.t[lvl] = e;
}

// P1: flood domain d to completion, U pixels are dummies.  A flood is a
// serial program whose every pop takes its own path (dummy or pixel, how
// many neighbours it pushes, which level comes next), so floods sharing a
// warp diverge on every pop and run one after another: each block runs ONE
// flood on one thread, and the SM's warp scheduler interleaves the floods
// instead (measured on 64 tiles, one at a time: P1 468 / 383 / 304 / 271 ms
// and P3 316 / 238 / 144 / 109 ms with 32 / 8 / 2 / 1 floods per block).
// The flood keeps its queue heads and tails in shared memory (kQPitch ints):
// every pop and push touches them, and thread-private local memory would
// share the L1 with the flood's global reads.
constexpr int kP1Threads = 1, kQPitch = 513;
constexpr size_t kP1Smem = sizeof(int) * kP1Threads * kQPitch;
__device__ void phase1_domain(const PW &a, int d, Q &q);
// Size-ordered dispatch: the floods start longest first, so that the longest
// chains are not left to the end of the launch: the ids are bucketed by work
// class (the leading-zero count of the work: a factor of two per class) and
// thread t of the launch takes the t-th id.  Which thread floods which domain
// does not change any result (every flood writes only its own domain's
// records).
// mode 0: domains, work = pixels + reserved dummy slots (P1);
// mode 1: P3 groups (mcount > 0), work = their members' pixels.
__device__ __forceinline__ int flood_work(const PW &a, int d, int mode) {
    if (mode == 0) return a.dsize[d] + a.ducnt[d];
    const int nm = a.mcount[d];
    if (nm <= 0) return -1;
    const int *mem = a.mlist + a.moff[d];
    int w = 0;
    for (int m = 0; m < nm; ++m) w += a.dsize[mem[m]];
    return w;
}
__global__ void k_order_count(PW a, int mode) {
    const int nd = a.ctl[W_ND];
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        const int w = flood_work(a, d, mode);
        const int k = w < 0 ? -1 : __clz(w > 1 ? w : 1);
        a.okey[d] = k;
        if (k >= 0) atomicAdd(a.obucket + k, 1);
    }
}
__global__ void k_order_scan(PW a) {  // one warp
    const int lane = threadIdx.x;
    const int v = a.obucket[lane];
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    a.obucket[32 + lane] = x - v;  // exclusive offset of class `lane`
    a.obucket[lane] = 0;           // reused as the fill counter
    if (lane == 31) a.ctl[W_NORD] = x;
}
__global__ void k_order_scatter(PW a) {
    const int nd = a.ctl[W_ND];
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        const int k = a.okey[d];
        if (k >= 0) a.ord[a.obucket[32 + k] + atomicAdd(a.obucket + k, 1)] = d;
    }
}

__global__ void __launch_bounds__(kP1Threads) k_phase1(PW a) {
    extern __shared__ int qsm[];
    const int nd = a.ctl[W_NORD];
    Q q;
    q.h = qsm + threadIdx.x * kQPitch;
    q.t = q.h + 256;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nd; t += gridDim.x * blockDim.x)
        phase1_domain(a, a.ord[t], q);
}

__device__ void phase1_domain(const PW &a, int d, Q &q) {
    q_init(q);
    const int W = a.W, n = a.n;
    for (int y = a.bby0[d]; y <= a.bby1[d]; ++y)
        for (int x = a.bbx0[d]; x <= a.bbx1[d]; ++x) {
            int p = y * W + x;
            if (a.dom[p] != d || !(a.flags[p] & F_INIT)) continue;
            int lv = a.initlvl[p];
            a.rparent[p] = -1;
            a.rmeta[p] = lv;
            q_push(q, a.next, lv, p);
            a.lab[p] = IN_QUEUE;
        }
    int active = 0, runmax = -1, lasttop = -1, local = 0, seq = 0;
    const int base = a.doff[d];
    int dslot = a.duoff[d];  // this domain's next dummy slot
    for (;;) {
        while (active < 256 && q.h[active] < 0) ++active;
        if (active == 256) break;
        // the pop's reads first (the queue link, the entry and, for a pixel, its
        // neighbourhood), so that they travel together
        int e = q.h[active];
        const int nx = a.next[e];
        int meta = a.rmeta[e];
        const int p = e;
        const int nb[4] = {p - 1, p + 1, p - W, p + W};
        Nb4 nv;
        uint32_t c = 0;
        if (e < n) {
            load_nb(a, nb, nv);
            c = __ldg(a.col + p);
        }
        q.h[active] = nx;
        if (nx < 0) q.t[active] = -1;
        int lv = m_level(meta);
        if (e >= n) {  // dummy U entry: position only
            int k = e - n;
            a.dseq[k] = seq++;
            a.rlocal[e] = local;
            int top = lv >= runmax;
            a.rmeta[e] = meta | (top << 8);
            a.rorigin[e] = top ? e : lasttop;
            continue;
        }
        seq++;
        int top = lv >= runmax;
        if (top) {
            runmax = lv;
            lasttop = p;
        }
        a.rmeta[p] = meta | (top << 8);
        a.rorigin[p] = lasttop;
        a.rlocal[p] = local;
        a.popl[base + local] = p;
        local++;
        int lb = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint8_t fq = nv.f[k];
            int t = 0;
            if (fq & F_BORDER) continue;
            if (!(fq & F_UNK)) t = nv.mk[k];
            else if (fq & F_FG) t = nv.lab[k];
            if (t > 0) {
                if (lb == 0) lb = t;
                else if (t != lb) lb = WSHED;
            }
        }
        a.lab[p] = lb;
        if (lb <= 0) {
            if (lb == 0) set_fallback(a, 9);
            continue;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int qq = nb[k];
            const uint8_t fq = nv.f[k];
            if (!(fq & F_UNK)) continue;
            if (fq & F_U) {
                if (fq & F_INIT) continue;  // queued from the start
                // already pushed by this domain from another side: a pixel of d
                // beside qq has popped with a label (the first such pixel pushed it)
                const int nq[4] = {qq - 1, qq + 1, qq - W, qq + W};
                int d2[4], l2q[4];
#pragma unroll
                for (int s2 = 0; s2 < 4; ++s2) {
                    d2[s2] = __ldg(a.dom + nq[s2]);
                    l2q[s2] = a.lab[nq[s2]];
                }
                bool mine = false;
#pragma unroll
                for (int s2 = 0; s2 < 4; ++s2)
                    if (nq[s2] != p && d2[s2] == d && l2q[s2] > 0) mine = true;
                if (mine) continue;
                const int kk = dslot++;
                if (kk >= a.pc) {
                    set_fallback(a, 4);
                    continue;
                }
                const int id = n + kk;
                const int l2 = cdiff(c, nv.col[k]);
                a.dpix[kk] = qq;
                a.ddom[kk] = d;
                a.rparent[id] = p;
                a.rmeta[id] = l2 | (k << 9);
                a.rlocal[id] = -1;
                q_push(q, a.next, l2, id);
                if (l2 < active) active = l2;
                continue;
            }
            if (nv.lab[k] != 0) continue;
            int l2 = cdiff(c, nv.col[k]);
            a.rparent[qq] = p;
            a.rmeta[qq] = l2 | (k << 9);
            q_push(q, a.next, l2, qq);
            if (l2 < active) active = l2;
            a.lab[qq] = IN_QUEUE;
        }
    }
    a.npop[d] = local;
}

// ---------------------------------------------------------------- ordering --
// x, y: top-level entries of different domains.  true if x pops first.
__device__ bool cmp_top(const PW &a, int x, int y) {
    for (int guard = 0; guard < (1 << 26); ++guard) {
        int mx = a.rmeta[x], my = a.rmeta[y];
        int lx = m_level(mx), ly = m_level(my);
        if (lx != ly) return lx < ly;
        int px = a.rparent[x], py = a.rparent[y];
        if (px < 0 && py < 0) return x < y;  // initial entries: raster order
        if (px < 0) return true;
        if (py < 0) return false;
        x = a.rorigin[px];
        y = a.rorigin[py];
    }
    set_fallback(a, 10);
    return false;
}
// push time of entry x before that of entry y (x, y of different domains or
// of the same domain); parents are real pops
__device__ bool push_before(const PW &a, int x, int dx, int y, int dy) {
    int px = a.rparent[x], py = a.rparent[y];
    if (px < 0 && py < 0) return x < y;  // both initial (raster); only real pixels are initial here
    if (px < 0) return true;
    if (py < 0) return false;
    if (dx == dy) {
        if (px == py) return m_dir(a.rmeta[x]) < m_dir(a.rmeta[y]);
        return a.rlocal[px] < a.rlocal[py];
    }
    return cmp_top(a, a.rorigin[px], a.rorigin[py]);
}

// true entry of each U pixel: the earliest of its dummies
__global__ void k_true_dummies(PW a) {
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += gridDim.x * blockDim.x) {
        if (!(a.flags[u] & F_U)) continue;
        if (a.flags[u] & F_INIT) {
            // initial U entry: a top-level entry of its own
            a.rparent[u] = -1;
            a.rmeta[u] = a.initlvl[u] | (1 << 8);
            a.rorigin[u] = u;
            a.rlocal[u] = 0;
            continue;
        }
        int best = a.utrue[u];
        if (best < 0) continue;
        for (int e = a.dnextu[best - a.n]; e >= 0; e = a.dnextu[e - a.n]) {
            if (push_before(a, e, a.ddom[e - a.n], best, a.ddom[best - a.n])) best = e;
        }
        a.utrue[u] = best;
        int k = best - a.n;
        atomicMin(a.dfirst + a.ddom[k], ((unsigned long long)(unsigned)a.dseq[k] << 32) | (unsigned)best);
    }
}

__global__ void k_candidates(PW a) {
    const int nd = a.ctl[W_ND];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        if (i < nd && a.dfirst[i] != ~0ull) {
            int e = (int)(a.dfirst[i] & 0xffffffffu);
            a.cand[atomicAdd(a.ctl + W_NCAND, 1)] = e;
        }
        if ((a.flags[i] & F_U) && (a.flags[i] & F_INIT)) a.cand[atomicAdd(a.ctl + W_NCAND, 1)] = i;
    }
}

// single CTA: the earliest candidate pop
__global__ void __launch_bounds__(1024) k_first_event(PW a) {
    __shared__ int sh[1024];
    const int nc = a.ctl[W_NCAND];
    int best = -1;
    for (int i = threadIdx.x; i < nc; i += blockDim.x) {
        int e = a.cand[i];
        if (best < 0 || cmp_top(a, a.rorigin[e], a.rorigin[best])) best = e;
    }
    sh[threadIdx.x] = best;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            int x = sh[threadIdx.x], y = sh[threadIdx.x + s];
            if (x < 0 || (y >= 0 && cmp_top(a, a.rorigin[y], a.rorigin[x]))) sh[threadIdx.x] = y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        int e = sh[0];
        a.ctl[W_E] = e;
        a.ctl[W_EVENT] = e >= 0;
        if (e >= 0) {
            int ep = e >= a.n ? a.dpix[e - a.n] : e;
            a.ctl[W_EP] = ep;
            a.ctl[W_DOME] = e >= a.n ? a.ddom[e - a.n] : -1;
            a.ctl[W_LE] = m_level(a.rmeta[e]);
            if (m_level(a.rmeta[e]) < 1) set_fallback(a, 1);
        }
    }
}

__global__ void k_cuts(PW a) {
    const int nd = a.ctl[W_ND];
    if (!a.ctl[W_EVENT] || a.ctl[W_FALLBACK]) return;
    const int e = a.ctl[W_E];
    const int oe = a.rorigin[e];
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        if (d == a.ctl[W_DOME]) {
            a.cut[d] = a.rlocal[e];
            continue;
        }
        int lo = 0, hi = a.npop[d];  // first index whose pop is not before e
        const int base = a.doff[d];
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            int p = a.popl[base + mid];
            if (cmp_top(a, a.rorigin[p], oe)) lo = mid + 1;
            else hi = mid;
        }
        a.cut[d] = lo;
    }
}

// state of every pixel at T_e
__global__ void k_state(PW a) {
    if (!a.ctl[W_EVENT] || a.ctl[W_FALLBACK]) return;
    const int ep = a.ctl[W_EP];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        uint8_t f = a.flags[p];
        uint8_t s = 0;
        if (f & F_FG) {
            int d = a.dom[p];
            int lc = a.rlocal[p];
            bool popped = lc >= 0 && lc < a.cut[d];
            if (popped) s |= S_POPPED;
            else {
                int par = a.rparent[p];
                bool pushed = par == -1 || (par >= 0 && a.rlocal[par] >= 0 && a.rlocal[par] < a.cut[d]);
                if (pushed) s |= S_QUEUED;
            }
        } else if (f & F_U) {
            if (p == ep) {
                s |= S_R;
            } else if (f & F_INIT) {
                s |= S_QUEUED;
            } else {
                int e = a.utrue[p];
                if (e >= 0) {
                    int par = a.rparent[e];
                    int dd = a.ddom[e - a.n];
                    if (a.rlocal[par] < a.cut[dd]) s |= S_QUEUED;
                }
            }
        }
        a.st[p] = s;
    }
}

__global__ void k_event_label(PW a) {
    if (threadIdx.x || blockIdx.x) return;
    if (!a.ctl[W_EVENT] || a.ctl[W_FALLBACK]) return;
    const int ep = a.ctl[W_EP];
    const int W = a.W;
    const int nb[4] = {ep - 1, ep + 1, ep - W, ep + W};
    int lb = 0;
    for (int k = 0; k < 4; ++k) {
        int q = nb[k];
        uint8_t f = a.flags[q];
        int t = 0;
        if (f & F_BORDER) continue;
        if (!(f & F_UNK)) t = a.mk[q];
        else if ((f & F_FG) && (a.st[q] & S_POPPED)) t = a.lab[q];
        if (t > 0) {
            if (lb == 0) lb = t;
            else if (t != lb) lb = WSHED;
        }
    }
    a.ctl[W_X] = lb;
    if (lb <= 0) set_fallback(a, 2);
}

// ------------------------------------------------------ rank-ordered BFS ----
__device__ int cta_exclusive_scan(int v, int *sh, int &total) {
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
    total = sh[32];
    __syncthreads();
    return r;
}

// Neighbour classes of every pixel R can contain (a black unknown pixel not
// queued at T_e, e included): bit k (k = left, right, up, down) when the
// neighbour in direction k is a black unknown pixel R may still enter, bit
// 4 + k when it is an fg pixel R would push (neither popped nor queued at
// T_e).  Both are fixed during the BFS, so a frontier pixel costs one byte.
__global__ void k_bfs_prep(PW a, uint8_t *nbm) {
    const bool on = a.ctl[W_EVENT] && !a.ctl[W_FALLBACK];
    const int off[4] = {-1, 1, -a.W, a.W};
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        const uint8_t f = a.flags[p];
        uint8_t m = 0;
        if (on && (f & F_U) && !(f & F_BORDER) && !(a.st[p] & S_QUEUED)) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int q = p + off[k];
                const uint8_t fq = a.flags[q], sq = a.st[q];
                if (!(fq & F_UNK)) continue;
                if (fq & F_U) {
                    if (!(sq & (S_QUEUED | S_R))) m |= (uint8_t)(1u << k);
                } else if (!(sq & (S_POPPED | S_QUEUED))) {
                    m |= (uint8_t)(16u << k);
                }
            }
        }
        nbm[p] = m;
    }
}

// FIFO BFS from e over black unknown pixels that are not queued at T_e.  A
// pixel joins the next frontier through the earliest frontier pixel that
// touches it, in the order (frontier position, direction).  Claims use
// atomicMin with the key 4 * key(entry) + direction, where key(entry) grows
// with the entry's frontier position and from layer to layer, so a pixel
// claimed in an earlier layer keeps its key and is never taken again, and the
// smallest key of a layer is its FIFO owner.  Every fg neighbour that is
// neither popped nor queued at T_e records the smallest key that touches it:
// the order in which R pushes it (keys are only compared, never decoded).
//
// One thread-block cluster runs the BFS (up to 16 small CTAs, so that other
// streams' kernels keep the rest of each SM), one cluster barrier per layer.
// After the barrier every CTA knows every CTA's entry count of the current
// frontier (each CTA pushed its count into all CTAs' shared memory) and takes
// an equal contiguous chunk of it; the claims of the whole frontier are
// complete, so it reads the claims of its chunk's candidates, compacts its
// winners in order into its own segment of the next frontier, and at once
// issues the winners' claims.  A winner's key needs no other CTA's count: it
// is its slot, base + segment * capacity + position, which orders entries as
// their frontier positions do (segments follow chunk order) and exceeds every
// key of the layer before (base grows by the layer's whole slot range).
// Counts are double-buffered by layer parity, so a CTA that runs ahead into
// the next layer never overwrites counts another CTA has yet to read.
// While the segments stay balanced (the largest within a quarter of an equal
// share), each CTA takes its own segment as its next chunk straight from its
// shared memory, with no global round trip; otherwise the chunks are restaged
// from the global frontier.  Who processes an entry never changes its key.
constexpr int kBfsThreads = 256, kBfsCtaItems = 4096, kBfsMaxCluster = 16;
constexpr size_t kBfsSmem = 2 * kBfsCtaItems * (sizeof(int) + 1) + 4 * kBfsCtaItems;  // dynamic shared memory

__global__ void __launch_bounds__(kBfsThreads) k_bfs(PW a, const uint8_t *__restrict__ nbm) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks(), me = (int)cl.block_rank();
    __shared__ int sh[40];
    __shared__ int tots[2][kBfsMaxCluster];   // entries of every CTA's segment, by layer parity
    __shared__ int offs[kBfsMaxCluster + 1];  // where each CTA's segment starts in frontier order
    __shared__ int s_mx;                      // the largest segment
    extern __shared__ __align__(16) unsigned char bfs_dyn[];
    int *s_rb = reinterpret_cast<int *>(bfs_dyn);                   // [2][kBfsCtaItems]: chunk pixels, next segment
    uint8_t *s_mb = bfs_dyn + 2 * kBfsCtaItems * sizeof(int);         // [2][kBfsCtaItems]: their neighbour classes
    uint8_t *s_nm = s_mb + 2 * kBfsCtaItems;                          // [kBfsCtaItems * 4]: classes of the winners
    const bool on = a.ctl[W_EVENT] && !a.ctl[W_FALLBACK];
    const int W = a.W;
    const int off[4] = {-1, 1, -W, W};
    // frontier entries carry their pixel's neighbour classes (one load less per layer)
    unsigned long long *Fc = reinterpret_cast<unsigned long long *>(a.fr0);
    unsigned long long *Fn = reinterpret_cast<unsigned long long *>(a.fr1);
    if (threadIdx.x < kBfsMaxCluster) tots[0][threadIdx.x] = threadIdx.x == 0 ? 1 : 0;
    if (threadIdx.x == 0 && me == 0 && on) {  // the seed: key 0, its claims before the first barrier
        const int ep = a.ctl[W_EP];
        const unsigned m = nbm[ep];
        Fc[0] = (unsigned)ep | ((unsigned long long)m << 32);
        for (int k = 0; k < 4; ++k) {
            if (m & (1u << k)) atomicMin(a.claim + ep + off[k], k);
            if (m & (16u << k)) atomicMin(a.inj + ep + off[k], k);
        }
    }
    long long base = 0;  // key of slot 0 of the current frontier
    int prevcap = 1;     // slots per segment of the current frontier
    int layer = 0;
    int cb = 0;          // which half of s_rb / s_mb holds this CTA's own segment
    if (threadIdx.x == 0 && me == 0 && on) {
        s_rb[0] = a.ctl[W_EP];
        s_mb[0] = nbm[s_rb[0]];
    }
    if (!on) {
        cl.sync();
        return;
    }
    constexpr long long kKeyLimit = (INT_MAX - 4) / 4;
    for (;; ++layer) {
        cl.sync();  // the frontier, its counts and its claims are complete
        const int par = layer & 1;
        if (threadIdx.x < 32) {  // every CTA's count, then a warp scan
            const int lane = threadIdx.x;
            const int v = lane < C ? tots[par][lane] : 0;
            int x = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, d);
                if (lane >= d) x += y;
            }
            if (lane <= C) offs[lane] = x - v;  // exclusive prefix; offs[C] = total
            int mx = v;
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
            if (lane == 0) s_mx = mx;
        }
        __syncthreads();
        const int s = offs[C];
        if (s == 0) break;
        const int per_cta = (s + C - 1) / C;
        const bool local = s_mx <= per_cta + per_cta / 4 + 16 && s_mx <= kBfsCtaItems;
        const int segcap = 4 * (local ? s_mx : per_cta);
        const long long nbase = base + (long long)C * prevcap;  // keys of the next frontier start here
        if (per_cta > kBfsCtaItems || (int64_t)segcap * C > (int64_t)a.n ||
            nbase + (long long)C * segcap > kKeyLimit) {
            if (me == 0 && threadIdx.x == 0) set_fallback(a, 9);  // frontier too wide: serial flood
            break;
        }
        int *s_r = s_rb + cb * kBfsCtaItems;
        uint8_t *s_m = s_mb + cb * kBfsCtaItems;
        int lo, cnt;
        if (local) {  // this CTA's own segment, already in shared memory
            lo = offs[me];
            cnt = offs[me + 1] - lo;
        } else {  // an equal chunk, staged from the global frontier (read in order: coalesced)
            lo = min(s, me * per_cta);
            cnt = min(s, lo + per_cta) - lo;
            int seg = 0;
            for (int i = lo + threadIdx.x; i < lo + cnt; i += kBfsThreads) {
                while (i >= offs[seg + 1]) ++seg;
                const unsigned long long e = __ldcg(Fc + seg * prevcap + (i - offs[seg]));
                s_r[i - lo] = (int)(unsigned)e;
                s_m[i - lo] = (uint8_t)(e >> 32);
            }
            __syncthreads();
        }
        // the segment of the chunk's first entry: this CTA's own in a local
        // layer (no walk over the counts), else found by the walk below
        int seg = local ? me : 0;
        const int pt = (cnt + kBfsThreads - 1) / kBfsThreads;
        const int j0 = threadIdx.x * pt;
        unsigned long long win = 0;
        for (int j = 0; j < pt && j0 + j < cnt; ++j) {
            const int r = s_r[j0 + j];
            const unsigned m = s_m[j0 + j];
            const int i = lo + j0 + j;  // frontier position: slot seg * prevcap + (i - offs[seg])
            while (i >= offs[seg + 1]) ++seg;
            const int key0 = (int)(base + (long long)seg * prevcap + (i - offs[seg])) * 4;
            int cl4[4];
            uint8_t nm4[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {  // both loads of every candidate issued together
                cl4[k] = (m & (1u << k)) ? __ldcg(a.claim + r + off[k]) : -1;
                nm4[k] = (m & (1u << k)) ? nbm[r + off[k]] : 0;
            }
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if ((m & (1u << k)) && cl4[k] == key0 + k) {
                    win |= 1ull << (j * 4 + k);
                    s_nm[(j0 + j) * 4 + k] = nm4[k];
                }
        }
        int total;
        int pos = cta_exclusive_scan(__popcll(win), sh, total);
        while (win) {
            const int b = __ffsll((long long)win) - 1;
            win &= win - 1;
            const int q = s_r[j0 + (b >> 2)] + off[b & 3];
            const unsigned m = s_nm[j0 * 4 + b];
            Fn[me * segcap + pos] = (unsigned)q | ((unsigned long long)m << 32);
            if (pos < kBfsCtaItems) {  // this CTA's next segment, for a balanced next layer
                s_rb[(cb ^ 1) * kBfsCtaItems + pos] = q;
                s_mb[(cb ^ 1) * kBfsCtaItems + pos] = (uint8_t)m;
            }
            const int key0 = (int)(nbase + (long long)me * segcap + pos) * 4;  // the winner's slot
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (m & (1u << k)) atomicMin(a.claim + q + off[k], key0 + k);
                if (m & (16u << k)) atomicMin(a.inj + q + off[k], key0 + k);
            }
            ++pos;
        }
        if (threadIdx.x < C) *cl.map_shared_rank(&tots[par ^ 1][me], threadIdx.x) = total;  // push the count to all
        unsigned long long *t = Fc;
        Fc = Fn;
        Fn = t;
        prevcap = segcap;
        base = nbase;
        cb ^= 1;
    }
    cl.sync();  // no CTA leaves while another may still push into its shared counts
    if (me == 0 && threadIdx.x == 0) {
        a.ctl[W_LAYERS] = layer;
        a.ctl[W_BFSCTAS] = C;
    }
}

// R: every pixel the BFS claimed (the seed is marked by k_state)
__global__ void k_mark_r(PW a) {
    if (!a.ctl[W_EVENT] || a.ctl[W_FALLBACK]) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x)
        if (a.claim[p] != INT_MAX) a.st[p] |= S_R;
}

// shells: U pixels queued at T_e
__global__ void k_shells(PW a) {
    if (!a.ctl[W_EVENT] || a.ctl[W_FALLBACK]) return;
    const int X = a.ctl[W_X];
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += gridDim.x * blockDim.x) {
        if (!(a.flags[u] & F_U)) continue;
        uint8_t s = a.st[u];
        if (!(s & S_QUEUED)) continue;
        const int nb[4] = {u - 1, u + 1, u - a.W, u + a.W};
        bool adjR = false;
        int mk1 = 0;
        bool two = false;
        for (int k = 0; k < 4; ++k) {
            int q = nb[k];
            if (a.st[q] & S_R) adjR = true;
            uint8_t f = a.flags[q];
            if (!(f & (F_UNK | F_BORDER))) {
                int m = a.mk[q];
                if (mk1 == 0) mk1 = m;
                else if (m != mk1) two = true;
            }
        }
        int Y;
        int owner = -1;
        if (a.flags[u] & F_INIT) {
            Y = mk1;
        } else {
            int e = a.utrue[u];
            Y = a.lab[a.rparent[e]];
            owner = a.ddom[e - a.n];
        }
        if ((adjR && Y > 0 && Y != X) || two) {
            a.st[u] = s | S_CERTAIN;
            continue;
        }
        if (owner < 0) {
            set_fallback(a, 3);
            continue;
        }
        a.st[u] = s | S_ACTIVE;
        a.uown[u] = owner;
    }
}

__global__ void k_pocket_img(PW a, uint8_t *img) {
    const bool on = a.ctl[W_EVENT] && !a.ctl[W_FALLBACK];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        bool pk = on && (a.flags[p] & F_U) && !(a.st[p] & (S_QUEUED | S_R));
        img[p] = pk ? 1 : 0;
        if (pk) a.st[p] |= S_POCKET;
    }
}

__device__ __forceinline__ int sfind(int *par, int x) {
    for (;;) {
        int p = __ldcg(par + x);
        if (p == x) return x;
        x = p;
    }
}
// Domain-group union.  Its retries are bounded; a union abandoned when the
// bound runs out would leave a wrong flood group, so it sends the flood to
// the serial path instead (fallback code 14), which needs no groups.
__device__ void sunite(const PW &a, int *par, int a_, int b_) {
    for (int guard = 0; guard < (1 << 24); ++guard) {
        a_ = sfind(par, a_);
        b_ = sfind(par, b_);
        if (a_ == b_) return;
        if (a_ < b_) {
            int t = a_;
            a_ = b_;
            b_ = t;
        }
        int old = atomicMin(par + a_, b_);
        if (old == a_) return;
        a_ = old;
    }
    set_fallback(a, 14);
}

// pocket owners: first domain (or active-shell owner) touching the pocket;
// every other one is merged with it
__global__ void k_pocket_owner(PW a, int *powner) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        if (!(a.st[p] & S_POCKET)) continue;
        int r = a.proot[p];
        const int nb[4] = {p - 1, p + 1, p - a.W, p + a.W};
        for (int k = 0; k < 4; ++k) {
            int q = nb[k];
            int d = -1;
            if (a.flags[q] & F_FG) d = a.dom[q];
            else if (a.st[q] & S_ACTIVE) d = a.uown[q];
            else if (a.st[q] & S_R) set_fallback(a, 7);
            if (d < 0) continue;
            int old = atomicCAS(powner + r, -1, d);
            if (old != -1 && old != d) sunite(a, a.sup, old, d);
        }
    }
}
__global__ void k_shell_unions(PW a, const int *powner) {
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < a.n; u += gridDim.x * blockDim.x) {
        if (a.st[u] & S_POCKET) {
            int o = powner[a.proot[u]];
            a.uown[u] = o;  // -1: never entered
            continue;
        }
        if (!(a.st[u] & S_ACTIVE)) continue;
        int o = a.uown[u];
        const int nb[4] = {u - 1, u + 1, u - a.W, u + a.W};
        for (int k = 0; k < 4; ++k) {
            int q = nb[k];
            if (a.flags[q] & F_FG) sunite(a, a.sup, o, a.dom[q]);
            else if (a.st[q] & S_ACTIVE) sunite(a, a.sup, o, a.uown[q]);
            else if ((a.st[q] & S_POCKET) && powner[a.proot[q]] >= 0) sunite(a, a.sup, o, powner[a.proot[q]]);
        }
    }
}

__global__ void k_sup_flatten(PW a) {
    const int nd = a.ctl[W_ND];
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x)
        a.sup[d] = sfind(a.sup, d);
}
__global__ void k_groups(PW a) {
    const int nd = a.ctl[W_ND];
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        int r = sfind(a.sup, d);
        atomicAdd(a.mcount + r, 1);
    }
}
__global__ void k_groups2(PW a) {
    const int nd = a.ctl[W_ND];
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        int r = sfind(a.sup, d);
        a.mlist[a.moff[r] + atomicAdd(a.mfill + r, 1)] = d;
    }
}
__global__ void k_inj_count(PW a, int pass) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        if (a.inj[p] == INT_MAX) continue;
        int r = a.sup[a.dom[p]];
        if (pass == 0) atomicAdd(a.icount + r, 1);
        else a.ilist[a.ioff[r] + atomicAdd(a.ifill + r, 1)] = p;
    }
}
// A group of one domain starts P3 from the domain's state at T_e, read from
// P1's records instead of replaying its flood: popped pixels keep their P1
// labels, pixels queued at T_e are IN_QUEUE, the rest 0; an active shell the
// domain owns becomes a real entry with its true dummy's pusher and level.
// (A shell whose dummy popped before the domain's cut is a U pop before T_e:
// the exactness condition the replay checks, so the serial flood takes over.)
__global__ void k_p3_state(PW a) {
    if (!a.ctl[W_EVENT] || a.ctl[W_FALLBACK]) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        const uint8_t f = a.flags[p];
        if (f & F_FG) {
            if (a.mcount[a.sup[a.dom[p]]] != 1) continue;  // several members: P3 replays them
            const uint8_t s = a.st[p];
            if (s & S_POPPED) continue;
            a.lab[p] = (s & S_QUEUED) ? IN_QUEUE : 0;
        } else if (f & F_U) {
            if (!(a.st[p] & S_ACTIVE)) continue;
            const int te = a.utrue[p];
            if (te < a.n) continue;
            const int d = a.ddom[te - a.n];
            if (a.mcount[a.sup[d]] != 1) continue;
            if (a.rlocal[te] < a.cut[d]) {
                set_fallback(a, 11);
                continue;
            }
            a.lab[p] = IN_QUEUE;
            a.rparent[p] = a.rparent[te];
            a.rmeta[p] = a.rmeta[te] & ~(1 << 8);
        }
    }
}

// the flood group owning each pixel (the owned() test of P3, precomputed)
__global__ void k_pixel_groups(PW a) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        const uint8_t f = a.flags[p];
        int g = -1;
        if (f & F_FG) {
            g = a.sup[a.dom[p]];
        } else if (f & F_U) {
            const int o = a.uown[p];
            if (o >= 0 && (a.st[p] & (S_ACTIVE | S_POCKET))) g = a.sup[o];
        }
        a.grp[p] = g;
    }
}
__global__ void k_reset_owned_u(PW a) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x)
        if ((a.st[p] & (S_ACTIVE | S_POCKET)) && a.uown[p] >= 0) a.lab[p] = 0;
}

// ---------------------------------------------------------------- P3 --------

// replay domain d up to its T_e state (pre-T_e rules)
__device__ bool replay(const PW &a, int d, Q &q, int &active) {
    const int W = a.W;
    for (int y = a.bby0[d]; y <= a.bby1[d]; ++y)
        for (int x = a.bbx0[d]; x <= a.bbx1[d]; ++x) {
            int p = y * W + x;
            if (a.dom[p] == d) a.lab[p] = 0;
        }
    for (int y = a.bby0[d]; y <= a.bby1[d]; ++y)
        for (int x = a.bbx0[d]; x <= a.bbx1[d]; ++x) {
            int p = y * W + x;
            if (a.dom[p] != d || !(a.flags[p] & F_INIT)) continue;
            q_push(q, a.next, a.initlvl[p], p);
            a.lab[p] = IN_QUEUE;
        }
    active = 0;
    const int cutd = a.cut[d];
    for (int local = 0; local < cutd;) {
        while (active < 256 && q.h[active] < 0) ++active;
        if (active == 256) return false;
        int e = q.h[active];
        const int nx = a.next[e];
        const int p = e;
        const int nb[4] = {p - 1, p + 1, p - W, p + W};
        Nb4 nv;
        load_nb(a, nb, nv);
        const uint32_t c = __ldg(a.col + p);
        const uint8_t fp = __ldg((const unsigned char *)a.flags + p);
        q.h[active] = nx;
        if (nx < 0) q.t[active] = -1;
        if (!(fp & F_FG)) return false;  // no U pop before T_e
        ++local;
        int lb = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint8_t fq = nv.f[k];
            int t = 0;
            if (fq & F_BORDER) continue;
            if (!(fq & F_UNK)) t = nv.mk[k];
            else if (fq & F_FG) t = nv.lab[k];
            if (t > 0) {
                if (lb == 0) lb = t;
                else if (t != lb) lb = WSHED;
            }
        }
        a.lab[p] = lb;
        if (lb == 0) return false;
        if (lb == WSHED) continue;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int qq = nb[k];
            const uint8_t fq = nv.f[k];
            if (!(fq & F_UNK)) continue;
            if (fq & F_U) {
                if (!(a.st[qq] & S_ACTIVE)) continue;
                int te = a.utrue[qq];
                if (te < a.n || a.ddom[te - a.n] != d) continue;
                if (nv.lab[k] != 0) continue;
                int l2 = cdiff(c, nv.col[k]);
                a.rparent[qq] = p;
                a.rmeta[qq] = l2 | (k << 9);
                q_push(q, a.next, l2, qq);
                if (l2 < active) active = l2;
                a.lab[qq] = IN_QUEUE;
                continue;
            }
            if (nv.lab[k] != 0) continue;
            int l2 = cdiff(c, nv.col[k]);
            q_push(q, a.next, l2, qq);
            if (l2 < active) active = l2;
            a.lab[qq] = IN_QUEUE;
        }
    }
    return true;
}

// The queue of domain d at T_e, from P1's records: the entries queued at T_e
// in the order the flood pushed them — first the initial ones (raster order),
// then, pop by pop up to the cut, the neighbours each pop pushed (direction
// order).  The reads of one pop do not depend on the previous pop's, so the
// walk streams instead of replaying the flood's dependent chain.
__device__ void queue_at_te(const PW &a, int d, Q &q) {
    const int W = a.W, n = a.n;
    for (int y = a.bby0[d]; y <= a.bby1[d]; ++y)
        for (int x = a.bbx0[d]; x <= a.bbx1[d]; ++x) {
            const int p = y * W + x;
            if (__ldg(a.dom + p) != d) continue;
            if ((__ldg((const unsigned char *)a.flags + p) & F_INIT) &&
                (__ldg((const unsigned char *)a.st + p) & S_QUEUED))
                q_push(q, a.next, __ldg((const unsigned char *)a.initlvl + p), p);
        }
    const int base = a.doff[d], cutd = a.cut[d];
#pragma unroll 2
    for (int i = 0; i < cutd; ++i) {
        const int p = __ldg(a.popl + base + i);
        const int nb[4] = {p - 1, p + 1, p - W, p + W};
        uint8_t f[4], sq[4];
        int par[4], te[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            f[k] = __ldg((const unsigned char *)a.flags + nb[k]);
            sq[k] = __ldg((const unsigned char *)a.st + nb[k]);
            par[k] = __ldg(a.rparent + nb[k]);
            te[k] = __ldg(a.utrue + nb[k]);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int qq = nb[k];
            if (f[k] & F_FG) {
                if ((sq[k] & S_QUEUED) && par[k] == p) q_push(q, a.next, m_level(__ldg(a.rmeta + qq)), qq);
            } else if ((f[k] & F_U) && (sq[k] & S_ACTIVE) && te[k] >= n) {
                if (__ldg(a.ddom + te[k] - n) == d && __ldg(a.rparent + te[k]) == p)
                    q_push(q, a.next, m_level(__ldg(a.rmeta + te[k])), qq);
            }
        }
    }
}

// P3: one thread per flood group, the group's queue in shared memory as in
// P1 (the members' queues of a multi-member merge stay in local memory)
__device__ void phase3_group(const PW &a, int S, Q &q);
__global__ void __launch_bounds__(kP1Threads) k_phase3(PW a) {
    extern __shared__ int qsm[];
    const int ng = a.ctl[W_NORD];  // the groups, longest first (k_order_*, mode 1)
    if (a.ctl[W_FALLBACK] || !a.ctl[W_EVENT]) return;
    Q q;
    q.h = qsm + threadIdx.x * kQPitch;
    q.t = q.h + 256;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x)
        phase3_group(a, a.ord[t], q);
}
__device__ void phase3_group(const PW &a, int S, Q &q) {
    const int nm = a.mcount[S];
    const int *mem = a.mlist + a.moff[S];
    const int X = a.ctl[W_X];
    const int W = a.W;
    q_init(q);
    int active = 0;
    if (nm == 1) {
        queue_at_te(a, mem[0], q);  // labels and shells were set by k_p3_state
        active = 0;
    } else {
        // replay every member, collect pending entries, merge them by push time
        int total = 0;
        for (int m = 0; m < nm; ++m) total += a.dsize[mem[m]] + 4 * a.dsize[mem[m]];
        int pb = atomicAdd(a.ctl + W_PEND, total);
        if (pb + total > a.n) {
            set_fallback(a, 6);
            return;
        }
        int *pend = a.pend + pb, *tmp = a.pend2 + pb;
        int np = 0;
        for (int m = 0; m < nm; ++m) {
            int qmh[256], qmt[256];
            Q qm{qmh, qmt};
            q_init(qm);
            int act = 0;
            if (!replay(a, mem[m], qm, act)) {
                set_fallback(a, 11);
                return;
            }
            for (int lv = 0; lv < 256; ++lv)
                for (int e = qm.h[lv]; e >= 0; e = a.next[e]) pend[np++] = e;
        }
        // bottom-up merge sort by (level, push time)
        for (int w = 1; w < np; w <<= 1) {
            for (int lo = 0; lo < np; lo += 2 * w) {
                int mid = min(lo + w, np), hi = min(lo + 2 * w, np);
                int i = lo, j = mid, k = lo;
                while (i < mid && j < hi) {
                    int x = pend[i], y = pend[j];
                    int lx = m_level(a.rmeta[x]), ly = m_level(a.rmeta[y]);
                    int dx = (a.flags[x] & F_FG) ? a.dom[x] : a.ddom[a.utrue[x] - a.n];
                    int dy = (a.flags[y] & F_FG) ? a.dom[y] : a.ddom[a.utrue[y] - a.n];
                    bool yfirst = ly < lx || (ly == lx && push_before(a, y, dy, x, dx));
                    tmp[k++] = yfirst ? pend[j++] : pend[i++];
                }
                while (i < mid) tmp[k++] = pend[i++];
                while (j < hi) tmp[k++] = pend[j++];
                for (int t = lo; t < hi; ++t) pend[t] = tmp[t];
            }
        }
        for (int i = 0; i < np; ++i) {
            int e = pend[i];
            q_push(q, a.next, m_level(a.rmeta[e]), e);
        }
        active = 0;
    }
    // T_e: R's pushes into this group, in BFS order
    {
        const int ni = a.icount[S];
        int *il = a.ilist + a.ioff[S];
        for (int i = 1; i < ni; ++i) {  // insertion sort by BFS key
            int v = il[i], kv = a.inj[v], j = i - 1;
            while (j >= 0 && a.inj[il[j]] > kv) {
                il[j + 1] = il[j];
                --j;
            }
            il[j + 1] = v;
        }
        for (int i = 0; i < ni; ++i) {
            int p = il[i];
            if (a.lab[p] != 0) {
                set_fallback(a, 12);
                return;
            }
            int l2 = cdiff(a.col[p], 0u);
            q_push(q, a.next, l2, p);
            a.lab[p] = IN_QUEUE;
            if (l2 < active) active = l2;
        }
    }
    // flood after T_e
    for (long long guard = 0;; ++guard) {
        while (active < 256 && q.h[active] < 0) ++active;
        if (active == 256) break;
        int e = q.h[active];
        const int nx = a.next[e];
        const int p = e;
        const int nb[4] = {p - 1, p + 1, p - W, p + W};
        Nb4 nv;
        load_nb(a, nb, nv);
        uint8_t sq[4];
        int gq[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            sq[k] = __ldg((const unsigned char *)a.st + nb[k]);
            gq[k] = __ldg(a.grp + nb[k]);
        }
        const uint32_t c = __ldg(a.col + p);
        q.h[active] = nx;
        if (nx < 0) q.t[active] = -1;
        int lb = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint8_t fq = nv.f[k];
            int t = 0;
            if (fq & F_BORDER) continue;
            if (!(fq & F_UNK)) t = nv.mk[k];
            else if (sq[k] & S_R) t = X;
            else if (gq[k] == S) t = nv.lab[k];
            if (t > 0) {
                if (lb == 0) lb = t;
                else if (t != lb) lb = WSHED;
            }
        }
        a.lab[p] = lb;
        if (lb == 0) {
            set_fallback(a, 13);
            return;
        }
        if (lb == WSHED) continue;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            int qq = nb[k];
            const uint8_t fq = nv.f[k];
            if (!(fq & F_UNK)) continue;
            if (sq[k] & (S_R | S_CERTAIN)) continue;
            if (gq[k] != S) {
                set_fallback(a, 5);
                return;
            }
            if (nv.lab[k] != 0) continue;
            int l2 = cdiff(c, nv.col[k]);
            q_push(q, a.next, l2, qq);
            if (l2 < active) active = l2;
            a.lab[qq] = IN_QUEUE;
        }
    }
}

// final padded labels
__global__ void k_assemble(PW a) {
    const int event = a.ctl[W_EVENT];
    const int X = a.ctl[W_X];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += gridDim.x * blockDim.x) {
        uint8_t f = a.flags[p];
        int v;
        if (f & F_BORDER) v = WSHED;
        else if (!(f & F_UNK)) v = a.mk[p];
        else if (f & F_FG) v = a.lab[p];
        else if (!event) v = 0;
        else {
            uint8_t s = a.st[p];
            if (s & S_R) v = X;
            else if (s & S_CERTAIN) v = WSHED;
            else if ((s & (S_ACTIVE | S_POCKET)) && a.uown[p] >= 0) v = a.lab[p];
            else v = 0;
        }
        a.outp[p] = v == IN_QUEUE ? 0 : v;
    }
}

// ------------------------------------------------------------- fallback -----
__global__ void k_copy_if(const int *mk, int *outp, int n, const int *flag) {
    if (*flag == 0) return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) outp[p] = mk[p];
}

__global__ void k_serial(int *m, const uint32_t *col, int *next, int H, int W, long long budget, int *status,
                         const int *flag) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (flag && *flag == 0) return;
    int qh[256], qt[256];
    for (int i = 0; i < 256; ++i) qh[i] = qt[i] = -1;
    auto push = [&](int idx, int ofs) {
        next[ofs] = -1;
        if (qt[idx] < 0) qh[idx] = ofs;
        else next[qt[idx]] = ofs;
        qt[idx] = ofs;
    };
    for (int j = 0; j < W; ++j) m[j] = m[j + (int64_t)W * (H - 1)] = WSHED;
    for (int i = 1; i < H - 1; ++i) {
        int *row = m + (int64_t)i * W;
        row[0] = row[W - 1] = WSHED;
        for (int j = 1; j < W - 1; ++j) {
            int *p = row + j;
            if (p[0] < 0) p[0] = 0;
            if (p[0] == 0 && (p[-1] > 0 || p[1] > 0 || p[-W] > 0 || p[W] > 0)) {
                int ofs = i * W + j;
                uint32_t c = col[ofs];
                int idx = 256, t;
                if (p[-1] > 0) idx = cdiff(c, col[ofs - 1]);
                if (p[1] > 0) {
                    t = cdiff(c, col[ofs + 1]);
                    idx = idx < t ? idx : t;
                }
                if (p[-W] > 0) {
                    t = cdiff(c, col[ofs - W]);
                    idx = idx < t ? idx : t;
                }
                if (p[W] > 0) {
                    t = cdiff(c, col[ofs + W]);
                    idx = idx < t ? idx : t;
                }
                push(idx, ofs);
                p[0] = IN_QUEUE;
            }
        }
    }
    int active = 0;
    while (active < 256 && qh[active] < 0) ++active;
    if (active == 256) return;
    long long steps = 0;
    for (;;) {
        if (qh[active] < 0) {
            int i;
            for (i = active + 1; i < 256; ++i)
                if (qh[i] >= 0) break;
            if (i == 256) break;
            active = i;
        }
        if (++steps > budget) {
            atomicOr(status, DEV_TIMEOUT);
            return;
        }
        int ofs = qh[active];
        qh[active] = next[ofs];
        if (qh[active] < 0) qt[active] = -1;
        int *p = m + ofs;
        int lab = 0, t;
        t = p[-1];
        if (t > 0) lab = t;
        t = p[1];
        if (t > 0) {
            if (lab == 0) lab = t;
            else if (t != lab) lab = WSHED;
        }
        t = p[-W];
        if (t > 0) {
            if (lab == 0) lab = t;
            else if (t != lab) lab = WSHED;
        }
        t = p[W];
        if (t > 0) {
            if (lab == 0) lab = t;
            else if (t != lab) lab = WSHED;
        }
        p[0] = lab;
        if (lab == WSHED) continue;
        uint32_t c = col[ofs];
        if (p[-1] == 0) {
            t = cdiff(c, col[ofs - 1]);
            push(t, ofs - 1);
            active = active < t ? active : t;
            p[-1] = IN_QUEUE;
        }
        if (p[1] == 0) {
            t = cdiff(c, col[ofs + 1]);
            push(t, ofs + 1);
            active = active < t ? active : t;
            p[1] = IN_QUEUE;
        }
        if (p[-W] == 0) {
            t = cdiff(c, col[ofs - W]);
            push(t, ofs - W);
            active = active < t ? active : t;
            p[-W] = IN_QUEUE;
        }
        if (p[W] == 0) {
            t = cdiff(c, col[ofs + W]);
            push(t, ofs + W);
            active = active < t ? active : t;
            p[W] = IN_QUEUE;
        }
    }
}

int blocks(Ctx &c, int64_t n) {
    int64_t g = (n + kB - 1) / kB;
    int64_t cap = (int64_t)c.sm_count * 16;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

struct Carve {
    char *p;
    size_t used = 0;
    template <typename T>
    T *take(size_t count) {
        size_t b = (count * sizeof(T) + 255) & ~(size_t)255;
        T *r = reinterpret_cast<T *>(p + used);
        used += b;
        return r;
    }
};

void carve(PW &a, char *base, size_t *used_out) {
    const size_t n = (size_t)a.n, np = (size_t)a.n + a.pc, pc = (size_t)a.pc;
    Carve cv{base};
    a.flags = cv.take<uint8_t>(n);
    a.initlvl = cv.take<uint8_t>(n);
    a.st = cv.take<uint8_t>(n);
    a.fgimg = cv.take<uint8_t>(n);
    a.domroot = cv.take<int>(n);
    a.dom = cv.take<int>(n);
    a.lab = cv.take<int>(n);
    a.utrue = cv.take<int>(n);
    a.inj = cv.take<int>(n);
    a.claim = cv.take<int>(n);
    a.uown = cv.take<int>(n);
    a.proot = cv.take<int>(n);
    a.fr0 = cv.take<int>(2 * n);  // BFS frontier entries: pixel | neighbour classes << 32
    a.fr1 = cv.take<int>(2 * n);
    a.grp = a.fr0;  // the BFS frontier is no longer needed when P3 runs
    a.popl = cv.take<int>(n);
    a.isroot = cv.take<int>(n);
    a.rank = cv.take<int>(n);
    a.ducnt = a.isroot;  // the root flags are scanned into ranks before the domains are initialised
    a.duoff = a.rank;    // the ranks are read by k_domains only
    a.next = cv.take<int>(np);
    a.rparent = cv.take<int>(np);
    a.rlocal = cv.take<int>(np);
    a.rorigin = cv.take<int>(np);
    a.rmeta = cv.take<int>(np);
    a.dpix = cv.take<int>(pc);
    a.ddom = cv.take<int>(pc);
    a.dseq = cv.take<int>(pc);
    a.dnextu = cv.take<int>(pc);
    a.dsize = cv.take<int>(n);
    a.doff = cv.take<int>(n);
    a.bbx0 = cv.take<int>(n);
    a.bbx1 = cv.take<int>(n);
    a.bby0 = cv.take<int>(n);
    a.bby1 = cv.take<int>(n);
    a.npop = cv.take<int>(n);
    a.cut = cv.take<int>(n);
    a.sup = cv.take<int>(n);
    a.mcount = cv.take<int>(n);
    a.moff = cv.take<int>(n);
    a.mfill = cv.take<int>(n);
    a.mlist = cv.take<int>(n);
    a.icount = cv.take<int>(n);
    a.ioff = cv.take<int>(n);
    a.ifill = cv.take<int>(n);
    a.ilist = cv.take<int>(n);
    a.cand = cv.take<int>(n);
    a.pend = cv.take<int>(n);
    a.pend2 = cv.take<int>(n);
    a.dfirst = cv.take<unsigned long long>(n);
    a.ord = cv.take<int>(n);
    a.okey = cv.take<int>(n);
    a.obucket = cv.take<int>(64);
    *used_out = cv.used;
}

}  // namespace

size_t pws_workspace_bytes(int64_t npad) {
    PW a;
    a.n = (int)npad;
    a.pc = (int)(npad / 2 + 4096);
    size_t used = 0;
    carve(a, nullptr, &used);
    return used + 4096;
}

int ws_flood_serial_launch(Ctx &c, const int *mk, const uint32_t *col, int *outp, int H, int W, bool conditional,
                           cudaStream_t s) {
    const int n = H * W;
    int *flag = conditional ? c.ws.ctrl + C_WS + W_FALLBACK : nullptr;
    // the flood's links reuse the start of the workspace: nothing there is read
    // once the serial flood runs
    int *next = (int *)c.ws.wsb;
    if (conditional) {
        k_copy_if<<<blocks(c, n), kB, 0, s>>>(mk, outp, n, flag);
        NSG_COUNT_LAUNCH();
    } else {
        cudaMemcpyAsync(outp, mk, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    }
    k_serial<<<1, 32, 0, s>>>(outp, col, next, H, W, c.spin_budget * 64, c.ws.ctrl + C_STATUS, flag);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// The BFS cluster: 16 CTAs when the device can co-schedule them, else fewer.
static int launch_bfs(Ctx &c, const PW &a, const uint8_t *nbm, cudaStream_t s) {
    NSG_CUDA_TRY(c, cudaFuncSetAttribute(k_bfs, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    NSG_CUDA_TRY(c, cudaFuncSetAttribute(k_bfs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBfsSmem));
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    cfg.blockDim = dim3(kBfsThreads);
    cfg.dynamicSmemBytes = kBfsSmem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int cl = kBfsMaxCluster;
    if (c.bfs_max_cluster >= 1 && c.bfs_max_cluster < cl) cl = c.bfs_max_cluster;
    if (const char *e = getenv("NSG_BFS_CLUSTER")) {  // tuning knob: largest cluster to try
        const int v = atoi(e);
        if (v >= 1 && v <= kBfsMaxCluster) cl = v;
    }
    for (; cl > 1; cl /= 2) {
        cfg.gridDim = dim3(cl);
        attr[0].val.clusterDim.x = cl;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, k_bfs, &cfg) == cudaSuccess && nclusters >= 1) break;
        cudaGetLastError();
    }
    cfg.gridDim = dim3(cl);
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    NSG_CUDA_TRY(c, cudaLaunchKernelEx(&cfg, k_bfs, a, nbm));
    NSG_COUNT_LAUNCH();
    return NSG_SUCCESS;
}

// The dispatch list of the P1 (mode 0) or P3 (mode 1) floods, longest
// first, and its length on the host (*count; a readback, so this waits for
// the stream).  The flood kernels are launched with exactly the blocks that
// have floods: each block holds a queue table of shared memory, and a launch
// padded with empty blocks would wait, under load from the other tiles in
// flight, until every empty block found room on some SM.
static int order_floods(Ctx &c, PW &a, int mode, int *count, cudaStream_t s) {
    const int g = blocks(c, a.n);
    NSG_CUDA_TRY(c, cudaMemsetAsync(a.obucket, 0, 64 * sizeof(int), s));
    k_order_count<<<g, kB, 0, s>>>(a, mode);
    NSG_COUNT_LAUNCH();
    k_order_scan<<<1, 32, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_order_scatter<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl + C_WS + W_NORD, a.ctl + W_NORD, sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaStreamSynchronize(s));
    *count = c.ws.h_ctrl[C_WS + W_NORD];
    return NSG_SUCCESS;
}
static int flood_blocks(int count) {
    const int b = (count + kP1Threads - 1) / kP1Threads;
    return b < 1 ? 1 : b;
}

int pws_flood(Ctx &c, const int *mk, const uint32_t *col, int *outp, int H, int W, cudaStream_t s) {
    PW a;
    a.H = H;
    a.W = W;
    a.n = H * W;
    a.pc = a.n / 2 + 4096;
    a.mk = mk;
    a.col = col;
    a.outp = outp;
    a.ctl = c.ws.ctrl + C_WS;
    a.status = c.ws.ctrl + C_STATUS;
    size_t used = 0;
    carve(a, c.ws.wsb, &used);
    if (used > c.ws.wsb_bytes) {
        c.last_error = "watershed workspace too small";
        return NSG_ERR_OOM;
    }
    const int n = a.n;
    const int g = blocks(c, n);
    NSG_CUDA_TRY(c, cudaMemsetAsync(a.ctl, 0, 64 * sizeof(int), s));
    k_classify<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_TRY(ccl_u8(c, a.fgimg, a.domroot, H, W, 4, CCL_NONZERO, s));
    k_roots<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_TRY(exclusive_scan_i32(c, a.isroot, a.rank, n, a.ctl + W_ND, s));
    k_domain_init<<<g, kB, 0, s>>>(a, a.ctl + W_ND);
    NSG_COUNT_LAUNCH();
    k_domains<<<g, kB, 0, s>>>(a, a.ctl + W_ND);
    NSG_COUNT_LAUNCH();
    NSG_TRY(exclusive_scan_i32(c, a.dsize, a.doff, n, nullptr, s, a.ctl + W_ND));  // per-domain: nd entries
    k_udom_count<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_TRY(exclusive_scan_i32(c, a.ducnt, a.duoff, n, a.ctl + W_DTOT, s, a.ctl + W_ND));
    NSG_CUDA_TRY(c, cudaMemsetAsync(a.dpix, 0xff, sizeof(int) * (size_t)a.pc, s));  // -1: slot unused
    NSG_LAUNCH_CHECK(c);
    // P1: one thread per domain
    // per-domain kernels: grid-stride over the domain count (on the device); 64-thread
    // blocks, 4 per SM cover 38,912 domains at once (a 4096^2 tile has a few thousand)
    const int gd = c.sm_count * 4;
    int nflood = 0;
    NSG_TRY(order_floods(c, a, 0, &nflood, s));
    NSG_CUDA_TRY(c, cudaFuncSetAttribute(k_phase1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kP1Smem));
    k_phase1<<<flood_blocks(nflood), kP1Threads, kP1Smem, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    stage_mark(c, kStageWsP1, s);
    // P2
    k_dummy_lists<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_true_dummies<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_candidates<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_first_event<<<1, 1024, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_cuts<<<gd / 4, 256, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    k_state<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_event_label<<<1, 32, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_bfs_prep<<<g, kB, 0, s>>>(a, a.fgimg);  // the domain image is no longer needed
    NSG_COUNT_LAUNCH();
    NSG_TRY(launch_bfs(c, a, a.fgimg, s));
    NSG_LAUNCH_CHECK(c);
    k_mark_r<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    stage_mark(c, kStageWsBfs, s);
    k_shells<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    uint8_t *pimg = a.fgimg;  // reuse: the domain image is no longer needed
    k_pocket_img<<<g, kB, 0, s>>>(a, pimg);
    NSG_COUNT_LAUNCH();
    NSG_TRY(ccl_u8(c, pimg, a.proot, H, W, 4, CCL_NONZERO, s));
    int *powner = a.claim;  // BFS claims are no longer needed
    NSG_CUDA_TRY(c, cudaMemsetAsync(powner, 0xff, sizeof(int) * (size_t)n, s));
    k_pocket_owner<<<g, kB, 0, s>>>(a, powner);
    NSG_COUNT_LAUNCH();
    k_shell_unions<<<g, kB, 0, s>>>(a, powner);
    NSG_COUNT_LAUNCH();
    k_sup_flatten<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_groups<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_TRY(exclusive_scan_i32(c, a.mcount, a.moff, n, nullptr, s, a.ctl + W_ND));
    k_groups2<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_inj_count<<<g, kB, 0, s>>>(a, 0);
    NSG_COUNT_LAUNCH();
    NSG_TRY(exclusive_scan_i32(c, a.icount, a.ioff, n, nullptr, s, a.ctl + W_ND));
    k_inj_count<<<g, kB, 0, s>>>(a, 1);
    NSG_COUNT_LAUNCH();
    k_reset_owned_u<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_pixel_groups<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    k_p3_state<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_TRY(order_floods(c, a, 1, &nflood, s));
    NSG_CUDA_TRY(c, cudaFuncSetAttribute(k_phase3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kP1Smem));
    k_phase3<<<flood_blocks(nflood), kP1Threads, kP1Smem, s>>>(a);
    NSG_COUNT_LAUNCH();
    stage_mark(c, kStageWsP3, s);
    k_assemble<<<g, kB, 0, s>>>(a);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    // exact serial flood when a fast-path condition failed
    return ws_flood_serial_launch(c, mk, col, outp, H, W, true, s);
}

}  // namespace nsg
