// watershed.cu — nscale::watershed2 (MorphologicOperations.cpp:3717-3760):
// regional minima -> bwlabel2 labels (min raster index, 0 = "unknown" when the
// component holds pixel 0) -> pad labels with 0 and colours with 0 ->
// OpenCV Meyer flooding (cv::watershed, OpenCV 2.4.9) -> border fix
// (NeighborOperations.cpp:18-44) -> crop.
//
// Flooding order.  cv::watershed keeps 256 FIFO queues keyed by the colour
// difference max(|dB|,|dG|,|dR|) and always pops the lowest non-empty queue;
// ties are broken by FIFO order, so the labels depend on the exact order of
// pushes.  This file reproduces that order exactly: `ws_flood_serial` is the
// reference's queue discipline executed by one thread over the padded label
// image (intrusive FIFO lists, one `next` link per pixel since every pixel is
// queued at most once).
#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int WSHED = -1;
constexpr int IN_QUEUE = -2;

__global__ void ws_pack(const int *__restrict__ labels, const uint8_t *__restrict__ bgr, int rows, int cols,
                        int *__restrict__ mk, uint32_t *__restrict__ col) {
    const int W = cols + 2, H = rows + 2;
    int64_t n = (int64_t)W * H;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int y = (int)(i / W) - 1, x = (int)(i % W) - 1;
        if (y >= 0 && y < rows && x >= 0 && x < cols) {
            int64_t s = (int64_t)y * cols + x;
            mk[i] = labels[s];
            const uint8_t *p = bgr + 3 * s;
            col[i] = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16);
        } else {
            mk[i] = 0;
            col[i] = 0;
        }
    }
}

__device__ __forceinline__ int cdiff(uint32_t a, uint32_t b) {
    int db = abs((int)(a & 255) - (int)(b & 255));
    int dg = abs((int)((a >> 8) & 255) - (int)((b >> 8) & 255));
    int dr = abs((int)((a >> 16) & 255) - (int)((b >> 16) & 255));
    int d = db > dg ? db : dg;
    return d > dr ? d : dr;
}

// One thread: the reference's queue discipline, step for step.
__global__ void ws_flood_serial(int *__restrict__ m, const uint32_t *__restrict__ col, int *__restrict__ next,
                                int H, int W, long long budget, int *status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
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

// NeighborOperations::border<int>(padded, -1), then crop (y, x in the image)
__global__ void ws_border_crop(const int *__restrict__ m, int rows, int cols, int *__restrict__ out) {
    const int W = cols + 2;
    int64_t n = (int64_t)rows * cols;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int y = (int)(i / cols) + 1, x = (int)(i % cols) + 1;
        const int *p = m + (int64_t)y * W + x;
        const int *pm = p - W;
        int v = p[0];
        if (pm[0] == WSHED && v != WSHED &&
            ((pm[-1] != WSHED && p[-1] == WSHED) || (pm[1] != WSHED && p[1] == WSHED)))
            v = WSHED;
        out[i] = v;
    }
}

int blocks(Ctx &c, int64_t n) {
    int64_t g = (n + 255) / 256;
    int64_t cap = (int64_t)c.sm_count * 16;
    return (int)(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

// scratch: local extrema (f32[0..2], u8[0], i32[0..1], i32[5]); u8[1] minima;
// i32[2] minima labels; i32[3] padded markers; i32[4] padded colours;
// i32[0] queue links.
int watershed_dev(Ctx &c, const uint8_t *bgr, const float *img, int32_t *out, int rows, int cols, int conn,
                  cudaStream_t s) {
    uint8_t *minima = c.ws.u8[1];
    int *labels = c.ws.i32[2], *mk = c.ws.i32[3];
    uint32_t *colp = (uint32_t *)c.ws.i32[4];
    int *next = c.ws.i32[0];
    NSG_TRY(local_extrema_dev(c, img, minima, rows, cols, conn, true, s));
    NSG_TRY(bwlabel_dev(c, minima, labels, rows, cols, conn, s));
    int64_t np = (int64_t)(rows + 2) * (cols + 2);
    ws_pack<<<blocks(c, np), 256, 0, s>>>(labels, bgr, rows, cols, mk, colp);
    NSG_LAUNCH_CHECK(c);
    ws_flood_serial<<<1, 32, 0, s>>>(mk, colp, next, rows + 2, cols + 2, c.spin_budget * 64,
                                     c.ws.ctrl + C_STATUS);
    NSG_LAUNCH_CHECK(c);
    ws_border_crop<<<blocks(c, (int64_t)rows * cols), 256, 0, s>>>(mk, rows, cols, out);
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

}  // namespace nsg
