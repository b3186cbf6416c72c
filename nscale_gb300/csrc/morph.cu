// morph.cu — greyscale erosion / dilation with an arbitrary k x k
// structuring element (cv::erode / cv::dilate as morphOpen calls them,
// MorphologicOperations.cpp:3849-3882; 19x19 MATLAB disk HistologicalEntities.cpp:169-188;
// 3x3 cross HistologicalEntities.cpp:327, 498).
//
// Design: a structuring element whose rows are centred chords (the disk and
// the cross are) is applied as   out(y,x) = min_dy H_{w(dy)}(y+dy, x)   where
// H_w is the horizontal running min over [x-w, x+w].  Each CTA stages an
// input tile plus halo in shared memory (out-of-image samples are neutral:
// 255 for erode, 0 for dilate), builds H_w for every distinct chord width
// incrementally (H_{w+1} = min(H_w, x-w-1, x+w+1)), then combines rows.
// Other structuring elements take a generic tap-list path.
#include <string.h>

#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int TH = 32;    // output rows per CTA
constexpr int TW = 128;   // output cols per CTA
constexpr int kThreads = 256;
constexpr int kMaxW = 6;  // distinct chord widths held in shared memory

struct ChordSE {
    int r;                 // vertical radius (k/2)
    int R;                 // max half width
    int nw;                // number of distinct widths
    int w[kMaxW];          // distinct widths, ascending
    int8_t row_w[kMaxSE];  // per SE row: index into w[], -1 = empty row
};

template <bool IS_MAX>
__device__ __forceinline__ uint8_t op(uint8_t a, uint8_t b) {
    return IS_MAX ? (a > b ? a : b) : (a < b ? a : b);
}

template <bool IS_MAX>
__global__ void __launch_bounds__(kThreads) chord_kernel(const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                         int rows, int cols, ChordSE se) {
    extern __shared__ uint8_t smem[];
    const uint8_t neutral = IS_MAX ? 0 : 255;
    const int r = se.r, R = se.R;
    const int IH = TH + 2 * r, IW = TW + 2 * R;
    uint8_t *tile = smem;            // IH x IW
    uint8_t *hbuf = smem + IH * IW;  // nw x IH x TW
    const int y0 = blockIdx.y * TH, x0 = blockIdx.x * TW;
    for (int i = threadIdx.x; i < IH * IW; i += kThreads) {
        int ty = i / IW, tx = i - ty * IW;
        int y = y0 - r + ty, x = x0 - R + tx;
        tile[i] = (y >= 0 && y < rows && x >= 0 && x < cols) ? in[(int64_t)y * cols + x] : neutral;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < IH * TW; i += kThreads) {
        int ty = i / TW, tx = i - ty * TW;
        const uint8_t *t = tile + ty * IW + (tx + R);  // centre sample
        int w = se.w[0];
        uint8_t m = t[0];
        for (int d = 1; d <= w; ++d) m = op<IS_MAX>(m, op<IS_MAX>(t[-d], t[d]));
        hbuf[ty * TW + tx] = m;
        for (int j = 1; j < se.nw; ++j) {
            for (int d = w + 1; d <= se.w[j]; ++d) m = op<IS_MAX>(m, op<IS_MAX>(t[-d], t[d]));
            w = se.w[j];
            hbuf[(j * IH + ty) * TW + tx] = m;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TH * TW; i += kThreads) {
        int ty = i / TW, tx = i - ty * TW;
        int y = y0 + ty, x = x0 + tx;
        if (y >= rows || x >= cols) continue;
        uint8_t m = neutral;
        for (int dy = 0; dy <= 2 * r; ++dy) {
            int wi = se.row_w[dy];
            if (wi < 0) continue;
            m = op<IS_MAX>(m, hbuf[(wi * IH + ty + dy) * TW + tx]);
        }
        out[(int64_t)y * cols + x] = m;
    }
}

struct TapSE {
    int r;
    int n;
    int8_t dy[kMaxSE * kMaxSE];
    int8_t dx[kMaxSE * kMaxSE];
};

template <bool IS_MAX>
__global__ void __launch_bounds__(kThreads) tap_kernel(const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                       int rows, int cols, const TapSE *__restrict__ se) {
    extern __shared__ uint8_t smem[];
    const uint8_t neutral = IS_MAX ? 0 : 255;
    const int r = se->r;
    const int IH = TH + 2 * r, IW = TW + 2 * r;
    const int y0 = blockIdx.y * TH, x0 = blockIdx.x * TW;
    for (int i = threadIdx.x; i < IH * IW; i += kThreads) {
        int ty = i / IW, tx = i - ty * IW;
        int y = y0 - r + ty, x = x0 - r + tx;
        smem[i] = (y >= 0 && y < rows && x >= 0 && x < cols) ? in[(int64_t)y * cols + x] : neutral;
    }
    __syncthreads();
    const int n = se->n;
    for (int i = threadIdx.x; i < TH * TW; i += kThreads) {
        int ty = i / TW, tx = i - ty * TW;
        int y = y0 + ty, x = x0 + tx;
        if (y >= rows || x >= cols) continue;
        uint8_t m = neutral;
        for (int k = 0; k < n; ++k) m = op<IS_MAX>(m, smem[(ty + r + se->dy[k]) * IW + (tx + r + se->dx[k])]);
        out[(int64_t)y * cols + x] = m;
    }
}

}  // namespace

int morph_u8(Ctx &c, const uint8_t *in, uint8_t *out, int rows, int cols, const uint8_t *se_host, int k, bool is_max,
             cudaStream_t s) {
    if (!se_host || k < 1 || k > kMaxSE || (k % 2) == 0) {
        c.last_error = "structuring element must be k x k with odd k <= 31";
        return NSG_ERR_ARG;
    }
    const int r = k / 2;
    // chord decomposition
    ChordSE cs;
    memset(&cs, 0, sizeof(cs));
    cs.r = r;
    bool chords = true;
    int widths[kMaxSE];
    int nw = 0, R = 0;
    for (int row = 0; row < k; ++row) {
        int lo = -1, hi = -1, cnt = 0;
        for (int col = 0; col < k; ++col)
            if (se_host[row * k + col]) {
                if (lo < 0) lo = col;
                hi = col;
                ++cnt;
            }
        if (cnt == 0) {
            cs.row_w[row] = -1;
            continue;
        }
        if (cnt != hi - lo + 1 || (lo + hi) != 2 * r) {
            chords = false;
            break;
        }
        int w = r - lo;
        int idx = -1;
        for (int j = 0; j < nw; ++j)
            if (widths[j] == w) idx = j;
        if (idx < 0) {
            widths[nw] = w;
            idx = nw++;
        }
        cs.row_w[row] = (int8_t)idx;
        if (w > R) R = w;
    }
    if (chords && nw <= kMaxW) {
        // sort widths ascending and remap
        int order[kMaxSE];
        for (int j = 0; j < nw; ++j) order[j] = j;
        for (int a = 0; a < nw; ++a)
            for (int b = a + 1; b < nw; ++b)
                if (widths[order[b]] < widths[order[a]]) {
                    int t = order[a];
                    order[a] = order[b];
                    order[b] = t;
                }
        int rank[kMaxSE];
        for (int j = 0; j < nw; ++j) {
            cs.w[j] = widths[order[j]];
            rank[order[j]] = j;
        }
        for (int row = 0; row < k; ++row)
            if (cs.row_w[row] >= 0) cs.row_w[row] = (int8_t)rank[(int)cs.row_w[row]];
        cs.nw = nw;
        cs.R = R;
        int IH = TH + 2 * r, IW = TW + 2 * R;
        size_t smem = (size_t)IH * IW + (size_t)nw * IH * TW;
        dim3 grid((cols + TW - 1) / TW, (rows + TH - 1) / TH);
        if (smem > 48 * 1024) {
            // the device's opt-in maximum, the same from every caller: host
            // threads that open with different elements never lower the limit
            // under one another's launches
            int optin = 0;
            NSG_CUDA_TRY(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
            if ((int64_t)smem > optin) return NSG_ERR_ARG;
            NSG_CUDA_TRY(c, cudaFuncSetAttribute(chord_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 optin));
            NSG_CUDA_TRY(c, cudaFuncSetAttribute(chord_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 optin));
        }
        if (is_max)
            chord_kernel<true><<<grid, kThreads, smem, s>>>(in, out, rows, cols, cs);
        else
            chord_kernel<false><<<grid, kThreads, smem, s>>>(in, out, rows, cols, cs);
        NSG_COUNT_LAUNCH();
        NSG_LAUNCH_CHECK(c);
        return NSG_SUCCESS;
    }
    // generic taps (staged through the context's control area)
    static_assert(sizeof(TapSE) <= (kCtrlInts - C_QSLOTS) * 4, "tap list does not fit");
    TapSE ts;
    memset(&ts, 0, sizeof(ts));
    ts.r = r;
    for (int row = 0; row < k; ++row)
        for (int col = 0; col < k; ++col)
            if (se_host[row * k + col]) {
                ts.dy[ts.n] = (int8_t)(row - r);
                ts.dx[ts.n] = (int8_t)(col - r);
                ++ts.n;
            }
    TapSE *d_ts = (TapSE *)(c.ws.ctrl + C_QSLOTS);
    NSG_CUDA_TRY(c, cudaMemcpyAsync(d_ts, &ts, sizeof(ts), cudaMemcpyHostToDevice, s));
    int IH = TH + 2 * r, IW = TW + 2 * r;
    size_t smem = (size_t)IH * IW;
    dim3 grid((cols + TW - 1) / TW, (rows + TH - 1) / TH);
    if (is_max)
        tap_kernel<true><<<grid, kThreads, smem, s>>>(in, out, rows, cols, d_ts);
    else
        tap_kernel<false><<<grid, kThreads, smem, s>>>(in, out, rows, cols, d_ts);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    // the host copy of `ts` must outlive the async copy
    NSG_CUDA_TRY(c, cudaStreamSynchronize(s));
    return NSG_SUCCESS;
}

}  // namespace nsg
