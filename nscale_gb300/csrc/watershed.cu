// watershed.cu — nscale::watershed2 (MorphologicOperations.cpp:3717-3760):
// regional minima -> bwlabel2 labels (min raster index, 0 = "unknown" when the
// component holds pixel 0) -> pad labels with 0 and colours with 0 ->
// OpenCV Meyer flooding (cv::watershed, OpenCV 2.4.9) -> border fix
// (NeighborOperations.cpp:18-44) -> crop.
//
// Flooding order.  cv::watershed keeps 256 FIFO queues keyed by the colour
// difference max(|dB|,|dG|,|dR|) and always pops the lowest non-empty queue;
// ties are broken by FIFO order, so the labels depend on the exact order of
// pushes.  watershed_pws.cu reproduces that order exactly with a
// domain-parallel flood (and a serial flood as its verified fallback).
#include "nsg_internal.cuh"

namespace nsg {

namespace {

constexpr int WSHED = -1;

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
// i32[0] padded flood result; the watershed workspace.
int watershed_dev(Ctx &c, const uint8_t *bgr, const float *img, int32_t *out, int rows, int cols, int conn,
                  cudaStream_t s, bool img_negated) {
    uint8_t *minima = c.ws.u8[1];
    int *labels = c.ws.i32[2], *mk = c.ws.i32[3], *outp = c.ws.i32[0];
    uint32_t *colp = (uint32_t *)c.ws.i32[4];
    // localMinima(img) is localMaxima(-img) (MorphologicOperations.cpp:3839)
    NSG_TRY(local_extrema_dev(c, img, minima, rows, cols, conn, !img_negated, s));
    NSG_TRY(bwlabel_dev(c, minima, labels, rows, cols, conn, s));
    int64_t np = (int64_t)(rows + 2) * (cols + 2);
    ws_pack<<<blocks(c, np), 256, 0, s>>>(labels, bgr, rows, cols, mk, colp);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_TRY(pws_flood(c, mk, colp, outp, rows + 2, cols + 2, s));
    ws_border_crop<<<blocks(c, (int64_t)rows * cols), 256, 0, s>>>(outp, rows, cols, out);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// The same flood with the reference's queue discipline executed serially (one
// thread); kept callable for tests and as the fallback.
int watershed_serial_dev(Ctx &c, const uint8_t *bgr, const float *img, int32_t *out, int rows, int cols, int conn,
                         cudaStream_t s) {
    uint8_t *minima = c.ws.u8[1];
    int *labels = c.ws.i32[2], *mk = c.ws.i32[3], *outp = c.ws.i32[0];
    uint32_t *colp = (uint32_t *)c.ws.i32[4];
    NSG_TRY(local_extrema_dev(c, img, minima, rows, cols, conn, true, s));
    NSG_TRY(bwlabel_dev(c, minima, labels, rows, cols, conn, s));
    int64_t np = (int64_t)(rows + 2) * (cols + 2);
    ws_pack<<<blocks(c, np), 256, 0, s>>>(labels, bgr, rows, cols, mk, colp);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    NSG_TRY(ws_flood_serial_launch(c, mk, colp, outp, rows + 2, cols + 2, false, s));
    ws_border_crop<<<blocks(c, (int64_t)rows * cols), 256, 0, s>>>(outp, rows, cols, out);
    NSG_COUNT_LAUNCH();
    NSG_LAUNCH_CHECK(c);
    return NSG_SUCCESS;
}

// Fast-path diagnostics of the last watershed call (host copy of the control
// block): [0] fallback code (0 = domain-parallel path), [1] domains,
// [2] dummy entries, [6] level of the first background pop, [11] BFS layers.
int watershed_diag(Ctx &c, int *out16, cudaStream_t s) {
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl, c.ws.ctrl + C_WS, 13 * sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl + 14, c.ws.ctrl + C_WS + 12, sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl + 12, c.ws.ctrl + C_RSTATS, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl + 15, c.ws.ctrl + C_RSTATS + 3, sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaStreamSynchronize(s));
    for (int i = 0; i < 16; ++i) out16[i] = c.ws.h_ctrl[i];
    return NSG_SUCCESS;
}

}  // namespace nsg
