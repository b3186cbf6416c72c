// context.cu — workspace arena, status plumbing and small ABI helpers.
#include <stdlib.h>
#include <string.h>

#include <new>

#include "nsg_internal.cuh"

namespace nsg {

std::atomic<long long> g_kernel_launches{0};

int sync_status(Ctx &c, cudaStream_t s) {
    NSG_CUDA_TRY(c, cudaMemcpyAsync(c.ws.h_ctrl, c.ws.ctrl + C_STATUS, sizeof(int), cudaMemcpyDeviceToHost, s));
    NSG_CUDA_TRY(c, cudaStreamSynchronize(s));
    int st = c.ws.h_ctrl[0];
    if (st & DEV_QUEUE_FULL) {
        c.last_error = "device queue overflow";
        return NSG_ERR_QUEUE_FULL;
    }
    if (st & DEV_TIMEOUT) {
        c.last_error = "device wait exceeded its iteration budget";
        return NSG_ERR_TIMEOUT;
    }
    return NSG_SUCCESS;
}

int reset_status(Ctx &c, cudaStream_t s) {
    NSG_CUDA_TRY(c, cudaMemsetAsync(c.ws.ctrl + C_STATUS, 0, sizeof(int), s));
    return NSG_SUCCESS;
}

// sizes of the arena's slots, in carving order; returns the total
size_t arena_layout(int64_t max_pad, size_t *sizes) {
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t P = (size_t)max_pad;
    int ns = 0;
    for (int i = 0; i < 6; ++i) sizes[ns++] = al(P * 4);
    for (int i = 0; i < 3; ++i) sizes[ns++] = al(P * 4);
    for (int i = 0; i < 4; ++i) sizes[ns++] = al(P);
    for (int i = 0; i < 10; ++i) sizes[ns++] = al(P);
    for (int i = 0; i < 2; ++i) sizes[ns++] = al(P * 4);
    for (int i = 0; i < 2; ++i) sizes[ns++] = al(P * 4);
    sizes[ns++] = al(P * 3);                 // p_bgr
    sizes[ns++] = al(kCtrlInts * 4);         // ctrl
    sizes[ns++] = al(64 * 8);                // ctr64
    sizes[ns++] = al((P / 256 + 1024) * 4);  // scan_tmp
    sizes[ns++] = al(pws_workspace_bytes((int64_t)P));  // watershed workspace
    size_t total = 0;
    for (int i = 0; i < ns; ++i) total += sizes[i];
    return total;
}

size_t context_bytes_for(int max_rows, int max_cols) {
    size_t sizes[64];
    return arena_layout((int64_t)(max_rows + 2) * (max_cols + 2), sizes);
}

}  // namespace nsg

using namespace nsg;

extern "C" {

int nsg_version(void) { return 10000; }

void nsg_default_params(nsg_seg_params *p) {
    if (!p) return;
    p->blue = p->green = p->red = 220;
    p->T1 = 5.0;
    p->T2 = 4.0;
    p->G1 = 80;
    p->minSize = 11;
    p->maxSize = 1000;
    p->G2 = 45;
    p->minSizePl = 30;
    p->minSizeSeg = 21;
    p->maxSizeSeg = 1000;
    p->fillHolesConnectivity = 4;
    p->reconConnectivity = 8;
    p->watershedConnectivity = 8;
}

const char *nsg_status_string(int st) {
    switch (st) {
        case NSG_SUCCESS: return "SUCCESS";
        case NSG_BACKGROUND: return "BACKGROUND";
        case NSG_BACKGROUND_LIKELY: return "BACKGROUND_LIKELY";
        case NSG_NO_CANDIDATES_LEFT: return "NO_CANDIDATES_LEFT";
        case NSG_CONTINUE: return "CONTINUE";
        case NSG_INVALID_IMAGE: return "INVALID_IMAGE";
        case NSG_RUNTIME_FAILED: return "RUNTIME_FAILED";
        case NSG_ERR_ARG: return "ERR_ARG";
        case NSG_ERR_OOM: return "ERR_OOM";
        case NSG_ERR_TIMEOUT: return "ERR_TIMEOUT";
        case NSG_ERR_QUEUE_FULL: return "ERR_QUEUE_FULL";
        case NSG_ERR_CUDA: return "ERR_CUDA";
        case NSG_ERR_UNSUPPORTED: return "ERR_UNSUPPORTED";
        default: return "UNKNOWN";
    }
}

int nsg_context_create(nsg_context **out, int max_rows, int max_cols, int device) {
    if (!out || max_rows <= 0 || max_cols <= 0) return NSG_ERR_ARG;
    *out = nullptr;
    nsg_context *h = new (std::nothrow) nsg_context();
    if (!h) return NSG_ERR_OOM;
    Ctx &c = h->c;
    c.device = device;
    c.max_rows = max_rows;
    c.max_cols = max_cols;
    c.max_px = (int64_t)max_rows * max_cols;
    c.max_pad = (int64_t)(max_rows + 2) * (max_cols + 2);
    if (cudaSetDevice(device) != cudaSuccess) {
        delete h;
        return NSG_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, device);
    size_t sizes[64];
    const size_t total = arena_layout(c.max_pad, sizes);
    char *base = nullptr;
    if (cudaMalloc((void **)&base, total) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return NSG_ERR_OOM;
    }
    c.arena = base;
    c.arena_bytes = total;
    int k = 0;
    char *p = base;
    auto take = [&](void) {
        char *r = p;
        p += sizes[k++];
        return r;
    };
    for (int i = 0; i < 6; ++i) c.ws.i32[i] = (int32_t *)take();
    for (int i = 0; i < 3; ++i) c.ws.f32[i] = (float *)take();
    for (int i = 0; i < 4; ++i) c.ws.u8[i] = (uint8_t *)take();
    for (int i = 0; i < 10; ++i) c.ws.p_u8[i] = (uint8_t *)take();
    for (int i = 0; i < 2; ++i) c.ws.p_f32[i] = (float *)take();
    for (int i = 0; i < 2; ++i) c.ws.p_i32[i] = (int32_t *)take();
    c.ws.p_bgr = (uint8_t *)take();
    c.ws.ctrl = (int *)take();
    c.ws.ctr64 = (int64_t *)take();
    c.ws.scan_tmp = (int32_t *)take();
    c.ws.wsb_bytes = sizes[k];
    c.ws.wsb = take();
    if (cudaMallocHost((void **)&c.ws.h_ctrl, kCtrlInts * 4) != cudaSuccess ||
        cudaMallocHost((void **)&c.ws.h_ctr64, 64 * 8) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(base);
        delete h;
        return NSG_ERR_OOM;
    }
    cudaMemset(c.ws.ctrl, 0, kCtrlInts * 4);
    cudaMemset(c.ws.ctr64, 0, 64 * 8);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaFree(base);
        delete h;
        return NSG_ERR_CUDA;
    }
    *out = h;
    return NSG_SUCCESS;
}

int nsg_context_destroy(nsg_context *h) {
    if (!h) return NSG_ERR_ARG;
    Ctx &c = h->c;
    cudaSetDevice(c.device);
    cudaDeviceSynchronize();
    if (c.ev_counts) cudaEventDestroy(c.ev_counts);
    if (c.ws.h_ctrl) cudaFreeHost(c.ws.h_ctrl);
    if (c.ws.h_ctr64) cudaFreeHost(c.ws.h_ctr64);
    if (c.arena) cudaFree(c.arena);
    delete h;
    return NSG_SUCCESS;
}

const char *nsg_context_last_error(const nsg_context *h) { return h ? h->c.last_error.c_str() : "null context"; }

int nsg_context_set_tuning(nsg_context *h, const nsg_tuning *t) {
    if (!h || !t || t->recon_max_ctas < 0 || t->bfs_max_cluster < 0 || t->bfs_max_cluster > 16 ||
        t->recon_wl_phases < -1 || t->recon_wl_phases > 8)
        return NSG_ERR_ARG;
    h->c.recon_max_ctas = t->recon_max_ctas;
    h->c.bfs_max_cluster = t->bfs_max_cluster;
    h->c.recon_wl_phases = t->recon_wl_phases;
    return NSG_SUCCESS;
}

size_t nsg_context_bytes(const nsg_context *h) { return h ? h->c.arena_bytes : 0; }

int nsg_context_set_spin_budget(nsg_context *h, long long it) {
    if (!h) return NSG_ERR_ARG;
    h->c.spin_budget = it > 0 ? it : (1ll << 26);
    return NSG_SUCCESS;
}

void *nsg_alloc(size_t bytes) { return malloc(bytes ? bytes : 1); }

long long nsg_kernel_launches(void) { return g_kernel_launches.load(); }
void nsg_free(void *p) { free(p); }

}  // extern "C"
