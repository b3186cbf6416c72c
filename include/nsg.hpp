/*
 * nsg.hpp — C++ drop-in shim over libnsg.so with nscale's own names and
 * argument order, for C++ callers of the reference's segmentNuclei path,
 * without OpenCV.  Header-only; it calls only the C ABI of nsg.h and the CUDA
 * runtime (device buffers), so it links against libnsg.so and libcudart.
 *
 * Image types (in place of cv::Mat / cv::gpu::GpuMat):
 *   nscale::HostImage<T>   row-major host image (std::vector storage)
 *   nscale::DeviceImage<T> row-major device image, reference-counted like
 *                          cv::gpu::GpuMat (copies share the buffer)
 * Both carry rows, cols and channels (3 for a BGR tile, else 1).
 *
 * Names and argument order follow the reference:
 *   HistologicalEntities::segmentNuclei   HistologicalEntities.h:52-60
 *   HistologicalEntities::getRBC / getBackground  HistologicalEntities.h:44-51
 *   imreconstruct, imreconstructBinary, imfillHoles, bwselect, bwlabel2,
 *   bwareaopen2, imhmin, localMaxima, localMinima, watershed2, morphOpen
 *                                        MorphologicOperations.h:33-115
 *   PixelOperations::invert, ComputeInverseStainMatrix, ColorDeconv
 *                                        PixelOperations.h:37-58
 * Errors: segmentNuclei returns the reference's status values; a library
 * failure in any call throws nscale::Error (code = the NSG_ERR_* value), in
 * the place of the reference's cv::Exception from CV_Assert.  The bbox array
 * segmentNuclei returns is malloc'd, as the reference's: release it with
 * free() (or nsg_free).
 *
 * Work runs on one per-thread library context (workspace arena, grown to the
 * largest image seen) and on the legacy default stream, and every call
 * returns finished results, as the reference's calls do.
 */
#ifndef NSG_HPP
#define NSG_HPP

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nsg.h"

namespace nscale {

class Error : public std::runtime_error {
  public:
    Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

  private:
    int code_;
};

namespace detail {

inline void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(NSG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// The per-thread context: one workspace arena on the current device, grown
// (re-created) when an image does not fit.
class Ctx {
  public:
    ~Ctx() {
        if (h_) nsg_context_destroy(h_);
    }
    nsg_context *get(int rows, int cols) {
        int dev = 0;
        check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
        if (!h_ || dev != dev_ || (int64_t)rows * cols > (int64_t)r_ * c_ ||
            (int64_t)(rows + 2) * (cols + 2) > (int64_t)(r_ + 2) * (c_ + 2)) {
            const int r = rows > r_ ? rows : r_, c = cols > c_ ? cols : c_;
            if (h_) nsg_context_destroy(h_);
            h_ = nullptr;
            const int st = nsg_context_create(&h_, r, c, dev);
            if (st != NSG_SUCCESS) throw Error(st, "nsg_context_create failed");
            r_ = r, c_ = c, dev_ = dev;
        }
        return h_;
    }
    void check(int st) const {
        if (st < 0) throw Error(st, h_ ? nsg_context_last_error(h_) : nsg_status_string(st));
    }

  private:
    nsg_context *h_ = nullptr;
    int r_ = 0, c_ = 0, dev_ = -1;
};

inline Ctx &ctx() {
    static thread_local Ctx c;
    return c;
}

}  // namespace detail

template <typename T>
class HostImage {
  public:
    int rows = 0, cols = 0, channels = 1;
    std::vector<T> pixels;
    HostImage() {}
    HostImage(int r, int c, int ch = 1) : rows(r), cols(c), channels(ch), pixels((size_t)r * c * ch) {}
    T *data() { return pixels.data(); }
    const T *data() const { return pixels.data(); }
    bool empty() const { return pixels.empty(); }
};

template <typename T>
class DeviceImage {
  public:
    int rows = 0, cols = 0, channels = 1;
    DeviceImage() {}
    DeviceImage(int r, int c, int ch = 1) : rows(r), cols(c), channels(ch) {
        T *p = nullptr;
        if (size() > 0) detail::check_cuda(cudaMalloc((void **)&p, size() * sizeof(T)), "cudaMalloc");
        buf_ = std::shared_ptr<T>(p, [](T *q) {
            if (q) cudaFree(q);
        });
    }
    static DeviceImage upload(const HostImage<T> &h) {
        DeviceImage d(h.rows, h.cols, h.channels);
        if (d.size() > 0)
            detail::check_cuda(cudaMemcpy(d.data(), h.data(), d.size() * sizeof(T), cudaMemcpyHostToDevice),
                               "upload");
        return d;
    }
    HostImage<T> download() const {
        HostImage<T> h(rows, cols, channels);
        if (size() > 0)
            detail::check_cuda(cudaMemcpy(h.data(), data(), size() * sizeof(T), cudaMemcpyDeviceToHost), "download");
        return h;
    }
    T *data() const { return buf_.get(); }
    size_t size() const { return (size_t)rows * cols * channels; }
    bool empty() const { return size() == 0; }

  private:
    std::shared_ptr<T> buf_;
};

namespace detail {
template <typename T>
void same_shape(const DeviceImage<T> &a, const DeviceImage<T> &b) {
    if (a.rows != b.rows || a.cols != b.cols || a.channels != 1 || b.channels != 1)
        throw Error(NSG_ERR_ARG, "images must be single-channel and of one size");
}
template <typename T>
struct Recon;
template <>
struct Recon<uint8_t> {
    static int run(nsg_context *c, const uint8_t *m, const uint8_t *k, uint8_t *o, int r, int cl, int conn) {
        return nsg_imreconstruct_u8(c, m, k, o, r, cl, conn, nullptr);
    }
};
template <>
struct Recon<float> {
    static int run(nsg_context *c, const float *m, const float *k, float *o, int r, int cl, int conn) {
        return nsg_imreconstruct_f32(c, m, k, o, r, cl, conn, nullptr);
    }
};
inline int invert_n(nsg_context *c, const uint8_t *i, uint8_t *o, int64_t n) { return nsg_invert_u8(c, i, o, n, nullptr); }
inline int invert_n(nsg_context *c, const int32_t *i, int32_t *o, int64_t n) { return nsg_invert_i32(c, i, o, n, nullptr); }
inline int invert_n(nsg_context *c, const float *i, float *o, int64_t n) { return nsg_invert_f32(c, i, o, n, nullptr); }
}  // namespace detail

// ---- PixelOperations ---------------------------------------------------------
class PixelOperations {
  public:
    template <typename T>
    static DeviceImage<T> invert(const DeviceImage<T> &img) {
        DeviceImage<T> out(img.rows, img.cols, img.channels);
        auto &cx = detail::ctx();
        cx.check(detail::invert_n(cx.get(1, 1), img.data(), out.data(), (int64_t)img.size()));
        return out;
    }
    // rows of inv(normalised M) selected by b, row-major 2 x 3 (M, b NULL =
    // the feature pipeline's stains)
    static std::vector<float> ComputeInverseStainMatrix(const double *M9 = nullptr, const uint8_t *b3 = nullptr) {
        std::vector<float> q(6);
        const int st = nsg_stain_matrix(M9, b3, q.data());
        if (st != NSG_SUCCESS) throw Error(st, "singular stain matrix");
        return q;
    }
    static void ColorDeconv(const DeviceImage<uint8_t> &image, const std::vector<float> &Q, DeviceImage<uint8_t> &H,
                            DeviceImage<uint8_t> &E) {
        H = DeviceImage<uint8_t>(image.rows, image.cols);
        E = DeviceImage<uint8_t>(image.rows, image.cols);
        auto &cx = detail::ctx();
        cx.check(nsg_color_deconv(cx.get(image.rows, image.cols), image.data(), image.rows, image.cols, 0, Q.data(),
                                  H.data(), E.data(), nullptr));
    }
};

// ---- MorphologicOperations ---------------------------------------------------
template <typename T>
DeviceImage<T> imreconstruct(const DeviceImage<T> &seeds, const DeviceImage<T> &image, int connectivity) {
    detail::same_shape(seeds, image);
    DeviceImage<T> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(detail::Recon<T>::run(cx.get(image.rows, image.cols), seeds.data(), image.data(), out.data(), image.rows,
                                   image.cols, connectivity));
    return out;
}

template <typename T>
DeviceImage<T> imreconstructBinary(const DeviceImage<T> &seeds, const DeviceImage<T> &binaryImage, int connectivity) {
    static_assert(sizeof(T) == 1, "binary reconstruction runs on uint8 images");
    detail::same_shape(seeds, binaryImage);
    DeviceImage<T> out(binaryImage.rows, binaryImage.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_imreconstruct_binary_u8(cx.get(out.rows, out.cols), seeds.data(), binaryImage.data(), out.data(),
                                         out.rows, out.cols, connectivity, nullptr));
    return out;
}

template <typename T>
DeviceImage<T> imfillHoles(const DeviceImage<T> &image, bool binary, int connectivity) {
    static_assert(sizeof(T) == 1, "hole filling runs on uint8 images");
    if (!binary) throw Error(NSG_ERR_UNSUPPORTED, "imfillHoles: only the binary form is on the segmentNuclei path");
    DeviceImage<T> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_imfill_holes_u8(cx.get(out.rows, out.cols), image.data(), out.data(), out.rows, out.cols,
                                 connectivity, nullptr));
    return out;
}

template <typename T>
DeviceImage<T> bwselect(const DeviceImage<T> &binaryImage, const DeviceImage<T> &seeds, int connectivity) {
    static_assert(sizeof(T) == 1, "bwselect runs on uint8 images");
    detail::same_shape(binaryImage, seeds);
    DeviceImage<T> out(seeds.rows, seeds.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_bwselect_u8(cx.get(out.rows, out.cols), binaryImage.data(), seeds.data(), out.data(), out.rows,
                             out.cols, connectivity, nullptr));
    return out;
}

inline DeviceImage<int32_t> bwlabel2(const DeviceImage<uint8_t> &binaryImage, int connectivity, bool relab) {
    (void)relab;  // the reference's relabel step is disabled (MorphologicOperations.cpp:3105-3112)
    DeviceImage<int32_t> out(binaryImage.rows, binaryImage.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_bwlabel(cx.get(out.rows, out.cols), binaryImage.data(), out.data(), out.rows, out.cols, connectivity,
                         nullptr));
    return out;
}

inline DeviceImage<uint8_t> bwareaopen2(const DeviceImage<uint8_t> &image, bool labeled, bool flatten, int minSize,
                                        int maxSize, int connectivity, int &count) {
    if (labeled || !flatten)
        throw Error(NSG_ERR_UNSUPPORTED, "bwareaopen2: only (labeled=false, flatten=true) is on the path");
    DeviceImage<uint8_t> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_bwareaopen(cx.get(out.rows, out.cols), image.data(), out.data(), out.rows, out.cols, minSize, maxSize,
                            connectivity, &count, nullptr));
    return out;
}

template <typename T>
DeviceImage<T> imhmin(const DeviceImage<T> &image, T h, int connectivity) {
    static_assert(sizeof(T) == 4, "imhmin runs on float images on the path");
    DeviceImage<T> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_imhmin_f32(cx.get(out.rows, out.cols), image.data(), out.data(), out.rows, out.cols, (float)h,
                            connectivity, nullptr));
    return out;
}

template <typename T>
DeviceImage<uint8_t> localMaxima(const DeviceImage<T> &image, int connectivity) {
    DeviceImage<uint8_t> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_local_maxima_f32(cx.get(out.rows, out.cols), image.data(), out.data(), out.rows, out.cols,
                                  connectivity, nullptr));
    return out;
}

template <typename T>
DeviceImage<uint8_t> localMinima(const DeviceImage<T> &image, int connectivity) {
    DeviceImage<uint8_t> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_local_minima_f32(cx.get(out.rows, out.cols), image.data(), out.data(), out.rows, out.cols,
                                  connectivity, nullptr));
    return out;
}

inline DeviceImage<int32_t> watershed2(const DeviceImage<uint8_t> &origImage, const DeviceImage<float> &image,
                                       int connectivity) {
    if (origImage.channels != 3 || origImage.rows != image.rows || origImage.cols != image.cols)
        throw Error(NSG_ERR_ARG, "watershed2: a BGR image and a float image of one size");
    DeviceImage<int32_t> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_watershed(cx.get(out.rows, out.cols), origImage.data(), image.data(), out.data(), out.rows, out.cols,
                           connectivity, nullptr));
    return out;
}

// kernel: k x k host structuring element (non-zero = in the support)
template <typename T>
DeviceImage<T> morphOpen(const DeviceImage<T> &image, const HostImage<uint8_t> &kernel) {
    static_assert(sizeof(T) == 1, "morphOpen runs on uint8 images on the path");
    if (kernel.rows != kernel.cols || kernel.rows < 3 || kernel.rows % 2 == 0)
        throw Error(NSG_ERR_ARG, "morphOpen: the kernel must be square, odd and larger than 1");
    DeviceImage<T> out(image.rows, image.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_morph_open_u8(cx.get(out.rows, out.cols), image.data(), out.data(), out.rows, out.cols, kernel.data(),
                               kernel.rows, nullptr));
    return out;
}

inline DeviceImage<float> distanceTransform(const DeviceImage<uint8_t> &mask) {
    DeviceImage<float> out(mask.rows, mask.cols);
    auto &cx = detail::ctx();
    cx.check(nsg_dist_transform(cx.get(out.rows, out.cols), mask.data(), out.data(), out.rows, out.cols, nullptr));
    return out;
}

// ---- HistologicalEntities --------------------------------------------------------
class HistologicalEntities {
  public:
    static const int BACKGROUND = NSG_BACKGROUND;
    static const int BACKGROUND_LIKELY = NSG_BACKGROUND_LIKELY;
    static const int NO_CANDIDATES_LEFT = NSG_NO_CANDIDATES_LEFT;
    static const int INVALID_IMAGE = NSG_INVALID_IMAGE;
    static const int SUCCESS = NSG_SUCCESS;
    static const int CONTINUE = NSG_CONTINUE;
    static const int RUNTIME_FAILED = NSG_RUNTIME_FAILED;

    // segmentNuclei(img, output, compcount, bbox, ...) on a host BGR tile:
    // output = int32 labels (background -1, label = minimum raster index);
    // bbox = malloc'd int[5 * compcount] (label, minx, maxx, miny, maxy arrays)
    static int segmentNuclei(const HostImage<uint8_t> &img, HostImage<int32_t> &output, int &compcount, int *&bbox,
                             unsigned char blue = 220, unsigned char green = 220, unsigned char red = 220,
                             double T1 = 5.0, double T2 = 4.0, unsigned char G1 = 80, int minSize = 11,
                             int maxSize = 1000, unsigned char G2 = 45, int minSizePl = 30, int minSizeSeg = 21,
                             int maxSizeSeg = 1000, int fillHolesConnectivity = 4, int reconConnectivity = 8,
                             int watershedConnectivity = 8) {
        compcount = 0;
        bbox = nullptr;
        if (img.empty()) return INVALID_IMAGE;
        if (img.channels != 3) throw Error(NSG_ERR_ARG, "segmentNuclei: a 3-channel BGR tile");
        const nsg_seg_params p = params(blue, green, red, T1, T2, G1, minSize, maxSize, G2, minSizePl, minSizeSeg,
                                        maxSizeSeg, fillHolesConnectivity, reconConnectivity, watershedConnectivity);
        output = HostImage<int32_t>(img.rows, img.cols);
        auto &cx = detail::ctx();
        int32_t *b = nullptr;
        const int st = nsg_segment_nuclei_host(cx.get(img.rows, img.cols), img.data(), img.rows, img.cols, &p,
                                               output.data(), nullptr, &compcount, &b, nullptr);
        cx.check(st);
        bbox = b;
        return st;
    }
    // the mask overload (HistologicalEntities.cpp:600-664): the final uint8 mask
    static int segmentNuclei(const HostImage<uint8_t> &img, HostImage<uint8_t> &mask, unsigned char blue = 220,
                             unsigned char green = 220, unsigned char red = 220, double T1 = 5.0, double T2 = 4.0,
                             unsigned char G1 = 80, int minSize = 11, int maxSize = 1000, unsigned char G2 = 45,
                             int minSizePl = 30, int minSizeSeg = 21, int maxSizeSeg = 1000,
                             int fillHolesConnectivity = 4, int reconConnectivity = 8, int watershedConnectivity = 8) {
        if (img.empty()) return INVALID_IMAGE;
        if (img.channels != 3) throw Error(NSG_ERR_ARG, "segmentNuclei: a 3-channel BGR tile");
        const nsg_seg_params p = params(blue, green, red, T1, T2, G1, minSize, maxSize, G2, minSizePl, minSizeSeg,
                                        maxSizeSeg, fillHolesConnectivity, reconConnectivity, watershedConnectivity);
        mask = HostImage<uint8_t>(img.rows, img.cols);
        auto &cx = detail::ctx();
        const int st = nsg_segment_nuclei_host(cx.get(img.rows, img.cols), img.data(), img.rows, img.cols, &p, nullptr,
                                               mask.data(), nullptr, nullptr, nullptr);
        cx.check(st);
        return st;
    }
    // the same pipeline on a device-resident tile (the reference's GPU form,
    // nscale::gpu::HistologicalEntities::segmentNuclei, HistologicalEntities.h:83-91)
    static int segmentNuclei(const DeviceImage<uint8_t> &img, DeviceImage<int32_t> &output, int &compcount, int *&bbox,
                             const nsg_seg_params *p = nullptr) {
        compcount = 0;
        bbox = nullptr;
        if (img.empty()) return INVALID_IMAGE;
        output = DeviceImage<int32_t>(img.rows, img.cols);
        auto &cx = detail::ctx();
        int32_t *b = nullptr;
        const int st = nsg_segment_nuclei(cx.get(img.rows, img.cols), img.data(), img.rows, img.cols, 0, p,
                                          output.data(), nullptr, &compcount, &b, nullptr);
        cx.check(st);
        bbox = b;
        return st;
    }
    static DeviceImage<uint8_t> getBackground(const DeviceImage<uint8_t> &img, unsigned char blue = 220,
                                              unsigned char green = 220, unsigned char red = 220) {
        DeviceImage<uint8_t> out(img.rows, img.cols);
        auto &cx = detail::ctx();
        cx.check(nsg_get_background(cx.get(img.rows, img.cols), img.data(), img.rows, img.cols, blue, green, red,
                                    out.data(), nullptr, nullptr));
        return out;
    }
    static DeviceImage<uint8_t> getRBC(const DeviceImage<uint8_t> &img, double T1 = 5.0, double T2 = 4.0) {
        DeviceImage<uint8_t> out(img.rows, img.cols);
        auto &cx = detail::ctx();
        cx.check(nsg_get_rbc(cx.get(img.rows, img.cols), img.data(), img.rows, img.cols, T1, T2, out.data(), nullptr));
        return out;
    }

  private:
    static nsg_seg_params params(unsigned char blue, unsigned char green, unsigned char red, double T1, double T2,
                                 unsigned char G1, int minSize, int maxSize, unsigned char G2, int minSizePl,
                                 int minSizeSeg, int maxSizeSeg, int fill, int recon, int ws) {
        nsg_seg_params p;
        p.blue = blue, p.green = green, p.red = red, p.T1 = T1, p.T2 = T2, p.G1 = G1, p.minSize = minSize;
        p.maxSize = maxSize, p.G2 = G2, p.minSizePl = minSizePl, p.minSizeSeg = minSizeSeg, p.maxSizeSeg = maxSizeSeg;
        p.fillHolesConnectivity = fill, p.reconConnectivity = recon, p.watershedConnectivity = ws;
        return p;
    }
};

}  // namespace nscale

#endif
