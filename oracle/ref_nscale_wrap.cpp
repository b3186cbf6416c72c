// ref_nscale_wrap.cpp — C entry points over nscale's OWN CPU functions on the
// segmentNuclei path, compiled from the nscale sources (test infrastructure
// only: it checks the oracle; nothing in libnsg.so uses it).
//
// The function definitions come from oracle/_ref/ref_nscale_extract.inc,
// which ref_extract.py writes at build time from the nscale tree:
//   PixelOperations::invert<T>          PixelOperations.cpp:21-43
//   propagate<T>, imreconstruct<T>       MorphologicOperations.cpp:430-440, 1730-1903
//   propagateBinary<T>, imreconstructBinary<T>  :2745-2751, 2768-2909
//   imfillHoles<T>, bwselect<T>          :2939-3006, 3009-3031
//   bwlabel2, bwareaopen2                :3092-3117, 3281-3314 (over ConnComponents.cpp)
//   imhmin<T>                            :3342-3364
//   NeighborOperations::border<T>        NeighborOperations.cpp:17-44
//   localMaxima<T>, localMinima<T>       :3763-3845
//   watershed2                           :3717-3760
//   morphOpen<T>                         :3848-3882
//   HistologicalEntities::getRBC / getBackground (vector<Mat> overloads)
//                                        HistologicalEntities.cpp:33-81, 93-109
//   plFindNucleusCandidates, plSeparateNuclei, segmentNuclei (labels and
//   mask overloads)                      :115-304, 308-449, 473-598, 600-664
// They are compiled against cvstandin/cv_standin.hpp instead of OpenCV (not
// installed), whose distanceTransform and watershed are the oracle's
// restatements (nsg_oracle.c is linked in): what this library checks is
// nscale's own code around those two OpenCV calls, i.e. every stage's order,
// parameters, padding and thresholds.  The class declarations below carry
// only the members those definitions need, with the reference's signatures
// (PixelOperations.h:37-58, NeighborOperations.h:19-27,
// HistologicalEntities.h:29-69); the logger is never given (NULL).
#include <float.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <iostream>
#include <limits>
#include <queue>
#include <vector>

#include "../cvstandin/cv_standin.hpp"
#include "ConnComponents.h"
#include "TypeUtils.h"

namespace cci {
namespace common {
namespace event {
inline long long timestampInUS() { return 0; }
}  // namespace event
}  // namespace common
}  // namespace cci

namespace cciutils {
class SimpleCSVLogger {
  public:
    template <typename... A>
    void logTimeSinceLastLog(A...) {}
    template <typename... A>
    void log(A...) {}
    template <typename... A>
    void logT(A...) {}
    template <typename... A>
    void logT0(A...) {}
    template <typename... A>
    void logStart(A...) {}
    template <typename... A>
    void endSession(A...) {}
};
namespace cv {
class IntermediateResultHandler {
  public:
    virtual ~IntermediateResultHandler() {}
    virtual void saveIntermediate(const ::cv::Mat &, int) {}
};
}  // namespace cv
}  // namespace cciutils

namespace nscale {

using namespace cv;
using namespace std;

class PixelOperations {
  public:
    template <typename T>
    static Mat invert(const Mat &img);
};

class NeighborOperations {
  public:
    template <typename T>
    static Mat border(Mat &img, T background);
};

class HistologicalEntities {
  public:
    static const int BACKGROUND = 1;
    static const int BACKGROUND_LIKELY = 2;
    static const int NO_CANDIDATES_LEFT = 3;
    static const int INVALID_IMAGE = -1;
    static const int SUCCESS = 0;
    static const int CONTINUE = 4;
    static const int RUNTIME_FAILED = -2;
    static int segmentNuclei(const Mat &img, Mat &mask, int &compcount, int *&bbox, unsigned char blue = 220,
                             unsigned char green = 220, unsigned char red = 220, double T1 = 5.0, double T2 = 4.0,
                             unsigned char G1 = 80, int minSize = 11, int maxSize = 1000, unsigned char G2 = 45,
                             int minSizePl = 30, int minSizeSeg = 21, int maxSizeSeg = 1000,
                             int fillHolesConnectivity = 4, int reconConnectivity = 8, int watershedConnectivity = 8,
                             ::cciutils::SimpleCSVLogger *logger = NULL,
                             ::cciutils::cv::IntermediateResultHandler *iresHandler = NULL);
    static int segmentNuclei(const Mat &img, Mat &mask, unsigned char blue = 220, unsigned char green = 220,
                             unsigned char red = 220, double T1 = 5.0, double T2 = 4.0, unsigned char G1 = 80,
                             int minSize = 11, int maxSize = 1000, unsigned char G2 = 45, int minSizePl = 30,
                             int minSizeSeg = 21, int maxSizeSeg = 1000, int fillHolesConnectivity = 4,
                             int reconConnectivity = 8, int watershedConnectivity = 8,
                             ::cciutils::SimpleCSVLogger *logger = NULL,
                             ::cciutils::cv::IntermediateResultHandler *iresHandler = NULL);
    static int plFindNucleusCandidates(const Mat &img, Mat &seg_norbc, unsigned char blue = 220,
                                       unsigned char green = 220, unsigned char red = 220, double T1 = 5.0,
                                       double T2 = 4.0, unsigned char G1 = 80, int minSize = 11, int maxSize = 1000,
                                       unsigned char G2 = 45, int fillHolesConnectivity = 4,
                                       int reconConnectivity = 8, ::cciutils::SimpleCSVLogger *logger = NULL,
                                       ::cciutils::cv::IntermediateResultHandler *iresHandler = NULL);
    static int plSeparateNuclei(const Mat &img, const Mat &seg_open, Mat &seg_nonoverlap, int minSizePl = 30,
                                int watershedConnectivity = 8, ::cciutils::SimpleCSVLogger *logger = NULL,
                                ::cciutils::cv::IntermediateResultHandler *iresHandler = NULL);
    static Mat getRBC(const std::vector<Mat> &bgr, double T1, double T2,
                      ::cciutils::SimpleCSVLogger *logger = NULL,
                      ::cciutils::cv::IntermediateResultHandler *iresHandler = NULL);
    static Mat getBackground(const std::vector<Mat> &bgr, unsigned char blue, unsigned char green, unsigned char red,
                             ::cciutils::SimpleCSVLogger *logger = NULL,
                             ::cciutils::cv::IntermediateResultHandler *iresHandler = NULL);
};

template <typename T>
Mat imreconstruct(const Mat &seeds, const Mat &image, int connectivity);
template <typename T>
Mat imreconstructBinary(const Mat &seeds, const Mat &image, int connectivity);
template <typename T>
Mat bwselect(const Mat &binaryImage, const Mat &seeds, int connectivity);
template <typename T>
Mat morphOpen(const Mat &image, const Mat &kernel);

#include "ref_nscale_extract.inc"

}  // namespace nscale

namespace {

cv::Mat in_mat(const void *p, int rows, int cols, int type) {
    cv::Mat m(rows, cols, type);
    memcpy(m.data, p, (size_t)rows * m.step);
    return m;
}
void out_mat(const cv::Mat &m, void *dst) {
    const size_t w = (size_t)m.cols * m.elemSize();
    for (int y = 0; y < m.rows; ++y) memcpy((char *)dst + (size_t)y * w, m.ptr(y), w);
}

template <typename F>
int guarded(F f) {
    try {
        f();
        return 0;
    } catch (const std::exception &e) {
        std::cerr << "ref_nscale: " << e.what() << std::endl;
        return -1;
    }
}

}  // namespace

extern "C" {

int ref_imreconstruct_u8(const uint8_t *marker, const uint8_t *mask, int rows, int cols, int conn, uint8_t *out) {
    return guarded([&] {
        out_mat(nscale::imreconstruct<unsigned char>(in_mat(marker, rows, cols, CV_8U), in_mat(mask, rows, cols, CV_8U),
                                                     conn),
                out);
    });
}

int ref_imreconstruct_f32(const float *marker, const float *mask, int rows, int cols, int conn, float *out) {
    return guarded([&] {
        out_mat(nscale::imreconstruct<float>(in_mat(marker, rows, cols, CV_32F), in_mat(mask, rows, cols, CV_32F), conn),
                out);
    });
}

int ref_imreconstruct_binary_u8(const uint8_t *marker, const uint8_t *mask, int rows, int cols, int conn,
                                uint8_t *out) {
    return guarded([&] {
        out_mat(nscale::imreconstructBinary<unsigned char>(in_mat(marker, rows, cols, CV_8U),
                                                           in_mat(mask, rows, cols, CV_8U), conn),
                out);
    });
}

int ref_imfill_holes_u8(const uint8_t *img, int rows, int cols, int conn, uint8_t *out) {
    return guarded([&] {
        out_mat(nscale::imfillHoles<unsigned char>(in_mat(img, rows, cols, CV_8U), true, conn), out);
    });
}

int ref_bwselect_u8(const uint8_t *bw, const uint8_t *seeds, int rows, int cols, int conn, uint8_t *out) {
    return guarded([&] {
        out_mat(nscale::bwselect<unsigned char>(in_mat(bw, rows, cols, CV_8U), in_mat(seeds, rows, cols, CV_8U), conn),
                out);
    });
}

int ref_bwlabel2(const uint8_t *img, int rows, int cols, int conn, int32_t *out) {
    return guarded([&] { out_mat(nscale::bwlabel2(in_mat(img, rows, cols, CV_8U), conn, true), out); });
}

int ref_bwareaopen2(const uint8_t *img, int rows, int cols, int min_size, int max_size, int conn, uint8_t *out,
                    int *count) {
    return guarded([&] {
        int n = 0;
        out_mat(nscale::bwareaopen2(in_mat(img, rows, cols, CV_8U), false, true, min_size, max_size, conn, n), out);
        *count = n;
    });
}

int ref_imhmin_f32(const float *img, int rows, int cols, float h, int conn, float *out) {
    return guarded([&] { out_mat(nscale::imhmin<float>(in_mat(img, rows, cols, CV_32F), h, conn), out); });
}

// NeighborOperations::border on an int32 image (padded, as watershed2 calls
// it); rows 0 and columns 0 / cols-1 of the result are never written by the
// reference and come back as 0 here
int ref_border_i32(const int32_t *img, int rows, int cols, int32_t bg, int32_t *out) {
    return guarded([&] {
        cv::Mat m = in_mat(img, rows, cols, CV_32S);
        out_mat(nscale::NeighborOperations::border<int>(m, bg), out);
    });
}

int ref_get_rbc(const uint8_t *bgr, int rows, int cols, double T1, double T2, uint8_t *out) {
    return guarded([&] {
        std::vector<cv::Mat> ch;
        cv::split(in_mat(bgr, rows, cols, CV_8UC3), ch);
        out_mat(nscale::HistologicalEntities::getRBC(ch, T1, T2), out);
    });
}

int ref_get_background(const uint8_t *bgr, int rows, int cols, int blue, int green, int red, uint8_t *out) {
    return guarded([&] {
        std::vector<cv::Mat> ch;
        cv::split(in_mat(bgr, rows, cols, CV_8UC3), ch);
        out_mat(nscale::HistologicalEntities::getBackground(ch, (unsigned char)blue, (unsigned char)green,
                                                            (unsigned char)red),
                out);
    });
}

int ref_invert_u8(const uint8_t *in, int rows, int cols, uint8_t *out) {
    return guarded([&] { out_mat(nscale::PixelOperations::invert<unsigned char>(in_mat(in, rows, cols, CV_8U)), out); });
}
int ref_invert_i32(const int32_t *in, int rows, int cols, int32_t *out) {
    return guarded([&] { out_mat(nscale::PixelOperations::invert<int>(in_mat(in, rows, cols, CV_32S)), out); });
}
int ref_invert_f32(const float *in, int rows, int cols, float *out) {
    return guarded([&] { out_mat(nscale::PixelOperations::invert<float>(in_mat(in, rows, cols, CV_32F)), out); });
}

int ref_local_minima_f32(const float *img, int rows, int cols, int conn, uint8_t *out) {
    return guarded([&] { out_mat(nscale::localMinima<float>(in_mat(img, rows, cols, CV_32F), conn), out); });
}

int ref_morph_open_u8(const uint8_t *img, int rows, int cols, const uint8_t *se, int k, uint8_t *out) {
    return guarded([&] {
        out_mat(nscale::morphOpen<unsigned char>(in_mat(img, rows, cols, CV_8U), in_mat(se, k, k, CV_8U)), out);
    });
}

int ref_watershed2(const uint8_t *bgr, const float *img, int rows, int cols, int conn, int32_t *out) {
    return guarded([&] {
        cv::Mat_<float> f(in_mat(img, rows, cols, CV_32F));
        out_mat(nscale::watershed2(in_mat(bgr, rows, cols, CV_8UC3), f, conn), out);
    });
}

// segmentNuclei (HistologicalEntities.cpp:473-598): status; labels (when
// SUCCESS) and the reference's bounding-box output (its boundingBox call with
// bgval 0, HistologicalEntities.cpp:591) as up to `box_cap` entries of 5
// ints; then the mask overload (:600-664) on the same tile for the final mask.
int ref_segment_nuclei(const uint8_t *bgr, int rows, int cols, int blue, int green, int red, double T1, double T2,
                       int G1, int minSize, int maxSize, int G2, int minSizePl, int minSizeSeg, int maxSizeSeg,
                       int fillConn, int reconConn, int wsConn, int32_t *labels_out, uint8_t *mask_out,
                       int32_t *box_out, int box_cap, int *compcount, int *mask_status) {
    int status = -100;
    const int r = guarded([&] {
        cv::Mat img = in_mat(bgr, rows, cols, CV_8UC3);
        cv::Mat output;
        int cc = 0;
        int *bbox = NULL;
        status = nscale::HistologicalEntities::segmentNuclei(
            img, output, cc, bbox, (unsigned char)blue, (unsigned char)green, (unsigned char)red, T1, T2,
            (unsigned char)G1, minSize, maxSize, (unsigned char)G2, minSizePl, minSizeSeg, maxSizeSeg, fillConn,
            reconConn, wsConn);
        *compcount = cc;
        if (status == nscale::HistologicalEntities::SUCCESS) {
            out_mat(output, labels_out);
            for (int i = 0; i < 5 * cc && i < 5 * box_cap; ++i) box_out[i] = bbox[i];
        }
        free(bbox);
        cv::Mat mask;
        *mask_status = nscale::HistologicalEntities::segmentNuclei(
            img, mask, (unsigned char)blue, (unsigned char)green, (unsigned char)red, T1, T2, (unsigned char)G1,
            minSize, maxSize, (unsigned char)G2, minSizePl, minSizeSeg, maxSizeSeg, fillConn, reconConn, wsConn);
        if (*mask_status == nscale::HistologicalEntities::SUCCESS) out_mat(mask, mask_out);
    });
    return r == 0 ? status : -100;
}

}  // extern "C"
