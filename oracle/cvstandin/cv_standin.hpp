// cv_standin.hpp — a minimal, header-only stand-in for the few OpenCV 2.4
// types and calls that nscale's own morphology / pixel functions use, so that
// those functions can be compiled from the nscale sources and run as a
// reference build that checks the oracle (test infrastructure only; OpenCV is not installed).
//
// Only what the compiled nscale functions touch is here: a reference-counted
// row-major Mat with ROI views, Mat_<T>, Size / Range / Rect / Scalar,
// copyMakeBorder (constant border), copyTo (with and without a mask),
// convertTo, split, countNonZero, bitwise_not and the element-wise operators
// those functions apply (|, &, comparison with a scalar, Mat / Mat, Mat -
// scalar, scalar - Mat, -Mat, Mat + scalar).  Each follows OpenCV 2.4's
// documented arithmetic for the depths used: results saturate to the
// destination depth (round half to even for floating values into integers);
// a comparison of a CV_32F array with a scalar converts the scalar to float
// first; float division is computed in double and rounded to float (equal to
// float division, the double rounding being innocuous); negation of a float
// array is the scale path v * -1 + 0.  Comparisons give 255 / 0 CV_8U masks.
//
// The image-processing calls of the path: erode / dilate (minimum / maximum
// over the structuring element's support, samples outside the image
// ignored: OpenCV's default constant border is neutral for both),
// getStructuringElement(MORPH_ELLIPSE) (OpenCV 2.4's ellipse rows) and
// floodFill with FLOODFILL_FIXED_RANGE | FLOODFILL_MASK_ONLY (the seed's
// equal-valued region, 4- or 8-connected, among pixels whose mask is still 0)
// are written out here; distanceTransform (CV_DIST_L2, precise) and watershed
// call the oracle's restatements (orc_dist_transform, orc_cv_watershed), so
// that what this stand-in lets the nscale code check is nscale's own logic
// around those two calls.
#pragma once

#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <memory>
#include <stdexcept>
#include <vector>

typedef unsigned char uchar;
typedef unsigned short ushort;

#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_CN_SHIFT 3
#define CV_MAT_DEPTH(t) ((t) & 7)
#define CV_MAKETYPE(depth, cn) ((depth) + (((cn) - 1) << CV_CN_SHIFT))
#define CV_8UC1 CV_MAKETYPE(CV_8U, 1)
#define CV_8UC3 CV_MAKETYPE(CV_8U, 3)
#define CV_32SC1 CV_MAKETYPE(CV_32S, 1)
#define CV_32FC1 CV_MAKETYPE(CV_32F, 1)

#define CV_Assert(expr)                                                           \
    do {                                                                          \
        if (!(expr)) throw std::runtime_error("CV_Assert failed: " #expr);       \
    } while (0)

namespace cv {

enum { BORDER_CONSTANT = 0 };

extern "C" {
void orc_dist_transform(const uint8_t *mask, int rows, int cols, float *out);
void orc_cv_watershed(const uint8_t *img, int32_t *mask, int rows, int cols);
}

struct Size {
    int width = 0, height = 0;
    Size() {}
    Size(int w, int h) : width(w), height(h) {}
    int area() const { return width * height; }
    Size operator+(const Size &o) const { return Size(width + o.width, height + o.height); }
    bool operator==(const Size &o) const { return width == o.width && height == o.height; }
};
struct Range {
    int start, end;
    Range(int s, int e) : start(s), end(e) {}
};
struct Rect {
    int x, y, width, height;
    Rect(int x_, int y_, int w, int h) : x(x_), y(y_), width(w), height(h) {}
};
struct Point {
    int x, y;
    Point(int x_ = 0, int y_ = 0) : x(x_), y(y_) {}
};
struct Scalar {
    double v[4];
    Scalar(double a = 0) : v{a, 0, 0, 0} {}
    Scalar(double a, double b, double c, double d = 0) : v{a, b, c, d} {}
};
template <typename T>
struct Scalar_ : Scalar {
    Scalar_(T a = 0) : Scalar((double)a) {}
};

inline int depth_size(int depth) {
    static const int s[7] = {1, 1, 2, 2, 4, 4, 8};
    return s[depth];
}

// saturate_cast: round to nearest (half to even, as cvRound) into integers
template <typename T>
inline T sat(double v) {
    if (std::numeric_limits<T>::is_integer) {
        const double r = std::nearbyint(v);
        if (r < (double)std::numeric_limits<T>::min()) return std::numeric_limits<T>::min();
        if (r > (double)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
        return (T)r;
    }
    return (T)v;
}

class Mat {
  public:
    int rows = 0, cols = 0;
    uchar *data = nullptr;
    size_t step = 0;  // bytes per row

    Mat() {}
    Mat(int r, int c, int type) { create(r, c, type); }
    Mat(Size s, int type) { create(s.height, s.width, type); }
    Mat(Size s, int type, const Scalar &v) {
        create(s.height, s.width, type);
        set_to(v.v);
    }
    // a column vector holding a copy of the elements
    explicit Mat(const std::vector<uchar> &v) {
        create((int)v.size(), 1, CV_8U);
        if (!v.empty()) memcpy(data, v.data(), v.size());
    }
    // same elements, `rows_` rows (continuous matrices only)
    Mat reshape(int cn, int rows_) const {
        CV_Assert(cn == channels() && step == (size_t)cols * elemSize());
        Mat m(*this);
        const int total = rows * cols;
        m.rows = rows_;
        m.cols = total / rows_;
        m.step = (size_t)m.cols * elemSize();
        return m;
    }
    Mat(const Mat &m, const Range &rr, const Range &cr) : Mat(m) {
        rows = rr.end - rr.start;
        cols = cr.end - cr.start;
        data = m.data + (size_t)rr.start * m.step + (size_t)cr.start * m.elemSize();
    }

    void create(int r, int c, int type) {
        if (buf_ && r == rows && c == cols && type == type_ && step == (size_t)c * depth_size(CV_MAT_DEPTH(type)) *
                                                                         channels_of(type))
            return;
        type_ = type;
        rows = r;
        cols = c;
        step = (size_t)c * elemSize();
        buf_ = std::make_shared<std::vector<uchar>>((size_t)r * step + 1, 0);
        data = buf_->data();
    }
    void create(Size s, int type) { create(s.height, s.width, type); }
    void release() {
        buf_.reset();
        data = nullptr;
        rows = cols = 0;
    }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }

    Size size() const { return Size(cols, rows); }
    int type() const { return type_; }
    int depth() const { return CV_MAT_DEPTH(type_); }
    int channels() const { return channels_of(type_); }
    size_t elemSize() const { return (size_t)depth_size(depth()) * channels(); }

    template <typename T>
    T *ptr(int y) {
        return reinterpret_cast<T *>(data + (size_t)y * step);
    }
    template <typename T>
    const T *ptr(int y) const {
        return reinterpret_cast<const T *>(data + (size_t)y * step);
    }
    uchar *ptr(int y) { return data + (size_t)y * step; }
    const uchar *ptr(int y) const { return data + (size_t)y * step; }

    Mat operator()(const Range &rr, const Range &cr) const { return Mat(*this, rr, cr); }
    Mat operator()(const Rect &r) const { return Mat(*this, Range(r.y, r.y + r.height), Range(r.x, r.x + r.width)); }

    static Mat zeros(Size s, int type) { return Mat(s, type, Scalar(0)); }
    static Mat zeros(int r, int c, int type) { return Mat(Size(c, r), type, Scalar(0)); }

    Mat clone() const {
        Mat d(size(), type_);
        for (int y = 0; y < rows; ++y) memcpy(d.ptr(y), ptr(y), (size_t)cols * elemSize());
        return d;
    }
    void copyTo(Mat &dst) const {
        if (dst.data == data && dst.rows == rows && dst.cols == cols) return;
        Mat d = clone();
        dst = d;
    }
    // copy where mask != 0 (dst keeps its other pixels; a new dst starts at 0)
    void copyTo(Mat &dst, const Mat &mask) const {
        if (!(dst.size() == size()) || dst.type() != type_) dst = Mat::zeros(size(), type_);
        const size_t es = elemSize();
        for (int y = 0; y < rows; ++y)
            for (int x = 0; x < cols; ++x)
                if (mask.ptr<uchar>(y)[x]) memcpy(dst.ptr(y) + x * es, ptr(y) + x * es, es);
    }
    void convertTo(Mat &dst, int rtype, double alpha = 1, double beta = 0) const;

    double at_d(int y, int x) const {
        switch (depth()) {
            case CV_8U: return ptr<uchar>(y)[x];
            case CV_8S: return ptr<signed char>(y)[x];
            case CV_16U: return ptr<ushort>(y)[x];
            case CV_16S: return ptr<short>(y)[x];
            case CV_32S: return ptr<int>(y)[x];
            case CV_32F: return ptr<float>(y)[x];
            default: return ptr<double>(y)[x];
        }
    }
    void set_d(int y, int x, double v) {
        switch (depth()) {
            case CV_8U: ptr<uchar>(y)[x] = sat<uchar>(v); break;
            case CV_8S: ptr<signed char>(y)[x] = sat<signed char>(v); break;
            case CV_16U: ptr<ushort>(y)[x] = sat<ushort>(v); break;
            case CV_16S: ptr<short>(y)[x] = sat<short>(v); break;
            case CV_32S: ptr<int>(y)[x] = sat<int>(v); break;
            case CV_32F: ptr<float>(y)[x] = (float)v; break;
            default: ptr<double>(y)[x] = v;
        }
    }

  private:
    static int channels_of(int t) { return (t >> CV_CN_SHIFT) + 1; }
    void set_to(const double *v) {
        const int cn = channels();
        for (int y = 0; y < rows; ++y)
            for (int x = 0; x < cols * cn; ++x) set_d(y, x, v[x % cn]);
    }
    std::shared_ptr<std::vector<uchar>> buf_;
    int type_ = CV_8UC1;
};

template <typename T>
struct DepthOf;
template <> struct DepthOf<uchar> { enum { v = CV_8U }; };
template <> struct DepthOf<int> { enum { v = CV_32S }; };
template <> struct DepthOf<float> { enum { v = CV_32F }; };
template <> struct DepthOf<ushort> { enum { v = CV_16U }; };

template <typename T>
class Mat_ : public Mat {
  public:
    Mat_() {}
    Mat_(const Mat &m) : Mat(m) {}
    Mat_(int r, int c) : Mat(r, c, DepthOf<T>::v) {}
    explicit Mat_(Size s) : Mat(s, DepthOf<T>::v) {}
    static Mat_ zeros(Size s) { return Mat_(Mat::zeros(s, DepthOf<T>::v)); }
};

// u8 -> f32 and same-depth conversions, v * alpha + beta in the working type
// of OpenCV 2.4's cvtScale (float for a float destination, double otherwise)
inline void Mat::convertTo(Mat &dst, int rtype, double alpha, double beta) const {
    Mat d(size(), rtype < 0 ? type_ : rtype);
    const bool noscale = std::fabs(alpha - 1) < 2.220446049250313e-16 && std::fabs(beta) < 2.220446049250313e-16;
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x) {
            const double v = at_d(y, x);
            if (noscale) d.set_d(y, x, v);
            else if (d.depth() == CV_32F) d.set_d(y, x, (float)v * (float)alpha + (float)beta);
            else d.set_d(y, x, v * alpha + beta);
        }
    dst = d;
}

inline void copyMakeBorder(const Mat &src, Mat &dst, int top, int bottom, int left, int right, int border_type,
                           const Scalar &value) {
    CV_Assert(border_type == BORDER_CONSTANT);
    Mat d(Size(src.cols + left + right, src.rows + top + bottom), src.type(), value);
    const size_t es = src.elemSize();
    for (int y = 0; y < src.rows; ++y) memcpy(d.ptr(y + top) + (size_t)left * es, src.ptr(y), (size_t)src.cols * es);
    dst = d;
}

inline void split(const Mat &m, std::vector<Mat> &out) {
    const int cn = m.channels();
    out.assign(cn, Mat());
    for (int c = 0; c < cn; ++c) {
        out[c] = Mat(m.size(), CV_MAKETYPE(m.depth(), 1));
        for (int y = 0; y < m.rows; ++y)
            for (int x = 0; x < m.cols; ++x) out[c].ptr<uchar>(y)[x] = m.ptr<uchar>(y)[x * cn + c];
    }
}

inline int countNonZero(const Mat &m) {
    int n = 0;
    for (int y = 0; y < m.rows; ++y)
        for (int x = 0; x < m.cols; ++x) n += m.at_d(y, x) != 0;
    return n;
}

template <typename F>
inline Mat map1(const Mat &a, int rtype, F f) {
    Mat d(a.size(), rtype);
    for (int y = 0; y < a.rows; ++y)
        for (int x = 0; x < a.cols; ++x) d.set_d(y, x, f(a.at_d(y, x)));
    return d;
}
template <typename F>
inline Mat map2(const Mat &a, const Mat &b, F f) {
    CV_Assert(a.size() == b.size() && a.type() == b.type());
    Mat d(a.size(), a.type());
    for (int y = 0; y < a.rows; ++y)
        for (int x = 0; x < a.cols; ++x) d.set_d(y, x, f(a.at_d(y, x), b.at_d(y, x)));
    return d;
}

inline Mat operator|(const Mat &a, const Mat &b) {
    CV_Assert(a.size() == b.size() && a.type() == b.type());
    Mat d(a.size(), a.type());
    const size_t w = (size_t)a.cols * a.elemSize();
    for (int y = 0; y < a.rows; ++y)
        for (size_t i = 0; i < w; ++i) d.ptr(y)[i] = a.ptr(y)[i] | b.ptr(y)[i];
    return d;
}
inline Mat operator&(const Mat &a, const Mat &b) {
    CV_Assert(a.size() == b.size() && a.type() == b.type());
    Mat d(a.size(), a.type());
    const size_t w = (size_t)a.cols * a.elemSize();
    for (int y = 0; y < a.rows; ++y)
        for (size_t i = 0; i < w; ++i) d.ptr(y)[i] = a.ptr(y)[i] & b.ptr(y)[i];
    return d;
}
inline void bitwise_not(const Mat &a, Mat &dst) {
    Mat d(a.size(), a.type());
    const size_t w = (size_t)a.cols * a.elemSize();
    for (int y = 0; y < a.rows; ++y)
        for (size_t i = 0; i < w; ++i) d.ptr(y)[i] = (uchar)~a.ptr(y)[i];
    dst = d;
}

// comparison with a scalar: 255 where true
inline Mat operator>(const Mat &a, double s) {
    const bool f32 = a.depth() == CV_32F;
    const float sf = (float)s;
    return map1(a, CV_8U, [&](double v) { return (f32 ? ((float)v > sf) : (v > s)) ? 255.0 : 0.0; });
}

inline Mat operator/(const Mat &a, const Mat &b) {
    CV_Assert(a.depth() == CV_32F);
    return map2(a, b, [](double x, double y) { return y != 0 ? (double)(float)(x * 1.0 / y) : 0.0; });
}

// Mat - scalar and scalar - Mat: the scalar in the array's depth, the
// difference saturated (float arrays: float arithmetic)
inline Mat operator-(const Mat &a, double s) {
    if (a.depth() == CV_32F) {
        const float sf = (float)s;
        return map1(a, a.type(), [&](double v) { return (double)((float)v - sf); });
    }
    return map1(a, a.type(), [&](double v) { return v - s; });
}
inline Mat operator-(double s, const Mat &a) {
    if (a.depth() == CV_32F) {
        const float sf = (float)s;
        return map1(a, a.type(), [&](double v) { return (double)(sf - (float)v); });
    }
    return map1(a, a.type(), [&](double v) { return s - v; });
}
inline Mat operator-(const Mat &a) {
    if (a.depth() == CV_32F) return map1(a, a.type(), [](double v) { return (double)((float)v * -1.0f + 0.0f); });
    return map1(a, a.type(), [](double v) { return -v; });
}
// int arrays wrap like the 32-bit addition OpenCV 2.4 performs
inline Mat operator+(const Mat &a, int s) {
    if (a.depth() == CV_32S) {
        Mat d(a.size(), a.type());
        for (int y = 0; y < a.rows; ++y)
            for (int x = 0; x < a.cols; ++x)
                d.ptr<int>(y)[x] = (int)((uint32_t)a.ptr<int>(y)[x] + (uint32_t)s);
        return d;
    }
    return map1(a, a.type(), [&](double v) { return v + s; });
}

// element-wise comparisons: 255 where true
template <typename P>
inline Mat cmp_scalar(const Mat &a, double s, P pred) {
    const bool f32 = a.depth() == CV_32F;
    const double sv = f32 ? (double)(float)s : s;
    return map1(a, CV_8U, [&](double v) { return pred(v, sv) ? 255.0 : 0.0; });
}
inline Mat operator>=(const Mat &a, double s) { return cmp_scalar(a, s, [](double v, double t) { return v >= t; }); }
inline Mat operator==(const Mat &a, double s) { return cmp_scalar(a, s, [](double v, double t) { return v == t; }); }
inline Mat operator<(const Mat &a, const Mat &b) {
    CV_Assert(a.size() == b.size() && a.type() == b.type());
    Mat d(a.size(), CV_8U);
    for (int y = 0; y < a.rows; ++y)
        for (int x = 0; x < a.cols; ++x) d.ptr<uchar>(y)[x] = a.at_d(y, x) < b.at_d(y, x) ? 255 : 0;
    return d;
}
// Mat - Mat, saturated to the depth
inline Mat operator-(const Mat &a, const Mat &b) {
    if (a.depth() == CV_32F) return map2(a, b, [](double x, double y) { return (double)((float)x - (float)y); });
    return map2(a, b, [](double x, double y) { return x - y; });
}

inline void minMaxLoc(const Mat &a, double *mn, double *mx) {
    double lo = std::numeric_limits<double>::max(), hi = -lo;
    for (int y = 0; y < a.rows; ++y)
        for (int x = 0; x < a.cols; ++x) {
            lo = std::min(lo, a.at_d(y, x));
            hi = std::max(hi, a.at_d(y, x));
        }
    if (mn) *mn = lo;
    if (mx) *mx = hi;
}

enum { MORPH_RECT = 0, MORPH_CROSS = 1, MORPH_ELLIPSE = 2 };
// OpenCV 2.4 getStructuringElement(MORPH_ELLIPSE, size): row i covers
// columns c - dx .. c + dx with dx = round(c * sqrt((r^2 - dy^2) / r^2))
inline Mat getStructuringElement(int shape, Size ks) {
    CV_Assert(shape == MORPH_ELLIPSE);
    Mat k = Mat::zeros(ks, CV_8U);
    const int r = ks.height / 2, c = ks.width / 2;
    const double inv_r2 = r ? 1.0 / ((double)r * r) : 0;
    for (int i = 0; i < ks.height; ++i) {
        const int dy = i - r;
        int j1 = 0, j2 = 0;
        if (std::abs(dy) <= r) {
            const int dx = sat<int>(c * std::sqrt((r * r - dy * dy) * inv_r2));
            j1 = std::max(c - dx, 0);
            j2 = std::min(c + dx + 1, ks.width);
        }
        for (int j = j1; j < j2; ++j) k.ptr<uchar>(i)[j] = 1;
    }
    return k;
}

// min (erode) / max (dilate) over the kernel's non-zero support, anchored at
// its centre; samples outside the image do not take part
inline Mat morph_ext(const Mat &src, const Mat &kernel, bool is_max) {
    CV_Assert(src.depth() == CV_8U && src.channels() == 1);
    const int ay = kernel.rows / 2, ax = kernel.cols / 2;
    Mat d(src.size(), src.type());
    for (int y = 0; y < src.rows; ++y)
        for (int x = 0; x < src.cols; ++x) {
            int v = is_max ? 0 : 255;
            for (int i = 0; i < kernel.rows; ++i) {
                const int yy = y + i - ay;
                if (yy < 0 || yy >= src.rows) continue;
                for (int j = 0; j < kernel.cols; ++j) {
                    const int xx = x + j - ax;
                    if (xx < 0 || xx >= src.cols || !kernel.ptr<uchar>(i)[j]) continue;
                    const int s = src.ptr<uchar>(yy)[xx];
                    v = is_max ? std::max(v, s) : std::min(v, s);
                }
            }
            d.ptr<uchar>(y)[x] = (uchar)v;
        }
    return d;
}
inline void erode(const Mat &src, Mat &dst, const Mat &kernel) { dst = morph_ext(src, kernel, false); }
inline void dilate(const Mat &src, Mat &dst, const Mat &kernel) { dst = morph_ext(src, kernel, true); }

enum { CV_DIST_L2 = 2, CV_DIST_MASK_PRECISE = 0 };
inline void distanceTransform(const Mat &src, Mat &dst, int type, int mask_size) {
    CV_Assert(type == CV_DIST_L2 && mask_size == CV_DIST_MASK_PRECISE && src.depth() == CV_8U);
    Mat s = src.clone();
    Mat d(src.size(), CV_32F);
    orc_dist_transform(s.data, s.rows, s.cols, (float *)d.data);
    dst = d;
}

inline void watershed(const Mat &image, Mat &markers) {
    CV_Assert(image.type() == CV_8UC3 && markers.depth() == CV_32S && image.size() == markers.size());
    Mat img = image.clone();
    Mat m = markers.clone();
    orc_cv_watershed(img.data, (int32_t *)m.data, m.rows, m.cols);
    for (int y = 0; y < m.rows; ++y) memcpy(markers.ptr(y), m.ptr(y), (size_t)m.cols * 4);
}

enum { FLOODFILL_FIXED_RANGE = 1 << 16, FLOODFILL_MASK_ONLY = 1 << 17 };
// floodFill(image, mask, seed, newVal, rect, loDiff, upDiff, flags) for the
// fixed-range, mask-only form: every pixel connected to the seed (4 or 8 by
// flags & 255) through pixels whose value lies in [seed - lo, seed + up] and
// whose mask (one pixel larger on each side) is 0 gets mask value
// (flags >> 8) & 255 (1 when that is 0).  The image is not changed.
inline int floodFill(Mat &image, Mat &mask, Point seed, Scalar newVal, Rect *rect, Scalar lo, Scalar up, int flags) {
    (void)newVal;
    CV_Assert((flags & FLOODFILL_FIXED_RANGE) && (flags & FLOODFILL_MASK_ONLY) && image.channels() == 1);
    const int conn = flags & 255;
    int mval = (flags >> 8) & 255;
    if (mval == 0) mval = 1;
    CV_Assert(mask.rows == image.rows + 2 && mask.cols == image.cols + 2);
    const double s0 = image.at_d(seed.y, seed.x);
    const double vlo = s0 - lo.v[0], vhi = s0 + up.v[0];
    std::vector<Point> st;
    int n = 0, x0 = seed.x, x1 = seed.x, y0 = seed.y, y1 = seed.y;
    if (mask.ptr<uchar>(seed.y + 1)[seed.x + 1]) return 0;
    mask.ptr<uchar>(seed.y + 1)[seed.x + 1] = (uchar)mval;
    st.push_back(seed);
    while (!st.empty()) {
        const Point p = st.back();
        st.pop_back();
        ++n;
        x0 = std::min(x0, p.x), x1 = std::max(x1, p.x), y0 = std::min(y0, p.y), y1 = std::max(y1, p.y);
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                if ((dx == 0 && dy == 0) || (conn == 4 && dx != 0 && dy != 0)) continue;
                const int qx = p.x + dx, qy = p.y + dy;
                if (qx < 0 || qy < 0 || qx >= image.cols || qy >= image.rows) continue;
                uchar &mk = mask.ptr<uchar>(qy + 1)[qx + 1];
                if (mk) continue;
                const double v = image.at_d(qy, qx);
                if (v < vlo || v > vhi) continue;
                mk = (uchar)mval;
                st.push_back(Point(qx, qy));
            }
    }
    if (rect) *rect = Rect(x0, y0, x1 - x0 + 1, y1 - y0 + 1);
    return n;
}

}  // namespace cv
