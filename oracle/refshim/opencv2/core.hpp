// ORACLE (test infrastructure only): project-written stand-in for the parts of OpenCV's core module
// that the reference's SuBSENSE / PAWCS path uses, so that the reference's own sources compile
// without OpenCV (which is not installed). Written from OpenCV's documented semantics (types, Mat
// header/refcount semantics, saturate_cast rounding, element-wise ops); the image operations use the
// same definitions as the C restatement of the oracle (oracle/common.h). Parity of these definitions
// with a real OpenCV build is unpinned. Only 2-D matrices are supported.
#pragma once

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

typedef unsigned char uchar;
typedef signed char schar;
typedef unsigned short ushort;

#define CV_CN_SHIFT 3
#define CV_DEPTH_MAX (1 << CV_CN_SHIFT)
#define CV_MAT_DEPTH_MASK (CV_DEPTH_MAX - 1)
#define CV_MAT_DEPTH(flags) ((flags)&CV_MAT_DEPTH_MASK)
#define CV_MAKETYPE(depth, cn) (CV_MAT_DEPTH(depth) + (((cn)-1) << CV_CN_SHIFT))
#define CV_MAT_CN_MASK ((512 - 1) << CV_CN_SHIFT)
#define CV_MAT_CN(flags) ((((flags)&CV_MAT_CN_MASK) >> CV_CN_SHIFT) + 1)
#define CV_MAT_TYPE_MASK (CV_DEPTH_MAX * 512 - 1)
#define CV_MAT_TYPE(flags) ((flags)&CV_MAT_TYPE_MASK)
#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_8UC(n) CV_MAKETYPE(CV_8U, (n))
#define CV_8UC1 CV_8UC(1)
#define CV_8UC2 CV_8UC(2)
#define CV_8UC3 CV_8UC(3)
#define CV_8UC4 CV_8UC(4)
#define CV_16UC(n) CV_MAKETYPE(CV_16U, (n))
#define CV_16UC1 CV_16UC(1)
#define CV_16UC3 CV_16UC(3)
#define CV_16UC4 CV_16UC(4)
#define CV_16SC(n) CV_MAKETYPE(CV_16S, (n))
#define CV_32SC(n) CV_MAKETYPE(CV_32S, (n))
#define CV_32SC1 CV_32SC(1)
#define CV_32FC(n) CV_MAKETYPE(CV_32F, (n))
#define CV_32FC1 CV_32FC(1)
#define CV_32FC3 CV_32FC(3)
#define CV_64FC(n) CV_MAKETYPE(CV_64F, (n))
#define CV_64FC1 CV_64FC(1)

namespace cv {

inline size_t depth_bytes(int depth) {
    static const size_t b[8] = {1, 1, 2, 2, 4, 4, 8, 0};
    return b[depth & 7];
}

// ---- saturate_cast: integer targets round to nearest, ties to even (cvRound), then clamp ----
template <typename T>
inline T saturate_cast_i(long long v) {
    const long long lo = (long long)std::numeric_limits<T>::min(), hi = (long long)std::numeric_limits<T>::max();
    return (T)(v < lo ? lo : v > hi ? hi : v);
}
template <typename T, typename S>
inline T saturate_cast(S v) {
    if (std::is_integral<T>::value) {
        if (std::is_floating_point<S>::value) {
            return saturate_cast_i<T>((long long)std::nearbyint((double)v));
        }
        return saturate_cast_i<T>((long long)v);
    }
    return (T)v;
}

// ---- small value types ----
template <typename T>
struct Point_ {
    T x, y;
    Point_() : x(0), y(0) {}
    Point_(T x_, T y_) : x(x_), y(y_) {}
    template <typename U>
    operator Point_<U>() const {
        return Point_<U>((U)x, (U)y);
    }
};
typedef Point_<int> Point2i;
typedef Point_<float> Point2f;
typedef Point2i Point;

template <typename T>
struct Size_ {
    T width, height;
    Size_() : width(0), height(0) {}
    Size_(T w, T h) : width(w), height(h) {}
    T area() const { return width * height; }
    bool empty() const { return width <= 0 || height <= 0; }
};
template <typename T>
inline bool operator==(const Size_<T>& a, const Size_<T>& b) {
    return a.width == b.width && a.height == b.height;
}
template <typename T>
inline bool operator!=(const Size_<T>& a, const Size_<T>& b) {
    return !(a == b);
}
typedef Size_<int> Size2i;
typedef Size2i Size;

template <typename T>
struct Rect_ {
    T x, y, width, height;
    Rect_() : x(0), y(0), width(0), height(0) {}
    Rect_(T x_, T y_, T w, T h) : x(x_), y(y_), width(w), height(h) {}
    T area() const { return width * height; }
};
typedef Rect_<int> Rect;

struct Range {
    int start, end;
    Range() : start(0), end(0) {}
    Range(int s, int e) : start(s), end(e) {}
    static Range all() { return Range(INT_MIN, INT_MAX); }
};

template <typename T, int n>
struct Vec {
    T val[n];
    Vec() {
        for (int i = 0; i < n; ++i) val[i] = T(0);
    }
    Vec(T v0, T v1, T v2) {
        static_assert(n >= 3, "three values");
        for (int i = 0; i < n; ++i) val[i] = T(0);
        val[0] = v0;
        val[1] = v1;
        val[2] = v2;
    }
    T& operator[](int i) { return val[i]; }
    const T& operator[](int i) const { return val[i]; }
};
typedef Vec<uchar, 3> Vec3b;
typedef Vec<float, 3> Vec3f;

template <typename T>
struct Scalar_ : Vec<T, 4> {
    Scalar_() {}
    Scalar_(T v0, T v1 = 0, T v2 = 0, T v3 = 0) {
        this->val[0] = v0;
        this->val[1] = v1;
        this->val[2] = v2;
        this->val[3] = v3;
    }
    static Scalar_<T> all(T v) { return Scalar_<T>(v, v, v, v); }
    template <typename U>
    operator Scalar_<U>() const {
        return Scalar_<U>(saturate_cast<U>(this->val[0]), saturate_cast<U>(this->val[1]),
                          saturate_cast<U>(this->val[2]), saturate_cast<U>(this->val[3]));
    }
};
typedef Scalar_<double> Scalar;

// ---- Mat: 2-D, refcounted data, row step in bytes ----
struct MatStep {
    size_t p[2];
    MatStep() { p[0] = p[1] = 0; }
    size_t operator[](int i) const { return p[i]; }
    operator size_t() const { return p[0]; }
};

class _InputArray;
class _OutputArray;
typedef const _InputArray& InputArray;
typedef const _OutputArray& OutputArray;
typedef OutputArray InputOutputArray;

class Mat {
public:
    int flags = 0;  // type
    int dims = 0, rows = 0, cols = 0;
    uchar* data = nullptr;
    MatStep step;
    std::shared_ptr<std::vector<uchar>> buf;  // null for user data

    Mat() {}
    Mat(int r, int c, int type) { create(r, c, type); }
    Mat(Size sz, int type) { create(sz, type); }
    Mat(int r, int c, int type, const Scalar& s) {
        create(r, c, type);
        setTo(s);
    }
    Mat(Size sz, int type, const Scalar& s) {
        create(sz, type);
        setTo(s);
    }
    // header over user data (not owned)
    Mat(int r, int c, int type, void* d, size_t stp = 0) : flags(CV_MAT_TYPE(type)), dims(2), rows(r), cols(c) {
        data = (uchar*)d;
        step.p[1] = elemSize();
        step.p[0] = stp ? stp : (size_t)c * step.p[1];
    }
    Mat(Size sz, int type, void* d, size_t stp = 0) : Mat(sz.height, sz.width, type, d, stp) {}
    // region of interest: shares the data of m
    Mat(const Mat& m, const Rect& r) : Mat(m) {
        if (r.x < 0 || r.y < 0 || r.width < 0 || r.height < 0 || r.x + r.width > m.cols || r.y + r.height > m.rows)
            throw std::runtime_error("cv::Mat ROI out of bounds");
        data = m.data + (size_t)r.y * m.step.p[0] + (size_t)r.x * m.step.p[1];
        rows = r.height;
        cols = r.width;
    }

    int type() const { return CV_MAT_TYPE(flags); }
    int depth() const { return CV_MAT_DEPTH(flags); }
    int channels() const { return CV_MAT_CN(flags); }
    size_t elemSize1() const { return depth_bytes(depth()); }
    size_t elemSize() const { return elemSize1() * (size_t)channels(); }
    Size size() const { return Size(cols, rows); }
    bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
    size_t total() const { return (size_t)rows * (size_t)cols; }
    bool isContinuous() const { return rows <= 1 || step.p[0] == (size_t)cols * elemSize(); }

    // OpenCV semantics: a no-op when the size and type already match
    void create(int r, int c, int type) {
        type = CV_MAT_TYPE(type);
        if (data && r == rows && c == cols && type == this->type()) return;
        flags = type;
        dims = 2;
        rows = r;
        cols = c;
        step.p[1] = elemSize();
        step.p[0] = (size_t)c * step.p[1];
        buf = std::make_shared<std::vector<uchar>>((size_t)r * step.p[0] + 16, (uchar)0);
        data = buf->data();
    }
    void create(Size sz, int type) { create(sz.height, sz.width, type); }
    void release() {
        buf.reset();
        data = nullptr;
        rows = cols = 0;
    }

    template <typename T>
    T* ptr(int y = 0) {
        return (T*)(data + (size_t)y * step.p[0]);
    }
    template <typename T>
    const T* ptr(int y = 0) const {
        return (const T*)(data + (size_t)y * step.p[0]);
    }
    uchar* ptr(int y = 0) { return data + (size_t)y * step.p[0]; }
    const uchar* ptr(int y = 0) const { return data + (size_t)y * step.p[0]; }
    template <typename T>
    T& at(int y, int x) {
        return *(T*)(data + (size_t)y * step.p[0] + (size_t)x * sizeof(T));
    }
    template <typename T>
    const T& at(int y, int x) const {
        return *(const T*)(data + (size_t)y * step.p[0] + (size_t)x * sizeof(T));
    }
    template <typename T>
    T& at(int i) {
        return ((T*)data)[i];
    }
    template <typename T>
    const T& at(int i) const {
        return ((const T*)data)[i];
    }
    template <typename T>
    T& at(Point p) {
        return at<T>(p.y, p.x);
    }

    Mat clone() const {
        Mat m;
        copyTo(m);
        return m;
    }
    void copyTo(Mat& dst) const {
        if (empty()) {
            dst.release();
            return;
        }
        if (dst.data == data && dst.rows == rows && dst.cols == cols && dst.type() == type()) return;
        dst.create(rows, cols, type());
        const size_t rb = (size_t)cols * elemSize();
        for (int y = 0; y < rows; ++y) std::memmove(dst.ptr(y), ptr(y), rb);
    }
    inline void copyTo(OutputArray dst) const;
    // masked copy: elements where mask != 0
    void copyTo(Mat& dst, const Mat& mask) const {
        dst.create(rows, cols, type());
        const size_t es = elemSize();
        for (int y = 0; y < rows; ++y)
            for (int x = 0; x < cols; ++x)
                if (mask.ptr(y)[x]) std::memcpy(dst.ptr(y) + x * es, ptr(y) + x * es, es);
    }
    // every element set to the scalar, converted to the element type (saturate_cast)
    Mat& setTo(const Scalar& s) {
        const int cn = channels(), d = depth();
        for (int y = 0; y < rows; ++y) {
            uchar* row = ptr(y);
            for (int x = 0; x < cols; ++x)
                for (int c = 0; c < cn; ++c) {
                    const double v = s.val[c < 4 ? c : 3];
                    uchar* e = row + ((size_t)x * cn + c) * elemSize1();
                    switch (d) {
                        case CV_8U: *(uchar*)e = saturate_cast<uchar>(v); break;
                        case CV_8S: *(schar*)e = saturate_cast<schar>(v); break;
                        case CV_16U: *(ushort*)e = saturate_cast<ushort>(v); break;
                        case CV_16S: *(short*)e = saturate_cast<short>(v); break;
                        case CV_32S: *(int*)e = saturate_cast<int>(v); break;
                        case CV_32F: *(float*)e = (float)v; break;
                        default: *(double*)e = v; break;
                    }
                }
        }
        return *this;
    }
    template <typename T>
    Mat& operator=(const Scalar_<T>& s) {
        return setTo(Scalar((double)s.val[0], (double)s.val[1], (double)s.val[2], (double)s.val[3]));
    }
    Mat& operator=(const Mat&) = default;

    // dst = saturate_cast<rtype>(src*alpha + beta), element-wise in double
    inline void convertTo(OutputArray dst, int rtype, double alpha = 1, double beta = 0) const;
    void convertTo(Mat& dst, int rtype, double alpha = 1, double beta = 0) const {
        const int cn = channels();
        const int dd = rtype < 0 ? depth() : CV_MAT_DEPTH(rtype);
        Mat out(rows, cols, CV_MAKETYPE(dd, cn));
        for (int y = 0; y < rows; ++y)
            for (int i = 0; i < cols * cn; ++i) {
                const double v = get_d(y, i) * alpha + beta;
                out.put_d(y, i, v);
            }
        dst = out;
    }

    static Mat zeros(Size sz, int type) { return Mat(sz, type, Scalar(0)); }
    static Mat zeros(int r, int c, int type) { return Mat(r, c, type, Scalar(0)); }

    // element i of row y (channels interleaved) as double / stored with conversion
    double get_d(int y, int i) const {
        const uchar* e = ptr(y) + (size_t)i * elemSize1();
        switch (depth()) {
            case CV_8U: return *(const uchar*)e;
            case CV_8S: return *(const schar*)e;
            case CV_16U: return *(const ushort*)e;
            case CV_16S: return *(const short*)e;
            case CV_32S: return *(const int*)e;
            case CV_32F: return *(const float*)e;
            default: return *(const double*)e;
        }
    }
    void put_d(int y, int i, double v) {
        uchar* e = ptr(y) + (size_t)i * elemSize1();
        switch (depth()) {
            case CV_8U: *(uchar*)e = saturate_cast<uchar>(v); break;
            case CV_8S: *(schar*)e = saturate_cast<schar>(v); break;
            case CV_16U: *(ushort*)e = saturate_cast<ushort>(v); break;
            case CV_16S: *(short*)e = saturate_cast<short>(v); break;
            case CV_32S: *(int*)e = saturate_cast<int>(v); break;
            case CV_32F: *(float*)e = (float)v; break;
            default: *(double*)e = v; break;
        }
    }
};

template <typename T>
class Mat_ : public Mat {
public:
    Mat_() {}
    Mat_(const Mat& m) : Mat(m) {}
};

// fixed-size matrix (declared for the reference's utils headers; not used on the path)
template <typename T, int m, int n>
struct Matx {
    T val[m * n];
};

double norm(InputArray src, int normType);

// ---- InputArray / OutputArray: references to a Mat ----
class _InputArray {
public:
    _InputArray() : m_(nullptr) {}
    _InputArray(const Mat& m) : m_(&m) {}
    Mat getMat() const { return m_ ? *m_ : Mat(); }
    bool empty() const { return !m_ || m_->empty(); }
    Size size() const { return m_ ? m_->size() : Size(); }
    int type() const { return m_ ? m_->type() : 0; }

protected:
    const Mat* m_;
};

class _OutputArray : public _InputArray {
public:
    _OutputArray(Mat& m) : _InputArray(m) {}
    // a temporary header (a region of interest) written through
    _OutputArray(const Mat& m) : _InputArray(m) {}
    void create(Size sz, int type) const { mat().create(sz, type); }
    void create(int r, int c, int type) const { mat().create(r, c, type); }
    Mat& getMatRef() const { return mat(); }
    Mat getMat() const { return mat(); }
    void assign(const Mat& m) const { mat() = m; }

private:
    Mat& mat() const { return *const_cast<Mat*>(m_); }
};

inline const _InputArray& noArray() {
    static _InputArray none;
    return none;
}

inline void Mat::copyTo(OutputArray dst) const {
    Mat& d = dst.getMatRef();
    copyTo(d);
}
inline void Mat::convertTo(OutputArray dst, int rtype, double alpha, double beta) const {
    Mat& d = dst.getMatRef();
    convertTo(d, rtype, alpha, beta);
}

// ---- element-wise comparisons and scaling (evaluated at once; 255 where true) ----
template <typename F>
inline Mat cmp_scalar(const Mat& a, double s, F f) {
    Mat out(a.rows, a.cols, CV_8UC(a.channels()));
    for (int y = 0; y < a.rows; ++y)
        for (int i = 0; i < a.cols * a.channels(); ++i) out.ptr(y)[i] = f(a.get_d(y, i), s) ? 255 : 0;
    return out;
}
inline Mat operator<(const Mat& a, double s) { return cmp_scalar(a, s, [](double x, double v) { return x < v; }); }
inline Mat operator>(const Mat& a, double s) { return cmp_scalar(a, s, [](double x, double v) { return x > v; }); }
inline Mat operator==(const Mat& a, double s) { return cmp_scalar(a, s, [](double x, double v) { return x == v; }); }
inline Mat operator!=(const Mat& a, const Mat& b) {
    Mat out(a.rows, a.cols, CV_8UC(a.channels()));
    for (int y = 0; y < a.rows; ++y)
        for (int i = 0; i < a.cols * a.channels(); ++i) out.ptr(y)[i] = a.get_d(y, i) != b.get_d(y, i) ? 255 : 0;
    return out;
}
inline Mat operator&(const Mat& a, const Mat& b) {
    Mat out(a.rows, a.cols, a.type());
    const size_t rb = (size_t)a.cols * a.elemSize();
    for (int y = 0; y < a.rows; ++y)
        for (size_t i = 0; i < rb; ++i) out.ptr(y)[i] = a.ptr(y)[i] & b.ptr(y)[i];
    return out;
}
// A |= s: bitwise or with the scalar converted to the element type (8-bit matrices)
inline Mat& operator|=(Mat& a, double s) {
    if (a.depth() != CV_8U) throw std::runtime_error("operator|=: 8-bit matrices only");
    const uchar v = saturate_cast<uchar>(s);
    const size_t rb = (size_t)a.cols * a.elemSize();
    for (int y = 0; y < a.rows; ++y)
        for (size_t i = 0; i < rb; ++i) a.ptr(y)[i] |= v;
    return a;
}
// A / s: the scaling expression, evaluated as convertTo(same type, 1/s)
inline Mat operator/(const Mat& a, double s) {
    Mat out;
    a.convertTo(out, -1, 1.0 / s, 0.0);
    return out;
}

// ---- core functions ----
inline int countNonZero(InputArray src) {
    const Mat m = src.getMat();
    int n = 0;
    for (int y = 0; y < m.rows; ++y)
        for (int i = 0; i < m.cols * m.channels(); ++i) n += m.get_d(y, i) != 0;
    return n;
}

inline void split(const Mat& m, std::vector<Mat>& out) {
    const int cn = m.channels();
    out.assign(cn, Mat());
    for (int c = 0; c < cn; ++c) {
        out[c].create(m.rows, m.cols, CV_MAKETYPE(m.depth(), 1));
        for (int y = 0; y < m.rows; ++y)
            for (int x = 0; x < m.cols; ++x) out[c].put_d(y, x, m.get_d(y, x * cn + c));
    }
}

template <typename F>
inline void bitwise_bin(InputArray a_, InputArray b_, OutputArray d_, F f) {
    const Mat a = a_.getMat(), b = b_.getMat();
    Mat out(a.rows, a.cols, a.type());
    const size_t rb = (size_t)a.cols * a.elemSize();
    for (int y = 0; y < a.rows; ++y)
        for (size_t i = 0; i < rb; ++i) out.ptr(y)[i] = f(a.ptr(y)[i], b.ptr(y)[i]);
    Mat& d = d_.getMatRef();
    d.create(a.rows, a.cols, a.type());
    out.copyTo(d);
}
inline void bitwise_and(InputArray a, InputArray b, OutputArray d) {
    bitwise_bin(a, b, d, [](uchar x, uchar y) { return (uchar)(x & y); });
}
inline void bitwise_or(InputArray a, InputArray b, OutputArray d) {
    bitwise_bin(a, b, d, [](uchar x, uchar y) { return (uchar)(x | y); });
}
inline void bitwise_xor(InputArray a, InputArray b, OutputArray d) {
    bitwise_bin(a, b, d, [](uchar x, uchar y) { return (uchar)(x ^ y); });
}
inline void bitwise_not(InputArray a_, OutputArray d_) {
    const Mat a = a_.getMat();
    Mat out(a.rows, a.cols, a.type());
    const size_t rb = (size_t)a.cols * a.elemSize();
    for (int y = 0; y < a.rows; ++y)
        for (size_t i = 0; i < rb; ++i) out.ptr(y)[i] = (uchar)~a.ptr(y)[i];
    Mat& d = d_.getMatRef();
    d.create(a.rows, a.cols, a.type());
    out.copyTo(d);
}

// dst = src1*alpha + src2*beta + gamma. The restated case is src1 CV_32F, src2 CV_8U, dtype CV_32F:
// src2 is converted to float and the sum is taken in float with float weights, each product
// rounded separately (no fused multiply-add), as oracle/common.h add_weighted_mask.
// Two CV_8U sources with an 8-bit output: saturate(src1*alpha + src2*beta + gamma) in float, rounded
// half to even (the pairs PBAS adds, weights 0.5 and 0.5, give exact halves).
inline void addWeighted(InputArray s1_, double alpha, InputArray s2_, double beta, double gamma, OutputArray d_,
                        int dtype = -1) {
    const Mat s1 = s1_.getMat(), s2 = s2_.getMat();
    if (s1.depth() == CV_8U && s2.depth() == CV_8U && (dtype < 0 || CV_MAT_DEPTH(dtype) == CV_8U)) {
        const float fa = (float)alpha, fb = (float)beta, fg = (float)gamma;
        Mat out(s1.rows, s1.cols, s1.type());
        for (int y = 0; y < s1.rows; ++y)
            for (int i = 0; i < s1.cols * s1.channels(); ++i) {
                const float v = ((float)s1.ptr(y)[i] * fa + (float)s2.ptr(y)[i] * fb) + fg;
                const float r = std::nearbyint(v);
                out.ptr(y)[i] = (uchar)(r < 0.f ? 0.f : r > 255.f ? 255.f : r);
            }
        Mat& d = d_.getMatRef();
        d.create(s1.rows, s1.cols, s1.type());
        out.copyTo(d);
        return;
    }
    if (s1.depth() != CV_32F || (dtype >= 0 && CV_MAT_DEPTH(dtype) != CV_32F))
        throw std::runtime_error("addWeighted: only CV_32F outputs are supported");
    const float fa = (float)alpha, fb = (float)beta, fg = (float)gamma;
    Mat out(s1.rows, s1.cols, s1.type());
    for (int y = 0; y < s1.rows; ++y)
        for (int i = 0; i < s1.cols * s1.channels(); ++i) {
            const float t1 = (float)s1.get_d(y, i) * fa;
            const float t2 = (float)s2.get_d(y, i) * fb;
            out.ptr<float>(y)[i] = (t1 + t2) + fg;
        }
    Mat& d = d_.getMatRef();
    d.create(s1.rows, s1.cols, s1.type());
    out.copyTo(d);
}

// per-channel sum, accumulated in double in raster order
inline Scalar sum(InputArray src) {
    const Mat m = src.getMat();
    Scalar s(0, 0, 0, 0);
    const int cn = m.channels();
    for (int y = 0; y < m.rows; ++y)
        for (int x = 0; x < m.cols; ++x)
            for (int c = 0; c < cn && c < 4; ++c) s.val[c] += m.get_d(y, x * cn + c);
    return s;
}

inline void max(InputArray a_, InputArray b_, OutputArray d_) {
    const Mat a = a_.getMat(), b = b_.getMat();
    Mat out(a.rows, a.cols, a.type());
    for (int y = 0; y < a.rows; ++y)
        for (int i = 0; i < a.cols * a.channels(); ++i) out.put_d(y, i, std::max(a.get_d(y, i), b.get_d(y, i)));
    Mat& d = d_.getMatRef();
    d = out;
}

enum NormTypes { NORM_INF = 1, NORM_L1 = 2, NORM_L2 = 4, NORM_HAMMING = 6, NORM_MINMAX = 32 };
enum BorderTypes { BORDER_CONSTANT = 0, BORDER_REPLICATE = 1, BORDER_REFLECT = 2, BORDER_WRAP = 3, BORDER_REFLECT_101 = 4,
                   BORDER_DEFAULT = BORDER_REFLECT_101 };

// debug-display helpers the reference only calls in code compiled out here
void normalize(InputArray src, InputOutputArray dst, double alpha, double beta, int norm_type, int dtype = -1);

class Algorithm {
public:
    virtual ~Algorithm() {}
    virtual void clear() {}
    virtual bool empty() const { return false; }
};

// the reference writes log lines to a display helper's FileStorage; no display helper exists here
// (the pointer stays null), so this stream accepts and drops what it is given
class FileStorage {
public:
    template <typename T>
    FileStorage& operator<<(const T&) {
        return *this;
    }
};
class FileNode;

}  // namespace cv
