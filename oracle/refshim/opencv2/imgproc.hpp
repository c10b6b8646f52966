// ORACLE (test infrastructure only): project-written stand-in for the OpenCV imgproc operations
// that the reference's SuBSENSE / PAWCS path calls. Each definition is written from OpenCV's
// documented semantics and is the one the C restatement uses (oracle/common.h, oracle/subsense.c,
// oracle/pawcs.c); parity with a real OpenCV build is unpinned.
#pragma once

#include <deque>

#include "opencv2/core.hpp"

namespace cv {

enum MorphShapes { MORPH_RECT = 0, MORPH_CROSS = 1, MORPH_ELLIPSE = 2 };
enum MorphTypes { MORPH_ERODE = 0, MORPH_DILATE = 1, MORPH_OPEN = 2, MORPH_CLOSE = 3 };
enum InterpolationFlags { INTER_NEAREST = 0, INTER_LINEAR = 1, INTER_CUBIC = 2, INTER_AREA = 3 };
enum ColorConversionCodes { COLOR_GRAY2BGR = 8 };

inline Mat getStructuringElement(int shape, Size ksize, Point anchor = Point(-1, -1)) {
    if (shape != MORPH_RECT) throw std::runtime_error("getStructuringElement: only MORPH_RECT is supported");
    (void)anchor;
    return Mat(ksize, CV_8UC1, Scalar(1));
}

// half-width of the square window equivalent to `iterations` passes of `kernel` (empty: 3x3)
inline int morph_radius(InputArray kernel, int iterations) {
    int k = 3;
    if (!kernel.empty()) {
        const Mat m = kernel.getMat();
        if (m.rows != m.cols || !(m.rows & 1) || countNonZero(m) != m.rows * m.cols)
            throw std::runtime_error("morphology: only odd square rectangular kernels are supported");
        k = m.rows;
    }
    return (k / 2) * (iterations < 1 ? 1 : iterations);
}

// max (dilate) or min (erode) over the (2r+1)x(2r+1) window clipped to the image: with the default
// border value (morphologyDefaultBorderValue) pixels outside the image never win, and n passes of a
// 3x3 rectangle equal one (2n+1)x(2n+1) rectangle under that rule. 8-bit, single channel.
inline void morph_minmax(const Mat& src, Mat& dst, int r, bool is_max) {
    const int W = src.cols, H = src.rows;
    Mat tmp(H, W, CV_8UC1), out(H, W, CV_8UC1);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int v = is_max ? 0 : 255;
            for (int d = -r; d <= r; ++d) {
                const int xx = x + d;
                if (xx < 0 || xx >= W) continue;
                const int s = src.ptr(y)[xx];
                v = is_max ? std::max(v, s) : std::min(v, s);
            }
            tmp.ptr(y)[x] = (uchar)v;
        }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            int v = is_max ? 0 : 255;
            for (int d = -r; d <= r; ++d) {
                const int yy = y + d;
                if (yy < 0 || yy >= H) continue;
                const int s = tmp.ptr(yy)[x];
                v = is_max ? std::max(v, s) : std::min(v, s);
            }
            out.ptr(y)[x] = (uchar)v;
        }
    dst.create(H, W, CV_8UC1);
    out.copyTo(dst);
}

inline void dilate(InputArray src, OutputArray dst, InputArray kernel, Point anchor = Point(-1, -1),
                   int iterations = 1) {
    (void)anchor;
    const Mat s = src.getMat();
    if (s.type() != CV_8UC1) throw std::runtime_error("dilate: 8UC1 only");
    morph_minmax(s, dst.getMatRef(), morph_radius(kernel, iterations), true);
}
inline void erode(InputArray src, OutputArray dst, InputArray kernel, Point anchor = Point(-1, -1),
                  int iterations = 1) {
    (void)anchor;
    const Mat s = src.getMat();
    if (s.type() != CV_8UC1) throw std::runtime_error("erode: 8UC1 only");
    morph_minmax(s, dst.getMatRef(), morph_radius(kernel, iterations), false);
}
// closing: dilation then erosion with the same kernel
inline void morphologyEx(InputArray src, OutputArray dst, int op, InputArray kernel, Point anchor = Point(-1, -1),
                         int iterations = 1) {
    if (op != MORPH_CLOSE) throw std::runtime_error("morphologyEx: only MORPH_CLOSE is supported");
    Mat t;
    dilate(src, t, kernel, anchor, iterations);
    erode(t, dst, kernel, anchor, iterations);
}

// 4-connected flood fill with zero tolerances (the default flags and loDiff/upDiff): every pixel
// 4-connected to the seed through pixels equal to the seed's value takes newVal. 8UC1.
inline int floodFill(InputOutputArray image, Point seed, Scalar newVal) {
    Mat& m = image.getMatRef();
    if (m.type() != CV_8UC1) throw std::runtime_error("floodFill: 8UC1 only");
    const int W = m.cols, H = m.rows;
    if (seed.x < 0 || seed.y < 0 || seed.x >= W || seed.y >= H) return 0;
    const uchar v0 = m.ptr(seed.y)[seed.x];
    const uchar nv = saturate_cast<uchar>(newVal.val[0]);
    std::vector<uchar> seen((size_t)W * H, 0);
    std::deque<int> q;
    q.push_back(seed.y * W + seed.x);
    seen[(size_t)seed.y * W + seed.x] = 1;
    int n = 0;
    while (!q.empty()) {
        const int p = q.front();
        q.pop_front();
        const int x = p % W, y = p / W;
        m.ptr(y)[x] = nv;
        ++n;
        const int nx[4] = {x - 1, x + 1, x, x}, ny[4] = {y, y, y - 1, y + 1};
        for (int k = 0; k < 4; ++k) {
            if (nx[k] < 0 || ny[k] < 0 || nx[k] >= W || ny[k] >= H) continue;
            const size_t j = (size_t)ny[k] * W + nx[k];
            if (seen[j] || m.ptr(ny[k])[nx[k]] != v0) continue;
            seen[j] = 1;
            q.push_back((int)j);
        }
    }
    return n;
}

// BORDER_REFLECT_101 index (OpenCV's BORDER_DEFAULT): -1 -> 1, n -> n-2
inline int border_reflect101(int i, int n) {
    if (n == 1) return 0;
    while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - 2 - i;
    return i;
}

// cv::GaussianBlur of 8-bit images, 3x3 kernel, sigma 0, BORDER_DEFAULT: the kernel [1 2 1]/4 in both
// directions, whose 8-bit result is the exact weighted sum rounded half up: (sum(w*p) + 8) >> 4
inline void GaussianBlur(InputArray src_, OutputArray dst_, Size ksize, double sigmaX, double sigmaY = 0,
                         int borderType = BORDER_DEFAULT) {
    const Mat src = src_.getMat();
    if (src.depth() != CV_8U || ksize.width != 3 || ksize.height != 3 || sigmaX != 0 || sigmaY != 0 ||
        borderType != BORDER_DEFAULT)
        throw std::runtime_error("GaussianBlur: 8-bit, 3x3, sigma 0, BORDER_DEFAULT only");
    const int W = src.cols, H = src.rows, C = src.channels();
    static const int w[3] = {1, 2, 1};
    Mat out(H, W, src.type());
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < C; ++c) {
                int acc = 0;
                for (int j = -1; j <= 1; ++j)
                    for (int i = -1; i <= 1; ++i)
                        acc += w[j + 1] * w[i + 1] * src.ptr(border_reflect101(y + j, H))[border_reflect101(x + i, W) * C + c];
                out.ptr(y)[x * C + c] = (uchar)((acc + 8) >> 4);
            }
    Mat& dst = dst_.getMatRef();
    dst.create(H, W, src.type());
    out.copyTo(dst);
}

// cv::Scharr of an 8-bit image into CV_16S (dx = 1, dy = 0: [-3 0 3; -10 0 10; -3 0 3]; dx = 0, dy = 1:
// its transpose), scale 1, delta 0, BORDER_DEFAULT
inline void Scharr(InputArray src_, OutputArray dst_, int ddepth, int dx, int dy, double scale = 1, double delta = 0,
                   int borderType = BORDER_DEFAULT) {
    const Mat src = src_.getMat();
    if (src.depth() != CV_8U || ddepth != CV_16S || dx + dy != 1 || scale != 1 || delta != 0 ||
        borderType != BORDER_DEFAULT)
        throw std::runtime_error("Scharr: 8-bit into CV_16S, first derivative, scale 1, BORDER_DEFAULT only");
    const int W = src.cols, H = src.rows, C = src.channels();
    static const int ws[3] = {3, 10, 3};
    Mat out(H, W, CV_16SC(C));
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < C; ++c) {
                int g = 0;
                for (int k = -1; k <= 1; ++k) {
                    if (dx) {
                        const uchar* row = src.ptr(border_reflect101(y + k, H));
                        g += ws[k + 1] * ((int)row[border_reflect101(x + 1, W) * C + c] -
                                          (int)row[border_reflect101(x - 1, W) * C + c]);
                    } else {
                        const int xx = border_reflect101(x + k, W) * C + c;
                        g += ws[k + 1] * ((int)src.ptr(border_reflect101(y + 1, H))[xx] -
                                          (int)src.ptr(border_reflect101(y - 1, H))[xx]);
                    }
                }
                out.ptr<short>(y)[x * C + c] = (short)g;
            }
    Mat& dst = dst_.getMatRef();
    dst.create(H, W, CV_16SC(C));
    out.copyTo(dst);
}

// cv::convertScaleAbs of a CV_16S image (alpha 1, beta 0): |v| saturated to 255
inline void convertScaleAbs(InputArray src_, OutputArray dst_, double alpha = 1, double beta = 0) {
    const Mat src = src_.getMat();
    if (src.depth() != CV_16S || alpha != 1 || beta != 0) throw std::runtime_error("convertScaleAbs: CV_16S, alpha 1, beta 0 only");
    const int C = src.channels();
    Mat out(src.rows, src.cols, CV_8UC(C));
    for (int y = 0; y < src.rows; ++y)
        for (int i = 0; i < src.cols * C; ++i) {
            const int v = std::abs((int)src.ptr<short>(y)[i]);
            out.ptr(y)[i] = (uchar)(v > 255 ? 255 : v);
        }
    Mat& dst = dst_.getMatRef();
    dst.create(src.rows, src.cols, CV_8UC(C));
    out.copyTo(dst);
}

// cv::cvtColor for COLOR_GRAY2BGR only: the single channel repeated into three (8UC1 -> 8UC3)
inline void cvtColor(InputArray src_, OutputArray dst_, int code) {
    const Mat src = src_.getMat();
    if (code != COLOR_GRAY2BGR || src.type() != CV_8UC1) throw std::runtime_error("cvtColor: GRAY2BGR of 8UC1 only");
    Mat out(src.rows, src.cols, CV_8UC3);
    for (int y = 0; y < src.rows; ++y)
        for (int x = 0; x < src.cols; ++x)
            for (int c = 0; c < 3; ++c) out.ptr(y)[3 * x + c] = src.ptr(y)[x];
    Mat& dst = dst_.getMatRef();
    dst.create(src.rows, src.cols, CV_8UC3);
    out.copyTo(dst);
}

// median of the k x k window with BORDER_REPLICATE (k odd), 8UC1: a 256-bin histogram slid along
// each row
inline void medianBlur(InputArray src_, OutputArray dst_, int k) {
    const Mat src = src_.getMat();
    if (src.type() != CV_8UC1 || k < 1 || !(k & 1)) throw std::runtime_error("medianBlur: 8UC1, odd k");
    const int W = src.cols, H = src.rows, r = k / 2, half = k * k / 2;
    Mat out(H, W, CV_8UC1);
    auto at = [&](int y, int x) {
        y = y < 0 ? 0 : y >= H ? H - 1 : y;
        x = x < 0 ? 0 : x >= W ? W - 1 : x;
        return src.ptr(y)[x];
    };
    for (int y = 0; y < H; ++y) {
        int hist[256] = {0};
        for (int dy = -r; dy <= r; ++dy)
            for (int dx = -r; dx <= r; ++dx) ++hist[at(y + dy, dx)];
        for (int x = 0; x < W; ++x) {
            if (x > 0)
                for (int dy = -r; dy <= r; ++dy) {
                    --hist[at(y + dy, x - 1 - r)];
                    ++hist[at(y + dy, x + r)];
                }
            int acc = 0, v = 0;
            for (; v < 256; ++v) {
                acc += hist[v];
                if (acc > half) break;
            }
            out.ptr(y)[x] = (uchar)v;
        }
    }
    Mat& dst = dst_.getMatRef();
    dst.create(H, W, CV_8UC1);
    out.copyTo(dst);
}

// INTER_AREA when the source size is an integral multiple of the output (OpenCV's "area fast"
// case): each output element is saturate_cast(block sum * (1.f/area)), the sum in int (8-bit
// sources) or double (float sources); for other scales the exact area-weighted mean, rounded half to
// even (the same definition as oracle/common.h resize_area_u8). INTER_NEAREST: source x =
// floor(dx * (1/(dw/W))), clamped.
inline void resize(InputArray src_, OutputArray dst_, Size dsize, double fx = 0, double fy = 0,
                   int interpolation = INTER_LINEAR) {
    (void)fx;
    (void)fy;
    const Mat src = src_.getMat();
    const int W = src.cols, H = src.rows, cn = src.channels(), dw = dsize.width, dh = dsize.height;
    Mat out(dh, dw, src.type());
    if (interpolation == INTER_AREA && (dw <= 0 || dh <= 0)) throw std::runtime_error("resize: empty output size");
    if (interpolation == INTER_AREA && (W % dw || H % dh)) {
        // non-integral scale: the exact area-weighted mean of the source pixels under each output
        // pixel (overlaps are integers in units of 1/dw, 1/dh), rounded half to even; 8-bit only
        if (src.depth() != CV_8U) throw std::runtime_error("resize(INTER_AREA): non-integral scales of 8-bit images only");
        const unsigned long long den = (unsigned long long)W * (unsigned long long)H;
        for (int y = 0; y < dh; ++y)
            for (int x = 0; x < dw; ++x) {
                const long long x0 = (long long)x * W, x1 = x0 + W, y0 = (long long)y * H, y1 = y0 + H;
                const int i0 = (int)(x0 / dw), i1 = (int)((x1 + dw - 1) / dw);
                const int j0 = (int)(y0 / dh), j1 = (int)((y1 + dh - 1) / dh);
                for (int c = 0; c < cn; ++c) {
                    unsigned long long num = 0;
                    for (int j = j0; j < j1; ++j) {
                        const long long a = (long long)j * dh, b = a + dh;
                        const long long oy = std::min(b, y1) - std::max(a, y0);
                        unsigned long long row = 0;
                        for (int i = i0; i < i1; ++i) {
                            const long long cc = (long long)i * dw, d = cc + dw;
                            row += (unsigned long long)(std::min(d, x1) - std::max(cc, x0)) * src.ptr(j)[i * cn + c];
                        }
                        num += row * (unsigned long long)oy;
                    }
                    unsigned long long q = num / den;
                    const unsigned long long r2 = (num % den) * 2ull;
                    if (r2 > den || (r2 == den && (q & 1ull))) ++q;
                    out.ptr(y)[x * cn + c] = (uchar)std::min(q, 255ull);
                }
            }
    } else if (interpolation == INTER_AREA) {
        const int sx = W / dw, sy = H / dh;
        const float scale = 1.f / (float)(sx * sy);
        for (int y = 0; y < dh; ++y)
            for (int x = 0; x < dw; ++x)
                for (int c = 0; c < cn; ++c) {
                    if (src.depth() == CV_8U) {
                        int s = 0;
                        for (int yy = 0; yy < sy; ++yy)
                            for (int xx = 0; xx < sx; ++xx) s += src.ptr(y * sy + yy)[(x * sx + xx) * cn + c];
                        out.ptr(y)[x * cn + c] = saturate_cast<uchar>((float)s * scale);
                    } else {
                        double s = 0;
                        for (int yy = 0; yy < sy; ++yy)
                            for (int xx = 0; xx < sx; ++xx) s += src.get_d(y * sy + yy, (x * sx + xx) * cn + c);
                        out.put_d(y, x * cn + c, s * scale);
                    }
                }
    } else if (interpolation == INTER_NEAREST) {
        const double ifx = 1.0 / ((double)dw / W), ify = 1.0 / ((double)dh / H);
        const size_t es = src.elemSize();
        for (int y = 0; y < dh; ++y) {
            int syy = (int)std::floor(y * ify);
            syy = syy < H - 1 ? syy : H - 1;
            for (int x = 0; x < dw; ++x) {
                int sxx = (int)std::floor(x * ifx);
                sxx = sxx < W - 1 ? sxx : W - 1;
                std::memcpy(out.ptr(y) + x * es, src.ptr(syy) + sxx * es, es);
            }
        }
    } else {
        throw std::runtime_error("resize: only INTER_AREA and INTER_NEAREST are supported");
    }
    Mat& dst = dst_.getMatRef();
    dst.create(dh, dw, src.type());
    out.copyTo(dst);
}

// dst = src*a + dst*(1-a), a = (float)alpha, in float, each product rounded separately
inline void accumulateWeighted(InputArray src_, InputOutputArray dst_, double alpha, InputArray mask = noArray()) {
    if (!mask.empty()) throw std::runtime_error("accumulateWeighted: masks are not supported");
    const Mat src = src_.getMat();
    Mat& dst = dst_.getMatRef();
    const float a = (float)alpha, b = 1.0f - a;
    for (int y = 0; y < src.rows; ++y)
        for (int i = 0; i < src.cols * src.channels(); ++i) {
            float* d = dst.ptr<float>(y) + i;
            const float t1 = (float)src.get_d(y, i) * a;
            const float t2 = *d * b;
            *d = t1 + t2;
        }
}

// dst += src1*src2 where mask != 0, in float
inline void accumulateProduct(InputArray s1_, InputArray s2_, InputOutputArray dst_, InputArray mask_ = noArray()) {
    const Mat s1 = s1_.getMat(), s2 = s2_.getMat(), mask = mask_.getMat();
    Mat& dst = dst_.getMatRef();
    if (dst.depth() != CV_32F || dst.channels() != 1) throw std::runtime_error("accumulateProduct: 32FC1 only");
    for (int y = 0; y < dst.rows; ++y)
        for (int x = 0; x < dst.cols; ++x) {
            if (!mask.empty() && !mask.ptr(y)[x]) continue;
            const float prod = (float)s1.get_d(y, x) * (float)s2.get_d(y, x);
            float* d = dst.ptr<float>(y) + x;
            *d = *d + prod;
        }
}

// normalized 3x3 box filter with BORDER_REPLICATE on 32FC1, sums in double: per row
// s = v[x-1] + v[x] + v[x+1], per column t = s[y-1] + s[y] + s[y+1], dst = (float)(t * (1.0/9))
inline void blur(InputArray src_, OutputArray dst_, Size ksize, Point anchor = Point(-1, -1),
                 int borderType = BORDER_DEFAULT) {
    (void)anchor;
    const Mat src = src_.getMat();
    if (ksize.width != 3 || ksize.height != 3 || borderType != BORDER_REPLICATE || src.type() != CV_32FC1)
        throw std::runtime_error("blur: 3x3 BORDER_REPLICATE on 32FC1 only");
    const int w = src.cols, h = src.rows;
    std::vector<double> row((size_t)w * h);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const int x0 = x > 0 ? x - 1 : 0, x1 = x < w - 1 ? x + 1 : w - 1;
            const float* p = src.ptr<float>(y);
            row[(size_t)y * w + x] = ((double)p[x0] + (double)p[x]) + (double)p[x1];
        }
    Mat out(h, w, CV_32FC1);
    for (int y = 0; y < h; ++y) {
        const int y0 = y > 0 ? y - 1 : 0, y1 = y < h - 1 ? y + 1 : h - 1;
        for (int x = 0; x < w; ++x) {
            const double t = (row[(size_t)y0 * w + x] + row[(size_t)y * w + x]) + row[(size_t)y1 * w + x];
            out.ptr<float>(y)[x] = (float)(t * (1.0 / 9.0));
        }
    }
    Mat& dst = dst_.getMatRef();
    dst.create(h, w, CV_32FC1);
    out.copyTo(dst);
}

// drawing is only called in the reference's debug-display code, which is compiled out here
void circle(InputOutputArray img, Point center, int radius, const Scalar& color, int thickness = 1);

}  // namespace cv
