// Test infrastructure: a small OpenCV-shaped core (cv::Mat of one channel,
// Size, Point, Scalar, type macros) under which the reference's own
// src/lib/nldiffusion_functions.cpp and src/lib/utils.cpp compile unchanged
// (oracle/Makefile, target "ref").  Only what those files touch is
// declared; image filters route to the oracle's implementations
// (ref_shim.cpp), drawing and RANSAC are absent (they throw if called).
#ifndef AKO_REF_SHIM_CORE_HPP
#define AKO_REF_SHIM_CORE_HPP
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#define CV_8U 0
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_CN_SHIFT 3
#define CV_MAKETYPE(depth, cn) ((depth) + (((cn)-1) << CV_CN_SHIFT))
#define CV_8UC1 CV_MAKETYPE(CV_8U, 1)
#define CV_8UC3 CV_MAKETYPE(CV_8U, 3)
#define CV_32FC1 CV_MAKETYPE(CV_32F, 1)
#define CV_Assert(expr) \
  do {                  \
    if (!(expr)) throw std::runtime_error("CV_Assert failed: " #expr); \
  } while (0)

namespace cv {
typedef unsigned char uchar;

enum { BORDER_REPLICATE = 1, BORDER_DEFAULT = 4 };
enum { INTER_LINEAR = 1, INTER_AREA = 3 };

struct Size {
  int width = 0, height = 0;
  Size() {}
  Size(int w, int h) : width(w), height(h) {}
};
struct Point {
  int x = 0, y = 0;
  Point() {}
  Point(int x_, int y_) : x(x_), y(y_) {}
};
struct Point2f {
  float x = 0, y = 0;
  Point2f() {}
  Point2f(float x_, float y_) : x(x_), y(y_) {}
};
struct Scalar {
  double val[4] = {0, 0, 0, 0};
  Scalar() {}
  Scalar(double a, double b = 0, double c = 0, double d = 0) : val{a, b, c, d} {}
};

/* Dense matrix; element size from the type (1, 3 or 4 bytes per element). */
class Mat {
 public:
  int rows = 0, cols = 0;
  uchar *data = nullptr;
  size_t step = 0;

  Mat() {}
  Mat(int r, int c, int t) { create(r, c, t); }
  Mat(Size s, int t) { create(s.height, s.width, t); }
  Mat(int r, int c, int t, void *ext) : rows(r), cols(c), data((uchar *)ext), step((size_t)c * esz(t)), type_(t) {}
  static Mat zeros(int r, int c, int t)
  {
    Mat m(r, c, t);
    std::memset(m.data, 0, m.total_bytes());
    return m;
  }
  static Mat zeros(Size s, int t) { return zeros(s.height, s.width, t); }
  void create(int r, int c, int t)
  {
    rows = r;
    cols = c;
    type_ = t;
    step = (size_t)c * esz(t);
    buf_ = std::make_shared<std::vector<uchar>>(total_bytes() + 1);
    data = buf_->data();
  }
  int type() const { return type_; }
  Size size() const { return Size(cols, rows); }
  bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
  size_t total_bytes() const { return (size_t)rows * step; }
  template <typename T>
  T *ptr(int r)
  {
    return reinterpret_cast<T *>(data + (size_t)r * step);
  }
  template <typename T>
  const T *ptr(int r) const
  {
    return reinterpret_cast<const T *>(data + (size_t)r * step);
  }
  template <typename T>
  T &at(int r, int c)
  {
    return ptr<T>(r)[c];
  }
  template <typename T>
  const T &at(int r, int c) const
  {
    return ptr<T>(r)[c];
  }
  template <typename T>
  T &at(int i)
  {
    return cols == 1 ? ptr<T>(i)[0] : ptr<T>(0)[i];
  }
  template <typename T>
  const T &at(int i) const
  {
    return cols == 1 ? ptr<T>(i)[0] : ptr<T>(0)[i];
  }
  /* every element (float or uchar matrices) set to s.val[0] */
  Mat &operator=(const Scalar &s)
  {
    for (int r = 0; r < rows; r++)
      for (int c = 0; c < cols; c++) {
        if (type_ == CV_32F)
          at<float>(r, c) = (float)s.val[0];
        else
          ptr<uchar>(r)[c] = (uchar)s.val[0];
      }
    return *this;
  }
  void copyTo(Mat &m) const
  {
    Mat out(rows, cols, type_);
    for (int r = 0; r < rows; r++) std::memcpy(out.ptr<uchar>(r), ptr<uchar>(r), step);
    m = out;
  }
  Mat clone() const
  {
    Mat m;
    copyTo(m);
    return m;
  }

 private:
  static size_t esz(int t)
  {
    const int depth = t & 7, cn = 1 + (t >> CV_CN_SHIFT);
    return (size_t)cn * (depth == CV_32F || depth == CV_32S ? 4 : depth == CV_64F ? 8 : 1);
  }
  int type_ = CV_8U;
  std::shared_ptr<std::vector<uchar>> buf_;
};

/* Element-wise float arithmetic used by utils.cpp's visualisation helpers. */
inline Mat shim_map(const Mat &a, float (*f)(float, float), float b)
{
  Mat out(a.rows, a.cols, CV_32F);
  for (int r = 0; r < a.rows; r++)
    for (int c = 0; c < a.cols; c++) out.at<float>(r, c) = f(a.at<float>(r, c), b);
  return out;
}
inline Mat operator-(const Mat &a, float b)
{
  return shim_map(a, [](float x, float y) { return x - y; }, b);
}
inline Mat operator/(const Mat &a, float b)
{
  return shim_map(a, [](float x, float y) { return x / y; }, b);
}
inline Mat operator-(double a, const Mat &m)
{
  return shim_map(m, [](float x, float y) { return y - x; }, (float)a);
}
inline void exp(const Mat &src, Mat &dst)
{
  dst = shim_map(src, [](float x, float) { return std::exp(x); }, 0.f);
}

/* The OutputArray of getDerivKernels / compute_derivative_kernels. */
class _OutputArray {
 public:
  _OutputArray(Mat &m) : m_(&m) {}
  void create(int r, int c, int t, int = -1, bool = false, int = 0) const { m_->create(r, c, t); }
  Mat getMat() const { return *m_; }
  Mat &mat() const { return *m_; }

 private:
  Mat *m_;
};
typedef const _OutputArray &OutputArray;
}  // namespace cv
#endif
