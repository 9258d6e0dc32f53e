// Minimal stand-in with the shape of OpenCV's core API (cv::Mat with a
// MatStep row step, type macros as preprocessor constants, cv::Point2f),
// only so that include/libAKAZECU/AKAZE.h's AKZ_WITH_OPENCV branch can be
// compiled in a container without OpenCV.  Declarations only as far as the
// wrapper and the test program use them; not a reimplementation of OpenCV.
#ifndef AKZ_TEST_OPENCV_STUB_CORE_HPP
#define AKZ_TEST_OPENCV_STUB_CORE_HPP
#include <cstddef>
#include <memory>
#include <vector>

#define CV_8U 0
#define CV_32F 5
#define CV_CN_SHIFT 3
#define CV_MAKETYPE(depth, cn) ((depth) + (((cn)-1) << CV_CN_SHIFT))
#define CV_8UC1 CV_MAKETYPE(CV_8U, 1)
#define CV_8UC3 CV_MAKETYPE(CV_8U, 3)
#define CV_32FC1 CV_MAKETYPE(CV_32F, 1)

namespace cv {
typedef unsigned char uchar;
struct Point2f {
  float x, y;
  Point2f() : x(0), y(0) {}
  Point2f(float x_, float y_) : x(x_), y(y_) {}
};
struct MatStep {
  size_t p[2] = {0, 0};
  operator size_t() const { return p[0]; }
  size_t operator[](int i) const { return p[i]; }
};
class Mat {
 public:
  int flags = 0, dims = 2, rows = 0, cols = 0;
  uchar *data = nullptr;
  MatStep step;
  Mat() {}
  Mat(int r, int c, int type) { create(r, c, type); }
  Mat(int r, int c, int type, void *d, size_t st = 0) : flags(type), rows(r), cols(c), data((uchar *)d)
  {
    step.p[0] = st ? st : (size_t)c * esz(type);
    step.p[1] = esz(type);
  }
  void create(int r, int c, int type)
  {
    flags = type;
    rows = r;
    cols = c;
    step.p[0] = (size_t)c * esz(type);
    step.p[1] = esz(type);
    mem_ = std::make_shared<std::vector<uchar>>((size_t)r * step.p[0]);
    data = mem_->data();
  }
  int type() const { return flags; }
  bool empty() const { return data == nullptr || rows == 0; }
  uchar *ptr(int r) { return data + (size_t)r * step.p[0]; }
  const uchar *ptr(int r) const { return data + (size_t)r * step.p[0]; }
  void convertTo(Mat &m, int rtype, double alpha = 1, double beta = 0) const
  {
    Mat out(rows, cols, rtype);
    for (int r = 0; r < rows; r++)
      for (int c = 0; c < cols; c++)
        reinterpret_cast<float *>(out.ptr(r))[c] = (float)ptr(r)[c] * (float)alpha + (float)beta;
    m = out;
  }

 private:
  static size_t esz(int t) { return (t & 7) == CV_32F ? 4 : 1 * (size_t)(1 + (t >> CV_CN_SHIFT)); }
  std::shared_ptr<std::vector<uchar>> mem_;
};
}  // namespace cv
#endif
