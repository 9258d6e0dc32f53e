/*
 * libAKAZECU/AKAZE.h - header-only C++ face of akaze_gb300 with the
 * reference's class signatures (src/lib/AKAZE.h:27-143 of francoto/akaze),
 * so that code written against libAKAZECU compiles unchanged:
 *
 *   libAKAZECU::AKAZE evolution(options);
 *   evolution.Create_Nonlinear_Scale_Space(img_32);     // CV_32F in [0,1] or CV_8U
 *   evolution.Feature_Detection(kpts);                  // kpts stays empty, as in the reference
 *   evolution.Compute_Descriptors(kpts, desc);          // fills kpts and desc (n x 61 CV_8U)
 *   libAKAZECU::Matcher m; m.bfmatch(desc1, desc2, dmatches);
 *
 * With OpenCV available (define AKZ_WITH_OPENCV before including) the real
 * cv::Mat / cv::KeyPoint / cv::DMatch types are used; otherwise a minimal
 * layout-compatible subset is declared in namespace cv.  Errors throw
 * std::runtime_error carrying akz_last_error() (the reference exits).
 */
#ifndef LIBAKAZECU_AKAZE_H
#define LIBAKAZECU_AKAZE_H

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../akaze_gb300.h"

#ifdef AKZ_WITH_OPENCV
#include <opencv2/core/core.hpp>
#include <opencv2/features2d/features2d.hpp>
#else
namespace cv {
struct Point2f {
  float x = 0, y = 0;
};
struct KeyPoint { /* 28 bytes, the cv::KeyPoint layout */
  Point2f pt;
  float size = 0, angle = -1, response = 0;
  int octave = 0, class_id = -1;
};
struct DMatch {
  int queryIdx = -1, trainIdx = -1, imgIdx = -1;
  float distance = 0;
};
enum { CV_8U = 0, CV_32F = 5 };
/* Continuous single-channel matrix (rows x cols of CV_8U or CV_32F). */
class Mat {
 public:
  int rows = 0, cols = 0, type_ = CV_8U;
  unsigned char *data = nullptr;
  Mat() = default;
  Mat(int r, int c, int t) : rows(r), cols(c), type_(t), buf_(std::make_shared<std::vector<unsigned char>>((size_t)r * c * elem(t)))
  {
    data = buf_->data();
  }
  Mat(int r, int c, int t, void *ext) : rows(r), cols(c), type_(t), data((unsigned char *)ext) {}
  int type() const { return type_; }
  size_t step1() const { return (size_t)cols; }
  size_t elemSize() const { return elem(type_); }
  bool empty() const { return rows == 0 || cols == 0; }

 private:
  static size_t elem(int t) { return t == CV_32F ? 4 : 1; }
  std::shared_ptr<std::vector<unsigned char>> buf_;
};
}  // namespace cv
#endif

static_assert(sizeof(cv::KeyPoint) == sizeof(akz_keypoint), "cv::KeyPoint layout");
static_assert(sizeof(cv::DMatch) == sizeof(akz_dmatch), "cv::DMatch layout");

/* AKAZEOptions (AKAZEConfig.h:84-172) is the C struct with the reference's
 * setters; DIFFUSIVITY_TYPE / DESCRIPTOR_TYPE values are AKZ_* enums. */
struct AKAZEOptions : akz_options {
  AKAZEOptions() { akz_options_default(this); }
  void setWidth(int w) { img_width = w; }
  void setHeight(int h) { img_height = h; }
};
typedef akz_timing AKAZETiming;

namespace libAKAZECU {

inline void akz_throw(akz_status s)
{
  if (s != AKZ_OK) throw std::runtime_error(std::string("akaze_gb300: ") + akz_last_error());
}

class AKAZE {
 public:
  explicit AKAZE(const AKAZEOptions &options) : options_(options) { akz_throw(akz_create(&options_, &ctx_)); }
  ~AKAZE() { akz_destroy(ctx_); }
  AKAZE(const AKAZE &) = delete;
  AKAZE &operator=(const AKAZE &) = delete;

  /* AKAZE.cpp:211-276; returns 0 (errors throw). */
  int Create_Nonlinear_Scale_Space(const cv::Mat &img)
  {
    const int dtype = img.type() == cv::CV_32F ? AKZ_F32 : AKZ_U8;
    const size_t stride = (size_t)img.cols * (dtype == AKZ_F32 ? 4 : 1);
    akz_throw(akz_create_nonlinear_scale_space(ctx_, img.data, img.cols, img.rows, stride, dtype, 0));
    return 0;
  }
  /* AKAZE.cpp:316-378: like the reference, kpts is left for Compute_Descriptors. */
  void Feature_Detection(std::vector<cv::KeyPoint> &kpts)
  {
    (void)kpts;
    akz_throw(akz_feature_detection(ctx_, &n_));
  }
  /* AKAZE.cpp:405-449: kpts and desc (n x 61, CV_8U) are filled here. */
  void Compute_Descriptors(std::vector<cv::KeyPoint> &kpts, cv::Mat &desc)
  {
    kpts.resize((size_t)n_);
    desc = cv::Mat(n_, 61, cv::CV_8U);
    int n = 0;
    akz_throw(akz_compute_descriptors(ctx_, reinterpret_cast<akz_keypoint *>(kpts.data()), desc.data, n_, &n));
  }
  AKAZETiming Get_Computation_Times() const
  {
    akz_timing t;
    akz_get_timing(ctx_, &t);
    return t;
  }
  void Show_Computation_Times() const {}

 private:
  AKAZEOptions options_;
  akz_context *ctx_ = nullptr;
  int n_ = 0;
};

class Matcher {
 public:
  Matcher() { akz_throw(akz_matcher_create(&m_)); }
  ~Matcher() { akz_matcher_destroy(m_); }
  Matcher(const Matcher &) = delete;
  Matcher &operator=(const Matcher &) = delete;

  /* AKAZE.cpp:36-79: two matches per query row (best, second best). */
  void bfmatch(cv::Mat &desc_query, cv::Mat &desc_train, std::vector<std::vector<cv::DMatch>> &dmatches)
  {
    std::vector<akz_dmatch> out((size_t)desc_query.rows * 2);
    akz_throw(akz_matcher_bfmatch(m_, desc_query.data, desc_query.rows, desc_train.data, desc_train.rows,
                                  desc_query.cols, out.data()));
    dmatches.assign((size_t)desc_query.rows, std::vector<cv::DMatch>(2));
    for (int i = 0; i < desc_query.rows; i++)
      for (int k = 0; k < 2; k++) std::memcpy(static_cast<void *>(&dmatches[i][k]), &out[(size_t)2 * i + k], sizeof(cv::DMatch));
  }

 private:
  akz_matcher *m_ = nullptr;
};

}  // namespace libAKAZECU

#endif
