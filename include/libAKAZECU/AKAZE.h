/*
 * libAKAZECU/AKAZE.h - header-only C++ face of akaze_gb300 with the
 * reference's class and option signatures (src/lib/AKAZE.h:27-150 and
 * src/lib/AKAZEConfig.h:41-172 of francoto/akaze), so that code written
 * against libAKAZECU compiles unchanged:
 *
 *   AKAZEOptions options;                               // defaults of AKAZEConfig.h:86-111
 *   options.descriptor = DESCRIPTOR_TYPE(5);            // MLDB; DIFFUSIVITY_TYPE likewise
 *   options.img_width = img.cols; options.img_height = img.rows;
 *   img.convertTo(img_32, CV_32F, 1.0 / 255.0, 0);
 *   libAKAZECU::AKAZE evolution(options);
 *   evolution.Create_Nonlinear_Scale_Space(img_32);     // CV_32FC1 in [0,1] or CV_8UC1
 *   evolution.Feature_Detection(kpts);                  // kpts stays empty, as in the reference
 *   evolution.Compute_Descriptors(kpts, desc);          // fills kpts and desc (n x row bytes, CV_8U)
 *   libAKAZECU::Matcher m; m.bfmatch(desc1, desc2, dmatches);
 *
 * With OpenCV available (define AKZ_WITH_OPENCV before including) the real
 * cv::Mat / cv::KeyPoint / cv::DMatch types are used; otherwise a minimal
 * layout-compatible subset is declared in namespace cv, with OpenCV's type
 * macros (CV_8U, CV_32F, CV_8UC1, CV_32FC1).  Errors throw
 * std::runtime_error carrying akz_last_error() (the reference exits).
 */
#ifndef LIBAKAZECU_AKAZE_H
#define LIBAKAZECU_AKAZE_H

#include <cstddef>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../akaze_gb300.h"

#ifdef AKZ_WITH_OPENCV
#include <opencv2/core/core.hpp>
#include <opencv2/features2d/features2d.hpp>
#else
#ifndef CV_8U
#define CV_8U 0
#endif
#ifndef CV_32F
#define CV_32F 5
#endif
#ifndef CV_8UC1
#define CV_8UC1 CV_8U
#endif
#ifndef CV_32FC1
#define CV_32FC1 CV_32F
#endif
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
/* Single-channel matrix of CV_8UC1 or CV_32FC1 with a row step in bytes
 * (rows of an external buffer may be padded). */
class Mat {
 public:
  int rows = 0, cols = 0;
  unsigned char *data = nullptr;
  size_t step = 0;
  Mat() = default;
  Mat(int r, int c, int t) { create(r, c, t); }
  Mat(int r, int c, int t, void *ext, size_t step_bytes = 0)
      : rows(r), cols(c), data((unsigned char *)ext), step(step_bytes ? step_bytes : (size_t)c * elem(t)), type_(t)
  {
  }
  void create(int r, int c, int t)
  {
    rows = r;
    cols = c;
    type_ = t;
    step = (size_t)c * elem(t);
    buf_ = std::make_shared<std::vector<unsigned char>>((size_t)r * step);
    data = buf_->data();
  }
  int type() const { return type_; }
  size_t elemSize() const { return elem(type_); }
  bool empty() const { return rows == 0 || cols == 0; }
  bool isContinuous() const { return step == (size_t)cols * elem(type_); }
  unsigned char *ptr(int r) { return data + (size_t)r * step; }
  const unsigned char *ptr(int r) const { return data + (size_t)r * step; }
  /* dst = saturate(src * alpha + beta) in float arithmetic, as OpenCV's
   * 8U -> 32F convertTo with a scale (the demos' 1/255 conversion). */
  void convertTo(Mat &dst, int rtype, double alpha = 1, double beta = 0) const
  {
    if (rtype != CV_32F || type_ != CV_8U) throw std::invalid_argument("cv::Mat stub: only CV_8U -> CV_32F");
    Mat out(rows, cols, CV_32F);
    const float a = (float)alpha, b = (float)beta;
    for (int r = 0; r < rows; r++) {
      const unsigned char *s = ptr(r);
      float *d = reinterpret_cast<float *>(out.ptr(r));
      for (int c = 0; c < cols; c++) d[c] = (float)s[c] * a + b;
    }
    dst = out;
  }

 private:
  static size_t elem(int t) { return t == CV_32F ? 4 : 1; }
  int type_ = CV_8U;
  std::shared_ptr<std::vector<unsigned char>> buf_;
};
}  // namespace cv
#endif

static_assert(sizeof(cv::KeyPoint) == sizeof(akz_keypoint), "cv::KeyPoint layout");
static_assert(sizeof(cv::DMatch) == sizeof(akz_dmatch), "cv::DMatch layout");

/* DESCRIPTOR_TYPE, AKAZEConfig.h:41-48 (MLDB and MLDB_UPRIGHT are implemented). */
enum DESCRIPTOR_TYPE {
  SURF_UPRIGHT = AKZ_SURF_UPRIGHT,
  SURF = AKZ_SURF,
  MSURF_UPRIGHT = AKZ_MSURF_UPRIGHT,
  MSURF = AKZ_MSURF,
  MLDB_UPRIGHT = AKZ_MLDB_UPRIGHT,
  MLDB = AKZ_MLDB
};

/* DIFFUSIVITY_TYPE, AKAZEConfig.h:52-57. */
enum DIFFUSIVITY_TYPE { PM_G1 = AKZ_PM_G1, PM_G2 = AKZ_PM_G2, WEICKERT = AKZ_WEICKERT, CHARBONNIER = AKZ_CHARBONNIER };

/* AKAZETiming, AKAZEConfig.h:61-80: milliseconds per stage, zero at construction. */
struct AKAZETiming : akz_timing {
  AKAZETiming() : akz_timing{0, 0, 0, 0, 0, 0, 0} {}
  AKAZETiming(const akz_timing &t) : akz_timing(t) {}
};

/* AKAZEOptions, AKAZEConfig.h:84-172: the same fields, types and defaults
 * (enum-typed diffusivity and descriptor, bool flags), with the reference's
 * setters and stream output. */
struct AKAZEOptions {
  AKAZEOptions()
  {
    akz_options c;
    akz_options_default(&c);
    from_c(c);
  }
  void setWidth(int w) { img_width = w; }
  void setHeight(int h) { img_height = h; }

  int omin;
  int omax;
  int nsublevels;
  int img_width;
  int img_height;
  float soffset;
  float derivative_factor;
  float sderivatives;
  DIFFUSIVITY_TYPE diffusivity;
  float dthreshold;
  float min_dthreshold;
  DESCRIPTOR_TYPE descriptor;
  int descriptor_size;
  int descriptor_channels;
  int descriptor_pattern_size;
  float kcontrast;
  float kcontrast_percentile;
  size_t kcontrast_nbins;
  bool save_scale_space;
  bool save_keypoints;
  bool verbosity;
  int ncudaimages;
  int maxkeypoints;
  int extrema_3d; /* extension: akz_options.extrema_3d (0, the reference's 3x3 rule, by default) */
  int fast_math;  /* extension: akz_options.fast_math (0, the reference's arithmetic, by default) */

  akz_options to_c() const
  {
    akz_options c;
    akz_options_default(&c);
    c.omin = omin;
    c.omax = omax;
    c.nsublevels = nsublevels;
    c.img_width = img_width;
    c.img_height = img_height;
    c.soffset = soffset;
    c.derivative_factor = derivative_factor;
    c.sderivatives = sderivatives;
    c.diffusivity = (int)diffusivity;
    c.dthreshold = dthreshold;
    c.min_dthreshold = min_dthreshold;
    c.descriptor = (int)descriptor;
    c.descriptor_size = descriptor_size;
    c.descriptor_channels = descriptor_channels;
    c.descriptor_pattern_size = descriptor_pattern_size;
    c.kcontrast = kcontrast;
    c.kcontrast_percentile = kcontrast_percentile;
    c.kcontrast_nbins = kcontrast_nbins;
    c.save_scale_space = save_scale_space;
    c.save_keypoints = save_keypoints;
    c.verbosity = verbosity;
    c.ncudaimages = ncudaimages;
    c.maxkeypoints = maxkeypoints;
    c.extrema_3d = extrema_3d;
    c.fast_math = fast_math;
    return c;
  }
  void from_c(const akz_options &c)
  {
    omin = c.omin;
    omax = c.omax;
    nsublevels = c.nsublevels;
    img_width = c.img_width;
    img_height = c.img_height;
    soffset = c.soffset;
    derivative_factor = c.derivative_factor;
    sderivatives = c.sderivatives;
    diffusivity = DIFFUSIVITY_TYPE(c.diffusivity);
    dthreshold = c.dthreshold;
    min_dthreshold = c.min_dthreshold;
    descriptor = DESCRIPTOR_TYPE(c.descriptor);
    descriptor_size = c.descriptor_size;
    descriptor_channels = c.descriptor_channels;
    descriptor_pattern_size = c.descriptor_pattern_size;
    kcontrast = c.kcontrast;
    kcontrast_percentile = c.kcontrast_percentile;
    kcontrast_nbins = c.kcontrast_nbins;
    save_scale_space = c.save_scale_space != 0;
    save_keypoints = c.save_keypoints != 0;
    verbosity = c.verbosity != 0;
    ncudaimages = c.ncudaimages;
    maxkeypoints = c.maxkeypoints;
    extrema_3d = c.extrema_3d;
    fast_math = c.fast_math;
  }

  /* The option listing of AKAZEConfig.h:145-172: one "name =  value" line
   * per option, names left-aligned in 33 columns. */
  friend std::ostream &operator<<(std::ostream &os, const AKAZEOptions &akaze_options)
  {
    os << std::left;
    auto line = [&os](const char *name, auto value) { os << std::setw(33) << name << " =  " << value << std::endl; };
    line("akaze_options.omax", akaze_options.omax);
    line("akaze_options.nsublevels", akaze_options.nsublevels);
    line("akaze_options.soffset", akaze_options.soffset);
    line("akaze_options.sderivatives", akaze_options.sderivatives);
    line("akaze_options.diffusivity", (int)akaze_options.diffusivity);
    line("akaze_options.dthreshold", akaze_options.dthreshold);
    line("akaze_options.descriptor", (int)akaze_options.descriptor);
    line("akaze_options.descriptor_channels", akaze_options.descriptor_channels);
    line("akaze_options.descriptor_size", akaze_options.descriptor_size);
    line("akaze_options.save_scale_space", akaze_options.save_scale_space);
    line("akaze_options.verbosity", akaze_options.verbosity);
    return os;
  }
};

namespace libAKAZECU {

inline void akz_throw(akz_status s)
{
  if (s != AKZ_OK) throw std::runtime_error(std::string("akaze_gb300: ") + akz_last_error());
}

/* Declared by the reference (AKAZE.h:148) without a definition; here it
 * resets every option to the defaults of AKAZEConfig.h:86-111. */
inline void setDefaultAKAZEOptions(AKAZEOptions &options) { options = AKAZEOptions(); }

/* Bytes of one descriptor row for the options (AKAZE.cpp:412-423). */
inline int descriptor_row_bytes(const AKAZEOptions &o)
{
  const int bits = o.descriptor_size > 0 ? o.descriptor_size : (6 + 36 + 120) * o.descriptor_channels;
  return (bits + 7) / 8;
}

class AKAZE {
 public:
  explicit AKAZE(const AKAZEOptions &options) : options_(options)
  {
    const akz_options c = options_.to_c();
    akz_throw(akz_create(&c, &ctx_));
  }
  ~AKAZE() { akz_destroy(ctx_); }
  AKAZE(const AKAZE &) = delete;
  AKAZE &operator=(const AKAZE &) = delete;

  /* AKAZE.cpp:211-276 for a CV_32FC1 image in [0, 1] (the demos'
   * convertTo(img_32, CV_32F, 1.0/255.0)) or a CV_8UC1 image; rows are read
   * img.step bytes apart.  Returns 0 (errors throw). */
  int Create_Nonlinear_Scale_Space(const cv::Mat &img)
  {
    int dtype;
    if (img.type() == CV_32FC1)
      dtype = AKZ_F32;
    else if (img.type() == CV_8UC1)
      dtype = AKZ_U8;
    else
      throw std::invalid_argument("akaze_gb300: the image must be CV_8UC1 or CV_32FC1");
    const size_t stride = static_cast<size_t>(img.step);
    akz_throw(akz_create_nonlinear_scale_space(ctx_, img.data, img.cols, img.rows, stride, dtype, 0));
    return 0;
  }
  /* AKAZE.cpp:316-378: like the reference, kpts is left for Compute_Descriptors. */
  void Feature_Detection(std::vector<cv::KeyPoint> &kpts)
  {
    (void)kpts;
    akz_throw(akz_feature_detection(ctx_, &n_));
  }
  /* AKAZE.cpp:405-449: kpts and desc (n x descriptor_row_bytes, CV_8U) are
   * filled here. */
  void Compute_Descriptors(std::vector<cv::KeyPoint> &kpts, cv::Mat &desc)
  {
    const int rb = descriptor_row_bytes(options_);
    kpts.resize((size_t)n_);
    std::vector<unsigned char> rows((size_t)n_ * rb + 1);
    int n = 0;
    akz_throw(akz_compute_descriptors(ctx_, reinterpret_cast<akz_keypoint *>(kpts.data()), rows.data(), n_, &n));
    desc = cv::Mat(n_, rb, CV_8U);
    for (int i = 0; i < n_; i++) std::memcpy(desc.ptr(i), rows.data() + (size_t)i * rb, (size_t)rb);
  }
  AKAZETiming Get_Computation_Times() const
  {
    akz_timing t;
    if (akz_get_timing(ctx_, &t) != AKZ_OK) return AKAZETiming();
    return AKAZETiming(t);
  }
  /* AKAZE.cpp:486-495. */
  void Show_Computation_Times() const
  {
    const AKAZETiming t = Get_Computation_Times();
    std::cout << "(*) Time Scale Space: " << t.scale << std::endl;
    std::cout << "   - Time KContrast: " << t.kcontrast << std::endl;
    std::cout << "(*) Time Detector: " << t.detector << std::endl;
    std::cout << "   - Time Derivatives: " << t.derivatives << std::endl;
    std::cout << "   - Time Extrema: " << t.extrema << std::endl;
    std::cout << "   - Time Subpixel: " << t.subpixel << std::endl;
    std::cout << "(*) Time Descriptor: " << t.descriptor << std::endl;
    std::cout << std::endl;
  }

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

  /* AKAZE.cpp:36-79: two matches per query row (best, second best).  Rows
   * of either matrix are read desc.step bytes apart. */
  void bfmatch(cv::Mat &desc_query, cv::Mat &desc_train, std::vector<std::vector<cv::DMatch>> &dmatches)
  {
    const int rb = desc_query.cols;
    if (desc_train.rows > 0 && desc_train.cols != rb)
      throw std::invalid_argument("akaze_gb300: query and train descriptors differ in row size");
    std::vector<unsigned char> q, t;
    const unsigned char *qp = rows_of(desc_query, rb, q), *tp = rows_of(desc_train, rb, t);
    std::vector<akz_dmatch> out((size_t)desc_query.rows * 2);
    if (desc_query.rows > 0)
      akz_throw(akz_matcher_bfmatch(m_, qp, desc_query.rows, tp, desc_train.rows, rb, out.data()));
    dmatches.assign((size_t)desc_query.rows, std::vector<cv::DMatch>(2));
    for (int i = 0; i < desc_query.rows; i++)
      for (int k = 0; k < 2; k++) std::memcpy(static_cast<void *>(&dmatches[i][k]), &out[(size_t)2 * i + k], sizeof(cv::DMatch));
  }

  /* AKAZE.cpp:82-105: nq x 8 CV_32FC1 rows {queryIdx, trainIdx, 0, distance}
   * of the best and the second-best match. */
  cv::Mat bfmatch_(cv::Mat desc_query, cv::Mat desc_train)
  {
    std::vector<std::vector<cv::DMatch>> m;
    bfmatch(desc_query, desc_train, m);
    cv::Mat out((int)m.size(), 8, CV_32F);
    for (size_t i = 0; i < m.size(); i++) {
      float *r = reinterpret_cast<float *>(out.ptr((int)i));
      for (int k = 0; k < 2; k++) {
        r[4 * k + 0] = (float)m[i][k].queryIdx;
        r[4 * k + 1] = (float)m[i][k].trainIdx;
        r[4 * k + 2] = 0.f;
        r[4 * k + 3] = m[i][k].distance;
      }
    }
    return out;
  }

 private:
  /* Contiguous rows of rb bytes: the matrix itself, or a packed copy when
   * its rows are padded. */
  static const unsigned char *rows_of(const cv::Mat &m, int rb, std::vector<unsigned char> &copy)
  {
    if (m.rows == 0) return nullptr;
    if (static_cast<size_t>(m.step) == (size_t)rb) return m.data;
    copy.resize((size_t)m.rows * rb);
    for (int i = 0; i < m.rows; i++) std::memcpy(copy.data() + (size_t)i * rb, m.ptr(i), (size_t)rb);
    return copy.data();
  }
  akz_matcher *m_ = nullptr;
};

}  // namespace libAKAZECU

/* The free 2-NN matcher of cuda_akaze.h:28 (used by akaze_features.cpp:107),
 * through a Matcher that lives for the call. */
inline void MatchDescriptors(cv::Mat &desc_query, cv::Mat &desc_train, std::vector<std::vector<cv::DMatch>> &dmatches)
{
  libAKAZECU::Matcher m;
  m.bfmatch(desc_query, desc_train, dmatches);
}

#endif
