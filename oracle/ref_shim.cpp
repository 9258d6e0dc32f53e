// Test infrastructure: C entry points over the reference's own scale-space
// and evaluation code, src/lib/nldiffusion_functions.cpp and
// src/lib/utils.cpp, compiled in place from the reference tree by
// oracle/Makefile (target "ref") against the OpenCV-shaped headers in
// oracle/ref_shim/.  They let the tests compare the oracle's restatements
// with what the reference's code computes on the same planes:
//   pm_g2                 nldiffusion_functions.cpp:72-83
//   compute_k_percentile  nldiffusion_functions.cpp:121-201 (its Gaussian and
//                         Scharr run through the shim, i.e. the oracle's)
//   nld_step_scalar       nldiffusion_functions.cpp:213-317
//   gaussian_2D_convolution's kernel-size rule, :29-47 (recorded by the shim)
//   save_keypoints        utils.cpp:97-152
//   matches2points_nndr   utils.cpp:155-171
//   compute_inliers_homography  utils.cpp:203-243
// The cv:: functions below are the shim's: filters route to the oracle's
// plane routines, the rest throws.
#include <stdexcept>
#include <vector>

#include "nldiffusion_functions.h"
#include "opencv2/calib3d/calib3d.hpp"
#include "opencv2/imgproc/imgproc.hpp"
#include "utils.h"

extern "C" {
int ako_plane_gaussian(const float *src, float *dst, int w, int h, float sigma, int *ksize);
void ako_plane_scharr(const float *src, float *lx, float *ly, int w, int h);
void ako_plane_halfsample(const float *src, int sw, int sh, float *dst, int dw, int dh);
}

static int g_last_ksize_x = 0, g_last_ksize_y = 0;

namespace cv {
static void need_f32(const Mat &m, const char *what)
{
  if (m.type() != CV_32F) throw std::runtime_error(std::string(what) + ": the shim handles CV_32F planes only");
}

void GaussianBlur(const Mat &src, Mat &dst, Size ksize, double sigmaX, double sigmaY, int borderType)
{
  need_f32(src, "GaussianBlur");
  if (sigmaX != sigmaY || borderType != BORDER_REPLICATE) throw std::runtime_error("GaussianBlur: unsupported form");
  g_last_ksize_x = ksize.width;
  g_last_ksize_y = ksize.height;
  Mat out(src.rows, src.cols, CV_32F);
  int ks = 0;
  if (ako_plane_gaussian(src.ptr<float>(0), out.ptr<float>(0), src.cols, src.rows, (float)sigmaX, &ks) != 0)
    throw std::runtime_error("GaussianBlur: oracle failed");
  if (ks != ksize.width || ks != ksize.height)
    throw std::runtime_error("GaussianBlur: the reference's kernel size differs from the oracle's");
  dst = out;
}

void Scharr(const Mat &src, Mat &dst, int ddepth, int dx, int dy, double scale, double delta, int borderType)
{
  need_f32(src, "Scharr");
  if (ddepth != CV_32F || scale != 1.0 || delta != 0.0 || borderType != BORDER_DEFAULT || dx + dy != 1)
    throw std::runtime_error("Scharr: unsupported form");
  Mat lx(src.rows, src.cols, CV_32F), ly(src.rows, src.cols, CV_32F);
  ako_plane_scharr(src.ptr<float>(0), lx.ptr<float>(0), ly.ptr<float>(0), src.cols, src.rows);
  dst = dx ? lx : ly;
}

void sepFilter2D(const Mat &, Mat &, int, const Mat &, const Mat &)
{
  throw std::runtime_error("sepFilter2D: not provided by the shim");
}

void getDerivKernels(OutputArray, OutputArray, int, int, int, bool, int)
{
  throw std::runtime_error("getDerivKernels: not provided by the shim");
}

void resize(const Mat &src, Mat &dst, Size dsize, double, double, int interpolation)
{
  if (interpolation != INTER_AREA) throw std::runtime_error("resize: only INTER_AREA");
  need_f32(src, "resize");
  Mat out(dsize.height, dsize.width, CV_32F);
  ako_plane_halfsample(src.ptr<float>(0), src.cols, src.rows, out.ptr<float>(0), dsize.width, dsize.height);
  dst = out;
}

void circle(Mat &, Point, int, const Scalar &, int) { throw std::runtime_error("circle: drawing is not provided"); }
void line(Mat &, Point, Point, const Scalar &, int) { throw std::runtime_error("line: drawing is not provided"); }

Mat findHomography(const std::vector<Point2f> &, const std::vector<Point2f> &, int, double, Mat &)
{
  throw std::runtime_error("findHomography: not provided by the shim");
}
Mat findFundamentalMat(const std::vector<Point2f> &, const std::vector<Point2f> &, int, double, double, Mat &)
{
  throw std::runtime_error("findFundamentalMat: not provided by the shim");
}
}  // namespace cv

static cv::Mat wrap(const float *p, int w, int h) { return cv::Mat(h, w, CV_32F, const_cast<float *>(p)); }

extern "C" {

/* pm_g2 of the reference on (lx, ly) planes of w x h. */
int nldref_pm_g2(const float *lx, const float *ly, float *dst, int w, int h, float k)
{
  try {
    cv::Mat d = wrap(dst, w, h);
    pm_g2(wrap(lx, w, h), wrap(ly, w, h), d, k);
    return 0;
  } catch (...) {
    return -1;
  }
}

/* One nld_step_scalar of the reference, in place on Ld. */
int nldref_nld_step(float *Ld, const float *c, int w, int h, float stepsize)
{
  try {
    cv::Mat L = wrap(Ld, w, h), step = cv::Mat::zeros(h, w, CV_32F);
    nld_step_scalar(L, wrap(c, w, h), step, stepsize);
    return 0;
  } catch (...) {
    return -1;
  }
}

/* compute_k_percentile of the reference (ksize 0: its own kernel-size
 * rule); *ksize receives the kernel size it passed to GaussianBlur. */
float nldref_k_percentile(const float *img, int w, int h, float perc, float gscale, int nbins, int *ksize)
{
  try {
    g_last_ksize_x = g_last_ksize_y = 0;
    const float r = compute_k_percentile(wrap(img, w, h), perc, gscale, (size_t)nbins, 0, 0);
    if (ksize) *ksize = g_last_ksize_x == g_last_ksize_y ? g_last_ksize_x : -1;
    return r;
  } catch (...) {
    return -1.0f;
  }
}

/* gaussian_2D_convolution of the reference with ksize 0 (its own rule). */
int nldref_gaussian(const float *src, float *dst, int w, int h, float sigma, int *ksize)
{
  try {
    cv::Mat out;
    gaussian_2D_convolution(wrap(src, w, h), out, 0, 0, sigma);
    std::memcpy(dst, out.ptr<float>(0), sizeof(float) * (size_t)w * h);
    if (ksize) *ksize = g_last_ksize_x;
    return 0;
  } catch (...) {
    return -1;
  }
}

/* save_keypoints of the reference: kpts in the cv::KeyPoint layout, desc as
 * n x desc_cols bytes (CV_8U). */
int utilsref_save_keypoints(const char *path, const void *kpts, int n, const unsigned char *desc, int desc_cols, int save_desc)
{
  try {
    std::vector<cv::KeyPoint> k((size_t)n);
    if (n) std::memcpy(static_cast<void *>(k.data()), kpts, sizeof(cv::KeyPoint) * (size_t)n);
    cv::Mat d = desc_cols > 0 ? cv::Mat(n, desc_cols, CV_8U, const_cast<unsigned char *>(desc)) : cv::Mat();
    return save_keypoints(path, k, d, save_desc != 0);
  } catch (...) {
    return -2;
  }
}

/* matches2points_nndr + compute_inliers_homography of the reference, as
 * akaze_match.cpp:161-168 chains them.  matches: 2*nq cv::DMatch records
 * (best, second); kp_train / kp_query: the keypoint arrays the reference
 * calls train and query (it indexes train by queryIdx); H: 3x3 row-major
 * float.  pts receives the putative point pairs (x1, y1, x2, y2 per match),
 * inl the inlier pairs; returns the match count, *ninl the inlier count. */
int utilsref_nndr_inliers(const void *matches, int nq, const void *kp_train, int ntrain, const void *kp_query, int nquery,
                          const float *H, float nndr, float min_error, float *pts, float *inl, int *ninl)
{
  try {
    std::vector<std::vector<cv::DMatch>> m((size_t)nq, std::vector<cv::DMatch>(2));
    const cv::DMatch *mm = static_cast<const cv::DMatch *>(matches);
    for (int i = 0; i < nq; i++) m[i][0] = mm[2 * i], m[i][1] = mm[2 * i + 1];
    std::vector<cv::KeyPoint> tr((size_t)ntrain), qu((size_t)nquery);
    if (ntrain) std::memcpy(static_cast<void *>(tr.data()), kp_train, sizeof(cv::KeyPoint) * (size_t)ntrain);
    if (nquery) std::memcpy(static_cast<void *>(qu.data()), kp_query, sizeof(cv::KeyPoint) * (size_t)nquery);
    std::vector<cv::Point2f> pm, in;
    matches2points_nndr(tr, qu, m, pm, nndr);
    cv::Mat Hm(3, 3, CV_32F);
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) Hm.at<float>(r, c) = H[3 * r + c];
    compute_inliers_homography(pm, in, Hm, min_error);
    for (size_t i = 0; i < pm.size(); i++) pts[2 * i] = pm[i].x, pts[2 * i + 1] = pm[i].y;
    for (size_t i = 0; i < in.size(); i++) inl[2 * i] = in[i].x, inl[2 * i + 1] = in[i].y;
    *ninl = (int)(in.size() / 2);
    return (int)(pm.size() / 2);
  } catch (...) {
    return -1;
  }
}
}
