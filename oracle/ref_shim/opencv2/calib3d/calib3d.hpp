// Test infrastructure: RANSAC entry points named by the reference's
// utils.cpp; not used by the pinned functions and throw if called.
#ifndef AKO_REF_SHIM_CALIB3D_HPP
#define AKO_REF_SHIM_CALIB3D_HPP
#include <vector>
#include "../core/core.hpp"
namespace cv {
enum { RANSAC = 8, FM_RANSAC = 8 };
Mat findHomography(const std::vector<Point2f> &a, const std::vector<Point2f> &b, int method, double thr, Mat &mask);
Mat findFundamentalMat(const std::vector<Point2f> &a, const std::vector<Point2f> &b, int method, double thr, double conf,
                       Mat &mask);
}  // namespace cv
#endif
