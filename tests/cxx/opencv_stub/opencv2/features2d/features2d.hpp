// Minimal stand-in with the shape of OpenCV's cv::KeyPoint and cv::DMatch
// (field order and types), for compiling include/libAKAZECU/AKAZE.h's
// AKZ_WITH_OPENCV branch without OpenCV.  Not a reimplementation of OpenCV.
#ifndef AKZ_TEST_OPENCV_STUB_FEATURES2D_HPP
#define AKZ_TEST_OPENCV_STUB_FEATURES2D_HPP
#include "../core/core.hpp"
namespace cv {
class KeyPoint {
 public:
  KeyPoint() : pt(0, 0), size(0), angle(-1), response(0), octave(0), class_id(-1) {}
  Point2f pt;
  float size, angle, response;
  int octave, class_id;
};
struct DMatch {
  DMatch() : queryIdx(-1), trainIdx(-1), imgIdx(-1), distance(0) {}
  int queryIdx, trainIdx, imgIdx;
  float distance;
};
}  // namespace cv
#endif
