// Test infrastructure: cv::KeyPoint and cv::DMatch with OpenCV's field
// layout, for the reference's utils.cpp (see core.hpp).
#ifndef AKO_REF_SHIM_FEATURES2D_HPP
#define AKO_REF_SHIM_FEATURES2D_HPP
#include "../core/core.hpp"
namespace cv {
class KeyPoint {
 public:
  Point2f pt;
  float size = 0, angle = -1, response = 0;
  int octave = 0, class_id = -1;
};
struct DMatch {
  int queryIdx = -1, trainIdx = -1, imgIdx = -1;
  float distance = 0;
};
}  // namespace cv
#endif
