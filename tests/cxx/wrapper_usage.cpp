// Code written against the reference's libAKAZECU class API (the pattern of
// its akaze_features.cpp / akaze_match.cpp demos), compiled against
// include/libAKAZECU/AKAZE.h.  Built and linked on the CPU; main() is not
// run there (it needs a GPU).
#include <cstdio>
#include <vector>

#include "libAKAZECU/AKAZE.h"

int main(int argc, char **)
{
  if (argc < 2) return 0;
  const int w = 640, h = 480;
  std::vector<float> pixels((size_t)w * h, 0.5f);
  cv::Mat img_32(h, w, cv::CV_32F, pixels.data());

  AKAZEOptions options;
  options.setWidth(w);
  options.setHeight(h);
  libAKAZECU::AKAZE evolution(options);
  evolution.Create_Nonlinear_Scale_Space(img_32);
  std::vector<cv::KeyPoint> kpts;
  evolution.Feature_Detection(kpts);
  cv::Mat desc;
  evolution.Compute_Descriptors(kpts, desc);
  AKAZETiming t = evolution.Get_Computation_Times();
  evolution.Show_Computation_Times();

  libAKAZECU::Matcher matcher;
  std::vector<std::vector<cv::DMatch>> dmatches;
  matcher.bfmatch(desc, desc, dmatches);
  std::printf("%zu keypoints, %zu query rows, %.3f ms\n", kpts.size(), dmatches.size(), t.scale + t.detector + t.descriptor);
  return 0;
}
