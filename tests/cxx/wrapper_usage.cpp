// Code in the dialect of the reference's demos (src/akaze_features.cpp:55-107
// and :250-275, src/akaze_match.cpp:100-138): `using namespace libAKAZECU`,
// DESCRIPTOR_TYPE / DIFFUSIVITY_TYPE casts from the command line, the
// options printed with operator<<, unqualified CV_32F / CV_8UC1 macros,
// convertTo(img_32, CV_32F, 1.0 / 255.0, 0), the class API, the Matcher and
// the MatchDescriptors free function.  Compiled against
// include/libAKAZECU/AKAZE.h twice: with its own cv subset, and with
// AKZ_WITH_OPENCV against an OpenCV-shaped header.  Without --run it only
// parses the options and prints them (no GPU call), so the CPU tests can
// run it.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <vector>

#include "libAKAZECU/AKAZE.h"

using namespace std;
using namespace libAKAZECU;

static int parse_input_options(AKAZEOptions &options, int argc, char *argv[])
{
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "--descriptor")) {
      if (++i >= argc) return -1;
      options.descriptor = DESCRIPTOR_TYPE(atoi(argv[i]));
      if (options.descriptor < 0 || options.descriptor > MLDB) options.descriptor = MLDB;
    } else if (!strcmp(argv[i], "--diffusivity")) {
      if (++i >= argc) return -1;
      options.diffusivity = DIFFUSIVITY_TYPE(atoi(argv[i]));
    } else if (!strcmp(argv[i], "--descriptor_channels")) {
      if (++i >= argc) return -1;
      options.descriptor_channels = atoi(argv[i]);
    } else if (!strcmp(argv[i], "--descriptor_size")) {
      if (++i >= argc) return -1;
      options.descriptor_size = atoi(argv[i]);
    } else if (!strcmp(argv[i], "--omax")) {
      if (++i >= argc) return -1;
      options.omax = atoi(argv[i]);
    } else if (!strcmp(argv[i], "--verbose")) {
      options.verbosity = true;
    }
  }
  return 0;
}

int main(int argc, char *argv[])
{
  AKAZEOptions options;
  setDefaultAKAZEOptions(options);
  if (parse_input_options(options, argc, argv)) return -1;
  const bool run = argc > 1 && !strcmp(argv[argc - 1], "--run");
  if (options.verbosity || !run) {
    cout << "Check AKAZE options:" << endl;
    cout << options << endl;
  }
  if (options.diffusivity != PM_G2 && options.descriptor == MLDB_UPRIGHT) cout << "upright, other diffusivity" << endl;
  if (!run) return 0;

  // A 640x480 gray ramp with a bright square, converted as the demos do.
  cv::Mat img(480, 640, CV_8UC1);
  for (int y = 0; y < img.rows; y++)
    for (int x = 0; x < img.cols; x++) img.ptr(y)[x] = (unsigned char)((x / 4 + y / 8 + ((x / 40 + y / 40) % 2) * 90) & 255);
  cv::Mat img_32;
  img.convertTo(img_32, CV_32F, 1.0 / 255.0, 0);

  options.img_width = img.cols;
  options.img_height = img.rows;
  AKAZE evolution(options);
  vector<cv::KeyPoint> kpts;
  evolution.Create_Nonlinear_Scale_Space(img_32);
  evolution.Feature_Detection(kpts);
  cv::Mat desc;
  evolution.Compute_Descriptors(kpts, desc);
  evolution.Show_Computation_Times();
  AKAZETiming t = evolution.Get_Computation_Times();

  std::vector<std::vector<cv::DMatch> > dmatches;
  MatchDescriptors(desc, desc, dmatches);
  Matcher cuda_matcher;
  cuda_matcher.bfmatch(desc, desc, dmatches);
  cv::Mat m = cuda_matcher.bfmatch_(desc, desc);
  int self = 0;
  for (size_t i = 0; i < dmatches.size(); i++) self += dmatches[i][0].distance == 0;
  printf("%zu keypoints, %d x %d descriptors, %d self matches, %d x %d match rows, %.3f ms\n", kpts.size(), desc.rows,
         desc.cols, self, m.rows, m.cols, t.scale + t.detector + t.descriptor);
  return self == (int)kpts.size() ? 0 : 1;
}
