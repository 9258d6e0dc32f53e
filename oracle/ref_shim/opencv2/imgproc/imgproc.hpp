// Test infrastructure: the imgproc calls of the reference's
// nldiffusion_functions.cpp and utils.cpp, implemented in ref_shim.cpp by the
// oracle's own filters (see core.hpp).
#ifndef AKO_REF_SHIM_IMGPROC_HPP
#define AKO_REF_SHIM_IMGPROC_HPP
#include "../core/core.hpp"
namespace cv {
void GaussianBlur(const Mat &src, Mat &dst, Size ksize, double sigmaX, double sigmaY, int borderType);
void Scharr(const Mat &src, Mat &dst, int ddepth, int dx, int dy, double scale, double delta, int borderType);
void sepFilter2D(const Mat &src, Mat &dst, int ddepth, const Mat &kx, const Mat &ky);
void getDerivKernels(OutputArray kx, OutputArray ky, int dx, int dy, int ksize, bool normalize, int ktype);
void resize(const Mat &src, Mat &dst, Size dsize, double fx, double fy, int interpolation);
void circle(Mat &img, Point center, int radius, const Scalar &color, int thickness);
void line(Mat &img, Point a, Point b, const Scalar &color, int thickness);
}  // namespace cv
#endif
