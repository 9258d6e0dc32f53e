/*
 * akaze_oracle.h - CPU oracle for the A-KAZE detect + M-LDB describe + 2-NN
 * Hamming match path of francoto/akaze (libAKAZECU).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load this library, and only as the checker
 * (or as the timed CPU baseline).  The product library never links it.
 *
 * What it restates (file:line in the reference project):
 *   - level geometry and FED schedule: src/lib/AKAZE.cpp:146-197 and
 *     src/lib/fed.cpp:41-148 (pinned: the reference's own fed.cpp is compiled
 *     into oracle/_ref and compared in tests);
 *   - scale space (the reference's CPU functions): Gaussian
 *     src/lib/nldiffusion_functions.cpp:29-47, Scharr :50-53, pm_g2 :72-83,
 *     contrast percentile :121-201, FED step :213-317, half-sample :320-324,
 *     orchestration src/lib/AKAZE.cpp:211-276;
 *   - detector, suppression, orientation, M-LDB and matcher (no CPU code in
 *     the reference, so the CUDA math is restated): src/lib/cuda_akaze.cu
 *     :651-725, :727-806, :884-1070, :1074-1316, :2114-2167, :1420-1533,
 *     :1786-1807, :2034-2111, :1843-1967.
 *
 * Parity pinning: the FED schedule is pinned against the reference's compiled
 * fed.cpp.  The rest of the reference needs OpenCV (absent) and ships no golden
 * vectors, so the remaining stages are pinned only by hand-derived known-answer
 * tests; for those stages parity is "unpinned" beyond them.  OpenCV primitives
 * (GaussianBlur, Scharr, sepFilter2D, resize INTER_AREA, getGaussianKernel) are
 * restated from their documented semantics with a fixed evaluation order.
 */
#ifndef AKAZE_ORACLE_H
#define AKAZE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AKO_MAX_LEVELS 64

typedef struct {
  int omax;
  int nsublevels;
  float soffset;
  float derivative_factor;
  float sderivatives;
  int diffusivity; /* 0 PM_G1, 1 PM_G2, 2 WEICKERT, 3 CHARBONNIER */
  float dthreshold;
  float min_dthreshold;
  int descriptor; /* 4 MLDB_UPRIGHT, 5 MLDB */
  int descriptor_size;
  int descriptor_channels;
  int descriptor_pattern_size;
  float kcontrast_percentile;
  int kcontrast_nbins;
  int extrema_3d; /* 1: also a strict maximum over the adjacent levels of the octave */
} ako_options;

/* cv::KeyPoint layout (28 bytes). */
typedef struct {
  float x, y, size, angle, response;
  int32_t octave, class_id;
} ako_keypoint;

/* cv::DMatch layout (16 bytes). */
typedef struct {
  int32_t queryIdx, trainIdx, imgIdx;
  float distance;
} ako_dmatch;

typedef struct {
  int width, height, octave, sublevel;
  float esigma, etime;
  int deriv_step; /* sigma_size of the detector: fRound(esigma*df/2^o) */
  float size;     /* esigma * derivative_factor */
  float border;   /* extrema border */
  int nsteps;     /* FED steps from the previous level (0 for level 0) */
  float kcontrast;
} ako_level;

/* A raw scale-space extremum as the reference's FindExtrema writes it. */
typedef struct {
  int32_t x, y;     /* level coordinates */
  int32_t level, octave;
  float response;
  float size;       /* +-2*esigma*df, negative when the subpixel fit is weak */
  float octsub;     /* value stored in the float-punned octave field */
  float dst1;       /* value stored in the angle field (y offset) */
} ako_extremum;

typedef struct ako_ctx ako_ctx;

void ako_options_default(ako_options *o);
ako_ctx *ako_create(const ako_options *o, int width, int height);
void ako_destroy(ako_ctx *c);
void ako_set_threads(int n);

int ako_num_levels(const ako_ctx *c);
int ako_get_level(const ako_ctx *c, int level, ako_level *out);
int ako_get_tau(const ako_ctx *c, int level, float *tau, int cap);

/* fed.cpp:41-119 restated; returns n (0 on failure). */
int ako_fed_tau_by_process_time(float T, int M, float tau_max, int reordering, float *tau, int cap);
/* Gaussian taps used for sigma (nldiffusion_functions.cpp:29-47 size rule). */
int ako_gaussian_taps(float sigma, float *taps, int cap);

void ako_u8_to_unit(const uint8_t *src, float *dst, long n);

/* Scale space in FP32 (reference CPU semantics) and in FP64. img is HxW in [0,1]. */
int ako_build(ako_ctx *c, const float *img);
int ako_build_f64(ako_ctx *c, const float *img);
float ako_kcontrast(const ako_ctx *c);
double ako_kcontrast_f64(const ako_ctx *c);

enum { AKO_PLANE_LT = 0, AKO_PLANE_LSMOOTH = 1, AKO_PLANE_LFLOW = 2, AKO_PLANE_LX = 3, AKO_PLANE_LY = 4, AKO_PLANE_LDET = 5 };
int ako_get_plane(const ako_ctx *c, int level, int plane, float *out);
int ako_get_plane_f64(const ako_ctx *c, int level, double *out);

/* Detector + suppression + orientation; returns the number of keypoints. */
int ako_detect(ako_ctx *c);
int ako_num_extrema(const ako_ctx *c);
int ako_get_extrema(const ako_ctx *c, ako_extremum *out, int cap);
int ako_get_level_offsets(const ako_ctx *c, int *out, int cap);
int ako_get_nms_state(const ako_ctx *c, int *out, int cap);
int ako_num_keypoints(const ako_ctx *c);
int ako_get_keypoints(const ako_ctx *c, ako_keypoint *out, int cap);

/* M-LDB descriptors, 61 bytes per keypoint. */
int ako_describe(ako_ctx *c);
int ako_get_descriptors(const ako_ctx *c, uint8_t *out, int cap_rows);
/* bytes of one descriptor row after ako_describe */
int ako_descriptor_bytes(const ako_ctx *c);
/* the M-LDB comparison table (value indices 3*cell + channel) for channels
 * 1..3 and a descriptor_size (0: the full descriptor); returns its bits */
int ako_mldb_table(int channels, int nbits_subset, int *c1, int *c2);
/* the first n outputs of the GNU C library's rand() after srand(seed) */
int ako_glibc_rand_sequence(uint32_t seed, int *out, int n);

/* Whole path on one u8 image (timed CPU baseline). Returns keypoints or <0. */
int ako_run_u8(ako_ctx *c, const uint8_t *img);

/* Brute-force 2-NN Hamming match: out has 2*nq entries. */
int ako_bfmatch(const uint8_t *q, int nq, const uint8_t *t, int nt, int row_bytes, ako_dmatch *out);

/* The shared deterministic float routines (akaze_gb300/csrc/akz_fmath.h). */
float ako_atan2f(float y, float x);
void ako_sincosf(float x, float *s, float *c);
float ako_expf(float x);
float ako_recip1pf(float f);
/* The 486 M-LDB comparison pairs (value index cell*3+channel), bit order. */
int ako_descriptor_pairs(int *i1, int *i2);

#ifdef __cplusplus
}
#endif
#endif
