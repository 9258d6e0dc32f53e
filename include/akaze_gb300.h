/*
 * akaze_gb300.h - C ABI of the GB300 A-KAZE library (libakaze_gb300.so).
 *
 * Drop-in boundary for the libAKAZECU API of francoto/akaze
 * (src/lib/AKAZE.h, src/lib/AKAZEConfig.h): plain pointers and sizes, every
 * call returns an akz_status and never exits the process (the reference's
 * safeCall exits, src/lib/cudautils.h:15-20).  A header-only C++ wrapper with
 * the reference's class signatures lives in include/libAKAZECU/AKAZE.h.
 *
 * Threading: contexts, batches and matchers are independent; each owns its
 * device memory and its stream.  One object must not be used from two host
 * threads at once.
 */
#ifndef AKAZE_GB300_H
#define AKAZE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define AKZ_API __attribute__((visibility("default")))
#else
#define AKZ_API
#endif

typedef enum akz_status {
  AKZ_OK = 0,
  AKZ_ERR_INVALID_ARG = 1,
  AKZ_ERR_OOM = 2,
  AKZ_ERR_CUDA = 3,
  AKZ_ERR_OVERFLOW = 4,   /* more raw extrema than maxkeypoints: reported, never silently capped */
  AKZ_ERR_TIMEOUT = 5,    /* a bounded device loop gave up */
  AKZ_ERR_UNSUPPORTED = 6,
  AKZ_ERR_STATE = 7       /* call order (e.g. descriptors before detection) */
} akz_status;

/* DIFFUSIVITY_TYPE, AKAZEConfig.h:52-57 */
enum { AKZ_PM_G1 = 0, AKZ_PM_G2 = 1, AKZ_WEICKERT = 2, AKZ_CHARBONNIER = 3 };
/* DESCRIPTOR_TYPE, AKAZEConfig.h:41-48 (MLDB and MLDB_UPRIGHT are implemented) */
enum { AKZ_SURF_UPRIGHT = 0, AKZ_SURF = 1, AKZ_MSURF_UPRIGHT = 2, AKZ_MSURF = 3, AKZ_MLDB_UPRIGHT = 4, AKZ_MLDB = 5 };
/* input pixel types */
enum { AKZ_U8 = 0, AKZ_F32 = 1 };
/* planes of a scale-space level (for inspection) */
enum { AKZ_PLANE_LT = 0, AKZ_PLANE_LSMOOTH = 1, AKZ_PLANE_LX = 3, AKZ_PLANE_LY = 4 };

/* AKAZEOptions, AKAZEConfig.h:84-172, field for field (bool fields as int). */
typedef struct akz_options {
  int omin;
  int omax;
  int nsublevels;
  int img_width;
  int img_height;
  float soffset;
  float derivative_factor;
  float sderivatives;
  int diffusivity;
  float dthreshold;
  float min_dthreshold;
  int descriptor;
  int descriptor_size;
  int descriptor_channels;
  int descriptor_pattern_size;
  float kcontrast;
  float kcontrast_percentile;
  size_t kcontrast_nbins;
  int save_scale_space;
  int save_keypoints;
  int verbosity;
  int ncudaimages;
  int maxkeypoints; /* capacity of raw extrema per image */
  /* Extension (no AKAZEOptions field): the scale-space extrema rule.
   * 0 (default): the reference's FindExtrema (cuda_akaze.cu:727-774), a strict
   *   maximum over the 8 neighbours in the level, above the threshold.
   * 1: also a strict maximum over the 3 x 3 neighbourhoods of the level below
   *   and the level above in the same octave (26 neighbours; the first and
   *   last sublevel of an octave compare with the one adjacent level they
   *   have), the rule for which the reference passes, and leaves unused, the
   *   adjacent levels to FindExtrema (AKAZE.cpp:340-367, cuda_akaze.cu:727). */
  int extrema_3d;
  /* Extension: the arithmetic of the scale-space and detector kernels.
   * 0 (default): every float operation in the reference's order, rounded on
   *   its own, the PM-g2 reciprocal exactly as the reference's double
   *   division rounds (bit-identical to the CPU restatement).
   * 1: fused multiply-adds and the hardware reciprocal in those kernels; the
   *   results stay within levels 1e-4 relative, >= 99% of keypoints within
   *   0.5 px at the same level and descriptors within Hamming 2 of the
   *   reference arithmetic (tests/test_gpu_fast_math.py). */
  int fast_math;
} akz_options;

/* cv::KeyPoint layout (28 bytes): pt.x, pt.y, size, angle, response, octave, class_id. */
typedef struct akz_keypoint {
  float x, y, size, angle, response;
  int32_t octave, class_id;
} akz_keypoint;

/* cv::DMatch layout (16 bytes). */
typedef struct akz_dmatch {
  int32_t queryIdx, trainIdx, imgIdx;
  float distance;
} akz_dmatch;

/* AKAZETiming, AKAZEConfig.h:61-80 (milliseconds, device time of each stage). */
typedef struct akz_timing {
  double kcontrast, scale, derivatives, detector, extrema, subpixel, descriptor;
} akz_timing;

/* A raw scale-space extremum as the reference's FindExtrema stores it
 * (cuda_akaze.cu:758-769), before suppression; for inspection. */
typedef struct akz_extremum {
  int32_t x, y, level, octave;
  float response, size, octsub, dst1;
} akz_extremum;

typedef struct akz_context akz_context;
typedef struct akz_batch akz_batch;
typedef struct akz_matcher akz_matcher;

AKZ_API const char *akz_version(void);
/* Message of the last failing call on this host thread. */
AKZ_API const char *akz_last_error(void);

/* setDefaultAKAZEOptions / AKAZEOptions::AKAZEOptions (AKAZEConfig.h:86-111). */
AKZ_API akz_status akz_options_default(akz_options *opt);

/* Bytes of one descriptor row for the options, as Compute_Descriptors sizes
 * its output (AKAZE.cpp:412-423): ceil((6 + 36 + 120) * descriptor_channels
 * / 8) for the full M-LDB (21, 41 or 61), ceil(descriptor_size / 8) for the
 * random-bit subset.  On the device every row is 64 bytes, zero-padded. */
AKZ_API akz_status akz_descriptor_bytes(const akz_options *opt, int *bytes);

/* Level plan of an image, computed on the host without touching the GPU
 * (AKAZE.cpp:146-197, fed.cpp:41-148): level count, and for level >= 0 its
 * size, octave, sublevel, evolution sigma, detector step, extrema border and
 * FED step sizes (tau, up to tau_cap) that lead to it.  No counterpart in the
 * reference, which keeps the plan private. */
AKZ_API akz_status akz_plan_info(const akz_options *opt, int width, int height, int level, int *nlevels, int *lw,
                                 int *lh, int *octave, int *sublevel, float *esigma, int *deriv_step, float *border,
                                 float *tau, int tau_cap, int *nsteps);
/* Gaussian taps the library uses for sigma (nldiffusion_functions.cpp:33-43
 * kernel-size rule), for inspection. */
AKZ_API akz_status akz_gaussian_taps(float sigma, float *taps, int cap, int *ntaps);

/* ---- single image: libAKAZECU::AKAZE (AKAZE.h:58-143) ---------------- */

/* AKAZE::AKAZE(options) + Allocate_Memory_Evolution (AKAZE.cpp:126-208):
 * level geometry for options.img_width x img_height, device memory.  Image
 * sides from 16 to 32768 pixels; others are AKZ_ERR_INVALID_ARG (here and in
 * akz_batch_create). */
AKZ_API akz_status akz_create(const akz_options *opt, akz_context **out);
/* AKAZE::~AKAZE (AKAZE.cpp:140-143). */
AKZ_API akz_status akz_destroy(akz_context *ctx);
/* Run on a caller stream (cudaStream_t); NULL restores the context's own. */
AKZ_API akz_status akz_set_stream(akz_context *ctx, void *stream);
/* AKAZE::Create_Nonlinear_Scale_Space (AKAZE.cpp:211-276). img: width x height
 * pixels of AKZ_U8 (0..255) or AKZ_F32 (0..1), rows stride_bytes apart, in host
 * memory (on_device = 0) or device memory (on_device = 1). The size must equal
 * the size the context was created for. */
AKZ_API akz_status akz_create_nonlinear_scale_space(akz_context *ctx, const void *img, int width, int height,
                                                    size_t stride_bytes, int dtype, int on_device);
/* AKAZE::Feature_Detection (AKAZE.cpp:316-378): detector, extrema,
 * suppression; returns the number of keypoints. */
AKZ_API akz_status akz_feature_detection(akz_context *ctx, int *nkeypoints);
/* AKAZE::Compute_Descriptors (AKAZE.cpp:405-449): orientation + M-LDB;
 * copies min(n, capacity) keypoints and descriptor rows of
 * akz_descriptor_bytes() bytes (61 for the default options) to host memory
 * (either pointer may be NULL) and returns n. */
AKZ_API akz_status akz_compute_descriptors(akz_context *ctx, akz_keypoint *kpts, uint8_t *desc, int capacity, int *nkeypoints);
/* AKAZE::Get_Computation_Times (AKAZE.h:140-142). */
AKZ_API akz_status akz_get_timing(akz_context *ctx, akz_timing *t);

/* Inspection of the scale space and detector of a context. */
AKZ_API akz_status akz_num_levels(const akz_context *ctx, int *nlevels);
AKZ_API akz_status akz_level_info(const akz_context *ctx, int level, int *width, int *height, int *octave, int *sublevel,
                                  float *esigma, int *nsteps);
AKZ_API akz_status akz_get_level_plane(akz_context *ctx, int level, int plane, float *out);
AKZ_API akz_status akz_get_kcontrast(akz_context *ctx, float *kcontrast);
AKZ_API akz_status akz_get_extrema(akz_context *ctx, akz_extremum *out, int capacity, int *n);

/* ---- many images per launch (persistent, graph-replayed stages) -------- */

/* A batch of nimages images (1 .. 4096) of the given sizes (each >= 8x8),
 * processed by one launch per stage. */
AKZ_API akz_status akz_batch_create(const akz_options *opt, int nimages, const int *widths, const int *heights, akz_batch **out);
AKZ_API akz_status akz_batch_destroy(akz_batch *b);
AKZ_API akz_status akz_batch_set_stream(akz_batch *b, void *stream);
/* Copy u8 images (host pointers, rows strides[i] bytes apart; on_device = 1
 * for device pointers) into the batch's device staging. Asynchronous. */
AKZ_API akz_status akz_batch_upload(akz_batch *b, const uint8_t *const *images, const size_t *strides, int on_device);
/* Device address of image i's staging area (u8, pitch in bytes), for
 * producers that write the input on the device themselves. */
AKZ_API akz_status akz_batch_input(akz_batch *b, int i, uint8_t **dptr, size_t *pitch);
/* Detect + describe every staged image. Asynchronous on the batch stream. */
AKZ_API akz_status akz_batch_run(akz_batch *b);
/* Per-image keypoint counts (synchronises the stream). */
AKZ_API akz_status akz_batch_counts(akz_batch *b, int *counts);
/* Copy image i's keypoints and descriptor rows (akz_descriptor_bytes()
 * bytes each) to host memory (sync). */
AKZ_API akz_status akz_batch_results(akz_batch *b, int i, akz_keypoint *kpts, uint8_t *desc, int capacity, int *n);
/* Device addresses of image i's keypoints and 64-byte descriptor rows. */
AKZ_API akz_status akz_batch_device_results(akz_batch *b, int i, akz_keypoint **kpts, uint8_t **desc64);
/* Whole job: upload (host u8), run, counts, copy results out. */
AKZ_API akz_status akz_batch_detect_describe(akz_batch *b, const uint8_t *const *images, const size_t *strides,
                                             akz_keypoint *const *kpts, uint8_t *const *desc, const int *capacities,
                                             int *counts);
/* Scale-space level plane of image i (inspection). */
AKZ_API akz_status akz_batch_level_plane(akz_batch *b, int i, int level, int plane, float *out);
/* Number of kernels one akz_batch_run launches (no counterpart in the
 * reference; for launch accounting). */
AKZ_API akz_status akz_batch_kernel_count(const akz_batch *b, int *n);
/* One run without graph replay, timed per stage group with CUDA events on the
 * batch stream (no counterpart in the reference; the AKAZETiming of a batch):
 * stage_ms[0..6] = contrast, level 0, levels >= 1, detector, scan+extract,
 * suppression, orientation+M-LDB. Synchronises. */
AKZ_API akz_status akz_batch_profile(akz_batch *b, float *stage_ms, int n);

/* ---- matcher: libAKAZECU::Matcher (AKAZE.h:29-55) ---------------------- */

AKZ_API akz_status akz_matcher_create(akz_matcher **out);
AKZ_API akz_status akz_matcher_destroy(akz_matcher *m);
AKZ_API akz_status akz_matcher_set_stream(akz_matcher *m, void *stream);
/* Matcher::bfmatch (AKAZE.cpp:36-79): nq x row_bytes query rows against
 * nt x row_bytes train rows (host memory, row_bytes <= 64, zero-padded to
 * 64 bytes on the device); out receives 2*nq matches, best then second. */
AKZ_API akz_status akz_matcher_bfmatch(akz_matcher *m, const uint8_t *query, int nq, const uint8_t *train, int nt,
                                       int row_bytes, akz_dmatch *out);
/* Same on device buffers of 64-byte rows; out is device memory of 2*nq. */
AKZ_API akz_status akz_matcher_bfmatch_device(akz_matcher *m, const uint8_t *query64, int nq, const uint8_t *train64,
                                              int nt, akz_dmatch *out);

/* Allocation-free variant of akz_matcher_bfmatch_device (no counterpart in
 * the reference).  For callers that cannot allocate device memory, such as a
 * plugin inside a host that owns the whole device memory budget or a hot
 * path where cudaMalloc would synchronise: query64 (nq x 64 B), train64
 * (nt x 64 B) and out (2*nq matches) are caller-provided device buffers; the
 * scratch is a fixed 2 MiB device array inside the library, held by every
 * GPU that loads it until exit.  At most 131072 query rows per call (larger
 * nq returns AKZ_ERR_INVALID_ARG).  The first call on a device resolves the
 * array's address and keeps it for the life of the process; make that first
 * call before any stream capture, and do not call this entry point again
 * after a cudaDeviceReset in the same process (the kept address would then
 * be stale).  Calls
 * share the array, so calls that overlap on the GPU race: serialise them.
 * Runs on stream (a cudaStream_t; NULL for the legacy default stream) and
 * returns without synchronising. */
AKZ_API akz_status akz_matcher_bfmatch_noalloc(const uint8_t *query64, int nq, const uint8_t *train64, int nt,
                                              akz_dmatch *out, void *stream);

/* Pair-distance engine of the matcher calls above with at least 2^20 pairs
 * and 128 train rows (no counterpart in the reference; process-wide):
 * on = 1 (default) forms the distances with tcgen05 FP8 matrix multiplies,
 * popc(q) + sum_k b_k (1 - 2 a_k) exact in FP32, on = 0 with 16 xor + popc
 * per pair.  Both give the same matches bit for bit.
 * akz_matcher_tensor_status reports (and clears) whether a tensor-core
 * matcher kernel gave up waiting for its MMAs (synchronous). */
AKZ_API akz_status akz_matcher_set_tensor_cores(int on);
AKZ_API akz_status akz_matcher_tensor_status(int *timed_out);

/* Measurement helper for the matcher's roofline (no counterpart in the
 * reference, whose README.md:22 publishes no matcher figure): the sustained
 * rate of 32-bit (xor, popc, add) triples on the current GPU, from one timed
 * launch of iters iterations x 8 chains per thread on every SM.  A pair of
 * 64-byte rows costs 16 triples, so the matcher's peak in pairs/s is
 * *triples_per_s / 16.  Synchronises stream; allocates 4 bytes. */
AKZ_API akz_status akz_measure_popc_rate(int iters, double *triples_per_s, void *stream);

/* Self-check of the bounded mbarrier wait that the level kernel uses for its
 * TMA input and the tcgen05 kernels for their MMAs: one CTA polls an
 * mbarrier at most spin times.  With arrive = 0 nothing completes the
 * barrier and the wait must give up (*timed_out = 1); with arrive = 1 the
 * CTA's first thread completes it and the wait must succeed (*timed_out =
 * 0).  Synchronous; no fault, no hang. */
AKZ_API akz_status akz_selfcheck_bounded_wait(int arrive, int spin, int *timed_out);

/* Self-check of the tensor-core matcher's failure path (no counterpart in
 * the reference): one launch whose MMA warp issues nothing, with at most
 * spin polls per wait, so the wait for the first MMA batch runs out.
 * *timed_out = 1 when the kernel flagged it (and freed its tensor memory);
 * later matcher calls work as before.  Synchronous; allocates 40 KB; no
 * fault, no hang. */
AKZ_API akz_status akz_selfcheck_matcher_timeout(int spin, int *timed_out);

/* ------------------------------------------------------------------------ */
/* Learned FED surrogate (no counterpart in the reference; it replaces the
 * FED cycle of AKAZE.cpp:244-270 for octaves >= 1 when enabled).  A 5-layer
 * 3x3 convolutional net 3 -> 32 -> 32 -> 32 -> 32 -> 1 with ReLU maps a
 * level's starting image, its conductance and a feature of the level's FED
 * time span to the residual L_end - L_start, scaled by s_out.
 *
 * Training kernels, FP32 NCHW tensors on the device, valid convolutions,
 * weights [cout][cin][3][3], 1 <= cin, cout <= 32: */
AKZ_API akz_status akz_sg_conv_forward(const float *in, const float *w, const float *bias, float *out, int nb, int cin,
                                      int cout, int hi, int wi, int relu, void *stream);
/* din = (mask > 0) * dL/d(in); mask NULL for no ReLU factor */
AKZ_API akz_status akz_sg_conv_backward_data(const float *dout, const float *w, const float *mask, float *din, int nb,
                                            int cin, int cout, int hi, int wi, void *stream);
/* dw, db overwritten with the gradients summed over the batch */
AKZ_API akz_status akz_sg_conv_backward_weights(const float *in, const float *dout, float *dw, float *db, int nb, int cin,
                                               int cout, int hi, int wi, void *stream);
AKZ_API akz_status akz_sg_adam(float *param, const float *grad, float *m, float *v, int n, float lr, float beta1,
                              float beta2, float eps, int step, void *stream);
/* dout = scale * (out - target); loss_parts[0 .. nparts-1] receive partial
 * sums of (out - target)^2 */
AKZ_API akz_status akz_sg_mse_grad(const float *out, const float *target, float *dout, int n, float scale,
                                  float *loss_parts, int nparts, void *stream);

/* Inference on one level plane (BF16 tensor cores, FP32 accumulation),
 * replicate border: out = l0 + s_out * net(l0, g, dt_feature).  l0, g, out
 * are float planes with row pitch `pitch` elements; weights_bf16 holds
 * akz_sg_weight_elems() bf16 values (layer 1 [32][32] over the im2col index
 * tap*3 + channel, layers 2-4 [32][288] over tap*32 + ci, layer 5 [8][288]
 * with rows 1-7 zero), biases 4 x 32 + 8 floats; scratch holds
 * 2 * width * height * 64 bytes.  Weights and scratch 16-byte aligned.
 * Asynchronous on stream. */
AKZ_API size_t akz_sg_weight_elems(void);
/* Run the three 3 x 3 32 -> 32 layers of akz_sg_infer_level on tcgen05
 * tensor cores (persistent CTAs, a ring of input rows, TMEM accumulators,
 * one elected thread issuing the MMAs; on by default) or on mma.sync (0);
 * process-wide.  akz_sg_tcgen05_status reports (and clears) whether any of
 * those kernels gave up waiting for its MMAs. */
AKZ_API akz_status akz_sg_set_tcgen05(int on);
AKZ_API akz_status akz_sg_tcgen05_status(int *timed_out);

/* Use the surrogate for every level of octave >= first_octave of a batch
 * (weights_bf16 NULL: plain FED again).  weights_bf16 / biases are host
 * arrays in the layout of akz_sg_infer_level.  Per such level and image:
 * a zero-step FED launch forms Lsmooth, the conductance and the start image,
 * then the net writes the level.  With check_tol > 0, image 0's level is also
 * computed by plain FED and compared; if the max difference exceeds
 * check_tol (or is not finite), the level falls back to plain FED for every
 * image, decided on the device.  Rebuilds the batch's graph on the next run. */
AKZ_API akz_status akz_batch_set_surrogate(akz_batch *b, const uint16_t *weights_bf16, const float *biases, float s_out,
                                           int first_octave, float check_tol);
/* After a run: per level, image 0's max |surrogate - plain FED| (0 where no
 * check ran); *nlevels receives the level count. */
AKZ_API akz_status akz_batch_surrogate_errors(akz_batch *b, float *err, int cap, int *nlevels);
AKZ_API akz_status akz_sg_infer_level(const float *l0, const float *g, size_t pitch, int width, int height,
                                     float dt_feature, float s_out, const void *weights_bf16, const float *biases,
                                     void *scratch, float *out, void *stream);

/* Autotuner of the FED temporal-blocking depth (FED steps per level-kernel
 * launch, 4..8; no counterpart in the reference): on the uploaded images,
 * times every level of the scale-space stage at each depth and keeps the
 * fastest depth per level for later runs.  ms_per_depth (cap entries, may be
 * NULL) receives the stage time with every level at depth 4, 5, ...;
 * depths (ndepths entries, may be NULL) the depth chosen per level (0 for
 * level 0, -1 past the batch's last level).  Synchronises the batch's stream. */
AKZ_API akz_status akz_batch_autotune(akz_batch *b, float *ms_per_depth, int cap, int *depths, int ndepths);

/* Sets the FED blocking depth (4..8; 8 at creation) without timing. */
AKZ_API akz_status akz_batch_set_fed_depth(akz_batch *b, int depth);

/* Diagnostics of image i after a run (no counterpart in the reference):
 * raw extrema before suppression, keypoints after it, suppression rounds,
 * and the contrast factor.  Any pointer may be NULL; synchronises the
 * batch's stream. */
AKZ_API akz_status akz_batch_image_info(akz_batch *b, int i, int *nraw, int *nkp, int *rounds, float *kcontrast);

/* Cap on the suppression rounds of every image (default 2^20, far above the
 * n rounds the loop needs for n raw extrema).  An image that needs more
 * rounds stops suppressing and its results report AKZ_ERR_TIMEOUT; the batch
 * stays usable.  cap >= 1. */
AKZ_API akz_status akz_batch_set_nms_round_cap(akz_batch *b, int cap);

/* The two halves of akz_batch_detect_describe_packed, for overlapping
 * several batches (each on its own stream) and consecutive runs of one
 * batch from one host thread: akz_batch_submit enqueues the upload of the
 * host images, the batch's graph, the packing of its keypoints and
 * descriptor rows on the device and the read-back of the per-image counts,
 * and returns at once; akz_batch_collect_packed waits for the oldest
 * submitted run only and copies its packed results (on a copy stream of
 * the batch, so that a run submitted after it keeps computing).  Up to two
 * runs may be outstanding: the second one's upload and graph queue behind
 * the first on the batch's stream.  A third submit, or a collect without a
 * submit, is AKZ_ERR_STATE; akz_batch_detect_describe_packed needs no run
 * outstanding.  The host images of a run must stay unchanged until it is
 * collected.  The first submit allocates two result slots of maxkeypoints
 * rows per image (keypoint record + descriptor row each) and a second input
 * staging buffer: consecutive runs alternate between the two, each with its
 * own captured graph, so that a run's upload overlaps the run before it. */
AKZ_API akz_status akz_batch_submit(akz_batch *b, const uint8_t *const *images, const size_t *strides);
AKZ_API akz_status akz_batch_collect_packed(akz_batch *b, akz_keypoint *kpts, uint8_t *desc, int capacity, int *counts,
                                            int *total);

/* akz_batch_detect_describe with packed host output: kpts (capacity
 * records) and desc (capacity x akz_descriptor_bytes() bytes) receive every image's keypoints
 * and descriptors back to back, image i starting at row sum_{j<i} counts[j];
 * counts[i] receives image i's count and *total their sum.  If the sum
 * exceeds capacity nothing is copied and AKZ_ERR_OVERFLOW is returned (call
 * again with *total rows).  Two device-to-host copies per call. */
AKZ_API akz_status akz_batch_detect_describe_packed(akz_batch *b, const uint8_t *const *images, const size_t *strides,
                                                    akz_keypoint *kpts, uint8_t *desc, int capacity, int *counts,
                                                    int *total);

/* Self-check of the device's exact PM-g2 reciprocal (no counterpart in the
 * reference): out[i] = (float)(1 / (1 + (double)in[i])) as the level kernel
 * computes it, by its two-pixel routine (fn 0) or the scalar one (fn 1).
 * Device buffers; asynchronous on stream.  For tests of that exactness. */
AKZ_API akz_status akz_selfcheck_pm_g2(const float *in, float *out, int n, int fn, void *stream);

/* ---- evaluation and output ---------------------------------------------- */

/* NNDR matches and homography inliers of a 2-NN result, on the device:
 * matches2points_nndr + compute_inliers_homography (utils.cpp:154-243) as
 * akaze_match.cpp:161-168 uses them (nndr 0.8, min_error 2.5 there).
 * matches: 2*nq records as akz_matcher_bfmatch_device writes them (query i's
 * best, then second best); kp_query / kp_train: the keypoints of the query
 * and train images; H: 3x3 row-major homography (host) mapping query points
 * to train points.  status[i] = 0 (no NNDR match), 1 (match) or 2 (match and
 * inlier); counts[0] = matches, counts[1] = inliers.  The arithmetic is the
 * reference's: float NNDR and projection, the distance in double.  Device
 * pointers except H; asynchronous on stream. */
AKZ_API akz_status akz_nndr_homography_inliers(const akz_dmatch *matches, int nq, const akz_keypoint *kp_query,
                                               const akz_keypoint *kp_train, const float *H, float nndr,
                                               float min_error, int8_t *status, int *counts, void *stream);

/* save_keypoints (utils.cpp:97-152): the Krystian Mikolajczyk text format,
 * "x y 1/r^2 0 1/r^2 [descriptor bytes]" per keypoint with r = size, after a
 * header of the descriptor length (1 when save_desc is 0) and the count.
 * As in the reference, every row carries its desc_bytes descriptor bytes
 * whatever save_desc says (desc_bytes 0: none; desc may be NULL then, or
 * when n is 0).
 * Host memory. */
AKZ_API akz_status akz_save_keypoints(const char *path, const akz_keypoint *kpts, int n, const uint8_t *desc,
                                      int desc_bytes, int save_desc);

#ifdef __cplusplus
}
#endif
#endif
