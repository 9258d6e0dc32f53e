/*
 * akz_engine.cu - host side of libakaze_gb300: options, level plan, HBM
 * arena, stage launches, CUDA-graph replay and the C ABI of
 * include/akaze_gb300.h.
 *
 * Level geometry and FED schedule follow src/lib/AKAZE.cpp:146-197 and
 * src/lib/fed.cpp:41-148 of the reference; Gaussian taps and the contrast
 * pipeline follow src/lib/nldiffusion_functions.cpp.  Nothing here falls
 * back to CPU computation: every stage of the path runs as a kernel.
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/akaze_gb300.h"
#include "akz_fmath.h"
#include "akz_kernels.h"

cudaError_t akz_match_run(const void *dq, int nq, const void *dt, int nt, void *dout, void *partial, int nsplit, cudaStream_t s);
cudaError_t akz_sg_maxdiff(const float *a, const float *b, int pitch, int width, int height, float *slot, cudaStream_t s);
cudaError_t akz_launch_pack_results(const akz_tables &t, const akz_kp *kp, const uint32_t *desc, akz_kp *kp_out,
                                    uint8_t *desc_out, int row_bytes, cudaStream_t s);
extern "C" akz_status akz_sg_infer_level(const float *l0, const float *g, size_t pitch, int width, int height,
                                         float dt_feature, float s_out, const void *weights_bf16, const float *biases,
                                         void *scratch, float *out, void *stream);
extern "C" size_t akz_sg_weight_elems(void);
int akz_match_splits(int nq, int nt, int nsm);
size_t akz_match_partial_bytes(int nq, int nsplit);

/* ------------------------------------------------------------------------ */
/* errors                                                                   */

static thread_local std::string g_last_error;

static akz_status akz_fail(akz_status s, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

static akz_status akz_fail_cuda(cudaError_t e, const char *expr, const char *file, int line)
{
  return akz_fail(e == cudaErrorMemoryAllocation ? AKZ_ERR_OOM : AKZ_ERR_CUDA, "%s failed: %s (%s:%d)", expr,
                  cudaGetErrorString(e), file, line);
}

/* Records an error for akz_last_error from other translation units. */
akz_status akz_report(akz_status s, const char *msg) { return akz_fail(s, "%s", msg); }

#define CK(x)                                                                 \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) return akz_fail_cuda(e_, #x, __FILE__, __LINE__); \
  } while (0)

static float akz_ms(cudaEvent_t a, cudaEvent_t b)
{
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

/* ------------------------------------------------------------------------ */
/* plan                                                                     */

struct akz_geo {
  int w, h, octave, sublevel, deriv_step, nsteps;
  float esigma, etime, size, border;
};

static bool akz_is_prime(int number)
{
  if (number <= 1) return false;
  if (number == 2 || number == 3 || number == 5 || number == 7) return true;
  if ((number % 2) == 0 || (number % 3) == 0 || (number % 5) == 0 || (number % 7) == 0) return false;
  const int upper = (int)std::sqrt(number + 1.0);
  for (int d = 11; d <= upper; d += 2)
    if (number % d == 0) return false;
  return true;
}

/* fed.cpp:41-119 */
static int akz_fed_tau(float T, float tau_max, std::vector<float> &tau)
{
  const float t = T / 1.0f;
  const int n = (int)(std::ceil(std::sqrt(3.0 * t / tau_max + 0.25f) - 0.5f - 1.0e-8f) + 0.5f);
  const float scale = (float)(3.0 * t / (tau_max * (float)(n * (n + 1))));
  if (n <= 0) return 0;
  std::vector<float> tauh(n);
  const float c = 1.0f / (4.0f * (float)n + 2.0f);
  const float d = scale * tau_max / 2.0f;
  for (int k = 0; k < n; ++k) {
    const float h = (float)std::cos(M_PI * (double)(2.0f * (float)k + 1.0f) * (double)c);
    tauh[k] = d / (h * h);
  }
  tau.assign(n, 0.0f);
  if (n == 1) {
    tau[0] = tauh[0];
    return 1;
  }
  const int kappa = n / 2;
  int prime = n + 1;
  while (!akz_is_prime(prime)) prime++;
  for (int k = 0, l = 0; l < n; ++k, ++l) {
    int index;
    while ((index = ((k + 1) * kappa) % prime - 1) >= n) k++;
    tau[l] = tauh[index];
  }
  return n;
}

/* AKAZE.cpp:146-197 */
static void akz_plan_levels(const akz_options &o, int W, int H, std::vector<akz_geo> &L, std::vector<std::vector<float>> &tau)
{
  L.clear();
  tau.clear();
  for (int i = 0; i <= o.omax - 1; i++) {
    const float rfactor = (float)(1.0 / std::pow(2.0, i));
    const int lh = (int)((float)H * rfactor);
    const int lw = (int)((float)W * rfactor);
    if ((lw < 80 || lh < 40) && i != 0) break;
    for (int j = 0; j < o.nsublevels; j++) {
      akz_geo g;
      g.w = lw;
      g.h = lh;
      g.octave = i;
      g.sublevel = j;
      g.esigma = o.soffset * powf(2.0f, (float)j / (float)o.nsublevels + (float)i);
      g.etime = (float)(0.5 * (double)(g.esigma * g.esigma));
      const float ratio = powf(2.0f, (float)i);
      g.deriv_step = (int)(g.esigma * o.derivative_factor / ratio + 0.5f);
      g.size = g.esigma * o.derivative_factor;
      const float smax = (float)(10.0 * (double)sqrtf(2.0f));
      g.border = smax * (float)(int)(g.size / ratio + 0.5f);
      g.nsteps = 0;
      L.push_back(g);
    }
  }
  tau.resize(L.size());
  for (size_t i = 1; i < L.size(); i++) {
    const float ttime = L[i].etime - L[i - 1].etime;
    L[i].nsteps = akz_fed_tau(ttime, 0.25f, tau[i]);
  }
}

/* nldiffusion_functions.cpp:33-43 size rule; normalised exp(-x^2/2s^2) taps
 * computed in double and rounded to float. */
static int akz_gauss_taps(float sigma, float *taps)
{
  long ks = (long)std::ceil(2.0 * (1.0 + (sigma - 0.8) / (0.3)));
  if (ks % 2 == 0) ks += 1;
  const int R = (int)(ks / 2);
  if (R > (AKZ_MAX_TAPS - 1) / 2) return -1;
  double k[AKZ_MAX_TAPS];
  const double scale2 = -0.5 / ((double)sigma * (double)sigma);
  double sum = 0;
  for (int i = 0; i <= 2 * R; i++) {
    const double x = i - R;
    k[i] = std::exp(scale2 * x * x);
    sum += k[i];
  }
  for (int i = 0; i <= 2 * R; i++) taps[i] = (float)(k[i] / sum);
  return R;
}

/* Per-axis INTER_AREA tables for odd-size half-sampling, which the reference
 * does with cv::resize(INTER_AREA) (nldiffusion_functions.cpp:320-324).  To
 * give OpenCV's bits, the construction follows OpenCV's computeResizeAreaTab
 * (modules/imgproc/src/resize.cpp; OpenCV, Apache License 2.0 for 4.x,
 * 3-clause BSD before): destination cell [d*scale, (d+1)*scale) clipped to
 * the source, a leading and a trailing partial pixel kept only when their
 * overlap exceeds 1e-3, weights = overlap / cell width. */
static void akz_area_tab(int ssize, int dsize, std::vector<int> &start, std::vector<int> &si, std::vector<float> &alpha)
{
  const double scale = (double)ssize / dsize;
  for (int dx = 0; dx < dsize; dx++) {
    start.push_back((int)si.size());
    const double fsx1 = dx * scale;
    const double fsx2 = fsx1 + scale;
    const double cellWidth = std::min(scale, ssize - fsx1);
    int sx1 = (int)std::ceil(fsx1), sx2 = (int)std::floor(fsx2);
    sx2 = std::min(sx2, ssize - 1);
    sx1 = std::min(sx1, sx2);
    if (sx1 - fsx1 > 1e-3) {
      si.push_back(sx1 - 1);
      alpha.push_back((float)((sx1 - fsx1) / cellWidth));
    }
    for (int sx = sx1; sx < sx2; sx++) {
      si.push_back(sx);
      alpha.push_back((float)(1.0 / cellWidth));
    }
    if (fsx2 - sx2 > 1e-3) {
      si.push_back(sx2);
      alpha.push_back((float)(std::min(std::min(fsx2 - sx2, 1.), cellWidth) / cellWidth));
    }
  }
  start.push_back((int)si.size());
}

/* The GNU C library's rand() after srand(seed): its TYPE_3 additive
 * feedback generator, r[i] = r[i-31] + r[i-3] over a table seeded by
 * r[i] = 16807 r[i-1] mod (2^31 - 1), the first 310 sums discarded, outputs
 * r >> 1.  The reference draws its descriptor subsample with it
 * (srand(1024), AKAZE.cpp:535); restated so that the table does not depend
 * on, or disturb, the process's own rand() state. */
struct akz_libc_rand {
  uint32_t r[34];
  int i = 0;
  explicit akz_libc_rand(uint32_t seed)
  {
    uint32_t u[344];
    int64_t v = seed ? seed : 1;
    u[0] = (uint32_t)v;
    for (int k = 1; k < 31; k++) {
      v = (16807 * v) % 2147483647;
      u[k] = (uint32_t)v;
    }
    for (int k = 31; k < 34; k++) u[k] = u[k - 31];
    for (int k = 34; k < 344; k++) u[k] = u[k - 31] + u[k - 3];
    for (int k = 0; k < 34; k++) r[k] = u[310 + k];
  }
  int next()
  {
    const uint32_t v = r[(i + 3) % 34] + r[(i + 31) % 34];
    r[i] = v;
    i = (i + 1) % 34;
    return (int)(v >> 1);
  }
};

/* The M-LDB bit table: bit b compares cell sum c1[b] with c2[b] (index
 * 3 * cell + channel; cells 0-3 the 2x2 grid, 4-12 the 3x3, 13-28 the 4x4,
 * row-major with rows along the keypoint direction).  descriptor_size 0:
 * every pair of each grid per channel, (6 + 36 + 120) x channels bits
 * (AKAZE.cpp:412-418).  descriptor_size n: the random comparisons of
 * generateDescriptorSubsample (AKAZE.cpp:498-603), restated: picks from the
 * 162 grid pairs (forced to the first 6, then rand() % remaining, the picked
 * row replaced by the last live one), each pick's cells listed once as
 * samples and compared channel by channel, the first n comparisons kept; a
 * listed cell j of a g x g grid sits at row j % g, column j / g, as
 * upstream libAKAZE's Get_MLDB_Descriptor_Subset samples it.  Returns the
 * bit count. */
static int akz_mldb_table(int channels, int subset, unsigned char *c1, unsigned char *c2)
{
  static const int g0[3] = {0, 4, 13};
  int n = 0;
  if (subset <= 0) {
    for (int grid = 0; grid < 3; grid++) {
      const int gs = (grid + 2) * (grid + 2);
      for (int ch = 0; ch < channels; ch++)
        for (int j = 0; j < gs - 1; j++)
          for (int i = j + 1; i < gs; i++) {
            c1[n] = (unsigned char)(3 * (g0[grid] + j) + ch);
            c2[n] = (unsigned char)(3 * (g0[grid] + i) + ch);
            n++;
          }
    }
    return n;
  }
  struct pair3 {
    int grid, a, b;
  };
  std::vector<pair3> pairs;
  for (int grid = 0; grid < 3; grid++) {
    const int gs = (grid + 2) * (grid + 2);
    for (int a = 0; a < gs; a++)
      for (int b2 = a + 1; b2 < gs; b2++) pairs.push_back({grid, a, b2});
  }
  const int nf = (int)pairs.size();
  std::vector<std::pair<int, int>> listed; /* (grid, cell in the subset's order) */
  std::vector<int> cmp_a, cmp_b;          /* listed sample index, per comparison */
  std::vector<int> cmp_ch;
  akz_libc_rand rng(1024);
  const int picks = (subset + channels - 1) / channels;
  for (int i = 0; i < picks; i++) {
    int k = rng.next() % (nf - i);
    if (i < 6) k = i;
    int idx[2];
    for (int e = 0; e < 2; e++) {
      const std::pair<int, int> s(pairs[k].grid, e ? pairs[k].b : pairs[k].a);
      int j = 0;
      while (j < (int)listed.size() && listed[j] != s) j++;
      if (j == (int)listed.size()) listed.push_back(s);
      idx[e] = j;
    }
    for (int ch = 0; ch < channels; ch++) {
      cmp_a.push_back(idx[0]);
      cmp_b.push_back(idx[1]);
      cmp_ch.push_back(ch);
    }
    pairs[k] = pairs[nf - i - 1];
  }
  auto cell = [&](int s) {
    const int grid = listed[s].first, j = listed[s].second, g = grid + 2;
    return g0[grid] + (j % g) * g + j / g;
  };
  for (n = 0; n < subset; n++) {
    c1[n] = (unsigned char)(3 * cell(cmp_a[n]) + cmp_ch[n]);
    c2[n] = (unsigned char)(3 * cell(cmp_b[n]) + cmp_ch[n]);
  }
  return n;
}

static int akz_row_bytes(const akz_options *o)
{
  const int bits = o->descriptor_size > 0 ? o->descriptor_size : 162 * o->descriptor_channels;
  return (bits + 7) / 8;
}

static akz_status akz_validate(const akz_options *o)
{
  if (!o) return akz_fail(AKZ_ERR_INVALID_ARG, "options are NULL");
  if (o->omax < 1 || o->nsublevels < 1 || o->omax * o->nsublevels > AKZ_MAX_LEVELS)
    return akz_fail(AKZ_ERR_INVALID_ARG, "omax*nsublevels must be in [1, %d]", AKZ_MAX_LEVELS);
  if (!(o->soffset >= 0.65f) || !(o->soffset <= 5.5f)) return akz_fail(AKZ_ERR_INVALID_ARG, "soffset must be in [0.65, 5.5]");
  if (!(o->derivative_factor > 0.0f)) return akz_fail(AKZ_ERR_INVALID_ARG, "derivative_factor must be positive");
  if (o->diffusivity < 0 || o->diffusivity > 3) return akz_fail(AKZ_ERR_INVALID_ARG, "unknown diffusivity %d", o->diffusivity);
  if (o->descriptor != AKZ_MLDB && o->descriptor != AKZ_MLDB_UPRIGHT)
    return akz_fail(AKZ_ERR_UNSUPPORTED, "descriptor %d is not implemented (MLDB and MLDB_UPRIGHT are)", o->descriptor);
  if (o->descriptor_channels < 1 || o->descriptor_channels > 3)
    return akz_fail(AKZ_ERR_INVALID_ARG, "descriptor_channels %d: must be 1, 2 or 3", o->descriptor_channels);
  if (o->descriptor_size < 0 || o->descriptor_size > 162 * o->descriptor_channels)
    return akz_fail(AKZ_ERR_INVALID_ARG, "descriptor_size %d: must be 0 (full) or at most %d bits for %d channel(s)",
                    o->descriptor_size, 162 * o->descriptor_channels, o->descriptor_channels);
  if (o->descriptor_pattern_size < 1 || o->descriptor_pattern_size > 10)
    return akz_fail(AKZ_ERR_INVALID_ARG, "descriptor_pattern_size must be in [1, 10]");
  if (o->kcontrast_nbins < 1 || o->kcontrast_nbins > AKZ_MAX_NBINS)
    return akz_fail(AKZ_ERR_INVALID_ARG, "kcontrast_nbins must be in [1, %d]", AKZ_MAX_NBINS);
  if (!(o->kcontrast_percentile >= 0.0f && o->kcontrast_percentile <= 1.0f))
    return akz_fail(AKZ_ERR_INVALID_ARG, "kcontrast_percentile must be in [0, 1]");
  if (o->maxkeypoints < 1) return akz_fail(AKZ_ERR_INVALID_ARG, "maxkeypoints must be positive");
  if (o->extrema_3d != 0 && o->extrema_3d != 1) return akz_fail(AKZ_ERR_INVALID_ARG, "extrema_3d must be 0 or 1");
  if (o->fast_math != 0 && o->fast_math != 1) return akz_fail(AKZ_ERR_INVALID_ARG, "fast_math must be 0 or 1");
  return AKZ_OK;
}

/* ------------------------------------------------------------------------ */
/* batch                                                                    */

#define AKZ_DEPTH_MIN 4            /* smallest FED blocking depth the autotuner tries */
#define AKZ_MAX_STEPS_PER_LAUNCH 8 /* k_fed's largest depth */

struct akz_fed_launch {
  int seg_off, nsegs, ntiles, tw, th;
  akz_fed_params p;
};

struct akz_area_launch {
  int seg_off, nsegs, maxw, maxh;
};

struct akz_batch {
  akz_options opt;
  int nimg = 0;
  std::vector<int> W, H;
  std::vector<akz_image_desc> im;
  std::vector<akz_level_desc> lv;
  std::vector<std::vector<akz_geo>> geo;
  std::vector<std::vector<float>> tau; /* per level index */
  int maxlev = 0, max_step = 1, max_level_h = 1;
  float taps0[AKZ_MAX_TAPS], taps1[AKZ_MAX_TAPS];
  int R0 = 0;
  /* launches */
  std::vector<akz_tile_seg> segs;
  int contrast_off = 0, contrast_n = 0, contrast_tiles = 0;
  int gauss_off = 0, gauss_n = 0, gauss_tiles = 0;
  int l0_off = 0, l0_n = 0, l0_tiles = 0; /* k_level0 tiles */
  int detect_off = 0, detect_n = 0, detect_tiles = 0;
  int strip_off = 0, strip_n = 0, strip_tiles = 0;
  int extract_off = 0, extract_n = 0, extract_rows = 0;
  std::vector<std::vector<akz_fed_launch>> fed;  /* per level index: the launches in use */
  /* the level stage's launches for every FED blocking depth (most steps per
   * launch) AKZ_DEPTH_MIN .. AKZ_MAX_STEPS_PER_LAUNCH; akz_batch_autotune
   * picks one, the default is the largest */
  std::vector<std::vector<std::vector<akz_fed_launch>>> fed_alt;
  std::vector<int> fed_depth; /* per level */
  /* learned surrogate (akz_batch_set_surrogate): per level, the zero-step
   * launch that forms Lsmooth, the conductance and the start image, and the
   * plain chunks of image 0 into the check plane */
  std::vector<akz_fed_launch> sg_prep;
  std::vector<std::vector<akz_fed_launch>> sg_check;
  int sg_on = 0, sg_first_octave = 1;
  float sg_s_out = 0.0f, sg_tol = 0.0f;
  std::vector<float> sg_dtf;
  void *d_sg_w = nullptr, *d_sg_scratch = nullptr;
  float *d_sg_b = nullptr, *d_sg_chk = nullptr, *d_sg_err = nullptr;
  std::vector<akz_area_launch> area;              /* per level index (nsegs 0 when none) */
  std::vector<akz_area_seg> area_segs;
  std::vector<int> area_start, area_si;
  std::vector<float> area_alpha;
  /* device */
  char *arena = nullptr;
  size_t arena_bytes = 0;
  float *planes = nullptr;
  void *d_tmaps = nullptr; /* k_fed input boxes: 2 CUtensorMaps per level descriptor */
  uint8_t *u8 = nullptr;
  float *f32 = nullptr;
  size_t staging_elems = 0;
  akz_level_desc *d_lv = nullptr;
  akz_image_desc *d_im = nullptr;
  akz_image_stats *d_stats = nullptr;
  akz_tile_seg *d_segs = nullptr;
  akz_area_seg *d_area_segs = nullptr;
  int *d_area_start = nullptr, *d_area_si = nullptr;
  float *d_area_alpha = nullptr;
  unsigned int *d_hist = nullptr;
  float2 *d_kc = nullptr;
  uint32_t *d_bitmap = nullptr;
  size_t bitmap_words = 0;
  int *d_rowcnt = nullptr, *d_rowscan = nullptr;
  size_t rows_all = 0;
  akz_raw *d_raw = nullptr;
  int *d_state = nullptr, *d_aux = nullptr;
  signed char *d_dec = nullptr;
  akz_kp *d_kp = nullptr;
  uint32_t *d_desc = nullptr;
  int *d_nbr = nullptr;
  unsigned char *d_nbc = nullptr;
  unsigned char *d_cmp = nullptr; /* M-LDB bit table: 512 first then 512 second value indices */
  int nbits = 486, row_bytes = 61;
  /* akz_batch_submit / akz_batch_collect_packed: two result slots, each with
   * the packed keypoints and descriptor rows of one submitted run (room for
   * every image at its keypoint capacity), its counts read back into pinned
   * memory, and an event; up to two runs outstanding, collected in order */
  void *d_slot[2] = {nullptr, nullptr};
  akz_image_stats *h_slot_stats[2] = {nullptr, nullptr};
  cudaEvent_t ev_slot[2] = {nullptr, nullptr};
  cudaStream_t copy_stream = nullptr;
  /* submitted runs alternate between two input staging buffers (the
   * arena's and d_stage2), each with its own graph: a run's images go up on
   * up_stream while the run before it computes */
  uint8_t *d_stage2 = nullptr;
  cudaStream_t up_stream = nullptr;
  cudaEvent_t ev_stage_full[2] = {nullptr, nullptr}, ev_stage_free[2] = {nullptr, nullptr};
  int stage_next = 0;
  bool slots_ready = false;
  int sub_first = 0, sub_n = 0; /* slot of the oldest outstanding run, runs outstanding */
  size_t raw_all = 0;
  int input_f32 = 0;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  /* captured graphs of the whole run, one per input staging buffer (0: the
   * arena's, 1: the submit path's second one), for the input kind and
   * stream they were captured with */
  struct akz_graph_entry {
    cudaGraphExec_t g = nullptr;
    int f32 = -1;
    cudaStream_t s = nullptr;
  };
  akz_graph_entry graphs[2];
  uint8_t *u8_arena = nullptr; /* the arena's staging buffer (u8 points to it outside akz_batch_submit) */
  akz_image_stats *h_stats = nullptr;
  int nsm = 152;
  int nms_round_cap = 1 << 20; /* suppression rounds before AKZ_ERR_TIMEOUT */
  cudaEvent_t ev[8] = {}; /* stage timing */
};

static size_t akz_align(size_t v, size_t a) { return (v + a - 1) / a * a; }

static akz_tables akz_make_tables(const akz_batch *b)
{
  akz_tables t;
  t.lv = b->d_lv;
  t.im = b->d_im;
  t.stats = b->d_stats;
  t.planes = b->planes;
  t.u8 = b->u8;
  t.f32 = b->f32;
  t.input_f32 = b->input_f32;
  t.nimg = b->nimg;
  return t;
}

static void akz_batch_free(akz_batch *b)
{
  if (!b) return;
  for (auto &ge : b->graphs)
    if (ge.g) cudaGraphExecDestroy(ge.g);
  if (b->arena) cudaFree(b->arena);
  for (void *q : {(void *)b->d_sg_w, b->d_sg_scratch, (void *)b->d_sg_b, (void *)b->d_sg_chk, (void *)b->d_sg_err,
                  b->d_slot[0], b->d_slot[1], (void *)b->d_stage2, b->d_tmaps})
    if (q) cudaFree(q);
  if (b->f32) cudaFree(b->f32);
  if (b->h_stats) cudaFreeHost(b->h_stats);
  for (int k = 0; k < 2; k++) {
    if (b->h_slot_stats[k]) cudaFreeHost(b->h_slot_stats[k]);
    if (b->ev_slot[k]) cudaEventDestroy(b->ev_slot[k]);
  }
  if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
  if (b->up_stream) cudaStreamDestroy(b->up_stream);
  for (cudaEvent_t e : {b->ev_stage_full[0], b->ev_stage_full[1], b->ev_stage_free[0], b->ev_stage_free[1]})
    if (e) cudaEventDestroy(e);
  for (auto &e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

/* The TMA descriptors of k_fed's input boxes: for every level descriptor,
 * its Lt plane and its image's T2 plane at the level's size and pitch, each
 * read in boxes of AKZ_FED_BOX_W x AKZ_FED_BOX_H floats with zero fill
 * outside the plane (the kernel replaces it by the replicate border).  The
 * encoder is the driver's cuTensorMapEncodeTiled, reached through the
 * runtime's entry-point query (no link against the driver library). */
static PFN_cuTensorMapEncodeTiled_v12000 akz_tmap_encoder()
{
  static std::mutex mu;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  if (!fn) {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)f;
  }
  return fn;
}

static akz_status akz_build_tensor_maps(akz_batch *b)
{
  const PFN_cuTensorMapEncodeTiled_v12000 enc = akz_tmap_encoder();
  if (!enc) return akz_fail(AKZ_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const size_t nl = b->lv.size();
  std::vector<CUtensorMap> maps(2 * nl);
  for (size_t l = 0; l < nl; l++) {
    const akz_level_desc &L = b->lv[l];
    const akz_image_desc &I = b->im[L.image];
    const cuuint64_t dims[2] = {(cuuint64_t)L.width, (cuuint64_t)L.height};
    const cuuint64_t strides[1] = {(cuuint64_t)L.pitch * sizeof(float)};
    const cuuint32_t box[2] = {AKZ_FED_BOX_W, AKZ_FED_BOX_H}, estr[2] = {1, 1};
    float *bases[2] = {b->planes + L.lt, b->planes + I.t2};
    for (int k = 0; k < 2; k++) {
      const CUresult r = enc(&maps[2 * l + k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, bases[k], dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return akz_fail(AKZ_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) for level %zu", (int)r, l);
    }
  }
  static_assert(sizeof(CUtensorMap) == 128, "k_fed indexes tensor maps at a 128-byte stride");
  CK(cudaMalloc(&b->d_tmaps, maps.size() * sizeof(CUtensorMap)));
  CK(cudaMemcpy(b->d_tmaps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
  return AKZ_OK;
}

static akz_status akz_batch_build(const akz_options *opt, int n, const int *Ws, const int *Hs, akz_batch **out)
{
  akz_status st = akz_validate(opt);
  if (st != AKZ_OK) return st;
  if (n < 1 || !Ws || !Hs || !out) return akz_fail(AKZ_ERR_INVALID_ARG, "batch needs at least one image and size arrays");
  if (n > AKZ_FIT_MAXIMG) return akz_fail(AKZ_ERR_INVALID_ARG, "a batch holds at most %d images", AKZ_FIT_MAXIMG);
  akz_batch *b = new (std::nothrow) akz_batch();
  if (!b) return akz_fail(AKZ_ERR_OOM, "host allocation failed");
  b->opt = *opt;
  b->nimg = n;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->nsm, cudaDevAttrMultiProcessorCount, dev);
  b->R0 = akz_gauss_taps(opt->soffset, b->taps0);
  if (akz_gauss_taps(1.0f, b->taps1) != 2 || b->R0 < 0) {
    akz_batch_free(b);
    return akz_fail(AKZ_ERR_INVALID_ARG, "Gaussian radius out of range");
  }
  /* geometry */
  b->geo.resize(n);
  for (int i = 0; i < n; i++) {
    if (Ws[i] < 16 || Hs[i] < 16 || Ws[i] > 32768 || Hs[i] > 32768) {
      akz_batch_free(b);
      return akz_fail(AKZ_ERR_INVALID_ARG, "image %d: size %dx%d outside [16, 32768]", i, Ws[i], Hs[i]);
    }
    b->W.push_back(Ws[i]);
    b->H.push_back(Hs[i]);
    std::vector<std::vector<float>> tau;
    akz_plan_levels(*opt, Ws[i], Hs[i], b->geo[i], tau);
    if ((int)b->geo[i].size() > b->maxlev) {
      b->maxlev = (int)b->geo[i].size();
      b->tau = tau;
    }
    for (auto &g : b->geo[i]) {
      if (g.deriv_step < 1 || g.w < 2 * g.deriv_step + 2 || g.h < 2 * g.deriv_step + 2) {
        akz_batch_free(b);
        return akz_fail(AKZ_ERR_INVALID_ARG, "image %d: level %dx%d too small for derivative step %d", i, g.w, g.h, g.deriv_step);
      }
      b->max_step = std::max(b->max_step, g.deriv_step);
      b->max_level_h = std::max(b->max_level_h, g.h);
    }
  }
  if (b->max_step > 16) {
    akz_batch_free(b);
    return akz_fail(AKZ_ERR_UNSUPPORTED, "derivative step %d above 16", b->max_step);
  }
  /* arena layout */
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = akz_align(off + bytes, 256);
    return o;
  };
  size_t plane_floats = 0;
  long long rows = 0;
  size_t bitmap = 0, raw = 0, staging = 0;
  for (int i = 0; i < n; i++) {
    akz_image_desc I;
    memset(&I, 0, sizeof(I));
    I.width = Ws[i];
    I.height = Hs[i];
    I.nlev = (int)b->geo[i].size();
    I.first_level = (int)b->lv.size();
    I.u8_pitch = (int)akz_align(Ws[i], 16);
    I.u8_off = (long long)staging;
    staging += (size_t)I.u8_pitch * Hs[i];
    I.rows_base = rows;
    int rt = 0;
    for (int l = 0; l < I.nlev; l++) {
      const akz_geo &g = b->geo[i][l];
      akz_level_desc L;
      memset(&L, 0, sizeof(L));
      L.width = g.w;
      L.height = g.h;
      L.pitch = (int)akz_align(g.w, 32);
      L.image = i;
      L.level = l;
      L.octave = g.octave;
      L.sublevel = g.sublevel;
      L.deriv_step = g.deriv_step;
      L.border = g.border;
      L.size = g.size;
      const size_t pf = (size_t)L.pitch * g.h;
      L.lt = (long long)plane_floats;
      plane_floats += pf;
      if (l == 0) {
        L.ls = L.lt;
      } else {
        L.ls = (long long)plane_floats;
        plane_floats += pf;
      }
      L.lx = (long long)plane_floats; /* Lx, Ly interleaved: (Lx, Ly) pairs, row pitch 2 * pitch */
      L.ly = L.lx + 1;
      plane_floats += 2 * pf;
      L.ldet = -1;
      if (opt->extrema_3d) { /* the 3 x 3 x 3 rule reads the adjacent levels' determinants */
        L.ldet = (long long)plane_floats;
        plane_floats += pf;
      }
      L.rows = rows + rt;
      rt += g.h;
      L.bitmap_pitch = (g.w + 31) / 32;
      L.bitmap = (long long)bitmap;
      bitmap += (size_t)L.bitmap_pitch * g.h;
      b->lv.push_back(L);
    }
    I.rows_total = rt;
    rows += rt + 1;
    const size_t p0 = (size_t)akz_align(Ws[i], 32) * Hs[i];
    I.t1 = (long long)plane_floats;
    plane_floats += p0;
    I.t2 = (long long)plane_floats;
    plane_floats += p0;
    I.g = (long long)plane_floats;
    plane_floats += p0;
    I.raw_cap = opt->maxkeypoints;
    I.kp_cap = opt->maxkeypoints;
    I.raw_base = (long long)raw;
    I.kp_base = (long long)raw;
    raw += (size_t)opt->maxkeypoints;
    b->im.push_back(I);
  }
  b->rows_all = (size_t)rows;
  b->bitmap_words = bitmap;
  b->raw_all = raw;
  b->staging_elems = staging;

  /* launch segments */
  auto add_tiles = [&](int ld_or_img, int w, int h, int tw, int th, int aux, int &ntiles) {
    akz_tile_seg s;
    s.level_desc = ld_or_img;
    s.tiles_x = (w + tw - 1) / tw;
    s.tile_begin = ntiles;
    s.aux = aux;
    ntiles += s.tiles_x * ((h + th - 1) / th);
    b->segs.push_back(s);
  };
  b->contrast_off = (int)b->segs.size();
  for (int i = 0; i < n; i++) add_tiles(i, Ws[i], Hs[i], AKZ_CONTRAST_TW, AKZ_CONTRAST_TH, 0, b->contrast_tiles);
  b->contrast_n = (int)b->segs.size() - b->contrast_off;
  b->gauss_off = (int)b->segs.size();
  for (int i = 0; i < n; i++) add_tiles(b->im[i].first_level, Ws[i], Hs[i], AKZ_GAUSS_TW, AKZ_GAUSS_TH, 0, b->gauss_tiles);
  b->gauss_n = (int)b->segs.size() - b->gauss_off;
  b->l0_off = (int)b->segs.size();
  for (int i = 0; i < n; i++) add_tiles(b->im[i].first_level, Ws[i], Hs[i], AKZ_L0_TW, AKZ_L0_TH, 0, b->l0_tiles);
  b->l0_n = (int)b->segs.size() - b->l0_off;

  b->fed.resize(b->maxlev);
  b->fed_alt.assign(AKZ_MAX_STEPS_PER_LAUNCH - AKZ_DEPTH_MIN + 1, std::vector<std::vector<akz_fed_launch>>(b->maxlev));
  b->area.resize(b->maxlev);
  b->sg_prep.resize(b->maxlev);
  b->sg_check.resize(b->maxlev);
  for (int l = 1; l < b->maxlev; l++) {
    const int nsteps = (int)b->tau[l].size();
    /* area tables for octave starts whose predecessor is not exactly 2x */
    akz_area_launch al{(int)b->area_segs.size(), 0, 0, 0};
    for (int i = 0; i < n; i++) {
      if (b->im[i].nlev <= l) continue;
      const akz_geo &g = b->geo[i][l], &gp = b->geo[i][l - 1];
      if (g.octave > gp.octave && !(gp.w == 2 * g.w && gp.h == 2 * g.h)) {
        akz_area_seg as;
        as.ld = b->im[i].first_level + l;
        as.xs = (int)b->area_start.size();
        akz_area_tab(gp.w, g.w, b->area_start, b->area_si, b->area_alpha);
        as.ys = (int)b->area_start.size();
        akz_area_tab(gp.h, g.h, b->area_start, b->area_si, b->area_alpha);
        as.pad = 0;
        b->area_segs.push_back(as);
        al.nsegs++;
        al.maxw = std::max(al.maxw, g.w);
        al.maxh = std::max(al.maxh, g.h);
      }
    }
    b->area[l] = al;
    /* FED chunks of at most `depth` steps; with chk, the same chunks for
     * image 0 alone, the last one into the check plane */
    auto chunks = [&](int depth, std::vector<akz_fed_launch> &out, std::vector<akz_fed_launch> *chk) {
      const int nch = std::max(1, (nsteps + depth - 1) / depth);
      int done = 0;
      for (int c = 0; c < nch; c++) {
        const int steps = (nsteps - done + (nch - c) - 1) / (nch - c);
        akz_fed_launch fl;
        memset(&fl, 0, sizeof(fl));
        fl.tw = akz_fed_tile_w(steps); /* k_fed region is 128 x 40 = tile +- steps (aligned) */
        fl.th = akz_fed_tile_h(steps);
        fl.seg_off = (int)b->segs.size();
        for (int i = 0; i < n; i++) {
          if (b->im[i].nlev <= l) continue;
          const akz_geo &g = b->geo[i][l], &gp = b->geo[i][l - 1];
          int src = 0;
          if (g.octave > gp.octave) src = (gp.w == 2 * g.w && gp.h == 2 * g.h) ? 1 : 2;
          add_tiles(b->im[i].first_level + l, g.w, g.h, fl.tw, fl.th, src, fl.ntiles);
        }
        fl.nsegs = (int)b->segs.size() - fl.seg_off;
        fl.p.steps = steps;
        fl.p.first = c == 0;
        fl.p.src = c == 0 ? 0 : ((c - 1) % 2 == 0 ? 1 : 2);
        fl.p.dst = c == nch - 1 ? 0 : (c % 2 == 0 ? 1 : 2);
        fl.p.write_g = (c == 0 && nch > 1) ? 1 : 0;
        fl.p.diffusivity = opt->diffusivity;
        for (int k = 0; k < 5; k++) fl.p.taps1[k] = b->taps1[k];
        for (int k = 0; k < steps; k++) fl.p.h[k] = 0.5f * b->tau[l][done + k];
        done += steps;
        out.push_back(fl);
        if (!chk) continue;
        akz_fed_launch cl = fl;
        cl.seg_off = (int)b->segs.size();
        cl.ntiles = 0;
        if (b->im[0].nlev > l) {
          const akz_geo &g = b->geo[0][l], &gp = b->geo[0][l - 1];
          int src = 0;
          if (g.octave > gp.octave) src = (gp.w == 2 * g.w && gp.h == 2 * g.h) ? 1 : 2;
          add_tiles(b->im[0].first_level + l, g.w, g.h, cl.tw, cl.th, src, cl.ntiles);
        }
        cl.nsegs = (int)b->segs.size() - cl.seg_off;
        if (c == nch - 1) cl.p.dst = 3;
        chk->push_back(cl);
      }
    };
    for (int depth = AKZ_DEPTH_MIN; depth < AKZ_MAX_STEPS_PER_LAUNCH; depth++)
      chunks(depth, b->fed_alt[depth - AKZ_DEPTH_MIN][l], nullptr);
    chunks(AKZ_MAX_STEPS_PER_LAUNCH, b->fed[l], &b->sg_check[l]);
    /* zero FED steps over 128 x 40 tiles: Lsmooth, the conductance (kept)
     * and the start image in Lt */
    akz_fed_launch pl;
    memset(&pl, 0, sizeof(pl));
    pl.tw = akz_fed_tile_w(0);
    pl.th = akz_fed_tile_h(0);
    pl.seg_off = (int)b->segs.size();
    for (int i = 0; i < n; i++) {
      if (b->im[i].nlev <= l) continue;
      const akz_geo &g = b->geo[i][l], &gp = b->geo[i][l - 1];
      int src = 0;
      if (g.octave > gp.octave) src = (gp.w == 2 * g.w && gp.h == 2 * g.h) ? 1 : 2;
      add_tiles(b->im[i].first_level + l, g.w, g.h, pl.tw, pl.th, src, pl.ntiles);
    }
    pl.nsegs = (int)b->segs.size() - pl.seg_off;
    pl.p.steps = 0;
    pl.p.first = 1;
    pl.p.dst = 0;
    pl.p.write_g = 1;
    pl.p.diffusivity = opt->diffusivity;
    for (int k = 0; k < 5; k++) pl.p.taps1[k] = b->taps1[k];
    b->sg_prep[l] = pl;
    b->fed_alt[AKZ_MAX_STEPS_PER_LAUNCH - AKZ_DEPTH_MIN][l] = b->fed[l];
  }
  b->fed_depth.assign(b->maxlev, AKZ_MAX_STEPS_PER_LAUNCH);
  /* detector: the streaming strip kernel for steps 2..4, tiles otherwise */
  b->strip_off = (int)b->segs.size();
  for (int i = 0; i < n; i++)
    for (int l = 0; l < b->im[i].nlev; l++) {
      const int tw = akz_strip_tile_width(b->geo[i][l].deriv_step);
      if (tw > 0) add_tiles(b->im[i].first_level + l, b->geo[i][l].w, b->geo[i][l].h, tw, AKZ_STRIP_CH, 0, b->strip_tiles);
    }
  b->strip_n = (int)b->segs.size() - b->strip_off;
  b->detect_off = (int)b->segs.size();
  for (int i = 0; i < n; i++)
    for (int l = 0; l < b->im[i].nlev; l++)
      if (akz_strip_tile_width(b->geo[i][l].deriv_step) == 0)
        add_tiles(b->im[i].first_level + l, b->geo[i][l].w, b->geo[i][l].h, AKZ_DETECT_TW, AKZ_DETECT_TH, 0,
                  b->detect_tiles);
  b->detect_n = (int)b->segs.size() - b->detect_off;
  b->extract_off = (int)b->segs.size();
  for (int i = 0; i < n; i++)
    for (int l = 0; l < b->im[i].nlev; l++) {
      akz_tile_seg s;
      s.level_desc = b->im[i].first_level + l;
      s.tiles_x = 1;
      s.tile_begin = b->extract_rows;
      s.aux = 0;
      b->extract_rows += b->geo[i][l].h;
      b->segs.push_back(s);
    }
  b->extract_n = (int)b->segs.size() - b->extract_off;

  /* arena */
  const size_t o_planes = take(plane_floats * sizeof(float));
  const size_t o_u8 = take(staging);
  const size_t o_lv = take(b->lv.size() * sizeof(akz_level_desc));
  const size_t o_im = take(b->im.size() * sizeof(akz_image_desc));
  const size_t o_stats = take((size_t)n * sizeof(akz_image_stats));
  const size_t o_segs = take(b->segs.size() * sizeof(akz_tile_seg));
  const size_t o_aseg = take(std::max<size_t>(1, b->area_segs.size()) * sizeof(akz_area_seg));
  const size_t o_astart = take(std::max<size_t>(1, b->area_start.size()) * sizeof(int));
  const size_t o_asi = take(std::max<size_t>(1, b->area_si.size()) * sizeof(int));
  const size_t o_aalpha = take(std::max<size_t>(1, b->area_alpha.size()) * sizeof(float));
  const size_t o_hist = take((size_t)n * opt->kcontrast_nbins * sizeof(unsigned int));
  const size_t o_kc = take((size_t)n * 16 * sizeof(float2));
  const size_t o_bitmap = take(bitmap * sizeof(uint32_t));
  const size_t o_rowcnt = take(b->rows_all * sizeof(int));
  const size_t o_rowscan = take(b->rows_all * sizeof(int));
  const size_t o_raw = take(raw * sizeof(akz_raw));
  const size_t o_state = take(raw * sizeof(int));
  const size_t o_aux = take(raw * sizeof(int));
  const size_t o_dec = take(raw);
  const size_t o_kp = take(raw * sizeof(akz_kp));
  const size_t o_desc = take(raw * 64);
  const size_t o_nbr = take(raw * AKZ_NMS_NB * sizeof(int));
  const size_t o_nbc = take(raw);
  const size_t o_cmp = take(1024);
  b->arena_bytes = off;
  cudaError_t e = cudaMalloc(&b->arena, b->arena_bytes);
  if (e != cudaSuccess) {
    akz_batch_free(b);
    return akz_fail(AKZ_ERR_OOM, "cudaMalloc of %.1f MB failed: %s", b->arena_bytes / 1048576.0, cudaGetErrorString(e));
  }
  char *a = b->arena;
  b->planes = (float *)(a + o_planes);
  b->u8 = (uint8_t *)(a + o_u8);
  b->u8_arena = b->u8;
  b->d_lv = (akz_level_desc *)(a + o_lv);
  b->d_im = (akz_image_desc *)(a + o_im);
  b->d_stats = (akz_image_stats *)(a + o_stats);
  b->d_segs = (akz_tile_seg *)(a + o_segs);
  b->d_area_segs = (akz_area_seg *)(a + o_aseg);
  b->d_area_start = (int *)(a + o_astart);
  b->d_area_si = (int *)(a + o_asi);
  b->d_area_alpha = (float *)(a + o_aalpha);
  b->d_hist = (unsigned int *)(a + o_hist);
  b->d_kc = (float2 *)(a + o_kc);
  b->d_bitmap = (uint32_t *)(a + o_bitmap);
  b->d_rowcnt = (int *)(a + o_rowcnt);
  b->d_rowscan = (int *)(a + o_rowscan);
  b->d_raw = (akz_raw *)(a + o_raw);
  b->d_state = (int *)(a + o_state);
  b->d_aux = (int *)(a + o_aux);
  b->d_dec = (signed char *)(a + o_dec);
  b->d_kp = (akz_kp *)(a + o_kp);
  b->d_desc = (uint32_t *)(a + o_desc);
  b->d_nbr = (int *)(a + o_nbr);
  b->d_nbc = (unsigned char *)(a + o_nbc);
  b->d_cmp = (unsigned char *)(a + o_cmp);
  {
    unsigned char cmp[1024] = {0};
    b->nbits = akz_mldb_table(b->opt.descriptor_channels, b->opt.descriptor_size, cmp, cmp + 512);
    b->row_bytes = akz_row_bytes(&b->opt);
    e = cudaMemcpy(b->d_cmp, cmp, sizeof(cmp), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_stats, (size_t)n * sizeof(akz_image_stats));
  for (auto &ev : b->ev)
    if (e == cudaSuccess) e = cudaEventCreate(&ev);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_lv, b->lv.data(), b->lv.size() * sizeof(akz_level_desc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_im, b->im.data(), b->im.size() * sizeof(akz_image_desc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_segs, b->segs.data(), b->segs.size() * sizeof(akz_tile_seg), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !b->area_segs.empty()) {
    e = cudaMemcpy(b->d_area_segs, b->area_segs.data(), b->area_segs.size() * sizeof(akz_area_seg), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_area_start, b->area_start.data(), b->area_start.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_area_si, b->area_si.data(), b->area_si.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_area_alpha, b->area_alpha.data(), b->area_alpha.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemset(b->u8, 0, staging);
  if (e != cudaSuccess) {
    akz_batch_free(b);
    return akz_fail_cuda(e, "batch set-up", __FILE__, __LINE__);
  }
  if (e == cudaSuccess) {
    const akz_status ts = akz_build_tensor_maps(b);
    if (ts != AKZ_OK) {
      akz_batch_free(b);
      return ts;
    }
  }
  b->stream = b->own_stream;
  *out = b;
  return AKZ_OK;
}

/* stage groups ------------------------------------------------------------ */

/* pe: events of the level-0 split (profile); lev: one event per level,
 * recorded when that level is done (level 0 included) */
static akz_status akz_stage_scale(akz_batch *b, cudaStream_t s, cudaEvent_t *pe = nullptr, cudaEvent_t *lev = nullptr)
{
  const akz_tables t = akz_make_tables(b);
  if (b->sg_on) CK(cudaMemsetAsync(b->d_sg_err, 0, (size_t)b->maxlev * sizeof(float), s));
  CK(cudaMemsetAsync(b->d_stats, 0, (size_t)b->nimg * sizeof(akz_image_stats), s));
  CK(cudaMemsetAsync(b->d_hist, 0, (size_t)b->nimg * b->opt.kcontrast_nbins * sizeof(unsigned int), s));
  const float inv255 = (float)(1.0 / 255.0);
  if (b->R0 <= 4) {
    /* level 0 and the contrast gradient from one staging of the input */
    akz_level0_params lp;
    lp.t = t;
    lp.segs = b->d_segs + b->l0_off;
    lp.nsegs = b->l0_n;
    lp.inv255 = inv255;
    for (int k = 0; k < 5; k++) lp.taps0[k] = k < 4 - b->R0 ? 0.0f : b->taps0[k - (4 - b->R0)];
    for (int k = 0; k < 3; k++) lp.taps1[k] = b->taps1[k];
    lp.nbins = (int)b->opt.kcontrast_nbins;
    lp.hist = b->d_hist;
    lp.fused = b->opt.fast_math;
    CK(akz_launch_level0(lp, b->l0_tiles, s));
    CK(akz_launch_contrast_final(t, b->d_hist, lp.nbins, b->opt.kcontrast_percentile, b->d_kc, s));
    if (pe) {
      CK(cudaEventRecord(pe[1], s));
      CK(cudaEventRecord(pe[2], s));
    }
  } else {
    akz_contrast_params cp;
    cp.t = t;
    cp.segs = b->d_segs + b->contrast_off;
    cp.nsegs = b->contrast_n;
    cp.nbins = (int)b->opt.kcontrast_nbins;
    cp.hist = b->d_hist;
    cp.inv255 = inv255;
    for (int k = 0; k < 5; k++) cp.taps[k] = b->taps1[k];
    CK(akz_launch_contrast(cp, b->contrast_tiles, 0, s));
    CK(akz_launch_contrast(cp, b->contrast_tiles, 1, s));
    CK(akz_launch_contrast_final(t, b->d_hist, cp.nbins, b->opt.kcontrast_percentile, b->d_kc, s));
    if (pe) CK(cudaEventRecord(pe[1], s));
    akz_gauss_params gp;
    gp.t = t;
    gp.segs = b->d_segs + b->gauss_off;
    gp.nsegs = b->gauss_n;
    gp.inv255 = inv255;
    gp.R = b->R0;
    for (int k = 0; k <= 2 * b->R0; k++) gp.taps[k] = b->taps0[k];
    CK(akz_launch_gauss0(gp, b->gauss_tiles, s));
    if (pe) CK(cudaEventRecord(pe[2], s));
  }
  if (lev) CK(cudaEventRecord(lev[0], s));
  for (int l = 1; l < b->maxlev; l++) {
    if (b->area[l].nsegs > 0) {
      akz_area_params ap;
      ap.t = t;
      ap.segs = b->d_area_segs + b->area[l].seg_off;
      ap.nsegs = b->area[l].nsegs;
      ap.start = b->d_area_start;
      ap.si = b->d_area_si;
      ap.alpha = b->d_area_alpha;
      CK(akz_launch_area(ap, b->area[l].maxw, b->area[l].maxh, s));
    }
    auto run_fed = [&](const akz_fed_launch &fl, const float *gate) -> cudaError_t {
      if (fl.ntiles <= 0) return cudaSuccess;
      akz_fed_params p = fl.p;
      p.t = t;
      p.segs = b->d_segs + fl.seg_off;
      p.nsegs = fl.nsegs;
      p.kc = b->d_kc;
      p.tmaps = b->d_tmaps;
      p.chk = b->d_sg_chk;
      p.gate = gate;
      p.gate_tol = b->sg_tol;
      p.fused = b->opt.fast_math;
      return akz_launch_fed(p, fl.ntiles, fl.tw, fl.th, s);
    };
    if (!b->sg_on || l / b->opt.nsublevels < b->sg_first_octave) {
      for (auto &fl : b->fed[l]) CK(run_fed(fl, nullptr));
      if (lev) CK(cudaEventRecord(lev[l], s));
      continue;
    }
    /* learned surrogate: start image, Lsmooth and conductance, then the net
     * in place on every image; with a tolerance, image 0 is also run through
     * the plain chunks into the check plane, compared, and the plain launches
     * of the level follow behind a device-side gate on that comparison */
    CK(run_fed(b->sg_prep[l], nullptr));
    for (int i = 0; i < b->nimg; i++) {
      if (b->im[i].nlev <= l) continue;
      const akz_level_desc &L = b->lv[b->im[i].first_level + l];
      float *lt = b->planes + L.lt;
      const akz_status st = akz_sg_infer_level(lt, b->planes + b->im[i].g, (size_t)L.pitch, L.width, L.height,
                                               b->sg_dtf[l], b->sg_s_out, b->d_sg_w, b->d_sg_b, b->d_sg_scratch, lt, s);
      if (st != AKZ_OK) return st;
    }
    if (b->sg_tol > 0.0f && b->im[0].nlev > l) {
      for (auto &cl : b->sg_check[l]) CK(run_fed(cl, nullptr));
      const akz_level_desc &L0 = b->lv[b->im[0].first_level + l];
      CK(akz_sg_maxdiff(b->d_sg_chk, b->planes + L0.lt, L0.pitch, L0.width, L0.height, b->d_sg_err + l, s));
      for (auto &fl : b->fed[l]) CK(run_fed(fl, b->d_sg_err + l));
    }
    if (lev) CK(cudaEventRecord(lev[l], s));
  }
  return AKZ_OK;
}

static akz_status akz_stage_detect(akz_batch *b, cudaStream_t s, cudaEvent_t *pe = nullptr)
{
  const akz_tables t = akz_make_tables(b);
  const float w = (float)(10.0 / 3.0);
  const float fac1 = (float)(1.0 / (2.0 * ((double)w + 2.0)));
  const float fac2 = w * fac1;
  CK(cudaMemsetAsync(b->d_bitmap, 0, b->bitmap_words * sizeof(uint32_t), s));
  CK(cudaMemsetAsync(b->d_rowcnt, 0, b->rows_all * sizeof(int), s));
  akz_detect_params dp;
  dp.t = t;
  dp.segs = b->d_segs + b->detect_off;
  dp.nsegs = b->detect_n;
  dp.bitmap = b->d_bitmap;
  dp.rowcnt = b->d_rowcnt;
  dp.thr = std::max(b->opt.dthreshold, b->opt.min_dthreshold);
  dp.fac1 = fac1;
  dp.fac2 = fac2;
  dp.store_det = b->opt.extrema_3d;
  dp.fused = b->opt.fast_math;
  CK(akz_launch_detect(dp, b->detect_tiles, b->max_step, s));
  dp.segs = b->d_segs + b->strip_off;
  dp.nsegs = b->strip_n;
  CK(akz_launch_detect_strip(dp, b->strip_tiles, s));
  if (b->opt.extrema_3d) CK(akz_launch_extrema3d(dp, (int)b->lv.size(), b->max_level_h, s));
  if (pe) CK(cudaEventRecord(pe[4], s));
  CK(akz_launch_rowscan(t, b->d_rowcnt, b->d_rowscan, s));
  akz_extract_params ep;
  ep.t = t;
  ep.segs = b->d_segs + b->extract_off;
  ep.nsegs = b->extract_n;
  ep.bitmap = b->d_bitmap;
  ep.rowscan = b->d_rowscan;
  ep.raw = b->d_raw;
  ep.fac1 = fac1;
  ep.fac2 = fac2;
  CK(akz_launch_extract(ep, b->extract_rows, s));
  if (pe) CK(cudaEventRecord(pe[5], s));
  akz_nms_params np;
  np.t = t;
  np.rowscan = b->d_rowscan;
  np.raw = b->d_raw;
  np.state = b->d_state;
  np.aux = b->d_aux;
  np.decision = b->d_dec;
  np.kp = b->d_kp;
  np.max_rounds = b->nms_round_cap;
  np.nbr = b->d_nbr;
  np.nbc = b->d_nbc;
  CK(akz_launch_nms(np, s));
  return AKZ_OK;
}

static akz_status akz_stage_describe(akz_batch *b, cudaStream_t s)
{
  akz_describe_params p;
  p.t = akz_make_tables(b);
  p.kp = b->d_kp;
  p.desc = b->d_desc;
  p.upright = b->opt.descriptor == AKZ_MLDB_UPRIGHT;
  p.pattern_size = b->opt.descriptor_pattern_size;
  p.channels = b->opt.descriptor_channels;
  p.nbits = b->nbits;
  p.cmp1 = b->d_cmp;
  p.cmp2 = b->d_cmp + 512;
  /* exp(-r2/12.5) with the shared deterministic exp (the CPU restatement
   * uses the same routine), so the weights are identical on every host */
  for (int r2 = 0; r2 < 36; r2++) p.gw[r2] = akz_expf((float)(-r2) / (2.5f * 2.5f * 2.0f));
  CK(akz_launch_describe(p, 8 * b->nsm, s));
  return AKZ_OK;
}

static akz_status akz_run_all(akz_batch *b, cudaStream_t s)
{
  akz_status st = akz_stage_scale(b, s);
  if (st == AKZ_OK) st = akz_stage_detect(b, s);
  if (st == AKZ_OK) st = akz_stage_describe(b, s);
  return st;
}

/* drops the captured graphs (after a change of the launches they hold) */
static void akz_drop_graphs(akz_batch *b)
{
  for (auto &ge : b->graphs) {
    if (ge.g) cudaGraphExecDestroy(ge.g);
    ge.g = nullptr;
  }
}

/* Whole-batch run, captured once per input staging buffer into a CUDA graph
 * and replayed. */
static akz_status akz_batch_launch(akz_batch *b)
{
  cudaStream_t s = b->stream;
  akz_batch::akz_graph_entry &ge = b->graphs[b->u8 == b->u8_arena ? 0 : 1];
  if (ge.g && (ge.f32 != b->input_f32 || ge.s != s)) {
    cudaGraphExecDestroy(ge.g);
    ge.g = nullptr;
  }
  if (!ge.g) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    akz_status st = akz_run_all(b, s);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st != AKZ_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return akz_fail_cuda(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    e = cudaGraphInstantiate(&ge.g, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      ge.g = nullptr;
      return akz_fail_cuda(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    ge.f32 = b->input_f32;
    ge.s = s;
  }
  CK(cudaGraphLaunch(ge.g, s));
  return AKZ_OK;
}

static akz_status akz_batch_sync_stats(akz_batch *b)
{
  CK(cudaMemcpyAsync(b->h_stats, b->d_stats, (size_t)b->nimg * sizeof(akz_image_stats), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->nimg; i++) {
    if (b->h_stats[i].overflow)
      return akz_fail(AKZ_ERR_OVERFLOW, "image %d: %d raw extrema exceed maxkeypoints=%d", i, b->h_stats[i].nraw, b->opt.maxkeypoints);
    if (b->h_stats[i].status == AKZ_ERR_TIMEOUT) return akz_fail(AKZ_ERR_TIMEOUT, "image %d: suppression did not settle", i);
  }
  return AKZ_OK;
}

static akz_status akz_copy_results(akz_batch *b, int i, akz_keypoint *kpts, uint8_t *desc, int capacity, int *n)
{
  const int nk = b->h_stats[i].nkp;
  const int m = std::min(nk, std::max(capacity, 0));
  const akz_image_desc &I = b->im[i];
  if (m > 0 && kpts) CK(cudaMemcpyAsync(kpts, b->d_kp + I.kp_base, (size_t)m * sizeof(akz_kp), cudaMemcpyDeviceToHost, b->stream));
  if (m > 0 && desc)
    CK(cudaMemcpy2DAsync(desc, b->row_bytes, (const uint8_t *)b->d_desc + (size_t)I.kp_base * 64, 64, b->row_bytes, m,
                         cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (n) *n = nk;
  return AKZ_OK;
}

/* ------------------------------------------------------------------------ */
/* single-image context                                                     */

struct akz_context {
  akz_batch *b = nullptr;
  int have_scale = 0, have_detect = 0;
  akz_timing timing;
  float *f32 = nullptr;
};

#define AKZ_GUARD(c)                                                                  \
  do {                                                                                \
    if (!(c)) return akz_fail(AKZ_ERR_INVALID_ARG, "%s: NULL handle", __func__); \
  } while (0)

extern "C" {

AKZ_API const char *akz_version(void) { return "akaze_gb300 0.1 (sm_103a)"; }
AKZ_API const char *akz_last_error(void) { return g_last_error.c_str(); }

AKZ_API akz_status akz_options_default(akz_options *o)
{
  if (!o) return akz_fail(AKZ_ERR_INVALID_ARG, "options are NULL");
  memset(o, 0, sizeof(*o));
  o->soffset = 1.6f;
  o->derivative_factor = 1.5f;
  o->omax = 4;
  o->nsublevels = 4;
  o->dthreshold = 0.001f;
  o->min_dthreshold = 0.00001f;
  o->diffusivity = AKZ_PM_G2;
  o->descriptor = AKZ_MLDB;
  o->descriptor_size = 0;
  o->descriptor_channels = 3;
  o->descriptor_pattern_size = 10;
  o->sderivatives = 1.0f;
  o->kcontrast = 0.001f;
  o->kcontrast_percentile = 0.7f;
  o->kcontrast_nbins = 300;
  o->ncudaimages = 4;
  o->maxkeypoints = 16 * 8192;
  o->extrema_3d = 0;
  o->fast_math = 0;
  return AKZ_OK;
}

AKZ_API akz_status akz_descriptor_bytes(const akz_options *opt, int *bytes)
{
  if (!bytes) return akz_fail(AKZ_ERR_INVALID_ARG, "bytes is NULL");
  akz_status st = akz_validate(opt);
  if (st != AKZ_OK) return st;
  *bytes = akz_row_bytes(opt);
  return AKZ_OK;
}

AKZ_API akz_status akz_plan_info(const akz_options *opt, int width, int height, int level, int *nlevels, int *lw, int *lh,
                                 int *octave, int *sublevel, float *esigma, int *deriv_step, float *border, float *tau,
                                 int tau_cap, int *nsteps)
{
  akz_status st = akz_validate(opt);
  if (st != AKZ_OK) return st;
  if (width < 1 || height < 1) return akz_fail(AKZ_ERR_INVALID_ARG, "bad image size");
  std::vector<akz_geo> L;
  std::vector<std::vector<float>> tv;
  akz_plan_levels(*opt, width, height, L, tv);
  if (nlevels) *nlevels = (int)L.size();
  if (level < 0) return AKZ_OK;
  if (level >= (int)L.size()) return akz_fail(AKZ_ERR_INVALID_ARG, "level %d out of range", level);
  const akz_geo &g = L[level];
  if (lw) *lw = g.w;
  if (lh) *lh = g.h;
  if (octave) *octave = g.octave;
  if (sublevel) *sublevel = g.sublevel;
  if (esigma) *esigma = g.esigma;
  if (deriv_step) *deriv_step = g.deriv_step;
  if (border) *border = g.border;
  if (nsteps) *nsteps = g.nsteps;
  if (tau)
    for (int k = 0; k < g.nsteps && k < tau_cap; k++) tau[k] = tv[level][k];
  return AKZ_OK;
}

AKZ_API akz_status akz_gaussian_taps(float sigma, float *taps, int cap, int *ntaps)
{
  float t[AKZ_MAX_TAPS];
  const int R = akz_gauss_taps(sigma, t);
  if (R < 0) return akz_fail(AKZ_ERR_INVALID_ARG, "Gaussian radius out of range");
  if (ntaps) *ntaps = 2 * R + 1;
  for (int i = 0; i <= 2 * R && i < cap; i++) taps[i] = t[i];
  return AKZ_OK;
}

AKZ_API akz_status akz_create(const akz_options *opt, akz_context **out)
{
  if (!opt || !out) return akz_fail(AKZ_ERR_INVALID_ARG, "akz_create: NULL argument");
  akz_context *c = new (std::nothrow) akz_context();
  if (!c) return akz_fail(AKZ_ERR_OOM, "host allocation failed");
  memset(&c->timing, 0, sizeof(c->timing));
  const int w = opt->img_width, h = opt->img_height;
  akz_status st = akz_batch_build(opt, 1, &w, &h, &c->b);
  if (st != AKZ_OK) {
    delete c;
    return st;
  }
  *out = c;
  return AKZ_OK;
}

AKZ_API akz_status akz_destroy(akz_context *c)
{
  if (!c) return AKZ_OK;
  if (c->f32) cudaFree(c->f32);
  akz_batch_free(c->b);
  delete c;
  return AKZ_OK;
}

AKZ_API akz_status akz_set_stream(akz_context *c, void *stream)
{
  AKZ_GUARD(c);
  c->b->stream = stream ? (cudaStream_t)stream : c->b->own_stream;
  return AKZ_OK;
}

AKZ_API akz_status akz_create_nonlinear_scale_space(akz_context *c, const void *img, int width, int height, size_t stride,
                                                    int dtype, int on_device)
{
  AKZ_GUARD(c);
  akz_batch *b = c->b;
  if (!img) return akz_fail(AKZ_ERR_INVALID_ARG, "image is NULL");
  if (width != b->W[0] || height != b->H[0])
    return akz_fail(AKZ_ERR_INVALID_ARG, "image is %dx%d but the context was created for %dx%d", width, height, b->W[0], b->H[0]);
  if (dtype != AKZ_U8 && dtype != AKZ_F32) return akz_fail(AKZ_ERR_INVALID_ARG, "unknown dtype %d", dtype);
  const size_t elem = dtype == AKZ_U8 ? 1 : 4;
  if (stride < (size_t)width * elem) return akz_fail(AKZ_ERR_INVALID_ARG, "stride %zu below the row size", stride);
  cudaStream_t s = b->stream;
  const akz_image_desc &I = b->im[0];
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (dtype == AKZ_U8) {
    CK(cudaMemcpy2DAsync(b->u8 + I.u8_off, I.u8_pitch, img, stride, width, height, kind, s));
    b->input_f32 = 0;
  } else {
    if (!b->f32) CK(cudaMalloc(&b->f32, b->staging_elems * sizeof(float)));
    CK(cudaMemcpy2DAsync(b->f32 + I.u8_off, (size_t)I.u8_pitch * 4, img, stride, (size_t)width * 4, height, kind, s));
    b->input_f32 = 1;
  }
  CK(cudaEventRecord(b->ev[0], s));
  akz_status st = akz_stage_scale(b, s);
  if (st != AKZ_OK) return st;
  CK(cudaEventRecord(b->ev[1], s));
  CK(cudaEventSynchronize(b->ev[1]));
  c->timing.kcontrast = 0.0;
  c->timing.scale = akz_ms(b->ev[0], b->ev[1]);
  c->have_scale = 1;
  c->have_detect = 0;
  return AKZ_OK;
}

AKZ_API akz_status akz_feature_detection(akz_context *c, int *n)
{
  AKZ_GUARD(c);
  if (!c->have_scale) return akz_fail(AKZ_ERR_STATE, "Feature_Detection before Create_Nonlinear_Scale_Space");
  akz_batch *b = c->b;
  CK(cudaEventRecord(b->ev[2], b->stream));
  akz_status st = akz_stage_detect(b, b->stream);
  if (st != AKZ_OK) return st;
  CK(cudaEventRecord(b->ev[3], b->stream));
  st = akz_batch_sync_stats(b);
  if (st != AKZ_OK) return st;
  c->timing.detector = akz_ms(b->ev[2], b->ev[3]);
  c->timing.derivatives = 0.0;
  c->timing.extrema = c->timing.detector;
  c->have_detect = 1;
  if (n) *n = b->h_stats[0].nkp;
  return AKZ_OK;
}

AKZ_API akz_status akz_compute_descriptors(akz_context *c, akz_keypoint *kpts, uint8_t *desc, int capacity, int *n)
{
  AKZ_GUARD(c);
  if (!c->have_detect) return akz_fail(AKZ_ERR_STATE, "Compute_Descriptors before Feature_Detection");
  akz_batch *b = c->b;
  CK(cudaEventRecord(b->ev[4], b->stream));
  akz_status st = akz_stage_describe(b, b->stream);
  if (st != AKZ_OK) return st;
  CK(cudaEventRecord(b->ev[5], b->stream));
  st = akz_copy_results(b, 0, kpts, desc, capacity, n);
  if (st != AKZ_OK) return st;
  c->timing.descriptor = akz_ms(b->ev[4], b->ev[5]);
  return AKZ_OK;
}

AKZ_API akz_status akz_get_timing(akz_context *c, akz_timing *t)
{
  AKZ_GUARD(c);
  if (!t) return akz_fail(AKZ_ERR_INVALID_ARG, "timing is NULL");
  *t = c->timing;
  return AKZ_OK;
}

AKZ_API akz_status akz_num_levels(const akz_context *c, int *n)
{
  AKZ_GUARD(c);
  if (n) *n = c->b->im[0].nlev;
  return AKZ_OK;
}

AKZ_API akz_status akz_level_info(const akz_context *c, int level, int *w, int *h, int *octave, int *sublevel, float *esigma, int *nsteps)
{
  AKZ_GUARD(c);
  const akz_batch *b = c->b;
  if (level < 0 || level >= b->im[0].nlev) return akz_fail(AKZ_ERR_INVALID_ARG, "level %d out of range", level);
  const akz_geo &g = b->geo[0][level];
  if (w) *w = g.w;
  if (h) *h = g.h;
  if (octave) *octave = g.octave;
  if (sublevel) *sublevel = g.sublevel;
  if (esigma) *esigma = g.esigma;
  if (nsteps) *nsteps = g.nsteps;
  return AKZ_OK;
}

static akz_status akz_plane_out(akz_batch *b, int i, int level, int plane, float *out)
{
  if (i < 0 || i >= b->nimg) return akz_fail(AKZ_ERR_INVALID_ARG, "image %d out of range", i);
  if (level < 0 || level >= b->im[i].nlev) return akz_fail(AKZ_ERR_INVALID_ARG, "level %d out of range", level);
  if (!out) return akz_fail(AKZ_ERR_INVALID_ARG, "output is NULL");
  const akz_level_desc &L = b->lv[b->im[i].first_level + level];
  long long off;
  switch (plane) {
    case AKZ_PLANE_LT: off = L.lt; break;
    case AKZ_PLANE_LSMOOTH: off = L.ls; break;
    case AKZ_PLANE_LX:
    case AKZ_PLANE_LY: {
      /* the interleaved (Lx, Ly) plane, split on the host */
      std::vector<float> tmp((size_t)2 * L.width * L.height);
      CK(cudaMemcpy2DAsync(tmp.data(), (size_t)L.width * 8, b->planes + L.lx, (size_t)L.pitch * 8, (size_t)L.width * 8,
                           L.height, cudaMemcpyDeviceToHost, b->stream));
      CK(cudaStreamSynchronize(b->stream));
      const int k = plane == AKZ_PLANE_LY ? 1 : 0;
      for (size_t q = 0; q < (size_t)L.width * L.height; q++) out[q] = tmp[2 * q + k];
      return AKZ_OK;
    }
    default: return akz_fail(AKZ_ERR_INVALID_ARG, "unknown plane %d", plane);
  }
  CK(cudaMemcpy2DAsync(out, (size_t)L.width * 4, b->planes + off, (size_t)L.pitch * 4, (size_t)L.width * 4, L.height,
                       cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return AKZ_OK;
}

AKZ_API akz_status akz_get_level_plane(akz_context *c, int level, int plane, float *out)
{
  AKZ_GUARD(c);
  if (!c->have_scale) return akz_fail(AKZ_ERR_STATE, "no scale space yet");
  return akz_plane_out(c->b, 0, level, plane, out);
}

AKZ_API akz_status akz_get_kcontrast(akz_context *c, float *k)
{
  AKZ_GUARD(c);
  if (!c->have_scale) return akz_fail(AKZ_ERR_STATE, "no scale space yet");
  akz_image_stats s;
  CK(cudaMemcpyAsync(&s, c->b->d_stats, sizeof(s), cudaMemcpyDeviceToHost, c->b->stream));
  CK(cudaStreamSynchronize(c->b->stream));
  if (k) *k = s.kcontrast;
  return AKZ_OK;
}

AKZ_API akz_status akz_get_extrema(akz_context *c, akz_extremum *out, int cap, int *n)
{
  AKZ_GUARD(c);
  if (!c->have_detect) return akz_fail(AKZ_ERR_STATE, "no detection yet");
  akz_batch *b = c->b;
  const int nr = b->h_stats[0].nraw;
  const int m = std::min(nr, std::max(cap, 0));
  if (m > 0 && out) {
    CK(cudaMemcpyAsync(out, b->d_raw + b->im[0].raw_base, (size_t)m * sizeof(akz_raw), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
  }
  if (n) *n = nr;
  return AKZ_OK;
}

/* ---- batch ---------------------------------------------------------------- */

AKZ_API akz_status akz_batch_create(const akz_options *opt, int n, const int *w, const int *h, akz_batch **out)
{
  if (!out) return akz_fail(AKZ_ERR_INVALID_ARG, "akz_batch_create: NULL output");
  return akz_batch_build(opt, n, w, h, out);
}

AKZ_API akz_status akz_batch_destroy(akz_batch *b)
{
  akz_batch_free(b);
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_set_stream(akz_batch *b, void *stream)
{
  AKZ_GUARD(b);
  b->stream = stream ? (cudaStream_t)stream : b->own_stream;
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_upload(akz_batch *b, const uint8_t *const *images, const size_t *strides, int on_device)
{
  AKZ_GUARD(b);
  if (!images || !strides) return akz_fail(AKZ_ERR_INVALID_ARG, "images/strides are NULL");
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  for (int i = 0; i < b->nimg; i++) {
    if (!images[i] || strides[i] < (size_t)b->W[i]) return akz_fail(AKZ_ERR_INVALID_ARG, "image %d: bad pointer or stride", i);
    const akz_image_desc &I = b->im[i];
    CK(cudaMemcpy2DAsync(b->u8 + I.u8_off, I.u8_pitch, images[i], strides[i], b->W[i], b->H[i], kind, b->stream));
  }
  b->input_f32 = 0;
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_input(akz_batch *b, int i, uint8_t **dptr, size_t *pitch)
{
  AKZ_GUARD(b);
  if (i < 0 || i >= b->nimg) return akz_fail(AKZ_ERR_INVALID_ARG, "image %d out of range", i);
  if (dptr) *dptr = b->u8 + b->im[i].u8_off;
  if (pitch) *pitch = (size_t)b->im[i].u8_pitch;
  b->input_f32 = 0;
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_run(akz_batch *b)
{
  AKZ_GUARD(b);
  return akz_batch_launch(b);
}

AKZ_API akz_status akz_batch_counts(akz_batch *b, int *counts)
{
  AKZ_GUARD(b);
  akz_status st = akz_batch_sync_stats(b);
  if (st != AKZ_OK) return st;
  if (counts)
    for (int i = 0; i < b->nimg; i++) counts[i] = b->h_stats[i].nkp;
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_results(akz_batch *b, int i, akz_keypoint *kpts, uint8_t *desc, int capacity, int *n)
{
  AKZ_GUARD(b);
  if (i < 0 || i >= b->nimg) return akz_fail(AKZ_ERR_INVALID_ARG, "image %d out of range", i);
  akz_status st = akz_batch_sync_stats(b);
  if (st != AKZ_OK) return st;
  return akz_copy_results(b, i, kpts, desc, capacity, n);
}

AKZ_API akz_status akz_batch_device_results(akz_batch *b, int i, akz_keypoint **kpts, uint8_t **desc64)
{
  AKZ_GUARD(b);
  if (i < 0 || i >= b->nimg) return akz_fail(AKZ_ERR_INVALID_ARG, "image %d out of range", i);
  if (kpts) *kpts = (akz_keypoint *)(b->d_kp + b->im[i].kp_base);
  if (desc64) *desc64 = (uint8_t *)b->d_desc + (size_t)b->im[i].kp_base * 64;
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_detect_describe(akz_batch *b, const uint8_t *const *images, const size_t *strides,
                                             akz_keypoint *const *kpts, uint8_t *const *desc, const int *caps, int *counts)
{
  AKZ_GUARD(b);
  akz_status st = akz_batch_upload(b, images, strides, 0);
  if (st == AKZ_OK) st = akz_batch_launch(b);
  if (st == AKZ_OK) st = akz_batch_sync_stats(b);
  if (st != AKZ_OK) return st;
  for (int i = 0; i < b->nimg; i++) {
    const int nk = b->h_stats[i].nkp;
    const int m = std::min(nk, caps ? std::max(caps[i], 0) : 0);
    const akz_image_desc &I = b->im[i];
    if (m > 0 && kpts && kpts[i])
      CK(cudaMemcpyAsync(kpts[i], b->d_kp + I.kp_base, (size_t)m * sizeof(akz_kp), cudaMemcpyDeviceToHost, b->stream));
    if (m > 0 && desc && desc[i])
      CK(cudaMemcpy2DAsync(desc[i], b->row_bytes, (const uint8_t *)b->d_desc + (size_t)I.kp_base * 64, 64, b->row_bytes,
                           m, cudaMemcpyDeviceToHost, b->stream));
    if (counts) counts[i] = nk;
  }
  CK(cudaStreamSynchronize(b->stream));
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_image_info(akz_batch *b, int i, int *nraw, int *nkp, int *rounds, float *kcontrast)
{
  AKZ_GUARD(b);
  if (i < 0 || i >= b->nimg) return akz_fail(AKZ_ERR_INVALID_ARG, "akz_batch_image_info: image %d out of range", i);
  akz_image_stats st;
  CK(cudaMemcpyAsync(&st, b->d_stats + i, sizeof(st), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (nraw) *nraw = st.nraw;
  if (nkp) *nkp = st.nkp;
  if (rounds) *rounds = st.nms_rounds;
  if (kcontrast) *kcontrast = st.kcontrast;
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_submit(akz_batch *b, const uint8_t *const *images, const size_t *strides)
{
  AKZ_GUARD(b);
  if (b->sub_n == 2) return akz_fail(AKZ_ERR_STATE, "akz_batch_submit: two runs outstanding, collect one first");
  if (!b->slots_ready) { /* first use */
    const size_t bytes = b->raw_all * (sizeof(akz_kp) + (size_t)b->row_bytes);
    for (int k = 0; k < 2; k++) {
      if (!b->d_slot[k]) CK(cudaMalloc(&b->d_slot[k], std::max<size_t>(bytes, 1)));
      if (!b->h_slot_stats[k]) CK(cudaMallocHost(&b->h_slot_stats[k], (size_t)b->nimg * sizeof(akz_image_stats)));
      if (!b->ev_slot[k]) CK(cudaEventCreateWithFlags(&b->ev_slot[k], cudaEventDisableTiming));
    }
    if (!b->copy_stream) CK(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking));
    if (!b->up_stream) CK(cudaStreamCreateWithFlags(&b->up_stream, cudaStreamNonBlocking));
    if (!b->d_stage2) CK(cudaMalloc(&b->d_stage2, std::max<size_t>(b->staging_elems, 1)));
    for (int k = 0; k < 2; k++) {
      if (!b->ev_stage_full[k]) CK(cudaEventCreateWithFlags(&b->ev_stage_full[k], cudaEventDisableTiming));
      if (!b->ev_stage_free[k]) CK(cudaEventCreateWithFlags(&b->ev_stage_free[k], cudaEventDisableTiming));
    }
    b->slots_ready = true;
  }
  if (!images || !strides) return akz_fail(AKZ_ERR_INVALID_ARG, "images/strides are NULL");
  for (int i = 0; i < b->nimg; i++)
    if (!images[i] || strides[i] < (size_t)b->W[i]) return akz_fail(AKZ_ERR_INVALID_ARG, "image %d: bad pointer or stride", i);
  const int slot = (b->sub_first + b->sub_n) & 1;
  /* the host images go up into staging buffer q once the graph that last
   * read it (two runs back) is done, beside the previous run's graph; this
   * run's graph, captured for buffer q, waits for them and, in the batch's
   * stream order, for the previous run's pack, which has read the keypoints
   * and descriptors */
  const int q = b->stage_next;
  uint8_t *stage = q ? b->d_stage2 : b->u8_arena;
  CK(cudaStreamWaitEvent(b->up_stream, b->ev_stage_free[q], 0));
  for (int i = 0; i < b->nimg; i++) {
    const akz_image_desc &I = b->im[i];
    CK(cudaMemcpy2DAsync(stage + I.u8_off, I.u8_pitch, images[i], strides[i], b->W[i], b->H[i], cudaMemcpyHostToDevice,
                         b->up_stream));
  }
  CK(cudaEventRecord(b->ev_stage_full[q], b->up_stream));
  CK(cudaStreamWaitEvent(b->stream, b->ev_stage_full[q], 0));
  b->input_f32 = 0;
  b->u8 = stage;
  const akz_status st = akz_batch_launch(b);
  b->u8 = b->u8_arena;
  if (st != AKZ_OK) return st;
  CK(cudaEventRecord(b->ev_stage_free[q], b->stream));
  b->stage_next = q ^ 1;
  akz_kp *pk = (akz_kp *)b->d_slot[slot];
  uint8_t *pd = (uint8_t *)(pk + b->raw_all);
  CK(akz_launch_pack_results(akz_make_tables(b), b->d_kp, b->d_desc, pk, pd, b->row_bytes, b->stream));
  CK(cudaMemcpyAsync(b->h_slot_stats[slot], b->d_stats, (size_t)b->nimg * sizeof(akz_image_stats), cudaMemcpyDeviceToHost,
                     b->stream));
  CK(cudaEventRecord(b->ev_slot[slot], b->stream));
  b->sub_n++;
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_collect_packed(akz_batch *b, akz_keypoint *kpts, uint8_t *desc, int capacity, int *counts,
                                            int *total)
{
  AKZ_GUARD(b);
  if (!counts || !total || capacity < 0) return akz_fail(AKZ_ERR_INVALID_ARG, "akz_batch_collect_packed: bad arguments");
  if (b->sub_n == 0) return akz_fail(AKZ_ERR_STATE, "akz_batch_collect_packed: nothing submitted");
  const int slot = b->sub_first;
  b->sub_first ^= 1;
  b->sub_n--;
  CK(cudaEventSynchronize(b->ev_slot[slot]));
  const akz_image_stats *hs = b->h_slot_stats[slot];
  for (int i = 0; i < b->nimg; i++) {
    if (hs[i].overflow)
      return akz_fail(AKZ_ERR_OVERFLOW, "image %d: %d raw extrema exceed maxkeypoints=%d", i, hs[i].nraw, b->opt.maxkeypoints);
    if (hs[i].status == AKZ_ERR_TIMEOUT) return akz_fail(AKZ_ERR_TIMEOUT, "image %d: suppression did not settle", i);
  }
  long long n = 0;
  for (int i = 0; i < b->nimg; i++) {
    counts[i] = hs[i].nkp;
    n += counts[i];
  }
  *total = (int)n;
  if (n > capacity)
    return akz_fail(AKZ_ERR_OVERFLOW, "akz_batch_collect_packed: %lld keypoints exceed the capacity %d", n, capacity);
  if (n == 0) return AKZ_OK;
  /* on the copy stream, beside the next run's graph */
  const akz_kp *pk = (const akz_kp *)b->d_slot[slot];
  const uint8_t *pd = (const uint8_t *)(pk + b->raw_all);
  if (kpts) CK(cudaMemcpyAsync(kpts, pk, (size_t)n * sizeof(akz_kp), cudaMemcpyDeviceToHost, b->copy_stream));
  if (desc) CK(cudaMemcpyAsync(desc, pd, (size_t)n * b->row_bytes, cudaMemcpyDeviceToHost, b->copy_stream));
  CK(cudaStreamSynchronize(b->copy_stream));
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_detect_describe_packed(akz_batch *b, const uint8_t *const *images, const size_t *strides,
                                                    akz_keypoint *kpts, uint8_t *desc, int capacity, int *counts,
                                                    int *total)
{
  AKZ_GUARD(b);
  if (!counts || !total || capacity < 0) return akz_fail(AKZ_ERR_INVALID_ARG, "akz_batch_detect_describe_packed: bad arguments");
  if (b->sub_n) return akz_fail(AKZ_ERR_STATE, "akz_batch_detect_describe_packed: a submitted run is not collected");
  const akz_status st = akz_batch_submit(b, images, strides);
  if (st != AKZ_OK) return st;
  return akz_batch_collect_packed(b, kpts, desc, capacity, counts, total);
}

AKZ_API akz_status akz_batch_level_plane(akz_batch *b, int i, int level, int plane, float *out)
{
  AKZ_GUARD(b);
  return akz_plane_out(b, i, level, plane, out);
}

/* Number of kernels one akz_batch_run launches. */
static int akz_batch_nkernels(const akz_batch *b)
{
  /* level 0 + contrast: k_level0, k_contrast_hist, k_contrast_final
   * (radius <= 4), else k_contrast x2, k_contrast_final, k_gauss0; then the
   * detector (strip and/or tile kernel), k_rowscan, k_extract, k_extract_fit,
   * k_nms, k_describe */
  int n = (b->R0 <= 4 ? 3 : 4) + 5 + (b->strip_tiles > 0) + (b->detect_tiles > 0);
  for (int l = 1; l < b->maxlev; l++) {
    n += b->area[l].nsegs > 0 ? 1 : 0;
    if (b->sg_on && l / b->opt.nsublevels >= b->sg_first_octave) {
      n += 1 + 6 * b->nimg; /* zero-step prologue, per image im2col + 5 GEMMs */
      if (b->sg_tol > 0.0f) n += (int)b->sg_check[l].size() + 1 + (int)b->fed[l].size();
    } else {
      n += (int)b->fed[l].size();
    }
  }
  return n;
}

AKZ_API akz_status akz_batch_kernel_count(const akz_batch *b, int *n)
{
  AKZ_GUARD(b);
  if (n) *n = akz_batch_nkernels(b);
  return AKZ_OK;
}

/* One run without the graph, with events between stage groups; stage_ms
 * receives up to 7 entries: contrast, level 0, levels 1.., detector,
 * scan+extract, suppression, orientation+M-LDB. */
AKZ_API akz_status akz_batch_profile(akz_batch *b, float *stage_ms, int n)
{
  AKZ_GUARD(b);
  cudaStream_t s = b->stream;
  cudaEvent_t *pe = b->ev;
  CK(cudaEventRecord(pe[0], s));
  akz_status st = akz_stage_scale(b, s, pe);
  if (st != AKZ_OK) return st;
  CK(cudaEventRecord(pe[3], s));
  st = akz_stage_detect(b, s, pe);
  if (st != AKZ_OK) return st;
  CK(cudaEventRecord(pe[6], s));
  st = akz_stage_describe(b, s);
  if (st != AKZ_OK) return st;
  CK(cudaEventRecord(pe[7], s));
  CK(cudaEventSynchronize(pe[7]));
  for (int k = 0; k < 7 && k < n; k++) stage_ms[k] = akz_ms(pe[k], pe[k + 1]);
  return AKZ_OK;
}

/* ---- matcher ------------------------------------------------------------ */

struct akz_matcher {
  cudaStream_t stream = nullptr, own = nullptr;
  void *dq = nullptr, *dt = nullptr, *dout = nullptr, *dpart = nullptr;
  size_t capq = 0, capt = 0, capout = 0, cappart = 0;
  int nsm = 152;
};

AKZ_API akz_status akz_matcher_create(akz_matcher **out)
{
  if (!out) return akz_fail(AKZ_ERR_INVALID_ARG, "akz_matcher_create: NULL output");
  akz_matcher *m = new (std::nothrow) akz_matcher();
  if (!m) return akz_fail(AKZ_ERR_OOM, "host allocation failed");
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaStreamCreateWithFlags(&m->own, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete m;
    return akz_fail_cuda(e, "cudaStreamCreate", __FILE__, __LINE__);
  }
  m->stream = m->own;
  *out = m;
  return AKZ_OK;
}

AKZ_API akz_status akz_matcher_destroy(akz_matcher *m)
{
  if (!m) return AKZ_OK;
  cudaFree(m->dq);
  cudaFree(m->dt);
  cudaFree(m->dout);
  cudaFree(m->dpart);
  if (m->own) cudaStreamDestroy(m->own);
  delete m;
  return AKZ_OK;
}

AKZ_API akz_status akz_matcher_set_stream(akz_matcher *m, void *stream)
{
  AKZ_GUARD(m);
  m->stream = stream ? (cudaStream_t)stream : m->own;
  return AKZ_OK;
}

static akz_status akz_grow(void **p, size_t *cap, size_t need)
{
  if (need <= *cap) return AKZ_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  const size_t n = std::max<size_t>(need, 4096);
  CK(cudaMalloc(p, n));
  *cap = n;
  return AKZ_OK;
}

static akz_status akz_match_device(akz_matcher *m, const void *dq, int nq, const void *dt, int nt, void *dout)
{
  const int ns = akz_match_splits(nq, nt, m->nsm);
  if (ns > 1) {
    akz_status st = akz_grow(&m->dpart, &m->cappart, akz_match_partial_bytes(nq, ns));
    if (st != AKZ_OK) return st;
  }
  CK(akz_match_run(dq, nq, dt, nt, dout, m->dpart, ns, m->stream));
  return AKZ_OK;
}

AKZ_API akz_status akz_matcher_bfmatch(akz_matcher *m, const uint8_t *q, int nq, const uint8_t *t, int nt, int row_bytes, akz_dmatch *out)
{
  AKZ_GUARD(m);
  if (nq < 0 || nt < 0 || row_bytes < 1 || row_bytes > 64) return akz_fail(AKZ_ERR_INVALID_ARG, "bad matcher sizes");
  if ((nq > 0 && (!q || !out)) || (nt > 0 && !t)) return akz_fail(AKZ_ERR_INVALID_ARG, "NULL matcher buffer");
  if (nq == 0) return AKZ_OK;
  akz_status st = akz_grow(&m->dq, &m->capq, (size_t)nq * 64);
  if (st == AKZ_OK) st = akz_grow(&m->dt, &m->capt, (size_t)std::max(nt, 1) * 64);
  if (st == AKZ_OK) st = akz_grow(&m->dout, &m->capout, (size_t)nq * 2 * sizeof(akz_dmatch));
  if (st != AKZ_OK) return st;
  CK(cudaMemsetAsync(m->dq, 0, (size_t)nq * 64, m->stream));
  CK(cudaMemcpy2DAsync(m->dq, 64, q, row_bytes, row_bytes, nq, cudaMemcpyHostToDevice, m->stream));
  if (nt > 0) {
    CK(cudaMemsetAsync(m->dt, 0, (size_t)nt * 64, m->stream));
    CK(cudaMemcpy2DAsync(m->dt, 64, t, row_bytes, row_bytes, nt, cudaMemcpyHostToDevice, m->stream));
  }
  st = akz_match_device(m, m->dq, nq, m->dt, nt, m->dout);
  if (st != AKZ_OK) return st;
  CK(cudaMemcpyAsync(out, m->dout, (size_t)nq * 2 * sizeof(akz_dmatch), cudaMemcpyDeviceToHost, m->stream));
  CK(cudaStreamSynchronize(m->stream));
  return AKZ_OK;
}

AKZ_API akz_status akz_matcher_bfmatch_device(akz_matcher *m, const uint8_t *q64, int nq, const uint8_t *t64, int nt, akz_dmatch *out)
{
  AKZ_GUARD(m);
  if (nq < 0 || nt < 0) return akz_fail(AKZ_ERR_INVALID_ARG, "bad matcher sizes");
  if (nq == 0) return AKZ_OK;
  if (!q64 || !out || (nt > 0 && !t64)) return akz_fail(AKZ_ERR_INVALID_ARG, "NULL matcher buffer");
  return akz_match_device(m, q64, nq, t64, nt, out);
}

static void akz_use_fed_depths(akz_batch *b)
{
  for (int l = 1; l < b->maxlev; l++) b->fed[l] = b->fed_alt[b->fed_depth[l] - AKZ_DEPTH_MIN][l];
  akz_drop_graphs(b); /* the captured graphs hold the old launches */
}

AKZ_API akz_status akz_batch_set_nms_round_cap(akz_batch *b, int cap)
{
  AKZ_GUARD(b);
  if (cap < 1) return akz_report(AKZ_ERR_INVALID_ARG, "akz_batch_set_nms_round_cap: cap must be >= 1");
  b->nms_round_cap = cap;
  akz_drop_graphs(b); /* the captured graphs hold the old cap */
  return AKZ_OK;
}

AKZ_API akz_status akz_batch_set_fed_depth(akz_batch *b, int depth)
{
  AKZ_GUARD(b);
  if (depth < AKZ_DEPTH_MIN || depth > AKZ_MAX_STEPS_PER_LAUNCH)
    return akz_report(AKZ_ERR_INVALID_ARG, "akz_batch_set_fed_depth: depth must be 4..8");
  for (int l = 1; l < b->maxlev; l++) b->fed_depth[l] = depth;
  akz_use_fed_depths(b);
  return AKZ_OK;
}

/* FED blocking depth autotuner: times every level of the uploaded batch at
 * each depth (the levels' launches do not depend on one another's chunking)
 * and keeps the fastest depth per level. */
AKZ_API akz_status akz_batch_autotune(akz_batch *b, float *ms_per_depth, int cap, int *depths, int ndepths)
{
  AKZ_GUARD(b);
  const int nd = AKZ_MAX_STEPS_PER_LAUNCH - AKZ_DEPTH_MIN + 1, nl = b->maxlev;
  std::vector<cudaEvent_t> ev(nl + 1, nullptr);
  cudaError_t ce = cudaSuccess;
  for (auto &e : ev)
    if (ce == cudaSuccess) ce = cudaEventCreate(&e);
  std::vector<std::vector<float>> tl(nd, std::vector<float>(nl, 1e30f));
  std::vector<float> tot(nd, 1e30f);
  akz_status st = AKZ_OK;
  for (int k = 0; k < nd && ce == cudaSuccess && st == AKZ_OK; k++) {
    b->fed = b->fed_alt[k];
    for (int rep = 0; rep < 4 && ce == cudaSuccess && st == AKZ_OK; rep++) {
      ce = cudaEventRecord(ev[nl], b->stream);
      if (ce == cudaSuccess) st = akz_stage_scale(b, b->stream, nullptr, ev.data());
      if (ce == cudaSuccess && st == AKZ_OK) ce = cudaEventSynchronize(ev[nl - 1]);
      if (rep == 0) continue; /* the first repetition warms up */
      float ms = 0.0f;
      if (ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, ev[nl], ev[nl - 1]);
      tot[k] = std::min(tot[k], ms);
      for (int l = 1; l < nl && ce == cudaSuccess; l++) {
        ce = cudaEventElapsedTime(&ms, ev[l - 1], ev[l]);
        tl[k][l] = std::min(tl[k][l], ms);
      }
    }
  }
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  if (st != AKZ_OK) return st;
  if (ce != cudaSuccess) return akz_report(AKZ_ERR_CUDA, cudaGetErrorString(ce));
  for (int k = 0; k < nd && k < cap && ms_per_depth; k++) ms_per_depth[k] = tot[k];
  for (int l = 1; l < nl; l++) {
    int best = nd - 1;
    for (int k = 0; k < nd; k++)
      if (tl[k][l] < tl[best][l]) best = k;
    b->fed_depth[l] = AKZ_DEPTH_MIN + best;
  }
  for (int l = 0; l < ndepths && depths; l++) depths[l] = l < nl ? (l ? b->fed_depth[l] : 0) : -1;
  akz_use_fed_depths(b);
  return AKZ_OK;
}

/* Learned FED surrogate for the levels of octave >= first_octave
 * (weights_bf16 NULL turns it off). */
AKZ_API akz_status akz_batch_set_surrogate(akz_batch *b, const uint16_t *weights_bf16, const float *biases, float s_out,
                                           int first_octave, float check_tol)
{
  AKZ_GUARD(b);
  akz_drop_graphs(b);
  if (!weights_bf16) {
    b->sg_on = 0;
    return AKZ_OK;
  }
  if (!biases || first_octave < 1 || !(s_out == s_out) || !(check_tol >= 0.0f))
    return akz_fail(AKZ_ERR_INVALID_ARG, "akz_batch_set_surrogate: bad arguments");
  size_t scratch = 16, chk = 1;
  for (int i = 0; i < b->nimg; i++)
    for (int l = 0; l < b->im[i].nlev; l++) {
      if (l / b->opt.nsublevels < first_octave) continue;
      const akz_level_desc &L = b->lv[b->im[i].first_level + l];
      scratch = std::max(scratch, (size_t)2 * L.width * L.height * 64);
      if (i == 0) chk = std::max(chk, (size_t)L.pitch * L.height);
    }
  const size_t nw = akz_sg_weight_elems();
  if (!b->d_sg_w) {
    CK(cudaMalloc(&b->d_sg_w, nw * 2));
    CK(cudaMalloc((void **)&b->d_sg_b, 136 * sizeof(float)));
    CK(cudaMalloc((void **)&b->d_sg_err, (size_t)b->maxlev * sizeof(float)));
    CK(cudaMalloc(&b->d_sg_scratch, scratch));
    CK(cudaMalloc((void **)&b->d_sg_chk, chk * sizeof(float)));
  }
  CK(cudaMemcpy(b->d_sg_w, weights_bf16, nw * 2, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(b->d_sg_b, biases, 136 * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemset(b->d_sg_err, 0, (size_t)b->maxlev * sizeof(float)));
  b->sg_dtf.assign(b->maxlev, 0.0f);
  for (int l = 1; l < b->maxlev; l++) {
    int i = 0;
    while (i < b->nimg && b->im[i].nlev <= l) i++;
    if (i == b->nimg) continue;
    const double e1 = b->geo[i][l].esigma, e0 = b->geo[i][l - 1].esigma;
    b->sg_dtf[l] = (float)(0.25 * std::log2(std::max(0.5 * (e1 * e1 - e0 * e0), 1e-12)));
  }
  b->sg_on = 1;
  b->sg_first_octave = first_octave;
  b->sg_s_out = s_out;
  b->sg_tol = check_tol;
  return AKZ_OK;
}

/* Per level, the max |surrogate - plain FED| of image 0 in the last run
 * (0 for levels without a check); a level above the tolerance fell back to
 * plain FED for every image. */
AKZ_API akz_status akz_batch_surrogate_errors(akz_batch *b, float *err, int cap, int *nlevels)
{
  AKZ_GUARD(b);
  if (nlevels) *nlevels = b->maxlev;
  if (!err || cap <= 0) return AKZ_OK;
  if (!b->sg_on || !b->d_sg_err) {
    for (int l = 0; l < cap; l++) err[l] = 0.0f;
    return AKZ_OK;
  }
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaMemcpy(err, b->d_sg_err, (size_t)std::min(cap, b->maxlev) * sizeof(float), cudaMemcpyDeviceToHost));
  return AKZ_OK;
}

} /* extern "C" */
