// C ABI and the multi-pass plan executor.
//
// piv_plan_run restates PIVGPU.__call__ (gpu_process.py:564-647) for a batch
// of equally sized frame pairs, as a fixed sequence of kernel launches on one
// stream with no host synchronisation between them:
//   for each iteration k:
//     k > 0: predictor onto the grid (regrid when the window size changes,
//            gpu_process.py:730-742), frame deformation (gpu_process.py:1149-1192)
//     correlation + peak + subpixel (+ S2N)        (gpu_process.py:1021-1097)
//     u = u_corr (+ up)                            (gpu_process.py:631-632)
//     validation, replacement loop                 (gpu_process.py:744-834)
//     smoothn unless last                          (gpu_process.py:637-639, 836-845)
//   scaling                                        (gpu_process.py:641-643)
// Data-dependent branches of the reference (no outliers, singular spring
// system, GCV search) are decided on the device, so a run can be captured in a
// CUDA graph.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <array>
#include <map>
#include <mutex>
#include <vector>

#include "piv_common.cuh"
#include "piv_internal.h"

namespace piv {

static thread_local char g_last_error[512] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int set_cuda_error(cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? PIV_E_OOM : PIV_E_CUDA;
  return set_error(code, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

int sm_count() {
  static std::mutex mu;
  static int counts[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::lock_guard<std::mutex> lock(mu);
  if (counts[dev] == 0) {
    int c = 0;
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
    counts[dev] = c > 0 ? c : 1;
  }
  return counts[dev];
}

static size_t pixel_bytes(int pixel_type) {
  switch (pixel_type) {
    case PIV_PIXEL_U8: return 1;
    case PIV_PIXEL_U16: return 2;
    case PIV_PIXEL_F32: return 4;
    case PIV_PIXEL_F64: return 8;
    default: return 0;
  }
}

int field_geometry(int height, int width, int window_size, int search_size, double overlap_ratio, int center,
                   piv_geometry* g) {
  if (height <= 0 || width <= 0 || search_size <= 0 || window_size <= 0 || window_size > search_size)
    return set_error(PIV_E_ARG, "invalid geometry (frame %dx%d, window %d, search %d)", height, width, window_size,
                     search_size);
  if (!(overlap_ratio >= 0 && overlap_ratio < 1)) return set_error(PIV_E_ARG, "overlap_ratio must be in [0, 1)");
  const int overlap = (int)(overlap_ratio * search_size);  // int(overlap_ratio * search_size)
  const int spacing = search_size - overlap;
  if (height < search_size || width < search_size)
    return set_error(PIV_E_ARG, "frame %dx%d smaller than search size %d", height, width, search_size);
  g->height = height;
  g->width = width;
  g->search_size = search_size;
  g->window_size = window_size;
  g->spacing = spacing;
  // Python floor division of non-negative operands.
  g->m = (height - search_size) / spacing + 1;
  g->n = (width - search_size) / spacing + 1;
  if (center) {
    const int xr = width - (spacing * (g->n - 1) + search_size);
    const int yr = height - (spacing * (g->m - 1) + search_size);
    g->x_offset = xr / 2 + search_size % 2;
    g->y_offset = yr / 2 + search_size % 2;
  } else {
    g->x_offset = g->y_offset = 0;
  }
  return PIV_OK;
}

}  // namespace piv

using namespace piv;

struct IterState {
  piv_iteration it;
  piv_geometry g;
  int fp32;
  size_t mn;
  void* u_corr = nullptr;
  void* v_corr = nullptr;
  double* up = nullptr;
  double* vp = nullptr;
  double* u_rep = nullptr;
  double* v_rep = nullptr;
  double* u_out = nullptr;
  double* v_out = nullptr;
  uint8_t* val0 = nullptr;
  uint8_t* val = nullptr;
  double* smooth_p = nullptr;
  int* smooth_flags = nullptr;
  int* peak_i = nullptr;
  int* peak_j = nullptr;
  uint8_t* near_tie = nullptr;  // per window: near tie of the correlation peak
  void* s2n = nullptr;
  uint8_t* field_mask = nullptr;
  // Correlation launch variant (0 = default; set by piv_plan_autotune or
  // piv_plan_set_variant), the pass's arguments of the last run, and the
  // autotuner's per-variant times (ms, -1 = not timed).
  int corr_variant = 0;
  CorrArgs corr{};
  bool corr_valid = false;
  std::vector<float> tune_ms;
};

struct piv_plan {
  piv_config cfg;
  std::vector<piv_iteration> iters;
  std::vector<IterState> st;
  int device = 0;
  size_t bytes = 0;
  std::vector<void*> allocs;
  void* stage_a = nullptr;
  void* stage_b = nullptr;
  void* def_a = nullptr;
  void* def_b = nullptr;
  float* coef = nullptr;
  uint8_t* frame_mask = nullptr;
  void* corr_scratch = nullptr;
  size_t corr_scratch_bytes = 0;
  void* rep_scratch = nullptr;
  void* smooth_scratch = nullptr;
  double* rms_stats = nullptr;
  int* status = nullptr;      // device status word of bounded device-side waits
  int* tie_counts = nullptr;  // [n_iters] near-tie windows of the last run per iteration
  int* tie_list = nullptr;    // refined tensor form: near-tie windows of a pass (max_pairs * max windows) + count
  float* win_means = nullptr; // refined tensor form: window means of a pass (max_pairs * max windows * 2)
  uint8_t* outliers = nullptr;
  double* u_final = nullptr;
  double* v_final = nullptr;
  bool any_cubic = false;
  std::vector<uint8_t> host_mask;
  // Stage timing.
  bool timing = false;
  struct TimedRun {
    cudaEvent_t start;
    std::vector<int> ids;
    std::vector<cudaEvent_t> ev;
  };
  std::vector<TimedRun> timed;
  std::vector<cudaEvent_t> event_pool;
  // CUDA graph of one run.
  cudaGraphExec_t graph_exec = nullptr;
};

struct piv_batch {
  std::vector<piv_plan*> plans;       // one per frame size
  std::vector<cudaStream_t> streams;  // one per frame size
  std::vector<cudaEvent_t> done;      // one per frame size
  cudaEvent_t fork = nullptr;
  std::vector<int> corr_variant;      // per pass: launch variant of the joint correlation
  int joint = 1;                      // one correlation launch per pass over all sizes (tensor engines)
  cudaGraphExec_t graph_exec = nullptr;
};

static cudaEvent_t take_event(piv_plan* p) {
  if (!p->event_pool.empty()) {
    cudaEvent_t e = p->event_pool.back();
    p->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

static int plan_alloc(piv_plan* p, void** ptr, size_t bytes) {
  *ptr = nullptr;
  if (bytes == 0) return PIV_OK;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(PIV_E_OOM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
  }
  p->allocs.push_back(*ptr);
  p->bytes += bytes;
  return PIV_OK;
}

template <typename Ptr>
static int plan_alloc_t(piv_plan* p, Ptr** ptr, size_t count) {
  void* v = nullptr;
  int rc = plan_alloc(p, &v, count * sizeof(Ptr));
  *ptr = reinterpret_cast<Ptr*>(v);
  return rc;
}

static bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

// A geometry the correlation reads windows with: positive sizes and every
// search window inside the frame. The kernels read window rows without
// per-pixel frame checks. PIVFieldGPU's centred grid puts the last window
// one pixel past the frame's edge for an odd search size that leaves no
// spare pixel (gpu_process.py:932-933; the reference then stacks pixels it
// never wrote, gpu_process.py:1127,1443-1447); such a geometry is refused.
static int check_corr_geometry(const piv_geometry& g, int n_pairs) {
  if (n_pairs < 0) return set_error(PIV_E_ARG, "n_pairs %d is negative", n_pairs);
  if (g.height <= 0 || g.width <= 0 || g.search_size <= 0 || g.window_size <= 0 ||
      g.window_size > g.search_size || g.spacing <= 0 || g.m <= 0 || g.n <= 0)
    return set_error(PIV_E_ARG, "invalid geometry (frame %dx%d, search %d, window %d, spacing %d, field %dx%d)",
                     g.height, g.width, g.search_size, g.window_size, g.spacing, g.m, g.n);
  const long long y_end = (long long)(g.m - 1) * g.spacing + g.y_offset + g.search_size;
  const long long x_end = (long long)(g.n - 1) * g.spacing + g.x_offset + g.search_size;
  if (g.y_offset < 0 || g.x_offset < 0 || y_end > g.height || x_end > g.width)
    return set_error(PIV_E_UNSUPPORTED,
                     "windows outside the %dx%d frame (search %d, offset %d,%d, field %dx%d, spacing %d)", g.height,
                     g.width, g.search_size, g.y_offset, g.x_offset, g.m, g.n, g.spacing);
  return PIV_OK;
}

// The correlation engine of a pass and its launch variants.
static int run_corr(int dft_mode, const CorrArgs& c, int variant, cudaStream_t s) {
  if (correlate_tensor_supported(c, dft_mode)) return correlate_tensor(c, dft_mode, variant, s);
  return correlate_fft(c, variant, s);
}

static int corr_variant_count(int dft_mode, const CorrArgs& c) {
  const int n = correlate_tensor_supported(c, dft_mode) ? correlate_tensor_variant_count(c, dft_mode)
                                                        : correlate_fft_variant_count(c.fft_size, c.dtype);
  return n > 0 ? n : 1;
}

// Autotuner results shared by the plans of a process: a pass with the same
// engine, transform size, float type, window sizes, pixel type, row alignment
// and order of magnitude of windows reuses the choice without timing again.
using TuneKey = std::array<long long, 11>;
static std::mutex g_tune_mu;
static std::map<TuneKey, int> g_tune_cache;

static TuneKey tune_key(int dft_mode, const CorrArgs& c) {
  int dev = 0;
  cudaGetDevice(&dev);
  const long long wins = (long long)c.n_pairs * c.m * c.n;
  int bucket = 0;
  while ((1LL << bucket) < wins) ++bucket;
  const int engine = correlate_tensor_supported(c, dft_mode) ? dft_mode : PIV_DFT_FFT32;
  const long long align = ((uintptr_t)c.frame_a % 16 == 0 && (uintptr_t)c.frame_b % 16 == 0 ? 1 : 0) |
                          (c.width % 4 == 0 ? 2 : 0) | (c.width % 16 == 0 ? 4 : 0) |
                          (c.x_offset % 4 == 0 && c.spacing % 4 == 0 ? 8 : 0) |
                          (c.x_offset % 16 == 0 && c.spacing % 16 == 0 ? 16 : 0);
  return TuneKey{dev, engine, c.fft_size, c.dtype, c.ss, c.ws, c.pixel_type, align, bucket, c.s2n ? 1 : 0,
                 c.win_mask ? 1 : 0};
}

extern "C" {

int piv_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return PIV_E_ARG;
  strncpy(buf, g_last_error, len - 1);
  buf[len - 1] = 0;
  return PIV_OK;
}

int piv_memcpy(void* dst, const void* src, size_t bytes, int kind, void* stream) {
  if (bytes == 0) return PIV_OK;
  if (!dst || !src) return set_error(PIV_E_ARG, "NULL argument");
  const cudaMemcpyKind k = kind == 0 ? cudaMemcpyDeviceToHost : (kind == 1 ? cudaMemcpyHostToDevice
                                                                            : cudaMemcpyDeviceToDevice);
  cudaError_t e = stream ? cudaMemcpyAsync(dst, src, bytes, k, (cudaStream_t)stream) : cudaMemcpy(dst, src, bytes, k);
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "piv_memcpy");
}

int piv_field_geometry(int height, int width, int window_size, int search_size, double overlap_ratio, int center,
                       piv_geometry* geom) {
  if (!geom) return set_error(PIV_E_ARG, "geom is NULL");
  return field_geometry(height, width, window_size, search_size, overlap_ratio, center, geom);
}

void piv_plan_destroy(piv_plan* p) {
  if (!p) return;
  if (p->graph_exec) cudaGraphExecDestroy(p->graph_exec);
  for (auto& r : p->timed) {
    p->event_pool.push_back(r.start);
    for (auto e : r.ev) p->event_pool.push_back(e);
  }
  for (auto e : p->event_pool) cudaEventDestroy(e);
  for (void* a : p->allocs) cudaFree(a);
  delete p;
}

int piv_plan_set_timing(piv_plan* p, int enable) {
  if (!p) return set_error(PIV_E_ARG, "NULL plan");
  p->timing = enable != 0;
  return PIV_OK;
}

int piv_plan_stage_times(piv_plan* p, float* ms, int capacity, int* runs) {
  if (!p || !ms) return set_error(PIV_E_ARG, "NULL argument");
  const int need = (int)p->st.size() * PIV_STAGES + 2;
  if (capacity < need) return set_error(PIV_E_ARG, "stage_times needs capacity %d", need);
  for (int k = 0; k < need; ++k) ms[k] = 0.0f;
  int n = 0;
  for (auto& r : p->timed) {
    if (!r.ev.empty()) cudaEventSynchronize(r.ev.back());
    cudaEvent_t prev = r.start;
    for (size_t k = 0; k < r.ev.size(); ++k) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, prev, r.ev[k]);
      if (r.ids[k] >= 0 && r.ids[k] < need) ms[r.ids[k]] += t;
      prev = r.ev[k];
    }
    p->event_pool.push_back(r.start);
    for (auto e : r.ev) p->event_pool.push_back(e);
    ++n;
  }
  p->timed.clear();
  if (runs) *runs = n;
  return cudaGetLastError() == cudaSuccess ? PIV_OK : set_error(PIV_E_CUDA, "stage timing failed");
}

int piv_plan_create(const piv_config* cfg, piv_plan** out) {
  if (!cfg || !out) return set_error(PIV_E_ARG, "NULL argument");
  *out = nullptr;
  if (cfg->n_iters <= 0 || !cfg->iters) return set_error(PIV_E_ARG, "no iterations");
  if (cfg->max_pairs <= 0) return set_error(PIV_E_ARG, "max_pairs must be positive");
  if (pixel_bytes(cfg->pixel_type) == 0) return set_error(PIV_E_ARG, "unknown pixel_type %d", cfg->pixel_type);
  if (cfg->dtype != PIV_DTYPE_F32 && cfg->dtype != PIV_DTYPE_F64) return set_error(PIV_E_ARG, "unknown dtype");
  if (cfg->dft_mode < PIV_DFT_FFT32 || cfg->dft_mode > PIV_DFT_TENSOR_REFINED)
    return set_error(PIV_E_ARG, "unknown dft_mode %d", cfg->dft_mode);
  if (!(cfg->dt > 0) || !(cfg->scaling_par > 0)) return set_error(PIV_E_ARG, "dt and scaling_par must be > 0");
  piv_plan* p = new piv_plan();
  p->cfg = *cfg;
  p->iters.assign(cfg->iters, cfg->iters + cfg->n_iters);
  p->cfg.iters = p->iters.data();
  cudaGetDevice(&p->device);
  const int P = cfg->max_pairs, H = cfg->height, W = cfg->width;
  const size_t hw = (size_t)H * W;
  const size_t tsz = cfg->dtype == PIV_DTYPE_F64 ? 8 : 4;
  int rc = PIV_OK;
  if (cfg->mask) p->host_mask.assign(cfg->mask, cfg->mask + hw);
  p->st.resize(cfg->n_iters);
  size_t max_mn = 0;
  for (int k = 0; k < cfg->n_iters && rc == PIV_OK; ++k) {
    const piv_iteration& it = p->iters[k];
    IterState& s = p->st[k];
    s.it = it;
    rc = field_geometry(H, W, it.window_size, it.search_size, it.overlap_ratio, cfg->center, &s.g);
    if (rc == PIV_OK) rc = check_corr_geometry(s.g, 0);
    if (rc) break;
    if (!is_pow2(it.fft_size) || it.fft_size < it.search_size || it.fft_size > 256) {
      rc = set_error(PIV_E_UNSUPPORTED, "fft_size %d (search size %d) is not supported", it.fft_size,
                     it.search_size);
      break;
    }
    if (it.deforming_order == 3) p->any_cubic = true;
    s.fp32 = (cfg->dtype == PIV_DTYPE_F32 && k == 0) ? 1 : 0;
    s.mn = (size_t)s.g.m * s.g.n;
    if (s.mn > max_mn) max_mn = s.mn;
    const size_t cnt = s.mn * P;
    if ((rc = plan_alloc(p, &s.u_corr, cnt * tsz))) break;
    if ((rc = plan_alloc(p, &s.v_corr, cnt * tsz))) break;
    if (k > 0) {
      if ((rc = plan_alloc_t(p, &s.up, cnt))) break;
      if ((rc = plan_alloc_t(p, &s.vp, cnt))) break;
    }
    if ((rc = plan_alloc_t(p, &s.u_rep, cnt))) break;
    if ((rc = plan_alloc_t(p, &s.v_rep, cnt))) break;
    if (k < cfg->n_iters - 1) {
      if ((rc = plan_alloc_t(p, &s.u_out, cnt))) break;
      if ((rc = plan_alloc_t(p, &s.v_out, cnt))) break;
    } else {
      s.u_out = s.u_rep;
      s.v_out = s.v_rep;
    }
    if ((rc = plan_alloc_t(p, &s.val0, cnt))) break;
    if ((rc = plan_alloc_t(p, &s.val, cnt))) break;
    if ((rc = plan_alloc_t(p, &s.smooth_p, (size_t)P))) break;
    if ((rc = plan_alloc_t(p, &s.smooth_flags, (size_t)P))) break;
    cudaMemset(s.smooth_flags, 0, sizeof(int) * P);
    if ((rc = plan_alloc_t(p, &s.peak_i, cnt))) break;
    if ((rc = plan_alloc_t(p, &s.peak_j, cnt))) break;
    if ((rc = plan_alloc_t(p, &s.near_tie, cnt))) break;
    if (!isnan(it.s2n_tol) && (rc = plan_alloc(p, &s.s2n, cnt * tsz))) break;
    if (cfg->mask) {
      std::vector<uint8_t> fm(s.mn);
      for (int i = 0; i < s.g.m; ++i)
        for (int j = 0; j < s.g.n; ++j) {
          // mask[y.astype(int), x.astype(int)] at the window centres (gpu_process.py:951)
          const int y = (int)(float)((double)i * s.g.spacing + s.g.search_size / 2.0 + s.g.y_offset);
          const int x = (int)(float)((double)j * s.g.spacing + s.g.search_size / 2.0 + s.g.x_offset);
          fm[(size_t)i * s.g.n + j] = cfg->mask[(size_t)y * W + x] ? 1 : 0;
        }
      if ((rc = plan_alloc_t(p, &s.field_mask, s.mn))) break;
      cudaMemcpy(s.field_mask, fm.data(), s.mn, cudaMemcpyHostToDevice);
    }
    const size_t cs = correlate_fft_scratch_bytes(it.fft_size, cfg->dtype);
    if (cs > p->corr_scratch_bytes) p->corr_scratch_bytes = cs;
  }
  if (rc == PIV_OK) rc = plan_alloc(p, &p->stage_a, (size_t)P * hw * pixel_bytes(cfg->pixel_type));
  if (rc == PIV_OK) rc = plan_alloc(p, &p->stage_b, (size_t)P * hw * pixel_bytes(cfg->pixel_type));
  if (rc == PIV_OK && cfg->n_iters > 1) {
    rc = plan_alloc(p, &p->def_a, (size_t)P * hw * tsz);
    if (rc == PIV_OK) rc = plan_alloc(p, &p->def_b, (size_t)P * hw * tsz);
  }
  const size_t chw = (size_t)(cfg->height + 2 * kCoefPad) * (cfg->width + 2 * kCoefPad);  // padded coefficient frame
  if (rc == PIV_OK && p->any_cubic) rc = plan_alloc_t(p, &p->coef, 2 * (size_t)P * chw);
  if (rc == PIV_OK && cfg->mask) {
    rc = plan_alloc_t(p, &p->frame_mask, hw);
    if (rc == PIV_OK) cudaMemcpy(p->frame_mask, cfg->mask, hw, cudaMemcpyHostToDevice);
  }
  if (rc == PIV_OK) rc = plan_alloc(p, &p->corr_scratch, p->corr_scratch_bytes);
  if (rc == PIV_OK) rc = plan_alloc(p, &p->rep_scratch, replace_scratch_bytes(1, (int)max_mn, P));
  size_t sm_bytes = 0;
  for (auto& s : p->st) {
    const size_t b = smoothn_scratch_bytes(s.g.m, s.g.n, P);
    if (b > sm_bytes) sm_bytes = b;
  }
  if (rc == PIV_OK) rc = plan_alloc(p, &p->smooth_scratch, sm_bytes);
  if (rc == PIV_OK) rc = plan_alloc_t(p, &p->rms_stats, 4 * (size_t)P);
  if (rc == PIV_OK) {
    rc = plan_alloc_t(p, &p->status, 1);
    if (rc == PIV_OK) cudaMemset(p->status, 0, sizeof(int));
  }
  if (rc == PIV_OK) {
    rc = plan_alloc_t(p, &p->tie_counts, (size_t)cfg->n_iters);
    if (rc == PIV_OK) cudaMemset(p->tie_counts, 0, sizeof(int) * cfg->n_iters);
  }
  bool refine_buffers = cfg->dft_mode == PIV_DFT_TENSOR_REFINED;
  for (int k = 0; k < cfg->n_iters; ++k)  // the split form's 64-px passes take the refined path
    refine_buffers = refine_buffers || (cfg->dft_mode == PIV_DFT_TENSOR_SPLIT && p->iters[k].search_size == 64);
  if (rc == PIV_OK && refine_buffers) {
    rc = plan_alloc_t(p, &p->tie_list, max_mn * P + 1);
    if (rc == PIV_OK) rc = plan_alloc_t(p, &p->win_means, 2 * max_mn * P);
  }
  if (rc == PIV_OK) {
    const size_t cnt = p->st.back().mn * P;
    rc = plan_alloc_t(p, &p->outliers, cnt);
    if (rc == PIV_OK) rc = plan_alloc_t(p, &p->u_final, cnt);
    if (rc == PIV_OK) rc = plan_alloc_t(p, &p->v_final, cnt);
  }
  if (rc != PIV_OK) {
    piv_plan_destroy(p);
    return rc;
  }
  *out = p;
  return PIV_OK;
}

int piv_plan_field_shape(const piv_plan* p, int iter, int* m, int* n) {
  if (!p || !m || !n) return set_error(PIV_E_ARG, "NULL argument");
  if (iter < 0) iter += (int)p->st.size();
  if (iter < 0 || iter >= (int)p->st.size()) return set_error(PIV_E_ARG, "iteration %d out of range", iter);
  *m = p->st[iter].g.m;
  *n = p->st[iter].g.n;
  return PIV_OK;
}

int piv_plan_workspace_bytes(const piv_plan* p, size_t* bytes) {
  if (!p || !bytes) return set_error(PIV_E_ARG, "NULL argument");
  *bytes = p->bytes;
  return PIV_OK;
}

int piv_plan_iteration_view(const piv_plan* p, int iter, piv_iteration_view* v) {
  if (!p || !v) return set_error(PIV_E_ARG, "NULL argument");
  if (iter < 0 || iter >= (int)p->st.size()) return set_error(PIV_E_ARG, "iteration %d out of range", iter);
  const IterState& s = p->st[iter];
  v->m = s.g.m;
  v->n = s.g.n;
  v->u_corr = s.u_corr;
  v->v_corr = s.v_corr;
  v->up = s.up;
  v->vp = s.vp;
  v->u_rep = s.u_rep;
  v->v_rep = s.v_rep;
  v->u_out = s.u_out;
  v->v_out = s.v_out;
  v->val0 = s.val0;
  v->smooth_p = s.smooth_p;
  v->peak_i = s.peak_i;
  v->peak_j = s.peak_j;
  v->s2n = s.s2n;
  v->near_tie = s.near_tie;
  v->smooth_flags = s.smooth_flags;
  return PIV_OK;
}

#define PIV_TRY(expr)            \
  do {                           \
    int _rc = (expr);            \
    if (_rc != PIV_OK) return _rc; \
  } while (0)

static int cuda_ok(cudaError_t e, const char* what) { return e == cudaSuccess ? PIV_OK : set_cuda_error(e, what); }

__global__ void k_mask_frames(long long npix, int n_pairs, int pixel_bytes, const uint8_t* mask, void* a, void* b) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix * n_pairs) return;
  if (!mask[t % npix]) return;
  uint8_t* pa = (uint8_t*)a + t * pixel_bytes;
  uint8_t* pb = (uint8_t*)b + t * pixel_bytes;
  for (int k = 0; k < pixel_bytes; ++k) { pa[k] = 0; pb[k] = 0; }
}

// One run of a plan, split into the pieces a multi-size batch interleaves:
// run_begin (frame copies, masking), run_pre (predictor and deformation of
// pass k; fills the pass's correlation arguments), the correlation, run_post
// (validation, replacement, smoothing of pass k) and run_end (scaling, result
// copies). piv_plan_run calls them in order on one stream.
struct RunCtx {
  int n_pairs = 0;
  const void* fa = nullptr;
  const void* fb = nullptr;
  bool coef_ready = false;
  piv_plan::TimedRun* tr = nullptr;
};

static void mark(piv_plan* p, RunCtx& x, int id, cudaStream_t s) {
  if (!x.tr) return;
  cudaEvent_t e = take_event(p);
  cudaEventRecord(e, s);
  x.tr->ids.push_back(id);
  x.tr->ev.push_back(e);
}

static int run_begin(piv_plan* p, int n_pairs, const void* frames_a, const void* frames_b, int frames_on_host,
                     cudaStream_t s, RunCtx& x) {
  const piv_config& cfg = p->cfg;
  const size_t hw = (size_t)cfg.height * cfg.width;
  const size_t pb = pixel_bytes(cfg.pixel_type);
  x.n_pairs = n_pairs;
  x.coef_ready = false;
  x.tr = nullptr;
  if (p->timing) {
    p->timed.emplace_back();
    x.tr = &p->timed.back();
    x.tr->start = take_event(p);
    cudaEventRecord(x.tr->start, s);
  }
  x.fa = frames_a;
  x.fb = frames_b;
  PIV_TRY(cuda_ok(cudaMemsetAsync(p->tie_counts, 0, sizeof(int) * p->st.size(), s), "near-tie counters"));
  if (frames_on_host || p->frame_mask) {
    const cudaMemcpyKind kind = frames_on_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    PIV_TRY(cuda_ok(cudaMemcpyAsync(p->stage_a, frames_a, n_pairs * hw * pb, kind, s), "frame copy"));
    PIV_TRY(cuda_ok(cudaMemcpyAsync(p->stage_b, frames_b, n_pairs * hw * pb, kind, s), "frame copy"));
    x.fa = p->stage_a;
    x.fb = p->stage_b;
    if (p->frame_mask) {
      // mask_frames (gpu_process.py:682-688)
      const long long tot = (long long)hw * n_pairs;
      k_mask_frames<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>((long long)hw, n_pairs, (int)pb, p->frame_mask,
                                                                    p->stage_a, p->stage_b);
      PIV_TRY(cuda_ok(cudaGetLastError(), "k_mask_frames"));
    }
  }
  mark(p, x, (int)p->st.size() * PIV_STAGES, s);
  return PIV_OK;
}

static int run_pre(piv_plan* p, int k, RunCtx& x, cudaStream_t s, CorrArgs& c) {
  const piv_config& cfg = p->cfg;
  const int H = cfg.height, W = cfg.width;
  const size_t chw = (size_t)(H + 2 * kCoefPad) * (W + 2 * kCoefPad);  // padded coefficient frame
  const int n_pairs = x.n_pairs;
  IterState& st = p->st[k];
  const piv_iteration& it = st.it;
  const int cnt = (int)(st.mn * n_pairs);
  const void* ca = x.fa;
  const void* cb = x.fb;
  int c_pixel = cfg.pixel_type;
  if (k > 0) {
    IterState& pr = p->st[k - 1];
    if (pr.g.search_size != st.g.search_size) {
      PIV_TRY(regrid(pr.g, st.g, n_pairs, pr.u_out, pr.v_out, st.up, st.vp, s));
    } else {
      PIV_TRY(cuda_ok(cudaMemcpyAsync(st.up, pr.u_out, cnt * 8, cudaMemcpyDeviceToDevice, s), "predictor copy"));
      PIV_TRY(cuda_ok(cudaMemcpyAsync(st.vp, pr.v_out, cnt * 8, cudaMemcpyDeviceToDevice, s), "predictor copy"));
    }
    mark(p, x, k * PIV_STAGES + 0, s);
    if (it.deforming_order == 3 && !x.coef_ready) {
      PIV_TRY(spline_prefilter(H, W, n_pairs, x.fa, cfg.pixel_type, p->coef, s, kCoefPad));
      PIV_TRY(spline_prefilter(H, W, n_pairs, x.fb, cfg.pixel_type, p->coef + (size_t)cfg.max_pairs * chw, s,
                               kCoefPad));
      x.coef_ready = true;
    }
    DeformArgs d;
    d.geom = st.g;
    d.n_pairs = n_pairs;
    d.frames_a = x.fa;
    d.frames_b = x.fb;
    d.pixel_type = cfg.pixel_type;
    d.up = st.up;
    d.vp = st.vp;
    d.deforming_par = it.deforming_par;
    d.order = it.deforming_order == 3 ? 3 : 1;
    d.coef_a = p->coef;
    d.coef_b = p->coef ? p->coef + (size_t)cfg.max_pairs * chw : nullptr;
    d.coef_pad = kCoefPad;
    d.frame_mask = p->frame_mask;
    d.dtype = cfg.dtype;
    d.out_a = p->def_a;
    d.out_b = p->def_b;
    PIV_TRY(deform(d, s));
    mark(p, x, k * PIV_STAGES + 1, s);
    ca = p->def_a;
    cb = p->def_b;
    c_pixel = cfg.dtype == PIV_DTYPE_F64 ? PIV_PIXEL_F64 : PIV_PIXEL_F32;
  }
  c = CorrArgs{};
  c.frame_a = ca;
  c.frame_b = cb;
  c.pixel_type = c_pixel;
  c.height = H;
  c.width = W;
  c.ss = st.g.search_size;
  c.ws = st.g.window_size;
  c.spacing = st.g.spacing;
  c.m = st.g.m;
  c.n = st.g.n;
  c.x_offset = st.g.x_offset;
  c.y_offset = st.g.y_offset;
  c.n_pairs = n_pairs;
  c.fft_size = it.fft_size;
  c.normalize = it.normalize;
  c.subpixel = it.subpixel_method;
  c.dtype = cfg.dtype;
  c.win_mask = st.field_mask;
  c.u = st.u_corr;
  c.v = st.v_corr;
  c.peak_i = st.peak_i;
  c.peak_j = st.peak_j;
  c.s2n = st.s2n;
  c.s2n_method = it.s2n_method;
  c.s2n_size = it.s2n_size;
  c.scratch = p->corr_scratch;
  c.scratch_bytes = p->corr_scratch_bytes;
  c.maps = nullptr;
  c.status = p->status;
  c.near_tie = st.near_tie;
  c.tie_count = p->tie_counts + k;
  if (p->tie_list) {
    c.tie_list = p->tie_list + 1;
    c.tie_list_count = p->tie_list;
    c.win_means = p->win_means;
  }
  st.corr = c;
  st.corr_valid = true;
  return PIV_OK;
}

static int run_post(piv_plan* p, int k, RunCtx& x, cudaStream_t s) {
  const piv_config& cfg = p->cfg;
  const int n_pairs = x.n_pairs;
  const int n_it = (int)p->st.size();
  IterState& st = p->st[k];
  const piv_iteration& it = st.it;
  const int cnt = (int)(st.mn * n_pairs);
  PIV_TRY(combine_fields(cnt, st.u_corr, st.v_corr, cfg.dtype, st.up, st.vp, st.fp32, st.u_rep, st.v_rep, s));
  ValArgs va;
  va.m = st.g.m;
  va.n = st.g.n;
  va.n_pairs = n_pairs;
  va.u = st.u_rep;
  va.v = st.v_rep;
  va.s2n = st.s2n;
  va.s2n_dtype = cfg.dtype;
  va.size = it.validation_size;
  va.s2n_tol = it.s2n_tol;
  va.median_tol = it.median_tol;
  va.mad_tol = it.mad_tol;
  va.mean_tol = it.mean_tol;
  va.rms_tol = it.rms_tol;
  va.field_mask = st.field_mask;
  va.exclude = nullptr;
  va.fp32 = st.fp32;
  PIV_TRY(validate(va, st.val0, p->rms_stats, s));
  PIV_TRY(cuda_ok(cudaMemcpyAsync(st.val, st.val0, cnt, cudaMemcpyDeviceToDevice, s), "val copy"));
  mark(p, x, k * PIV_STAGES + 3, s);
  RepArgs ra;
  ra.val = va;
  ra.u = st.u_rep;
  ra.v = st.v_rep;
  ra.val_mask = st.val;
  ra.n_iters = it.num_replacing_iters;
  ra.method = it.replacing_method;
  ra.size = it.replacing_size;
  ra.revalidate = it.revalidate;
  ra.dtype = cfg.dtype;
  ra.scratch = p->rep_scratch;
  ra.status = p->status;
  PIV_TRY(replace(ra, s));
  if (k == n_it - 1) {
    va.u = st.u_rep;
    va.v = st.v_rep;
    PIV_TRY(validate(va, p->outliers, p->rms_stats, s));
  }
  mark(p, x, k * PIV_STAGES + 4, s);
  if (k != n_it - 1) {
    PIV_TRY(smoothn(st.g.m, st.g.n, n_pairs, st.u_rep, st.v_rep, st.u_out, st.v_out, st.field_mask,
                    it.smoothing_par, st.smooth_p, p->smooth_scratch, s, st.smooth_flags));
    mark(p, x, k * PIV_STAGES + 5, s);
  }
  return PIV_OK;
}

static int run_end(piv_plan* p, RunCtx& x, double* u, double* v, uint8_t* val_locations, uint8_t* outliers,
                   int outputs_on_host, cudaStream_t s) {
  const piv_config& cfg = p->cfg;
  IterState& last = p->st.back();
  const int cnt = (int)(last.mn * x.n_pairs);
  const double* ru = last.u_rep;
  const double* rv = last.v_rep;
  if (cfg.dt != 1 || cfg.scaling_par != 1) {
    PIV_TRY(scale_fields(cnt, last.u_rep, last.v_rep, cfg.scaling_par, cfg.dt, last.fp32, p->u_final, p->v_final, s));
    ru = p->u_final;
    rv = p->v_final;
  }
  const cudaMemcpyKind ok = outputs_on_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  PIV_TRY(cuda_ok(cudaMemcpyAsync(u, ru, cnt * 8, ok, s), "result copy"));
  PIV_TRY(cuda_ok(cudaMemcpyAsync(v, rv, cnt * 8, ok, s), "result copy"));
  if (val_locations) PIV_TRY(cuda_ok(cudaMemcpyAsync(val_locations, last.val0, cnt, ok, s), "result copy"));
  if (outliers) PIV_TRY(cuda_ok(cudaMemcpyAsync(outliers, p->outliers, cnt, ok, s), "result copy"));
  mark(p, x, (int)p->st.size() * PIV_STAGES + 1, s);
  return PIV_OK;
}

int piv_plan_run(piv_plan* p, int n_pairs, const void* frames_a, const void* frames_b, int frames_on_host, double* u,
                 double* v, uint8_t* val_locations, uint8_t* outliers, int outputs_on_host, void* stream_ptr) {
  if (!p || !frames_a || !frames_b || !u || !v) return set_error(PIV_E_ARG, "NULL argument");
  if (n_pairs <= 0 || n_pairs > p->cfg.max_pairs)
    return set_error(PIV_E_ARG, "n_pairs %d outside [1, max_pairs=%d]", n_pairs, p->cfg.max_pairs);
  cudaStream_t s = (cudaStream_t)stream_ptr;
  RunCtx x;
  PIV_TRY(run_begin(p, n_pairs, frames_a, frames_b, frames_on_host, s, x));
  for (int k = 0; k < (int)p->st.size(); ++k) {
    CorrArgs c;
    PIV_TRY(run_pre(p, k, x, s, c));
    PIV_TRY(run_corr(p->cfg.dft_mode, c, p->st[k].corr_variant, s));
    mark(p, x, k * PIV_STAGES + 2, s);
    PIV_TRY(run_post(p, k, x, s));
  }
  PIV_TRY(run_end(p, x, u, v, val_locations, outliers, outputs_on_host, s));
  if (outputs_on_host == 1) PIV_TRY(cuda_ok(cudaStreamSynchronize(s), "stream synchronize"));
  return cuda_ok(cudaGetLastError(), "piv_plan_run");
}

int piv_plan_graph_capture(piv_plan* p, int n_pairs, const void* frames_a, const void* frames_b, double* u,
                           double* v, uint8_t* val_locations, uint8_t* outliers, int* kernel_nodes,
                           void* stream_ptr) {
  if (!p) return set_error(PIV_E_ARG, "NULL plan");
  if (!stream_ptr) return set_error(PIV_E_ARG, "graph capture needs a non-default stream");
  cudaStream_t s = (cudaStream_t)stream_ptr;
  if (p->graph_exec) {
    cudaGraphExecDestroy(p->graph_exec);
    p->graph_exec = nullptr;
  }
  const bool saved = p->timing;
  p->timing = false;
  PIV_TRY(cuda_ok(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture"));
  int rc = piv_plan_run(p, n_pairs, frames_a, frames_b, 0, u, v, val_locations, outliers, 0, stream_ptr);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  p->timing = saved;
  if (rc != PIV_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return set_cuda_error(e, "cudaStreamEndCapture");
  if (kernel_nodes) {
    size_t n = 0;
    cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    cudaGraphGetNodes(graph, nodes.data(), &n);
    int k = 0;
    for (size_t i = 0; i < n; ++i) {
      cudaGraphNodeType t;
      cudaGraphNodeGetType(nodes[i], &t);
      if (t == cudaGraphNodeTypeKernel) ++k;
    }
    *kernel_nodes = k;
  }
  e = cudaGraphInstantiate(&p->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  return cuda_ok(e, "cudaGraphInstantiate");
}

int piv_plan_graph_launch(piv_plan* p, void* stream) {
  if (!p || !p->graph_exec) return set_error(PIV_E_ARG, "no captured graph");
  return cuda_ok(cudaGraphLaunch(p->graph_exec, (cudaStream_t)stream), "cudaGraphLaunch");
}

// ---------------------------------------------------------------------------
// Stage entry points.
// ---------------------------------------------------------------------------
int piv_correlate(const piv_geometry* g, int n_pairs, const void* frames_a, const void* frames_b, int pixel_type,
                  int dtype, int fft_size, int normalize, int subpixel_method, const uint8_t* win_mask, void* u,
                  void* v, int* peak_i, int* peak_j, int s2n_method, int s2n_size, void* s2n, int dft_mode,
                  void* stream) {
  if (!g || !frames_a || !frames_b || !u || !v) return set_error(PIV_E_ARG, "NULL argument");
  PIV_TRY(check_corr_geometry(*g, n_pairs));
  if (!is_pow2(fft_size) || fft_size < g->search_size || fft_size > 256)
    return set_error(PIV_E_UNSUPPORTED, "fft_size %d is not supported", fft_size);
  CorrArgs c{};
  c.frame_a = frames_a;
  c.frame_b = frames_b;
  c.pixel_type = pixel_type;
  c.height = g->height;
  c.width = g->width;
  c.ss = g->search_size;
  c.ws = g->window_size;
  c.spacing = g->spacing;
  c.m = g->m;
  c.n = g->n;
  c.x_offset = g->x_offset;
  c.y_offset = g->y_offset;
  c.n_pairs = n_pairs;
  c.fft_size = fft_size;
  c.normalize = normalize;
  c.subpixel = subpixel_method;
  c.dtype = dtype;
  c.win_mask = win_mask;
  c.u = u;
  c.v = v;
  c.peak_i = peak_i;
  c.peak_j = peak_j;
  c.s2n = s2n;
  c.s2n_method = s2n_method;
  c.s2n_size = s2n_size;
  c.scratch = nullptr;
  c.scratch_bytes = 0;
  c.maps = nullptr;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t need = correlate_fft_scratch_bytes(fft_size, dtype);
  if (correlate_tensor_supported(c, dft_mode)) {
    PIV_TRY(cuda_ok(cudaMallocAsync((void**)&c.status, sizeof(int), s), "cudaMallocAsync"));
    cudaMemsetAsync(c.status, 0, sizeof(int), s);
    int* peaks = nullptr;  // the refined form reads the peaks back: device peaks when the caller wants none
    const size_t cnt = (size_t)n_pairs * g->m * g->n;
    if ((dft_mode == PIV_DFT_TENSOR_REFINED || (dft_mode == PIV_DFT_TENSOR_SPLIT && c.ss == 64)) &&
        (!c.peak_i || !c.peak_j)) {
      PIV_TRY(cuda_ok(cudaMallocAsync((void**)&peaks, 2 * cnt * sizeof(int), s), "cudaMallocAsync"));
      if (!c.peak_i) c.peak_i = peaks;
      if (!c.peak_j) c.peak_j = peaks + cnt;
    }
    int rc = correlate_tensor(c, dft_mode, 0, s);
    int st = 0;
    cudaMemcpyAsync(&st, c.status, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(c.status, s);
    if (peaks) cudaFreeAsync(peaks, s);
    cudaStreamSynchronize(s);
    if (rc == PIV_OK && st != 0) rc = set_error(st, "tensor correlation: a bounded wait gave up");
    return rc;
  }
  if (need) {
    PIV_TRY(cuda_ok(cudaMallocAsync(&c.scratch, need, s), "cudaMallocAsync"));
    c.scratch_bytes = need;
  }
  int rc = correlate_fft(c, 0, s);
  if (c.scratch) cudaFreeAsync(c.scratch, s);
  return rc;
}

int piv_correlate_maps(const piv_geometry* g, int n_pairs, const void* frames_a, const void* frames_b,
                       int pixel_type, int dtype, int fft_size, int normalize, const uint8_t* win_mask, void* maps,
                       int dft_mode, void* stream) {
  if (!g || !frames_a || !frames_b || !maps) return set_error(PIV_E_ARG, "NULL argument");
  PIV_TRY(check_corr_geometry(*g, n_pairs));
  if (!is_pow2(fft_size) || fft_size < g->search_size || fft_size > 256)
    return set_error(PIV_E_UNSUPPORTED, "fft_size %d is not supported", fft_size);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t cnt = (size_t)n_pairs * g->m * g->n;
  const size_t tsz = dtype == PIV_DTYPE_F64 ? 8 : 4;
  void* u = nullptr;
  PIV_TRY(cuda_ok(cudaMallocAsync(&u, 2 * cnt * tsz, s), "cudaMallocAsync"));
  CorrArgs c{};
  c.frame_a = frames_a;
  c.frame_b = frames_b;
  c.pixel_type = pixel_type;
  c.height = g->height;
  c.width = g->width;
  c.ss = g->search_size;
  c.ws = g->window_size;
  c.spacing = g->spacing;
  c.m = g->m;
  c.n = g->n;
  c.x_offset = g->x_offset;
  c.y_offset = g->y_offset;
  c.n_pairs = n_pairs;
  c.fft_size = fft_size;
  c.normalize = normalize;
  c.subpixel = PIV_SUBPIXEL_GAUSSIAN;
  c.dtype = dtype;
  c.win_mask = win_mask;
  c.u = u;
  c.v = (char*)u + cnt * tsz;
  c.maps = maps;
  int rc;
  if (correlate_tensor_supported(c, dft_mode)) {
    PIV_TRY(cuda_ok(cudaMallocAsync((void**)&c.status, sizeof(int), s), "cudaMallocAsync"));
    cudaMemsetAsync(c.status, 0, sizeof(int), s);
    rc = correlate_tensor(c, dft_mode, 0, s);
    cudaFreeAsync(c.status, s);
    cudaFreeAsync(u, s);
    return rc;
  }
  const size_t need = correlate_fft_scratch_bytes(fft_size, dtype);
  if (need) {
    PIV_TRY(cuda_ok(cudaMallocAsync(&c.scratch, need, s), "cudaMallocAsync"));
    c.scratch_bytes = need;
  }
  rc = correlate_fft(c, 0, s);
  if (c.scratch) cudaFreeAsync(c.scratch, s);
  cudaFreeAsync(u, s);
  return rc;
}

int piv_regrid(const piv_geometry* src, const piv_geometry* dst, int n_pairs, const double* u_src,
               const double* v_src, double* u_dst, double* v_dst, void* stream) {
  if (!src || !dst || !u_src || !v_src || !u_dst || !v_dst) return set_error(PIV_E_ARG, "NULL argument");
  return regrid(*src, *dst, n_pairs, u_src, v_src, u_dst, v_dst, (cudaStream_t)stream);
}

int piv_deform(const piv_geometry* g, int n_pairs, const void* frames_a, const void* frames_b, int pixel_type,
               const double* up, const double* vp, double deforming_par, int deforming_order, const float* coef_a,
               const float* coef_b, const uint8_t* frame_mask, int dtype, void* out_a, void* out_b, void* stream) {
  if (!g || !frames_a || !frames_b || !up || !vp || !out_a || !out_b) return set_error(PIV_E_ARG, "NULL argument");
  DeformArgs d;
  d.geom = *g;
  d.n_pairs = n_pairs;
  d.frames_a = frames_a;
  d.frames_b = frames_b;
  d.pixel_type = pixel_type;
  d.up = up;
  d.vp = vp;
  d.deforming_par = deforming_par;
  d.order = deforming_order == 3 ? 3 : 1;
  d.coef_a = coef_a;
  d.coef_b = coef_b;
  d.coef_pad = 0;
  d.frame_mask = frame_mask;
  d.dtype = dtype;
  d.out_a = out_a;
  d.out_b = out_b;
  return deform(d, (cudaStream_t)stream);
}

int piv_spline_prefilter(int height, int width, int n_frames, const void* frames, int pixel_type, float* coef,
                         void* stream) {
  if (!frames || !coef) return set_error(PIV_E_ARG, "NULL argument");
  return spline_prefilter(height, width, n_frames, frames, pixel_type, coef, (cudaStream_t)stream);
}

int piv_validate(int m, int n, int n_pairs, const double* u, const double* v, const void* s2n, int s2n_dtype,
                 int size, double s2n_tol, double median_tol, double mad_tol, double mean_tol, double rms_tol,
                 const uint8_t* field_mask, const uint8_t* exclude, int fp32, uint8_t* val, void* stream) {
  if (!u || !v || !val) return set_error(PIV_E_ARG, "NULL argument");
  ValArgs a{m, n, n_pairs, u, v, s2n, s2n_dtype, size, s2n_tol, median_tol, mad_tol, mean_tol, rms_tol,
            field_mask, exclude, fp32};
  cudaStream_t s = (cudaStream_t)stream;
  double* stats = nullptr;
  if (!isnan(rms_tol)) PIV_TRY(cuda_ok(cudaMallocAsync((void**)&stats, 4 * 8 * (size_t)n_pairs, s), "cudaMallocAsync"));
  int rc = validate(a, val, stats, s);
  if (stats) cudaFreeAsync(stats, s);
  return rc;
}

int piv_replace(int m, int n, int n_pairs, double* u, double* v, uint8_t* val, const uint8_t* field_mask, int n_iters,
                int method, int size, int revalidate, const void* s2n, int s2n_dtype, int val_size, double s2n_tol,
                double median_tol, double mad_tol, double mean_tol, double rms_tol, int fp32, int dtype,
                void* stream) {
  if (!u || !v || !val) return set_error(PIV_E_ARG, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  RepArgs a;
  a.val = ValArgs{m, n, n_pairs, u, v, s2n, s2n_dtype, val_size, s2n_tol, median_tol, mad_tol, mean_tol, rms_tol,
                  field_mask, nullptr, fp32};
  a.u = u;
  a.v = v;
  a.val_mask = val;
  a.n_iters = n_iters;
  a.method = method;
  a.size = size;
  a.revalidate = revalidate;
  a.dtype = dtype;
  a.status = nullptr;
  const size_t need = replace_scratch_bytes(m, n, n_pairs);
  PIV_TRY(cuda_ok(cudaMallocAsync(&a.scratch, need, s), "cudaMallocAsync"));
  int rc = replace(a, s);
  cudaFreeAsync(a.scratch, s);
  return rc;
}

int piv_smoothn(int m, int n, int n_pairs, double* u, double* v, const uint8_t* field_mask, double sp, double* p_out,
                void* stream) {
  return piv_smoothn_flags(m, n, n_pairs, u, v, field_mask, sp, p_out, nullptr, stream);
}

int piv_smoothn_flags(int m, int n, int n_pairs, double* u, double* v, const uint8_t* field_mask, double sp,
                      double* p_out, int* flags_out, void* stream) {
  if (!u || !v) return set_error(PIV_E_ARG, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  void* scratch = nullptr;
  PIV_TRY(cuda_ok(cudaMallocAsync(&scratch, smoothn_scratch_bytes(m, n, n_pairs), s), "cudaMallocAsync"));
  int rc = smoothn(m, n, n_pairs, u, v, u, v, field_mask, sp, p_out, scratch, s, flags_out);
  cudaFreeAsync(scratch, s);
  return rc;
}

int piv_bounds_check(int* checked, int* violations) {
  if (!checked || !violations) return set_error(PIV_E_ARG, "NULL argument");
  PIV_TRY(cuda_ok(cudaDeviceSynchronize(), "device synchronize"));
  const int a = bounds_violations_tensor(), b = bounds_violations_refine();
  if (a == -2 || b == -2) return set_error(PIV_E_CUDA, "bounds counters could not be read");
  *checked = a >= 0 ? 1 : 0;
  *violations = (a > 0 ? a : 0) + (b > 0 ? b : 0);
  return PIV_OK;
}

int piv_plan_near_ties(piv_plan* plan, int* counts, int capacity, void* stream) {
  if (!plan || !counts) return set_error(PIV_E_ARG, "NULL argument");
  const int n = (int)plan->st.size() < capacity ? (int)plan->st.size() : capacity;
  if (n <= 0) return PIV_OK;
  cudaStream_t s = (cudaStream_t)stream;
  PIV_TRY(cuda_ok(cudaMemcpyAsync(counts, plan->tie_counts, sizeof(int) * n, cudaMemcpyDeviceToHost, s),
                  "near-tie copy"));
  return cuda_ok(cudaStreamSynchronize(s), "stream synchronize");
}

int piv_plan_status(piv_plan* plan, int* status, void* stream) {
  if (!plan || !status) return set_error(PIV_E_ARG, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  int word = 0;
  PIV_TRY(cuda_ok(cudaMemcpyAsync(&word, plan->status, sizeof(int), cudaMemcpyDeviceToHost, s), "status copy"));
  PIV_TRY(cuda_ok(cudaStreamSynchronize(s), "stream synchronize"));
  if (word != PIV_OK) PIV_TRY(cuda_ok(cudaMemsetAsync(plan->status, 0, sizeof(int), s), "status reset"));
  *status = word;
  return PIV_OK;
}

int piv_plan_autotune(piv_plan* p, int n_pairs, const void* frames_a, const void* frames_b, int frames_on_host,
                      int reps, void* stream_ptr) {
  if (!p || !frames_a || !frames_b) return set_error(PIV_E_ARG, "NULL argument");
  if (n_pairs <= 0 || n_pairs > p->cfg.max_pairs)
    return set_error(PIV_E_ARG, "n_pairs %d outside [1, max_pairs=%d]", n_pairs, p->cfg.max_pairs);
  if (reps <= 0) reps = 5;
  cudaStream_t s = (cudaStream_t)stream_ptr;
  // One run, so that every pass's inputs (the deformed frames of later
  // passes) are those of these frames.
  const size_t cnt = p->st.back().mn * (size_t)n_pairs;
  double* uv = nullptr;
  PIV_TRY(cuda_ok(cudaMallocAsync((void**)&uv, 2 * cnt * sizeof(double), s), "cudaMallocAsync"));
  int rc = piv_plan_run(p, n_pairs, frames_a, frames_b, frames_on_host, uv, uv + cnt, nullptr, nullptr, 0, stream_ptr);
  cudaFreeAsync(uv, s);
  if (rc != PIV_OK) return rc;
  PIV_TRY(cuda_ok(cudaStreamSynchronize(s), "stream synchronize"));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  PIV_TRY(cuda_ok(cudaEventCreate(&e0), "cudaEventCreate"));
  rc = cuda_ok(cudaEventCreate(&e1), "cudaEventCreate");
  for (size_t k = 0; rc == PIV_OK && k < p->st.size(); ++k) {
    IterState& st = p->st[k];
    const CorrArgs& c = st.corr;
    const int nv = corr_variant_count(p->cfg.dft_mode, c);
    st.tune_ms.assign(nv, -1.0f);
    const TuneKey key = tune_key(p->cfg.dft_mode, c);
    {
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto f = g_tune_cache.find(key);
      if (f != g_tune_cache.end() && f->second < nv) {
        st.corr_variant = f->second;
        continue;
      }
    }
    int best = 0;
    float best_ms = 0;
    for (int v = 0; v < nv && rc == PIV_OK; ++v) {
      rc = run_corr(p->cfg.dft_mode, c, v, s);  // warm-up, first-use configuration
      cudaEventRecord(e0, s);
      for (int r = 0; r < reps && rc == PIV_OK; ++r) rc = run_corr(p->cfg.dft_mode, c, v, s);
      cudaEventRecord(e1, s);
      if (rc == PIV_OK) rc = cuda_ok(cudaEventSynchronize(e1), "autotune");
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= reps;
      st.tune_ms[v] = ms;
      if (v == 0 || ms < best_ms) {
        best_ms = ms;
        best = v;
      }
    }
    if (rc != PIV_OK) break;
    st.corr_variant = best;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache[key] = best;
  }
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (rc != PIV_OK) return rc;
  int status = 0;
  PIV_TRY(piv_plan_status(p, &status, stream_ptr));
  if (status != PIV_OK) return set_error(status, "autotune: a bounded device-side wait gave up");
  if (p->graph_exec) {  // a captured run would keep the old variants
    cudaGraphExecDestroy(p->graph_exec);
    p->graph_exec = nullptr;
  }
  return PIV_OK;
}

int piv_plan_tuning(const piv_plan* p, int iter, int* variant, int* n_variants, float* ms, int capacity) {
  if (!p || !variant || !n_variants) return set_error(PIV_E_ARG, "NULL argument");
  if (iter < 0 || iter >= (int)p->st.size()) return set_error(PIV_E_ARG, "iteration %d out of range", iter);
  const IterState& st = p->st[iter];
  *variant = st.corr_variant;
  *n_variants = st.corr_valid ? corr_variant_count(p->cfg.dft_mode, st.corr) : 0;
  for (int v = 0; ms && v < capacity && v < *n_variants; ++v)
    ms[v] = v < (int)st.tune_ms.size() ? st.tune_ms[v] : -1.0f;
  return PIV_OK;
}

int piv_plan_variant_name(const piv_plan* p, int iter, int variant, char* buf, size_t len) {
  if (!p || !buf || len == 0) return set_error(PIV_E_ARG, "NULL argument");
  if (iter < 0 || iter >= (int)p->st.size()) return set_error(PIV_E_ARG, "iteration %d out of range", iter);
  const IterState& st = p->st[iter];
  if (!st.corr_valid) return set_error(PIV_E_ARG, "the plan has not run yet");
  const CorrArgs& c = st.corr;
  if (correlate_tensor_supported(c, p->cfg.dft_mode)) {
    int per_sm = 0, async = 0;
    if (correlate_tensor_variant_describe(c, p->cfg.dft_mode, variant, &per_sm, &async) != PIV_OK)
      return set_error(PIV_E_ARG, "variant %d out of range", variant);
    snprintf(buf, len, "tensor%s ss=%d N=%d, %d CTA/SM, %s staging",
             p->cfg.dft_mode == PIV_DFT_TENSOR_SPLIT ? (c.ss == 64 ? " refined (split form)" : " hi/lo")
             : p->cfg.dft_mode == PIV_DFT_TENSOR_REFINED ? " refined" : "", c.ss, c.fft_size, per_sm,
             async ? "async" : "sync");
  } else {
    int r1 = 0, r2 = 0, wpc = 0, nt = 0;
    if (correlate_fft_variant_describe(c.fft_size, c.dtype, variant, &r1, &r2, &wpc, &nt) != PIV_OK)
      return set_error(PIV_E_ARG, "variant %d out of range", variant);
    snprintf(buf, len, "fft%s N=%d, radix %dx%d, %d windows/CTA, %d threads", c.dtype == PIV_DTYPE_F64 ? "64" : "32",
             c.fft_size, r1, r2, wpc, nt);
  }
  return PIV_OK;
}

int piv_plan_set_variant(piv_plan* p, int iter, int variant) {
  if (!p) return set_error(PIV_E_ARG, "NULL plan");
  if (iter < 0 || iter >= (int)p->st.size()) return set_error(PIV_E_ARG, "iteration %d out of range", iter);
  IterState& st = p->st[iter];
  if (variant < 0 || (st.corr_valid && variant >= corr_variant_count(p->cfg.dft_mode, st.corr)))
    return set_error(PIV_E_ARG, "variant %d out of range", variant);
  st.corr_variant = variant;
  if (p->graph_exec) {
    cudaGraphExecDestroy(p->graph_exec);
    p->graph_exec = nullptr;
  }
  return PIV_OK;
}

int piv_selftest_bounded_wait(unsigned int max_polls, int* status, void* stream_ptr) {
  if (!status) return set_error(PIV_E_ARG, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream_ptr;
  int* dev = nullptr;
  PIV_TRY(cuda_ok(cudaMallocAsync((void**)&dev, sizeof(int), s), "cudaMallocAsync"));
  cudaMemsetAsync(dev, 0, sizeof(int), s);
  int rc = bounded_wait_probe(max_polls, dev, s);
  if (rc == PIV_OK) rc = cuda_ok(cudaMemcpyAsync(status, dev, sizeof(int), cudaMemcpyDeviceToHost, s), "status copy");
  cudaFreeAsync(dev, s);
  if (rc == PIV_OK) rc = cuda_ok(cudaStreamSynchronize(s), "stream synchronize");
  return rc;
}

void piv_autotune_cache_clear(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache.clear();
}

// ---------------------------------------------------------------------------
// Multi-size batches.
// ---------------------------------------------------------------------------
int piv_batch_create(const piv_config* cfgs, int n_cfgs, piv_batch** out) {
  if (!cfgs || !out || n_cfgs <= 0) return set_error(PIV_E_ARG, "NULL argument or no configuration");
  *out = nullptr;
  const piv_config& c0 = cfgs[0];
  for (int g = 1; g < n_cfgs; ++g) {
    const piv_config& c = cfgs[g];
    if (c.n_iters != c0.n_iters || c.dtype != c0.dtype || c.dft_mode != c0.dft_mode)
      return set_error(PIV_E_ARG, "batch configuration %d differs in passes, dtype or dft_mode", g);
    for (int k = 0; k < c0.n_iters; ++k) {
      const piv_iteration &a = c0.iters[k], &b = c.iters[k];
      if (a.search_size != b.search_size || a.window_size != b.window_size || a.fft_size != b.fft_size ||
          a.normalize != b.normalize || a.subpixel_method != b.subpixel_method || a.s2n_method != b.s2n_method)
        return set_error(PIV_E_ARG, "batch configuration %d differs from configuration 0 in pass %d", g, k);
    }
  }
  piv_batch* b = new piv_batch();
  int rc = PIV_OK;
  for (int g = 0; g < n_cfgs && rc == PIV_OK; ++g) {
    piv_plan* p = nullptr;
    rc = piv_plan_create(&cfgs[g], &p);
    if (rc == PIV_OK) b->plans.push_back(p);
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    if (rc == PIV_OK) rc = cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    if (rc == PIV_OK) b->streams.push_back(st);
    if (rc == PIV_OK) rc = cuda_ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
    if (rc == PIV_OK) b->done.push_back(ev);
  }
  if (rc == PIV_OK) rc = cuda_ok(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "cudaEventCreate");
  if (rc != PIV_OK) {
    piv_batch_destroy(b);
    return rc;
  }
  *out = b;
  return PIV_OK;
}

void piv_batch_destroy(piv_batch* b) {
  if (!b) return;
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  for (piv_plan* p : b->plans) piv_plan_destroy(p);
  for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
  for (cudaEvent_t ev : b->done) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  delete b;
}

int piv_batch_plan(piv_batch* b, int group, piv_plan** plan) {
  if (!b || !plan) return set_error(PIV_E_ARG, "NULL argument");
  if (group < 0 || group >= (int)b->plans.size()) return set_error(PIV_E_ARG, "group %d out of range", group);
  *plan = b->plans[group];
  return PIV_OK;
}

// Enqueues one batch run: every size group runs its stages on its own stream;
// a pass on a tensor engine joins the groups, launches one correlation over
// all their windows (up to kMaxCorrSegs sizes per launch) on `s` and forks
// again.
static int batch_enqueue(piv_batch* b, const int* n_pairs, const void* const* frames_a,
                         const void* const* frames_b, double* const* u, double* const* v,
                         uint8_t* const* val_locations, uint8_t* const* outliers, cudaStream_t s) {
  const int G = (int)b->plans.size();
  std::vector<int> act;  // groups with pairs in this run
  for (int g = 0; g < G; ++g) {
    if (n_pairs[g] < 0 || n_pairs[g] > b->plans[g]->cfg.max_pairs)
      return set_error(PIV_E_ARG, "group %d: n_pairs %d outside [0, %d]", g, n_pairs[g], b->plans[g]->cfg.max_pairs);
    if (n_pairs[g] == 0) continue;
    if (!frames_a[g] || !frames_b[g] || !u[g] || !v[g]) return set_error(PIV_E_ARG, "group %d: NULL argument", g);
    act.push_back(g);
  }
  if (act.empty()) return PIV_OK;
  std::vector<RunCtx> x(G);
  PIV_TRY(cuda_ok(cudaEventRecord(b->fork, s), "cudaEventRecord"));
  for (int g : act) {
    PIV_TRY(cuda_ok(cudaStreamWaitEvent(b->streams[g], b->fork, 0), "cudaStreamWaitEvent"));
    PIV_TRY(run_begin(b->plans[g], n_pairs[g], frames_a[g], frames_b[g], 0, b->streams[g], x[g]));
  }
  const int n_it = (int)b->plans[0]->st.size();
  const int mode = b->plans[0]->cfg.dft_mode;
  for (int k = 0; k < n_it; ++k) {
    std::vector<CorrArgs> cs(G);
    bool joint = b->joint != 0;
    for (int g : act) {
      PIV_TRY(run_pre(b->plans[g], k, x[g], b->streams[g], cs[g]));
      joint = joint && correlate_tensor_supported(cs[g], mode) && cs[g].pixel_type == cs[act[0]].pixel_type;
    }
    if (joint) {
      for (int g : act) {
        PIV_TRY(cuda_ok(cudaEventRecord(b->done[g], b->streams[g]), "cudaEventRecord"));
        PIV_TRY(cuda_ok(cudaStreamWaitEvent(s, b->done[g], 0), "cudaStreamWaitEvent"));
      }
      for (size_t c0 = 0; c0 < act.size(); c0 += kMaxCorrSegs) {
        CorrArgs m = cs[act[c0]];
        m.n_segs = 0;
        m.seg_windows = 0;
        for (size_t j = c0; j < act.size() && j < c0 + kMaxCorrSegs; ++j) {
          const CorrArgs& c = cs[act[j]];
          CorrSeg& q = m.segs[m.n_segs++];
          q.frame_a = c.frame_a;
          q.frame_b = c.frame_b;
          q.u = c.u;
          q.v = c.v;
          q.peak_i = c.peak_i;
          q.peak_j = c.peak_j;
          q.win_mask = c.win_mask;
          q.near_tie = c.near_tie;
          q.tie_count = c.tie_count;
          q.tie_list = c.tie_list;
          q.tie_list_count = c.tie_list_count;
          q.win_means = c.win_means;
          q.win0 = m.seg_windows;
          q.height = c.height;
          q.width = c.width;
          q.spacing = c.spacing;
          q.m = c.m;
          q.n = c.n;
          q.x_offset = c.x_offset;
          q.y_offset = c.y_offset;
          q.n_pairs = c.n_pairs;
          m.seg_windows += (long long)c.n_pairs * c.m * c.n;
        }
        const int var = k < (int)b->corr_variant.size() ? b->corr_variant[k] : 0;
        PIV_TRY(run_corr(mode, m, var, s));
      }
      PIV_TRY(cuda_ok(cudaEventRecord(b->fork, s), "cudaEventRecord"));
      for (int g : act) PIV_TRY(cuda_ok(cudaStreamWaitEvent(b->streams[g], b->fork, 0), "cudaStreamWaitEvent"));
    } else {
      for (int g : act) PIV_TRY(run_corr(mode, cs[g], b->plans[g]->st[k].corr_variant, b->streams[g]));
    }
    for (int g : act) PIV_TRY(run_post(b->plans[g], k, x[g], b->streams[g]));
  }
  for (int g : act) {
    PIV_TRY(run_end(b->plans[g], x[g], u[g], v[g], val_locations ? val_locations[g] : nullptr,
                    outliers ? outliers[g] : nullptr, 0, b->streams[g]));
    PIV_TRY(cuda_ok(cudaEventRecord(b->done[g], b->streams[g]), "cudaEventRecord"));
    PIV_TRY(cuda_ok(cudaStreamWaitEvent(s, b->done[g], 0), "cudaStreamWaitEvent"));
  }
  return PIV_OK;
}

int piv_batch_run(piv_batch* b, const int* n_pairs, const void* const* frames_a, const void* const* frames_b,
                  double* const* u, double* const* v, uint8_t* const* val_locations, uint8_t* const* outliers,
                  void* stream) {
  if (!b || !n_pairs || !frames_a || !frames_b || !u || !v) return set_error(PIV_E_ARG, "NULL argument");
  PIV_TRY(batch_enqueue(b, n_pairs, frames_a, frames_b, u, v, val_locations, outliers, (cudaStream_t)stream));
  return cuda_ok(cudaGetLastError(), "piv_batch_run");
}

int piv_batch_graph_capture(piv_batch* b, const int* n_pairs, const void* const* frames_a,
                            const void* const* frames_b, double* const* u, double* const* v,
                            uint8_t* const* val_locations, uint8_t* const* outliers, int* kernel_nodes,
                            void* stream) {
  if (!b || !n_pairs || !frames_a || !frames_b || !u || !v) return set_error(PIV_E_ARG, "NULL argument");
  if (!stream) return set_error(PIV_E_ARG, "graph capture needs a non-default stream");
  cudaStream_t s = (cudaStream_t)stream;
  if (b->graph_exec) {
    cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
  }
  PIV_TRY(cuda_ok(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture"));
  int rc = batch_enqueue(b, n_pairs, frames_a, frames_b, u, v, val_locations, outliers, s);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  if (rc != PIV_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return set_cuda_error(e, "cudaStreamEndCapture");
  if (kernel_nodes) {
    size_t n = 0;
    cudaGraphGetNodes(graph, nullptr, &n);
    std::vector<cudaGraphNode_t> nodes(n);
    cudaGraphGetNodes(graph, nodes.data(), &n);
    int kn = 0;
    for (size_t i = 0; i < n; ++i) {
      cudaGraphNodeType t;
      cudaGraphNodeGetType(nodes[i], &t);
      if (t == cudaGraphNodeTypeKernel) ++kn;
    }
    *kernel_nodes = kn;
  }
  e = cudaGraphInstantiate(&b->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  return cuda_ok(e, "cudaGraphInstantiate");
}

int piv_batch_graph_launch(piv_batch* b, void* stream) {
  if (!b || !b->graph_exec) return set_error(PIV_E_ARG, "no captured graph");
  return cuda_ok(cudaGraphLaunch(b->graph_exec, (cudaStream_t)stream), "cudaGraphLaunch");
}

int piv_batch_set_schedule(piv_batch* b, int joint) {
  if (!b) return set_error(PIV_E_ARG, "NULL batch");
  b->joint = joint != 0;
  if (b->graph_exec) {
    cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
  }
  return PIV_OK;
}

int piv_batch_status(piv_batch* b, int* status, void* stream) {
  if (!b || !status) return set_error(PIV_E_ARG, "NULL argument");
  int worst = PIV_OK;
  for (piv_plan* p : b->plans) {
    int st = PIV_OK;
    PIV_TRY(piv_plan_status(p, &st, stream));
    if (worst == PIV_OK) worst = st;
  }
  *status = worst;
  return PIV_OK;
}

}  // extern "C"
