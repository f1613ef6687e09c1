// Internal interfaces between the kernel files and the C-ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/piv_gb300.h"

namespace piv {

// Records an error message for piv_last_error() and returns `code`.
int set_error(int code, const char* fmt, ...);
int set_cuda_error(cudaError_t e, const char* what);

// Arguments of one correlation pass over n_pairs frame pairs.
// One frame geometry of a multi-geometry correlation launch: the windows of
// n_pairs pairs of one frame size, global windows [win0, win0 + n_pairs m n)
// of the launch, with their own frames and outputs.
struct CorrSeg {
  const void* frame_a;
  const void* frame_b;
  void* u;
  void* v;
  int* peak_i;
  int* peak_j;
  const uint8_t* win_mask;
  uint8_t* near_tie;  // per window: 1 where the top two map values are within the engine's tie tolerance; may be NULL
  int* tie_count;     // incremented once per near-tie window; may be NULL
  int* tie_list;      // refined form: scratch [n_pairs m n] for the near-tie windows' indices, and their count
  int* tie_list_count;
  float* win_means;   // refined form: [n_pairs m n][2] window means of frames a and b (written by the engine)
  long long win0;
  int height, width, spacing, m, n, x_offset, y_offset, n_pairs;
};
constexpr int kMaxCorrSegs = 8;

struct CorrArgs {
  const void* frame_a;
  const void* frame_b;
  int pixel_type;
  int height, width;
  int ss, ws, spacing, m, n, x_offset, y_offset;
  int n_pairs;
  int fft_size;
  int normalize;
  int subpixel;
  int dtype;
  const uint8_t* win_mask;
  void* u;
  void* v;
  int* peak_i;
  int* peak_j;
  void* s2n;
  int s2n_method;
  int s2n_size;
  void* scratch;        // device scratch for transforms that do not fit in shared memory
  size_t scratch_bytes;
  void* maps;           // optional [windows][N][N] output of the shifted correlation maps
  int* status;          // device word set to PIV_E_TIMEOUT when a bounded wait gives up (tensor engine)
  // Near ties: a window whose second-largest map value (at another lag; lags
  // without window overlap read as zero) is within tie_tol * |peak| of the
  // peak gets near_tie[window] = 1 and one increment of *tie_count (both may
  // be NULL). The engine launchers set tie_tol to the engine's map accuracy
  // (kTieTol*): such a window's integer peak is not resolved by the engine.
  uint8_t* near_tie;
  int* tie_count;
  float tie_tol;
  // FFT engine: with win_list, only the windows win_list[0 .. *win_count)
  // (window indices pair-major, as the outputs are indexed) are correlated.
  const int* win_list;
  const int* win_count;
  // Refined tensor form: scratch for the near-tie windows' indices (n_pairs m
  // n ints) and their count; when set, those windows are correlated again by
  // the float32 FFT engine, which resolves their integer peaks (NULL: they
  // keep the fp16 maps' peaks and are counted as near ties).
  int* tie_list;
  int* tie_list_count;
  // Refined tensor form: the fp16 engine writes each window's mean of frame a
  // and of frame b here ([n_pairs m n][2]), and the refinement reads them.
  float* win_means;
  // Multi-geometry launch (tensor engines): n_segs > 0 segments replace the
  // single geometry above (frames, sizes, outputs, mask; the window and search
  // sizes, pixel type and settings are shared), covering seg_windows windows
  // in total. The table travels in the kernel parameters.
  int n_segs;
  long long seg_windows;
  CorrSeg segs[kMaxCorrSegs];
};

// Relative tie tolerances of the engines (map error relative to the map
// maximum, with margin): float32 FFT and hi/lo split tensor products ~1e-6,
// float64 FFT ~1e-15, fp16-operand tensor products ~6e-4.
constexpr float kTieTolF32 = 1.0f / 131072.0f;        // 2^-17
constexpr float kTieTolF64 = 1.0f / 1099511627776.0f;  // 2^-40
constexpr float kTieTolF16 = 1.0f / 512.0f;            // 2^-9

// Launch variants (tile shape, radix split, CTAs per SM, staging) of the two
// engines; variant 0 is the default, and an out-of-range variant runs it.
int correlate_fft(const CorrArgs& a, int variant, cudaStream_t stream);
int correlate_fft_variant_count(int fft_size, int dtype);
int correlate_fft_variant_describe(int fft_size, int dtype, int variant, int* r1, int* r2, int* wpc, int* nt);
size_t correlate_fft_scratch_bytes(int fft_size, int dtype);  // the largest over the variants
// dft_mode: PIV_DFT_TENSOR or PIV_DFT_TENSOR_SPLIT.
int correlate_tensor(const CorrArgs& a, int dft_mode, int variant, cudaStream_t stream);
bool correlate_tensor_supported(const CorrArgs& a, int dft_mode);
int correlate_tensor_variant_count(const CorrArgs& a, int dft_mode);
int correlate_tensor_variant_describe(const CorrArgs& a, int dft_mode, int variant, int* per_sm, int* async);
// Peak refinement after a tensor-core pass (float32 fields, n_fft 2, window =
// search size of 16, 32 or 64 px, no S2N): the five values of the subpixel
// stencil around each window's integer peak (peak_i / peak_j, as the engine
// wrote them) are recomputed in float32 from the frames by direct sums, and
// u, v are rewritten from them.
bool refine_supported(const CorrArgs& a);
int refine_peaks(const CorrArgs& a, cudaStream_t stream);
// Violations counted by the checked build's index checks in the tensor-core
// and refinement kernels since the last call (the counters are reset); -1 in
// the normal build, -2 when the counter cannot be read.
int bounds_violations_tensor();
int bounds_violations_refine();
// Indices of the windows with near_tie set into list (window order not
// kept), their number into *count (reset first).
int compact_near_ties(const uint8_t* near_tie, long long windows, int* list, int* count, cudaStream_t stream);
// One bounded mbarrier wait that nothing completes; writes PIV_E_TIMEOUT to *status_dev.
int bounded_wait_probe(uint32_t max_polls, int* status_dev, cudaStream_t stream);

// Deformation.
struct DeformArgs {
  piv_geometry geom;
  int n_pairs;
  const void* frames_a;
  const void* frames_b;
  int pixel_type;
  const double* up;
  const double* vp;
  double deforming_par;
  int order;
  const float* coef_a;
  const float* coef_b;
  int coef_pad;  // 0: [pairs][H][W]; kCoefPad: [pairs][H + 4][W + 4] with a mirrored 2-pixel border
  const uint8_t* frame_mask;
  int dtype;
  void* out_a;
  void* out_b;
};
int deform(const DeformArgs& a, cudaStream_t stream);
int regrid(const piv_geometry& src, const piv_geometry& dst, int n_pairs, const double* u_src, const double* v_src,
           double* u_dst, double* v_dst, cudaStream_t stream);
// pad = 0: coef is [n_frames][height][width]; pad = kCoefPad: [n_frames][height
// + 4][width + 4], the frame at offset (2, 2) and the border holding the
// mirrored coefficients, so that cubic taps never need the mirror rule.
constexpr int kCoefPad = 2;
int spline_prefilter(int height, int width, int n_frames, const void* frames, int pixel_type, float* coef,
                     cudaStream_t stream, int pad = 0);

// Validation and replacement.
struct ValArgs {
  int m, n, n_pairs;
  const double* u;
  const double* v;
  const void* s2n;
  int s2n_dtype;
  int size;
  double s2n_tol, median_tol, mad_tol, mean_tol, rms_tol;
  const uint8_t* field_mask;  // [m][n] or NULL
  const uint8_t* exclude;     // [pairs][m][n] or NULL
  int fp32;
};
int validate(const ValArgs& a, uint8_t* val, double* rms_stats, cudaStream_t stream);

struct RepArgs {
  ValArgs val;                // revalidation settings (u/v/exclude ignored)
  double* u;
  double* v;
  uint8_t* val_mask;
  int n_iters, method, size, revalidate;
  int dtype;                  // dtype_f of the pipeline (float32 coefficient rounding)
  void* scratch;              // replace_scratch_bytes(m, n, n_pairs)
  int* status;                // device word set to PIV_E_TIMEOUT when a solve hits its cap; may be NULL
};
size_t replace_scratch_bytes(int m, int n, int n_pairs);
int replace(const RepArgs& a, cudaStream_t stream);

// Field combination before validation: u = u_corr (+ up), in float32 when fp32.
int combine_fields(int count, const void* u_corr, const void* v_corr, int corr_dtype, const double* up,
                   const double* vp, int fp32, double* u, double* v, cudaStream_t stream);

// smoothn.
size_t smoothn_scratch_bytes(int m, int n, int n_pairs);
// flags (device [n_pairs], may be NULL) receives the PIV_SMOOTH_* bits of each pair.
int smoothn(int m, int n, int n_pairs, const double* u_in, const double* v_in, double* u_out, double* v_out,
            const uint8_t* field_mask, double s, double* p_out, void* scratch, cudaStream_t stream,
            int* flags = nullptr);

// Final scaling u * scaling_par / dt (gpu_process.py:847-849).
int scale_fields(int count, const double* u, const double* v, double scaling, double dt, int fp32, double* uo,
                 double* vo, cudaStream_t stream);

}  // namespace piv
