/*
 * piv_gb300.h - C ABI of the GB300-native multi-pass PIV library (libpiv_gb300.so).
 *
 * The library replaces the device side of openpiv-python-gpu's PIV path:
 * PIVGPU.__call__ (openpiv_gpu/gpu_process.py:564-647) and everything it calls.
 * All pointers are plain host or device addresses; `stream` is a cudaStream_t
 * passed as void* (NULL = the legacy default stream). Every function returns a
 * status code (PIV_OK = 0); piv_last_error() returns the message of the last
 * failure on the calling thread.
 *
 * Field arrays are row-major [pair][m][n]. Frames are row-major [pair][H][W].
 * "None" for a tolerance or smoothing parameter is encoded as NaN.
 */
#ifndef PIV_GB300_H
#define PIV_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define PIV_OK 0
#define PIV_E_ARG 1         /* invalid argument (the Python layer raises AssertionError) */
#define PIV_E_OOM 2         /* device allocation failed */
#define PIV_E_CUDA 3        /* CUDA runtime error */
#define PIV_E_TIMEOUT 4     /* a bounded device-side iteration gave up */
#define PIV_E_UNSUPPORTED 6 /* configuration outside what the kernels implement */

/* Pixel types of input frames. */
#define PIV_PIXEL_U8 0
#define PIV_PIXEL_U16 1
#define PIV_PIXEL_F32 2
#define PIV_PIXEL_F64 3

/* Float type of the correlation (the reference's dtype_f). */
#define PIV_DTYPE_F32 0
#define PIV_DTYPE_F64 1

/* Subpixel methods (gpu_process.py:1276-1292). */
#define PIV_SUBPIXEL_GAUSSIAN 0
#define PIV_SUBPIXEL_PARABOLIC 1
#define PIV_SUBPIXEL_CENTROID 2

/* Signal-to-noise methods (gpu_process.py:1321-1330). */
#define PIV_S2N_PEAK2PEAK 0
#define PIV_S2N_PEAK2MEAN 1
#define PIV_S2N_PEAK2ENERGY 2

/* Replacement methods (gpu_validation.py:319-324). */
#define PIV_REPLACE_SPRING 0
#define PIV_REPLACE_MEDIAN 1
#define PIV_REPLACE_MEAN 2

/* Flag bits of smoothn per pair (the conditions of SmoothnGPU's log
 * messages, gpu_smoothn.py:218-222, 429-439). */
#define PIV_SMOOTH_S_LOWER 1     /* GCV: log10(s) within 0.1 of its lower bound */
#define PIV_SMOOTH_S_UPPER 2     /* GCV: log10(s) within 0.1 of its upper bound */
#define PIV_SMOOTH_MAX_ITERS 4   /* the weighted iteration reached its last allowed step (100) */

/* Correlation engines. */
#define PIV_DFT_FFT32 0          /* in-shared-memory FFT in the correlation float type */
#define PIV_DFT_TENSOR 1         /* tcgen05 tensor-core DFT: FP16 operands, FP32 accumulation
                                    (float32 passes with search 16, 32 or 64 px and n_fft 2;
                                    other passes use the FFT) */
#define PIV_DFT_TENSOR_SPLIT 2   /* as PIV_DFT_TENSOR with every operand split into FP16 hi and
                                    lo parts and three products per stage (compensated) for
                                    search 16 or 32 px; 64-px passes take the refined path of
                                    PIV_DFT_TENSOR_REFINED (float32 accuracy as well); other
                                    passes use the FFT */
#define PIV_DFT_TENSOR_REFINED 3 /* PIV_DFT_TENSOR's maps give each window's integer peak, then
                                    the five values of the subpixel fit are recomputed in float32
                                    by direct sums from the frames (float32 FFT accuracy of the
                                    fit; same passes as PIV_DFT_TENSOR, others use the FFT) */

/* Settings of one PIV iteration, the per-pass tuple entries of
 * PIVGPU.__init__ (gpu_process.py:497-546) expanded per iteration as the
 * reference's settings generators do (gpu_process.py:675-728). */
typedef struct piv_iteration {
    int search_size;          /* 2**(P-1-i) * min_search_size */
    int window_size;          /* == search_size except with shrink_ratio on iteration 0 (gpu_process.py:654-662) */
    double overlap_ratio;
    int fft_size;             /* N = 2**ceil(log2(search_size * n_fft)) (gpu_process.py:1102-1103) */
    int deforming_order;      /* 1: the reference's bilinear kernel; 3: cubic B-spline */
    double deforming_par;     /* 0 <= dp <= 1 (gpu_process.py:1165-1171) */
    int normalize;
    int subpixel_method;
    int s2n_method;
    int s2n_size;
    int validation_size;
    double s2n_tol, median_tol, mad_tol, mean_tol, rms_tol; /* NaN = None */
    int num_replacing_iters;
    int replacing_method;
    int replacing_size;
    int revalidate;
    double smoothing_par;     /* NaN = GCV (gpu_smoothn.py:114) */
} piv_iteration;

/* Whole-pipeline configuration: PIVGPU(frame_shape, min_search_size, **settings)
 * (gpu_process.py:465-562). */
typedef struct piv_config {
    int height, width;        /* frame_shape */
    int n_iters;              /* sum(search_size_iters) */
    const piv_iteration* iters;
    int center;
    double dt;
    double scaling_par;
    int dtype;                /* PIV_DTYPE_F32 / PIV_DTYPE_F64 */
    int pixel_type;           /* PIV_PIXEL_* of the frames given to piv_plan_run */
    int max_pairs;            /* pairs per piv_plan_run call; sizes the workspace */
    const uint8_t* mask;      /* host [height][width], nonzero = masked; NULL for none */
    int dft_mode;             /* PIV_DFT_* */
} piv_config;

typedef struct piv_plan piv_plan;

/* Builds a plan (the reference builds its PIVFieldGPU list once per instance,
 * gpu_process.py:560,649-673) and allocates every device workspace it needs for
 * up to max_pairs pairs. Replaces PIVGPU.__init__. */
int piv_plan_create(const piv_config* cfg, piv_plan** out);

/* Field shape (m, n) of iteration `iter` (PIVFieldGPU.field_shape, gpu_process.py:922-925). */
int piv_plan_field_shape(const piv_plan* plan, int iter, int* m, int* n);

/* Device bytes held by the plan. */
int piv_plan_workspace_bytes(const piv_plan* plan, size_t* bytes);

/* Runs the whole multi-pass pipeline on n_pairs frame pairs. Replaces
 * PIVGPU.__call__ (gpu_process.py:564-647) for a batch of pairs.
 *   frames_a, frames_b: [n_pairs][H][W] of cfg.pixel_type, host or device
 *                       (frames_on_host = 1: pageable or pinned host memory).
 *   u, v:               [n_pairs][m][n] float64 results of the last iteration
 *                       (scaled like scale_fields, gpu_process.py:847-849).
 *   val_locations:      [n_pairs][m][n] uint8, outliers found before replacement
 *                       in the last iteration (piv_gpu.val_locations); may be NULL.
 *   outliers:           [n_pairs][m][n] uint8, outliers left after replacement
 *                       (piv_gpu.outliers); may be NULL.
 * All kernels go to `stream`; with outputs_on_host = 1 the call returns after
 * the results are copied back, with outputs_on_host = 2 the copies to host
 * memory are queued on `stream` and the call returns at once (the caller
 * synchronises the stream before reading them: lets a caller upload the next
 * batch while this one runs), otherwise (device outputs) it returns without
 * synchronising. */
int piv_plan_run(piv_plan* plan, int n_pairs, const void* frames_a, const void* frames_b, int frames_on_host,
                 double* u, double* v, uint8_t* val_locations, uint8_t* outliers, int outputs_on_host,
                 void* stream);

/* Device status word of the plan's bounded device-side waits (the tensor-core
 * correlation's MMA completion waits, the spring solver's iteration cap):
 * PIV_OK, or PIV_E_TIMEOUT when a wait gave up since the last call (the word
 * is then reset). Synchronises `stream`. No counterpart in the reference,
 * whose CuPy calls have no device-side waits. */
int piv_plan_status(piv_plan* plan, int* status, void* stream);

/* Near ties of the correlation peaks of the last run, per iteration (counts
 * over all pairs; counts[k] for iteration k, up to `capacity` entries). A
 * window is a near tie when its second-largest correlation value, at another
 * lag (lags without window overlap read as zero), is within tol * |peak| of
 * the peak, tol being the engine's map accuracy: 2^-17 for the float32 FFT
 * and the hi/lo split tensor engines, 2^-40 for the float64 FFT, 2^-9 for the
 * fp16-operand tensor engine. Its integer peak location is then not resolved
 * by the engine and may differ from the reference's first argmax
 * (gpu_process.py:1248-1254); every other window's integer peak is expected
 * to be identical. Masked windows are never near ties. The per-window flags
 * are in piv_iteration_view.near_tie. Synchronises `stream`. */
int piv_plan_near_ties(piv_plan* plan, int* counts, int capacity, void* stream);

/* Autotuner (no counterpart in the reference, whose correlation is one cuFFT
 * call per pass). Runs the plan once on the given frames, then times every
 * launch variant of each pass's correlation engine on that pass's own inputs
 * (`reps` launches each after one warm-up, CUDA events on `stream`) and keeps
 * the fastest for later runs. Variants of the FFT engine differ in radix split
 * and tile shape (windows per CTA, threads per CTA) and agree up to rounding;
 * variants of the tensor engines differ in CTAs per SM and staging and give
 * identical results. Results are shared by the plans of the process (same
 * engine, sizes, pixel type, alignment and order of magnitude of windows skip
 * the timing). A captured graph of the plan is released. Synchronises
 * `stream`. */
int piv_plan_autotune(piv_plan* plan, int n_pairs, const void* frames_a, const void* frames_b, int frames_on_host,
                      int reps, void* stream);
/* Chosen variant of iteration `iter`, the number of variants of its engine
 * (0 before the first run) and the autotuner's time per variant in ms (-1 where
 * not timed), up to `capacity` entries. */
int piv_plan_tuning(const piv_plan* plan, int iter, int* variant, int* n_variants, float* ms, int capacity);
/* Human-readable description of variant `variant` of iteration `iter` (after a run). */
int piv_plan_variant_name(const piv_plan* plan, int iter, int variant, char* buf, size_t len);
/* Sets the variant of iteration `iter` (e.g. a choice saved from an earlier
 * autotune); an out-of-range variant is an error once the plan has run. */
int piv_plan_set_variant(piv_plan* plan, int iter, int variant);
/* Forgets the process-wide autotuner results. */
void piv_autotune_cache_clear(void);
/* Failure-detection self test: one bounded mbarrier wait that no arrival
 * completes (the primitive behind every tensor-core completion wait), run for
 * max_polls polls; *status receives the status word the kernel wrote,
 * PIV_E_TIMEOUT. The context stays usable afterwards. Synchronises `stream`.
 * No counterpart in the reference. */
int piv_selftest_bounded_wait(unsigned int max_polls, int* status, void* stream);

/* Multi-size batch: a submission of pairs of several frame sizes processed
 * together (the reference processes one pair per PIVGPU call,
 * gpu_process.py:564-647). One plan per frame size (configs[g]; every
 * configuration has the same passes: search, window and transform sizes,
 * normalisation, subpixel and S2N method, plus the same dtype and dft_mode).
 * A run gives each size group its own stream for its stages; a pass on a
 * tensor engine joins the groups and runs ONE correlation launch over the
 * windows of every pair of every size (a segment table of up to 8 sizes per
 * launch travels in the kernel parameters), then forks them again. Results
 * equal each group's piv_plan_run. */
typedef struct piv_batch piv_batch;
int piv_batch_create(const piv_config* configs, int n_configs, piv_batch** out);
void piv_batch_destroy(piv_batch* batch);
/* The plan of size group `group` (iteration views, tuning, status). */
int piv_batch_plan(piv_batch* batch, int group, piv_plan** plan);
/* Enqueues one run on `stream` with device frames and device outputs per
 * group (n_pairs[g] = 0 skips group g; val_locations / outliers may be NULL
 * or hold NULL entries). Does not synchronise. */
int piv_batch_run(piv_batch* batch, const int* n_pairs, const void* const* frames_a, const void* const* frames_b,
                  double* const* u, double* const* v, uint8_t* const* val_locations, uint8_t* const* outliers,
                  void* stream);
/* Captures one run as a CUDA graph (fixed pointers and pair counts);
 * kernel_nodes receives the number of kernel nodes. */
int piv_batch_graph_capture(piv_batch* batch, const int* n_pairs, const void* const* frames_a,
                            const void* const* frames_b, double* const* u, double* const* v,
                            uint8_t* const* val_locations, uint8_t* const* outliers, int* kernel_nodes,
                            void* stream);
int piv_batch_graph_launch(piv_batch* batch, void* stream);
/* Schedule of the correlation: joint = 1 (default) launches one correlation
 * per pass over every size on the tensor engines, after joining the size
 * groups' streams; joint = 0 keeps every size group on its own stream for
 * the whole run (one correlation launch per size and pass, overlapping the
 * other groups' stages). Results are the same; a captured graph is released. */
int piv_batch_set_schedule(piv_batch* batch, int joint);
/* Worst status word of the groups' plans (see piv_plan_status). */
int piv_batch_status(piv_batch* batch, int* status, void* stream);

/* Per-iteration intermediates of the last piv_plan_run (device pointers owned
 * by the plan, valid until the next run): correlation output u/v (dtype of the
 * correlation), predictor on the iteration's grid, fields after validation and
 * replacement, initial outlier mask and the smoothing exponent p = log10(s). */
typedef struct piv_iteration_view {
    int m, n;
    const void* u_corr; const void* v_corr; /* [pairs][m][n], float32 or float64 per dtype */
    const double* up; const double* vp;     /* predictor on this grid (NULL for iteration 0) */
    const double* u_rep; const double* v_rep;
    const double* u_out; const double* v_out; /* after smoothing (== u_rep on the last iteration) */
    const uint8_t* val0;
    const double* smooth_p;                 /* [pairs], NaN when no smoothing ran */
    const int* peak_i; const int* peak_j;   /* integer peak of each window (shifted map) */
    const void* s2n;                        /* [pairs][m][n] or NULL */
    const uint8_t* near_tie;                /* [pairs][m][n]: 1 where the peak is a near tie (piv_plan_near_ties) */
    const int* smooth_flags;                /* [pairs]: PIV_SMOOTH_* bits of this iteration's smoothing (0 when none ran) */
} piv_iteration_view;
int piv_plan_iteration_view(const piv_plan* plan, int iter, piv_iteration_view* out);

/* Releases every device resource of the plan. */
void piv_plan_destroy(piv_plan* plan);

/* CUDA-graph form of piv_plan_run (no counterpart in the reference, which
 * launches from Python with host synchronisations): captures one run on
 * device buffers into an executable graph held by the plan. kernel_nodes
 * (may be NULL) receives the number of kernel launches in one run. */
int piv_plan_graph_capture(piv_plan* plan, int n_pairs, const void* frames_a, const void* frames_b, double* u,
                           double* v, uint8_t* val_locations, uint8_t* outliers, int* kernel_nodes, void* stream);
/* Launches the captured graph on `stream`. */
int piv_plan_graph_launch(piv_plan* plan, void* stream);

/* Stage timing (instrumentation, no counterpart in the reference). With
 * timing on, piv_plan_run records CUDA events at every stage boundary.
 * piv_plan_stage_times waits for the recorded runs and returns the summed
 * milliseconds per stage: index k * PIV_STAGES + s for iteration k and stage
 * s (predictor, deform, correlate, validate, replace, smooth), then input
 * copy and output copy at n_iters * PIV_STAGES and + 1. It clears the sums and
 * returns the number of runs covered in *runs. */
#define PIV_STAGES 6
int piv_plan_set_timing(piv_plan* plan, int enable);
int piv_plan_stage_times(piv_plan* plan, float* ms, int capacity, int* runs);

/* Index checks of a checked build of this library (compiled with
 * -DPIV_BOUNDS_CHECK; a test and debugging aid, no counterpart in the
 * reference): *checked = 1 in such a build, where every shared-memory store,
 * asynchronous copy, TMEM load, window read and result write of the
 * tensor-core correlation and peak refinement kernels is checked against its
 * buffer, and a failed check skips the access and is counted; *violations
 * receives the count since the last call (then reset). The normal build
 * gives *checked = 0, *violations = 0. Synchronises the device. */
int piv_bounds_check(int* checked, int* violations);

/* Copies the message of the last failure on this thread into buf. */
int piv_last_error(char* buf, size_t len);

/* Plain memory copy for bindings that have no CUDA runtime binding of their
 * own (no counterpart in the reference, which copies through CuPy).
 * kind: 0 device->host, 1 host->device, 2 device->device. Synchronous when
 * stream is NULL. */
int piv_memcpy(void* dst, const void* src, size_t bytes, int kind, void* stream);

/* ------------------------------------------------------------------------
 * Stage entry points (device pointers). They back the component classes of
 * the Python layer and the stage-level parity tests.
 * ---------------------------------------------------------------------- */

/* Window geometry of one pass (PIVFieldGPU, gpu_process.py:897-961). */
typedef struct piv_geometry {
    int height, width;        /* frame shape */
    int search_size, window_size, spacing;
    int m, n;                 /* field shape */
    int x_offset, y_offset;
} piv_geometry;

/* Fills `geom` exactly as PIVFieldGPU does (gpu_process.py:897-938). */
int piv_field_geometry(int height, int width, int window_size, int search_size, double overlap_ratio,
                       int center, piv_geometry* geom);

/* Cross-correlation of every window pair of n_pairs frame pairs, first peak,
 * subpixel fit and displacement: CorrelationGPU.__call__ without deformation
 * (gpu_process.py:1021-1097, 1122-1147, 1201-1310) and, when s2n != NULL,
 * get_s2n_ratio (gpu_process.py:1312-1347).
 *   frames_*: device [n_pairs][H][W] of pixel_type; masked windows (win_mask[k]
 *   nonzero, may be NULL) produce NaN displacement and zero s2n.
 *   u, v, s2n: device [n_pairs][m][n] of dtype; peak_i/peak_j may be NULL.
 * Every search window of `geom` must lie inside the frame: a geometry whose
 * last window passes the frame's edge (piv_field_geometry's centred grid with
 * an odd search size and no spare pixel) gives PIV_E_UNSUPPORTED, inconsistent
 * sizes or a negative n_pairs PIV_E_ARG (also piv_correlate_maps; plans refuse
 * such passes at creation). */
int piv_correlate(const piv_geometry* geom, int n_pairs, const void* frames_a, const void* frames_b,
                  int pixel_type, int dtype, int fft_size, int normalize, int subpixel_method,
                  const uint8_t* win_mask, void* u, void* v, int* peak_i, int* peak_j,
                  int s2n_method, int s2n_size, void* s2n, int dft_mode, void* stream);

/* The fftshift-ed correlation maps of every window pair (the reference keeps
 * them as CorrelationGPU.corr, gpu_process.py:1086,1207-1220): device
 * [n_pairs][m][n][N][N] of dtype, N = fft_size. Same arguments as
 * piv_correlate. */
int piv_correlate_maps(const piv_geometry* geom, int n_pairs, const void* frames_a, const void* frames_b,
                       int pixel_type, int dtype, int fft_size, int normalize, const uint8_t* win_mask, void* maps,
                       int dft_mode, void* stream);

/* Linear interpolation of a field from grid `src` to the coordinates of grid
 * `dst`, with linear extrapolation (interpolate_displacement,
 * gpu_process.py:730-742). Device float64 [n_pairs][m][n]. */
int piv_regrid(const piv_geometry* src, const piv_geometry* dst, int n_pairs, const double* u_src,
               const double* v_src, double* u_dst, double* v_dst, void* stream);

/* Frame deformation by the predictor field on grid `geom` (deform_frame +
 * interpolate_frame, gpu_process.py:1149-1192, 1461-1547): frame A is sampled
 * at x + up*(dp-1), frame B at x + up*dp (0 < dp < 1), only B at dp == 1, only
 * A at dp == 0. Order 1 is the reference's bilinear kernel; order 3 samples the
 * cubic B-spline coefficient frames `coef_a/coef_b` (piv_spline_prefilter).
 * Outputs are device [n_pairs][H][W] in dtype; a frame that is not deformed is
 * copied (converted) from the input. frame_mask (device, may be NULL) zeroes
 * masked pixels. */
int piv_deform(const piv_geometry* geom, int n_pairs, const void* frames_a, const void* frames_b, int pixel_type,
               const double* up, const double* vp, double deforming_par, int deforming_order,
               const float* coef_a, const float* coef_b, const uint8_t* frame_mask, int dtype, void* out_a,
               void* out_b, void* stream);

/* Cubic B-spline interpolation coefficients of n_frames frames (mirror
 * boundary), float32 device [n_frames][H][W]. */
int piv_spline_prefilter(int height, int width, int n_frames, const void* frames, int pixel_type, float* coef,
                         void* stream);

/* Validation (ValidationGPU.__call__, gpu_validation.py:80-121) of n_pairs
 * field pairs. fp32 != 0 evaluates the tests in float32 like the reference does
 * before the first smoothing. field_mask/val_mask (device [m][n] and
 * [n_pairs][m][n]) may be NULL; a nonzero val_mask entry excludes the point
 * like the reference's `mask` argument. s2n may be NULL. */
int piv_validate(int m, int n, int n_pairs, const double* u, const double* v, const void* s2n, int s2n_dtype,
                 int size, double s2n_tol, double median_tol, double mad_tol, double mean_tol, double rms_tol,
                 const uint8_t* field_mask, const uint8_t* exclude, int fp32, uint8_t* val, void* stream);

/* Outlier replacement loop (PIVGPU.replace_outliers, gpu_process.py:788-834,
 * with ReplacementGPU, gpu_validation.py:245-415) in place on u/v; `val` is the
 * initial outlier mask and receives the final one. Validation settings are the
 * ones used for revalidation. */
int piv_replace(int m, int n, int n_pairs, double* u, double* v, uint8_t* val, const uint8_t* field_mask,
                int n_iters, int method, int size, int revalidate, const void* s2n, int s2n_dtype,
                int val_size, double s2n_tol, double median_tol, double mad_tol, double mean_tol, double rms_tol,
                int fp32, int dtype, void* stream);

/* smoothn of the two fields of each pair (SmoothnGPU(f_shape, mask, s)(u, v),
 * gpu_smoothn.py:123-231, non-robust, order 2) in float64, in place. s <= 0 or
 * NaN selects GCV. p_out (device [n_pairs], may be NULL) receives log10(s). */
int piv_smoothn(int m, int n, int n_pairs, double* u, double* v, const uint8_t* field_mask, double s,
                double* p_out, void* stream);

/* piv_smoothn that also writes, per pair, the PIV_SMOOTH_* flags behind
 * SmoothnGPU's log messages (gpu_smoothn.py:218-222, 429-439) to flags_out
 * (device [n_pairs]). */
int piv_smoothn_flags(int m, int n, int n_pairs, double* u, double* v, const uint8_t* field_mask, double s,
                      double* p_out, int* flags_out, void* stream);

/* piv_smoothn for callers that cannot allocate device memory while they run
 * (a fixed memory budget handed over at start-up, a real-time loop that must
 * not wait on the allocator, a host framework that owns every allocation).
 * No counterpart in the reference. Same arguments and results as
 * piv_smoothn, but the scratch is a fixed 4 MiB device array inside the
 * library (for example 4 pairs of 128 x 128 fields, or 2 pairs of 127 x 127
 * fields with a field mask, whose weighted iteration keeps more per pair);
 * larger requests, and shapes beyond 2^31 elements or 65535 pairs, fail with
 * PIV_E_ARG and a message. It calls no allocator. Each call made outside
 * stream capture looks up the array's device address in the current context
 * (so calls after a device reset use the reloaded array); a call made while
 * `stream` is being captured reuses the address of the device's last
 * uncaptured call, so make the first call on a device (and the first after a
 * device reset) before any stream capture. Calls share the array and find it
 * holding the previous call's contents: calls that overlap on the GPU (other
 * streams, other threads) race and must be serialised by the caller. */
int piv_smoothn_noalloc(int m, int n, int n_pairs, double* u, double* v, const uint8_t* field_mask, double s,
                        double* p_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PIV_GB300_H */
