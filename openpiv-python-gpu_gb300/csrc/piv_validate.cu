// Outlier validation and replacement on the device.
//
// Validation restates ValidationGPU (gpu_validation.py:80-243): local median,
// MAD and mean of the (2s+1)^2 neighbourhood without its centre (NaN padding
// and NaN values skipped), global mean/std for the RMS test, S2N threshold;
// the selected tests are OR-ed, then points excluded by the mask are cleared.
// Comparisons use strict '>' (or '<' for S2N) like the reference.
//
// Replacement restates PIVGPU.replace_outliers (gpu_process.py:788-834) and
// ReplacementGPU (gpu_validation.py:245-415) with one CTA per field pair:
// spring (the reference builds a sparse linear system and calls spsolve; here
// the same system, scaled to its symmetric form, is solved by conjugate
// gradients in float64), local median or local mean replacement, optional
// revalidation of the replaced points, and reset of unresolved points.
//
// `fp32` selects float32 arithmetic, which the reference uses for fields that
// have not been through smoothn yet (dtype_f float32, first iteration); the
// field arrays are float64 throughout and hold float32 values in that mode.
#include <math.h>

#include "piv_common.cuh"
#include "piv_internal.h"

namespace piv {

static constexpr int kMaxKernel = 7;                       // validation/replacement size <= 3
static constexpr int kMaxNbrs = kMaxKernel * kMaxKernel;   // values incl. centre

template <typename T>
PIV_D void sort_small(T* a, int n) {
  for (int i = 1; i < n; ++i) {
    T v = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > v) { a[j + 1] = a[j]; --j; }
    a[j + 1] = v;
  }
}

// nanmedian of n finite values (sorted in place): middle value, or the mean of
// the two middle values as (lo + hi) / 2 (numpy.ma.median); NaN when n == 0.
template <typename T>
PIV_D T median_of(T* a, int n) {
  if (n == 0) return (T)NAN;
  sort_small(a, n);
  const T lo = a[(n - 1) / 2], hi = a[n / 2];
  return mul_rn(add_rn(lo, hi), (T)0.5);  // exact: the same value as the division by 2
}

// numpy's pairwise summation (n <= 128 branch) of n values.
template <typename T>
PIV_D T pairwise_sum(const T* a, int n) {
  if (n < 8) {
    T r = (T)0;
    for (int i = 0; i < n; ++i) r = add_rn(r, a[i]);
    return r;
  }
  T r[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) r[j] = a[j];
  int i = 8;
  for (; i < n - (n % 8); i += 8) {
#pragma unroll
    for (int j = 0; j < 8; ++j) r[j] = add_rn(r[j], a[i + j]);
  }
  T res = add_rn(add_rn(add_rn(r[0], r[1]), add_rn(r[2], r[3])), add_rn(add_rn(r[4], r[5]), add_rn(r[6], r[7])));
  for (; i < n; ++i) res = add_rn(res, a[i]);
  return res;
}

template <typename T>
PIV_D T as_t(double v) { return (T)v; }

// Field value at (i, j) with NaN outside the field; `sub` replaces the value at
// points flagged in `subst` (outliers) by `sub_val` when non-null.
struct FieldView {
  const double* f;
  int m, n;
  const uint8_t* subst;  // may be null
  double sub_val;        // NaN or 0
};

template <typename T>
PIV_D T fv_at(const FieldView& v, int i, int j) {
  if (i < 0 || i >= v.m || j < 0 || j >= v.n) return (T)NAN;
  const int p = i * v.n + j;
  if (v.subst && v.subst[p]) return (T)v.sub_val;
  return (T)v.f[p];
}

// Order-preserving integer keys: signed comparison of the keys orders the
// values like the floating-point comparison (-0 sorts below +0). The sorting
// network then runs on the integer ALUs; float64 min/max are slow here.
PIV_D int sort_key(float v) {
  const int b = __float_as_int(v);
  return b ^ ((b >> 31) & 0x7fffffff);
}
PIV_D long long sort_key(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
PIV_D float key_value(int k) { return __int_as_float(k ^ ((k >> 31) & 0x7fffffff)); }
PIV_D double key_value(long long k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL)); }

// Median (kind 0) or MAD (kind 2, |v - med|) of the eight neighbours of (i, j)
// in registers: missing values sort last as +inf, a 19-comparator network
// (Batcher's odd-even merge) sorts their keys, and the middle pair of the cnt
// valid values is picked by selects. Same result as median_of on the valid
// values.
template <typename T>
PIV_D T median8(const FieldView& fv, int i, int j, int kind, T med) {
  using K = decltype(sort_key(T(0)));
  K a[8];
  int cnt = 0, k = 0;
#pragma unroll
  for (int di = -1; di <= 1; ++di)
#pragma unroll
    for (int dj = -1; dj <= 1; ++dj) {
      if (di == 0 && dj == 0) continue;
      T v = fv_at<T>(fv, i + di, j + dj);
      const bool ok = !is_nan(v);
      if (kind == 2) v = fabs(sub_rn(v, med));
      a[k++] = sort_key(ok ? v : (T)INFINITY);
      cnt += ok ? 1 : 0;
    }
  auto cx = [&](int x, int y) {
    const K lo = min(a[x], a[y]), hi = max(a[x], a[y]);
    a[x] = lo;
    a[y] = hi;
  };
  cx(0, 1); cx(2, 3); cx(4, 5); cx(6, 7);
  cx(0, 2); cx(1, 3); cx(4, 6); cx(5, 7);
  cx(1, 2); cx(5, 6);
  cx(0, 4); cx(1, 5); cx(2, 6); cx(3, 7);
  cx(2, 4); cx(3, 5);
  cx(1, 2); cx(3, 4); cx(5, 6);
  if (cnt == 0) return (T)NAN;
  const int il = (cnt - 1) / 2, ih = cnt / 2;
  K lo = a[0], hi = a[0];
#pragma unroll
  for (int q = 1; q < 8; ++q) {
    lo = il == q ? a[q] : lo;
    hi = ih == q ? a[q] : hi;
  }
  return mul_rn(add_rn(key_value(lo), key_value(hi)), (T)0.5);  // exact: the same value as the division by 2
}

// Neighbourhood statistics at (i, j): kind 0 median, 1 mean, 2 MAD (needs med).
template <typename T>
PIV_D T nbr_stat(const FieldView& fv, int i, int j, int s, int kind, T med) {
  if (s == 1 && kind != 1) return median8<T>(fv, i, j, kind, med);
  T vals[kMaxNbrs];
  const int k = 2 * s + 1;
  if (kind == 1) {
    // nanmean over the whole (2s+1)^2 kernel with the centre NaN: pairwise sum
    // of the kernel in row-major order with NaN -> 0, divided by the count.
    int cnt = 0;
    for (int di = 0; di < k; ++di)
      for (int dj = 0; dj < k; ++dj) {
        T v = (di == s && dj == s) ? (T)NAN : fv_at<T>(fv, i + di - s, j + dj - s);
        if (is_nan(v)) v = (T)0; else ++cnt;
        vals[di * k + dj] = v;
      }
    const T sum = pairwise_sum(vals, k * k);
    return cnt ? div_rn(sum, (T)cnt) : (T)NAN;
  }
  int cnt = 0;
  for (int di = -s; di <= s; ++di)
    for (int dj = -s; dj <= s; ++dj) {
      if (di == 0 && dj == 0) continue;
      T v = fv_at<T>(fv, i + di, j + dj);
      if (is_nan(v)) continue;
      vals[cnt++] = kind == 2 ? fabs(sub_rn(v, med)) : v;
    }
  return median_of(vals, cnt);
}

struct ValSettings {
  int size;
  double s2n_tol, median_tol, mad_tol, mean_tol, rms_tol;
  int fp32;
  const void* s2n;
  int s2n_dtype;
};

// Outlier test of point p of one pair. rms: {mean_u, std_u, mean_v, std_v}.
template <typename T>
PIV_D bool point_invalid(const ValSettings& s, const FieldView& fu, const FieldView& fv, long long s2n_index, int i,
                         int j, const double* rms) {
  const int p = i * fu.n + j;
  const T u = (T)fu.f[p], v = (T)fv.f[p];
  bool out = false;
  if (!isnan(s.s2n_tol) && s.s2n) {
    if (s.s2n_dtype == PIV_DTYPE_F64) out |= ((const double*)s.s2n)[s2n_index] < s.s2n_tol;
    else out |= ((const float*)s.s2n)[s2n_index] < (float)s.s2n_tol;
  }
  T mu = (T)NAN, mv = (T)NAN;
  const bool need_med = !isnan(s.median_tol) || !isnan(s.mad_tol);
  if (need_med) {
    mu = nbr_stat<T>(fu, i, j, s.size, 0, (T)0);
    mv = nbr_stat<T>(fv, i, j, s.size, 0, (T)0);
  }
  if (!isnan(s.median_tol)) {
    const T tol = (T)s.median_tol;
    out |= fabs(sub_rn(u, mu)) > tol || fabs(sub_rn(v, mv)) > tol;
  }
  if (!isnan(s.mad_tol)) {
    const T tol = (T)s.mad_tol;
    const T du = nbr_stat<T>(fu, i, j, s.size, 2, mu), dv = nbr_stat<T>(fv, i, j, s.size, 2, mv);
    out |= fabs(sub_rn(u, mu)) > mul_rn(tol, du) || fabs(sub_rn(v, mv)) > mul_rn(tol, dv);
  }
  if (!isnan(s.mean_tol)) {
    const T tol = (T)s.mean_tol;
    const T au = nbr_stat<T>(fu, i, j, s.size, 1, (T)0), av = nbr_stat<T>(fv, i, j, s.size, 1, (T)0);
    out |= fabs(sub_rn(u, au)) > tol || fabs(sub_rn(v, av)) > tol;
  }
  if (!isnan(s.rms_tol) && rms) {
    const T tol = (T)s.rms_tol;
    out |= fabs(sub_rn(u, (T)rms[0])) > mul_rn(tol, (T)rms[1]) || fabs(sub_rn(v, (T)rms[2])) > mul_rn(tol, (T)rms[3]);
  }
  return out;
}

// Per-pair nanmean / nanstd of u and v (RMS test), one CTA per pair.
template <typename T>
__global__ void k_field_stats(int m, int n, const double* __restrict__ u, const double* __restrict__ v, double* out) {
  __shared__ double red[3][32];
  const int pair = blockIdx.x;
  const long long off = (long long)pair * m * n;
  for (int f = 0; f < 2; ++f) {
    const double* x = (f == 0 ? u : v) + off;
    T s = 0;
    int c = 0;
    for (int p = threadIdx.x; p < m * n; p += blockDim.x) {
      const T val = (T)x[p];
      if (!is_nan(val)) { s += val; ++c; }
    }
    for (int o = 16; o > 0; o >>= 1) { s += __shfl_xor_sync(~0u, s, o); c += __shfl_xor_sync(~0u, c, o); }
    if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = (double)s; red[1][threadIdx.x >> 5] = c; }
    __syncthreads();
    __shared__ double mean_s, cnt_s;
    if (threadIdx.x == 0) {
      T ts = 0;
      double tc = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { ts += (T)red[0][w]; tc += red[1][w]; }
      mean_s = tc > 0 ? (double)(ts / (T)tc) : NAN;
      cnt_s = tc;
    }
    __syncthreads();
    const T mean = (T)mean_s;
    T q = 0;
    for (int p = threadIdx.x; p < m * n; p += blockDim.x) {
      const T val = (T)x[p];
      if (!is_nan(val)) { const T d = val - mean; q += d * d; }
    }
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(~0u, q, o);
    if ((threadIdx.x & 31) == 0) red[2][threadIdx.x >> 5] = (double)q;
    __syncthreads();
    if (threadIdx.x == 0) {
      T tq = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tq += (T)red[2][w];
      out[pair * 4 + 2 * f] = mean_s;
      out[pair * 4 + 2 * f + 1] = cnt_s > 0 ? (double)sqrt(tq / (T)cnt_s) : NAN;
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void k_validate(ValArgs a, uint8_t* __restrict__ val, const double* __restrict__ rms) {
  const long long npts = (long long)a.m * a.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * a.n_pairs) return;
  const int pair = (int)(t / npts);
  const int p = (int)(t % npts);
  if ((a.field_mask && a.field_mask[p]) || (a.exclude && a.exclude[t])) {
    val[t] = 0;
    return;
  }
  const long long off = (long long)pair * npts;
  FieldView fu{a.u + off, a.m, a.n, nullptr, 0.0}, fv{a.v + off, a.m, a.n, nullptr, 0.0};
  ValSettings s{a.size, a.s2n_tol, a.median_tol, a.mad_tol, a.mean_tol, a.rms_tol, a.fp32, a.s2n, a.s2n_dtype};
  val[t] = point_invalid<T>(s, fu, fv, t, p / a.n, p % a.n, rms ? rms + pair * 4 : nullptr) ? 1 : 0;
}

int validate(const ValArgs& a, uint8_t* val, double* rms_stats, cudaStream_t stream) {
  if (a.size > 3 || a.size < 1) return set_error(PIV_E_UNSUPPORTED, "validation_size %d (supported: 1..3)", a.size);
  const long long total = (long long)a.m * a.n * a.n_pairs;
  if (total == 0) return PIV_OK;
  const double* rms = nullptr;
  if (!isnan(a.rms_tol)) {
    if (!rms_stats) return set_error(PIV_E_ARG, "RMS validation needs a statistics buffer");
    if (a.fp32) k_field_stats<float><<<a.n_pairs, 256, 0, stream>>>(a.m, a.n, a.u, a.v, rms_stats);
    else k_field_stats<double><<<a.n_pairs, 256, 0, stream>>>(a.m, a.n, a.u, a.v, rms_stats);
    rms = rms_stats;
  }
  const int bs = 128;
  const unsigned grid = (unsigned)((total + bs - 1) / bs);
  if (a.fp32) k_validate<float><<<grid, bs, 0, stream>>>(a, val, rms);
  else k_validate<double><<<grid, bs, 0, stream>>>(a, val, rms);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_validate launch");
}

// ---------------------------------------------------------------------------
// Field combination u = u_corr (+ up).
// ---------------------------------------------------------------------------
__global__ void k_combine(long long count, const void* uc, const void* vc, int corr_dtype, const double* up,
                          const double* vp, double* u, double* v) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  double a, b;
  if (corr_dtype == PIV_DTYPE_F64) { a = ((const double*)uc)[t]; b = ((const double*)vc)[t]; }
  else { a = (double)((const float*)uc)[t]; b = (double)((const float*)vc)[t]; }
  if (up) { a = __dadd_rn(a, up[t]); b = __dadd_rn(b, vp[t]); }
  u[t] = a;
  v[t] = b;
}

int combine_fields(int count, const void* u_corr, const void* v_corr, int corr_dtype, const double* up,
                   const double* vp, int fp32, double* u, double* v, cudaStream_t stream) {
  (void)fp32;
  if (count == 0) return PIV_OK;
  k_combine<<<(count + 255) / 256, 256, 0, stream>>>(count, u_corr, v_corr, corr_dtype, up, vp, u, v);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_combine launch");
}

// (u * scaling) / dt in the field's float type.
__global__ void k_scale(long long count, const double* u, const double* v, double scaling, double dt, int fp32,
                        double* uo, double* vo) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  if (fp32) {
    uo[t] = (double)__fdiv_rn(__fmul_rn((float)u[t], (float)scaling), (float)dt);
    vo[t] = (double)__fdiv_rn(__fmul_rn((float)v[t], (float)scaling), (float)dt);
  } else {
    uo[t] = __ddiv_rn(__dmul_rn(u[t], scaling), dt);
    vo[t] = __ddiv_rn(__dmul_rn(v[t], scaling), dt);
  }
}

int scale_fields(int count, const double* u, const double* v, double scaling, double dt, int fp32, double* uo,
                 double* vo, cudaStream_t stream) {
  if (count == 0) return PIV_OK;
  k_scale<<<(count + 255) / 256, 256, 0, stream>>>(count, u, v, scaling, dt, fp32, uo, vo);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_scale launch");
}

// ---------------------------------------------------------------------------
// Replacement: one CTA per pair.
// ---------------------------------------------------------------------------
static constexpr int kRepThreads = 512;
static constexpr int kCgMaxIters = 20000;
// Up to kCgSmall outliers per pair, the conjugate-gradient vectors stay in
// registers (kCgPer per thread) and the search direction in shared memory.
static constexpr int kCgPer = 4;
static constexpr int kCgSmall = kRepThreads * kCgPer;

struct RepScratch {
  double* init_u;   // [mn]
  double* init_v;
  double* new_u;    // [mn] replacement values by outlier rank
  double* new_v;
  double* cg;       // 8 * [mn]: x_u, x_v, r_u, r_v, p_u, p_v, q_u, q_v
  double* dinv;     // [mn] spring row scale 1/c_r by outlier rank
  int* nbr;         // 4 * [mn] outlier ranks of the linked neighbours (-1: none)
  int* list;        // [mn] outlier positions
  int* rank;        // [mn] position -> outlier rank or -1
  uint8_t* flag;    // [mn] anchored / scratch flags
  uint8_t* val2;    // [mn] next validation mask
};

// Bytes of one pair's replacement scratch, rounded up to 256 so that every
// pair's block (and the doubles at its start) stays aligned.
PIV_HD size_t rep_scratch_stride(size_t mn) {
  return ((mn * (13 * sizeof(double) + 6 * sizeof(int) + 2) + 255) / 256) * 256;
}

size_t replace_scratch_bytes(int m, int n, int n_pairs) {
  return rep_scratch_stride((size_t)m * n) * (size_t)n_pairs;
}

static __device__ RepScratch rep_scratch(void* base, int mn, int pair) {
  char* p = (char*)base + rep_scratch_stride((size_t)mn) * pair;
  RepScratch s;
  s.init_u = (double*)p; p += mn * sizeof(double);
  s.init_v = (double*)p; p += mn * sizeof(double);
  s.new_u = (double*)p; p += mn * sizeof(double);
  s.new_v = (double*)p; p += mn * sizeof(double);
  s.cg = (double*)p; p += 8 * (size_t)mn * sizeof(double);
  s.dinv = (double*)p; p += mn * sizeof(double);
  s.nbr = (int*)p; p += 4 * (size_t)mn * sizeof(int);
  s.list = (int*)p; p += mn * sizeof(int);
  s.rank = (int*)p; p += mn * sizeof(int);
  s.flag = (uint8_t*)p; p += mn;
  s.val2 = (uint8_t*)p;
  return s;
}

// Block-wide sum of a double (all threads get the result).
PIV_D double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = 0;
  for (int k = 0; k < nw; ++k) t += red[k];
  return t;
}

// Block-wide sums of two doubles in one reduction (all threads get both). The
// warps' partial sums are combined by a shuffle tree rather than a serial
// chain: the conjugate-gradient loop waits on this twice per iteration.
PIV_D double2 block_sum2(double a, double b, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(~0u, a, o);
    b += __shfl_xor_sync(~0u, b, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) { red[w] = a; red[32 + w] = b; }
  __syncthreads();
  double ta = l < nw ? red[l] : 0.0, tb = l < nw ? red[32 + l] : 0.0;
  for (int o = 16; o > 0; o >>= 1) {
    ta += __shfl_xor_sync(~0u, ta, o);
    tb += __shfl_xor_sync(~0u, tb, o);
  }
  return make_double2(ta, tb);
}

// The first nwa warps of the block: a named barrier (id 1) among them, and
// sums of two doubles over them (every thread of the group gets both). With
// one warp the shuffle tree alone suffices. Float64 throughput on this GPU is
// a small fraction of float32, so work that only the warps holding data need
// is kept off the others.
PIV_D void group_bar(int nwa) {
  if (nwa == 1) __syncwarp();
  else asm volatile("bar.sync 1, %0;" ::"r"(nwa * 32) : "memory");
}

PIV_D double2 group_sum2(double a, double b, double* red, int nwa) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(~0u, a, o);
    b += __shfl_xor_sync(~0u, b, o);
  }
  if (nwa == 1) return make_double2(a, b);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { red[w] = a; red[32 + w] = b; }
  group_bar(nwa);
  double ta = l < nwa ? red[l] : 0.0, tb = l < nwa ? red[32 + l] : 0.0;
  for (int o = 16; o > 0; o >>= 1) {
    ta += __shfl_xor_sync(~0u, ta, o);
    tb += __shfl_xor_sync(~0u, tb, o);
  }
  group_bar(nwa);  // red is rewritten by the next call
  return make_double2(ta, tb);
}

PIV_D int block_count(int v, int* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  int t = 0;
  for (int k = 0; k < nw; ++k) t += red[k];
  return t;
}

// Stable compaction of the flagged positions into list (ascending), returns
// count; rank[p] = position in list, or -1. Each thread takes a contiguous
// range of the field, so one block-wide scan of the per-thread counts places
// every range (three barriers in all, whatever the field size).
PIV_D int block_compact(const uint8_t* flags, int mn, int* list, int* rank, int* red) {
  const int nt = blockDim.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = nt >> 5;
  const int per = (mn + nt - 1) / nt, p0 = tid * per, p1 = min(mn, p0 + per);
  int c = 0;
  for (int p = p0; p < p1; ++p) c += flags[p] ? 1 : 0;
  int x = c;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(~0u, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) red[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < nw ? red[lane] : 0, ts = t;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(~0u, ts, o);
      if (lane >= o) ts += y;
    }
    if (lane < nw) red[lane] = ts - t;  // exclusive prefix of the warps
    if (lane == 31) red[nw] = ts;       // total (nw <= 32)
  }
  __syncthreads();
  int pos = red[w] + x - c;
  for (int p = p0; p < p1; ++p) {
    if (flags[p]) { list[pos] = p; rank[p] = pos; ++pos; }
    else rank[p] = -1;
  }
  const int total = red[nw];
  __syncthreads();  // red is reused by the caller
  return total;
}

// Coefficient magnitude 1/n_r of the spring link (gpu_validation.py:365-371),
// rounded to the link matrix dtype.
PIV_D double spring_coef(int i, int j, int m, int n, int s, int dtype) {
  const bool ei = i < s || i >= m - s, ej = j < s || j >= n - s;
  double c = (ei && ej) ? 0.5 : ((ei || ej) ? 1.0 / 3.0 : 0.25);
  if (dtype == PIV_DTYPE_F32) c = (double)(float)c;
  return c;
}

// Spring right-hand side: mean over the four linked neighbours at distance s,
// outliers counted as 0, NaN and out-of-field ignored (gpu_validation.py:381-394).
template <typename T>
PIV_D T spring_rhs(const FieldView& fv, int i, int j, int s) {
  const int k = 2 * s + 1;
  T vals[kMaxNbrs];
  int cnt = 0;
  for (int q = 0; q < k * k; ++q) vals[q] = (T)0;
  const int di[4] = {0, s, s, 2 * s}, dj[4] = {s, 0, 2 * s, s};  // top, left, right, bottom (row-major)
  for (int e = 0; e < 4; ++e) {
    T v = fv_at<T>(fv, i + di[e] - s, j + dj[e] - s);
    if (!is_nan(v)) { vals[di[e] * k + dj[e]] = v; ++cnt; }
  }
  const T sum = pairwise_sum(vals, k * k);
  return cnt ? div_rn(sum, (T)cnt) : (T)NAN;
}

template <typename T>
__global__ void __launch_bounds__(kRepThreads) k_replace(RepArgs a, int* status) {
  __shared__ double red_d[64];
  __shared__ double cg_pu[kCgSmall], cg_pv[kCgSmall];
  __shared__ int red_i[40];
  const int pair = blockIdx.x;
  const int m = a.val.m, n = a.val.n, mn = m * n;
  const long long off = (long long)pair * mn;
  double* u = a.u + off;
  double* v = a.v + off;
  uint8_t* val = a.val_mask + off;
  const uint8_t* fmask = a.val.field_mask;
  RepScratch sc = rep_scratch(a.scratch, mn, pair);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int s = a.size;

  int cnt = 0;
  for (int p = tid; p < mn; p += nt) cnt += val[p] ? 1 : 0;
  cnt = block_count(cnt, red_i);
  if (cnt == 0 || a.n_iters == 0) return;
  for (int p = tid; p < mn; p += nt) { sc.init_u[p] = u[p]; sc.init_v[p] = v[p]; }
  __syncthreads();

  bool fill_nan = true;
  ValSettings vs{a.val.size, a.val.s2n_tol, a.val.median_tol, a.val.mad_tol, a.val.mean_tol, a.val.rms_tol,
                 a.val.fp32, a.val.s2n, a.val.s2n_dtype};
  for (int it = 0; it < a.n_iters; ++it) {
    const int nv = block_compact(val, mn, sc.list, sc.rank, red_i);
    if (nv == 0) break;
    // 1. Replacement values from the current fields.
    if (a.method == PIV_REPLACE_SPRING && nv <= kCgSmall) {
      // Conjugate gradients on (D - Adj) x = D rhs for both fields, run by the
      // nwa warps that hold outliers (outlier r = tid + k nt in registers, the
      // search direction p in shared memory); the other warps wait at the
      // block barrier below.
      const int nwa = min(nt >> 5, (nv + 31) >> 5);
      if ((tid >> 5) < nwa) {
        FieldView fu{u, m, n, val, 0.0}, fv{v, m, n, val, 0.0};
        double xu[kCgPer], xv[kCgPer], ru[kCgPer], rv[kCgPer], dd[kCgPer];
        int nb[kCgPer][4];
        double rr_u = 0, rr_v = 0;
#pragma unroll
        for (int k = 0; k < kCgPer; ++k) {
          const int r = tid + k * nt;
          xu[k] = xv[k] = ru[k] = rv[k] = dd[k] = 0;
          nb[k][0] = nb[k][1] = nb[k][2] = nb[k][3] = -1;
          if (r < nv) {
            const int p = sc.list[r], i = p / n, j = p % n;
            dd[k] = 1.0 / spring_coef(i, j, m, n, s, a.dtype);
            ru[k] = dd[k] * (double)spring_rhs<T>(fu, i, j, s);
            rv[k] = dd[k] * (double)spring_rhs<T>(fv, i, j, s);
            const int oi[4] = {-s, 0, 0, s}, oj[4] = {0, -s, s, 0};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const int ii = i + oi[e], jj = j + oj[e];
              nb[k][e] = (ii < 0 || ii >= m || jj < 0 || jj >= n) ? -1 : sc.rank[ii * n + jj];
            }
            cg_pu[r] = ru[k];
            cg_pv[r] = rv[k];
            rr_u += ru[k] * ru[k];
            rr_v += rv[k] * rv[k];
          }
        }
        group_bar(nwa);  // publishes cg_pu / cg_pv
        const double2 rr = group_sum2(rr_u, rr_v, red_d, nwa);
        rr_u = rr.x;
        rr_v = rr.y;
        const double tol_u = rr_u * 1e-28, tol_v = rr_v * 1e-28;
        bool done_u = rr_u <= tol_u || rr_u == 0, done_v = rr_v <= tol_v || rr_v == 0;
        int iter = 0;
        for (; iter < kCgMaxIters && !(done_u && done_v); ++iter) {
          double qu[kCgPer], qv[kCgPer], pq_u = 0, pq_v = 0;
#pragma unroll
          for (int k = 0; k < kCgPer; ++k) {
            const int r = tid + k * nt;
            qu[k] = qv[k] = 0;
            if (r < nv) {
              double au = dd[k] * cg_pu[r], av = dd[k] * cg_pv[r];
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const int q = nb[k][e];
                if (q >= 0) { au -= cg_pu[q]; av -= cg_pv[q]; }
              }
              qu[k] = au; qv[k] = av;
              pq_u += cg_pu[r] * au; pq_v += cg_pv[r] * av;
            }
          }
          const double2 pq = group_sum2(pq_u, pq_v, red_d, nwa);
          const double al_u = done_u ? 0.0 : rr_u / pq.x, al_v = done_v ? 0.0 : rr_v / pq.y;
          double nr_u = 0, nr_v = 0;
#pragma unroll
          for (int k = 0; k < kCgPer; ++k) {
            const int r = tid + k * nt;
            if (r < nv) {
              xu[k] += al_u * cg_pu[r]; xv[k] += al_v * cg_pv[r];
              ru[k] -= al_u * qu[k]; rv[k] -= al_v * qv[k];
              nr_u += ru[k] * ru[k]; nr_v += rv[k] * rv[k];
            }
          }
          const double2 nr = group_sum2(nr_u, nr_v, red_d, nwa);
          const double be_u = done_u ? 0.0 : nr.x / rr_u, be_v = done_v ? 0.0 : nr.y / rr_v;
          group_bar(nwa);  // every read of p in this iteration is done
#pragma unroll
          for (int k = 0; k < kCgPer; ++k) {
            const int r = tid + k * nt;
            if (r < nv) {
              if (!done_u) cg_pu[r] = ru[k] + be_u * cg_pu[r];
              if (!done_v) cg_pv[r] = rv[k] + be_v * cg_pv[r];
            }
          }
          rr_u = nr.x; rr_v = nr.y;
          done_u = done_u || rr_u <= tol_u;
          done_v = done_v || rr_v <= tol_v;
          group_bar(nwa);  // the new p is visible to the next product
        }
        if (iter >= kCgMaxIters && tid == 0 && status) atomicExch(status, PIV_E_TIMEOUT);
#pragma unroll
        for (int k = 0; k < kCgPer; ++k) {
          const int r = tid + k * nt;
          if (r < nv) { sc.new_u[r] = xu[k]; sc.new_v[r] = xv[k]; }
        }
      }
    } else if (a.method == PIV_REPLACE_SPRING) {
      FieldView fu{u, m, n, val, 0.0}, fv{v, m, n, val, 0.0};
      double* xu = sc.cg;
      double* xv = sc.cg + mn;
      double* ru = sc.cg + 2 * mn;
      double* rv = sc.cg + 3 * mn;
      double* pu = sc.cg + 4 * mn;
      double* pv = sc.cg + 5 * mn;
      double* qu = sc.cg + 6 * mn;
      double* qv = sc.cg + 7 * mn;
      // Row scale d_r = 1/c_r. A cluster of outliers with no other neighbour
      // (only possible when every point is an outlier) has a zero right-hand
      // side; CG leaves it at zero, the minimum-norm solution that the
      // reference's direct solve returns for this singular case.
      for (int r = tid; r < nv; r += nt) {
        const int p = sc.list[r], i = p / n, j = p % n;
        const double d = 1.0 / spring_coef(i, j, m, n, s, a.dtype);
        const double bu = (double)spring_rhs<T>(fu, i, j, s), bv = (double)spring_rhs<T>(fv, i, j, s);
        const double b1 = d * bu, b2 = d * bv;
        xu[r] = 0; xv[r] = 0;
        ru[r] = b1; rv[r] = b2;
        pu[r] = b1; pv[r] = b2;
        // The row's coupling to the other outliers, resolved once for the
        // iterations: scale and neighbour ranks.
        sc.dinv[r] = d;
        const int oi[4] = {-s, 0, 0, s}, oj[4] = {0, -s, s, 0};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int ii = i + oi[e], jj = j + oj[e];
          sc.nbr[e * mn + r] = (ii < 0 || ii >= m || jj < 0 || jj >= n) ? -1 : sc.rank[ii * n + jj];
        }
      }
      __syncthreads();
      {
        // Conjugate gradients on (D - Adj) x = D rhs for both fields at once.
        double rr_u = 0, rr_v = 0;
        for (int r = tid; r < nv; r += nt) { rr_u += ru[r] * ru[r]; rr_v += rv[r] * rv[r]; }
        const double2 rr = block_sum2(rr_u, rr_v, red_d);
        rr_u = rr.x;
        rr_v = rr.y;
        const double tol_u = rr_u * 1e-28, tol_v = rr_v * 1e-28;
        bool done_u = rr_u <= tol_u || rr_u == 0, done_v = rr_v <= tol_v || rr_v == 0;
        int iter = 0;
        for (; iter < kCgMaxIters && !(done_u && done_v); ++iter) {
          // q = A p
          double pq_u = 0, pq_v = 0;
          for (int r = tid; r < nv; r += nt) {
            const double d = sc.dinv[r];
            double au = d * pu[r], av = d * pv[r];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const int k = sc.nbr[e * mn + r];
              if (k >= 0) { au -= pu[k]; av -= pv[k]; }
            }
            qu[r] = au; qv[r] = av;
            pq_u += pu[r] * au; pq_v += pv[r] * av;
          }
          const double2 pq = block_sum2(pq_u, pq_v, red_d);
          const double al_u = done_u ? 0.0 : rr_u / pq.x, al_v = done_v ? 0.0 : rr_v / pq.y;
          double nr_u = 0, nr_v = 0;
          for (int r = tid; r < nv; r += nt) {
            xu[r] += al_u * pu[r]; xv[r] += al_v * pv[r];
            ru[r] -= al_u * qu[r]; rv[r] -= al_v * qv[r];
            nr_u += ru[r] * ru[r]; nr_v += rv[r] * rv[r];
          }
          const double2 nr = block_sum2(nr_u, nr_v, red_d);
          const double be_u = done_u ? 0.0 : nr.x / rr_u, be_v = done_v ? 0.0 : nr.y / rr_v;
          for (int r = tid; r < nv; r += nt) {
            if (!done_u) pu[r] = ru[r] + be_u * pu[r];
            if (!done_v) pv[r] = rv[r] + be_v * pv[r];
          }
          rr_u = nr.x; rr_v = nr.y;
          done_u = done_u || rr_u <= tol_u;
          done_v = done_v || rr_v <= tol_v;
          __syncthreads();
        }
        if (iter >= kCgMaxIters && tid == 0 && status) atomicExch(status, PIV_E_TIMEOUT);
        for (int r = tid; r < nv; r += nt) { sc.new_u[r] = xu[r]; sc.new_v[r] = xv[r]; }
      }
    } else {
      const double fill = fill_nan ? NAN : 0.0;
      FieldView fu{u, m, n, fill_nan ? val : nullptr, fill}, fv{v, m, n, fill_nan ? val : nullptr, fill};
      const int kind = a.method == PIV_REPLACE_MEDIAN ? 0 : 1;
      for (int r = tid; r < nv; r += nt) {
        const int p = sc.list[r], i = p / n, j = p % n;
        sc.new_u[r] = (double)nbr_stat<T>(fu, i, j, s, kind, (T)0);
        sc.new_v[r] = (double)nbr_stat<T>(fv, i, j, s, kind, (T)0);
      }
    }
    __syncthreads();
    // 2. Write the replacements (rounded to the field type).
    for (int r = tid; r < nv; r += nt) {
      const int p = sc.list[r];
      u[p] = (double)(T)sc.new_u[r];
      v[p] = (double)(T)sc.new_v[r];
    }
    __syncthreads();
    if (a.revalidate) {
      // Reset unresolved points, then revalidate the replaced points only.
      for (int r = tid; r < nv; r += nt) {
        const int p = sc.list[r];
        const bool unres = isnan(u[p]) || isnan(v[p]);
        sc.flag[p] = unres ? 1 : 0;
        if (unres) { u[p] = sc.init_u[p]; v[p] = sc.init_v[p]; }
      }
      __syncthreads();
      FieldView fu{u, m, n, nullptr, 0.0}, fv{v, m, n, nullptr, 0.0};
      for (int p = tid; p < mn; p += nt) {
        uint8_t nvl = 0;
        if (val[p] && !(fmask && fmask[p])) {
          nvl = point_invalid<T>(vs, fu, fv, off + p, p / n, p % n, nullptr) ? 1 : 0;
          nvl |= sc.flag[p];
        } else if (val[p]) {
          nvl = sc.flag[p];
        }
        sc.val2[p] = nvl;
      }
      __syncthreads();
      for (int p = tid; p < mn; p += nt) val[p] = sc.val2[p];
      __syncthreads();
    } else {
      fill_nan = false;
    }
  }
  if (!a.revalidate) {
    for (int p = tid; p < mn; p += nt) {
      if (val[p] && (isnan(u[p]) || isnan(v[p]))) { u[p] = sc.init_u[p]; v[p] = sc.init_v[p]; }
    }
  }
}

int replace(const RepArgs& a, cudaStream_t stream) {
  if (a.size > 3 || a.size < 1) return set_error(PIV_E_UNSUPPORTED, "replacing_size %d (supported: 1..3)", a.size);
  if (a.val.size > 3 || a.val.size < 1)
    return set_error(PIV_E_UNSUPPORTED, "validation_size %d (supported: 1..3)", a.val.size);
  if (!isnan(a.val.rms_tol) && a.revalidate)
    return set_error(PIV_E_UNSUPPORTED, "revalidation with rms_tol is not implemented");
  if (a.val.n_pairs == 0 || a.val.m * a.val.n == 0 || a.n_iters == 0) return PIV_OK;
  if (a.val.fp32) k_replace<float><<<a.val.n_pairs, kRepThreads, 0, stream>>>(a, a.status);
  else k_replace<double><<<a.val.n_pairs, kRepThreads, 0, stream>>>(a, a.status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_replace launch");
}

}  // namespace piv
