// smoothn for the two displacement fields of each pair, as PIVGPU uses it
// (SmoothnGPU(f_shape, mask, s)(u, v), gpu_smoothn.py:123-231: non-robust,
// order 2, equal weights): z = IDCT2(gamma * DCT2(f)), gamma = 1/(1 + s lambda^2),
// lambda = 2 (2 - cos(pi i/m) - cos(pi j/n)) (gpu_smoothn.py:340-351), one s
// shared by u and v. With s unset, p = log10(s) minimises the GCV score
// (gpu_smoothn.py:353-372) over [p_min, p_max] (gpu_smoothn.py:320-338): a
// 10-point scan (gpu_smoothn.py:182-188) followed by a bounded local search
// from the best scan point that keeps the scan point when its projected
// finite-difference gradient is below 1e-5 (the stopping test of the
// reference's L-BFGS-B call, gpu_smoothn.py:191-193).
//
// The orthonormal DCT-II/III pairs are float64 matrix products with cosine
// matrices built on the device; the GCV search runs in one CTA per pair.
#include <math.h>

#include <mutex>

#include "piv_common.cuh"
#include "piv_internal.h"

namespace piv {

struct SmoothScratch {
  double* fd;    // [pairs][2][mn] DCT coefficients of u and v
  double* tmp;   // [pairs][2][mn]
  double* f2;    // [pairs][mn] fd_u^2 + fd_v^2
  double* cm;    // [m][m]
  double* cn;    // [n][n]
  double* lam2;  // [mn]
  double* p;     // [pairs]
  float* f2f;    // [pairs][mn] f2 in float32 (the GCV search's fast score)
  float* lam2f;  // [mn] lam2 in float32
  float* cmf;    // [2][m][m] cm as hi/lo floats (the DCT lines' double-float products)
  float* cnf;    // [2][n][n]
};

static size_t align_up(size_t v) { return (v + 255) / 256 * 256; }

// Per-pair block of the weighted path: f, z, t, fd, tmp (2 mn doubles each),
// w (mn doubles), the column-nearest table (mn ints) and the hi/lo float
// split of a DCT input (2 mn floats).
static size_t weighted_pair_bytes(size_t mn) { return align_up(11 * mn * 8 + mn * 4 + 2 * mn * 4); }
// The DCT matrices of the weighted path as hi/lo float pairs (2 (m^2 + n^2) floats).
static size_t weighted_matrix_bytes(int m, int n) { return align_up(2 * ((size_t)m * m + (size_t)n * n) * 4); }

size_t smoothn_scratch_bytes(int m, int n, int n_pairs) {
  const size_t mn = (size_t)m * n;
  const size_t shared = align_up((size_t)m * m * 8) + align_up((size_t)n * n * 8) + align_up(mn * 8) +
                        align_up((size_t)n_pairs * 8);
  const size_t plain = align_up(2 * mn * n_pairs * 8) * 2 + align_up(mn * n_pairs * 8) + shared +
                       align_up(mn * n_pairs * 4) + align_up(mn * 4) + align_up((size_t)m * m * 8) +
                       align_up((size_t)n * n * 8);
  const size_t weighted = shared + weighted_matrix_bytes(m, n) + weighted_pair_bytes(mn) * n_pairs;
  return plain > weighted ? plain : weighted;
}

static SmoothScratch carve(void* base, int m, int n, int n_pairs) {
  const size_t mn = (size_t)m * n;
  char* p = (char*)base;
  SmoothScratch s;
  s.fd = (double*)p; p += align_up(2 * mn * n_pairs * 8);
  s.tmp = (double*)p; p += align_up(2 * mn * n_pairs * 8);
  s.f2 = (double*)p; p += align_up(mn * n_pairs * 8);
  s.cm = (double*)p; p += align_up((size_t)m * m * 8);
  s.cn = (double*)p; p += align_up((size_t)n * n * 8);
  s.lam2 = (double*)p; p += align_up(mn * 8);
  s.p = (double*)p; p += align_up((size_t)n_pairs * 8);
  s.f2f = (float*)p; p += align_up(mn * n_pairs * 4);
  s.lam2f = (float*)p; p += align_up(mn * 4);
  s.cmf = (float*)p; p += align_up((size_t)m * m * 8);
  s.cnf = (float*)p;
  return s;
}

// Orthonormal DCT-II matrix C[k][i] = s_k cos(pi (2i+1) k / (2 len)).
__global__ void k_dct_matrix(int len, double* c) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= len * len) return;
  const int k = t / len, i = t % len;
  const double sk = k == 0 ? sqrt(1.0 / len) : sqrt(2.0 / len);
  c[t] = sk * cospi((double)((2 * i + 1) * k) / (2.0 * len));
}

// lambda^2 with lambda = 2 (2 - (cos(pi i/m) + cos(pi j/n))).
__global__ void k_lambda2(int m, int n, double* lam2, float* lam2f = nullptr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m * n) return;
  const int i = t / n, j = t % n;
  const double l = 2.0 * (2.0 - (cos(M_PI * i / m) + cos(M_PI * j / n)));
  lam2[t] = l * l;
  if (lam2f) lam2f[t] = (float)(l * l);
}

// out[b][i][l] = sum_j in[b][i][j] * c[l][j]       (transform along rows, mode 0)
// out[b][i][l] = sum_j in[b][i][j] * c[j][l]       (inverse along rows, mode 1)
// out[b][k][j] = sum_i c[k][i] * in[b][i][j]       (transform along columns, mode 2)
// out[b][k][j] = sum_i c[i][k] * in[b][i][j]       (inverse along columns, mode 3)
__global__ void k_dct_apply(int m, int n, int batch, int mode, const double* __restrict__ c,
                            const double* __restrict__ in, double* __restrict__ out) {
  const long long mn = (long long)m * n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= mn * batch) return;
  const int b = (int)(t / mn);
  const int e = (int)(t % mn);
  const int r = e / n, col = e % n;
  const double* x = in + b * mn;
  double acc = 0.0;
  if (mode == 0) {
    for (int j = 0; j < n; ++j) acc = fma(x[r * n + j], c[col * n + j], acc);
  } else if (mode == 1) {
    for (int j = 0; j < n; ++j) acc = fma(x[r * n + j], c[j * n + col], acc);
  } else if (mode == 2) {
    for (int i = 0; i < m; ++i) acc = fma(c[r * m + i], x[i * n + col], acc);
  } else {
    for (int i = 0; i < m; ++i) acc = fma(c[i * m + r], x[i * n + col], acc);
  }
  out[t] = acc;
}

// The orthonormal DCT-II matrix has C[k][L-1-i] = (-1)^k C[k][i], so along a
// line of length L the forward transform needs only the sums x[i] + x[L-1-i]
// (even k) or differences (odd k) of the first L/2 positions, and the inverse
// gives x[i] and x[L-1-i] from one pass over the even and the odd k: half the
// float64 multiply-adds of the plain product. One CTA takes 32 lines staged
// in shared memory as [position][line]; `cols` selects lines along the
// columns of the [m][n] fields (stride n) instead of along the rows.
// Lines up to 90 long keep the staging under the default 48 KB of shared memory.
// x -> (hi, lo) float pairs: hi = (float)x, lo = (float)(x - hi).
__global__ void k_split_f64(int count, const double* __restrict__ x, float* __restrict__ hi, float* __restrict__ lo) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const float h = (float)x[t];
  hi[t] = h;
  lo[t] = (float)(x[t] - (double)h);
}

// Dot product of two hi/lo float vectors in float32 with error-free
// transformations: every product's rounding error is kept (fma), the cross
// terms a_hi b_lo + a_lo b_hi join a small-term sum, and the main sum is
// compensated (TwoSum). The result, (hi, lo), is within ~1e-13 of the float64
// dot product here (orthonormal cosine matrices, smooth fields), at a fraction
// of the cost of float64 FMAs on this GPU.
struct DfAcc {
  float s = 0.f, c = 0.f;
  PIV_D void add(float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    c += fmaf(ah, bh, -p) + fmaf(ah, bl, al * bh);
    const float t = s + p, bp = t - s;
    c += (s - (t - bp)) + (p - bp);
    s = t;
  }
  PIV_D void result(float& hi, float& lo) const {
    hi = s + c;
    lo = c - (hi - s);
  }
};

static constexpr int kDctLines = 32, kDctThreads = 256, kDctMaxLen = 90;

// DCT-II (or, INV, DCT-III) of kDctLines lines per CTA with the symmetric
// split of the cosine matrix (half the products). The products are
// double-float (DfAcc: hi/lo float pairs with error-free transformations,
// within ~1e-13 of float64); cf holds the matrix as [2][L][L] hi/lo floats.
template <bool INV>
__global__ void __launch_bounds__(kDctThreads) k_dct_lines(int m, int n, int batch, int cols, const float* __restrict__ cf,
                                                           const double* __restrict__ in, double* __restrict__ out) {
  extern __shared__ double dsm[];
  const int L = cols ? m : n;
  const long long mn = (long long)m * n;
  const long long n_lines = (long long)batch * (cols ? n : m);
  const long long l0 = (long long)blockIdx.x * kDctLines;
  constexpr int S = kDctLines + 1;           // odd stride: conflict-free rows of 32 lines
  double* xs = dsm;                          // [L][S] doubles
  const int h = L / 2, hc = (L + 1) / 2;
  float* fs = reinterpret_cast<float*>(dsm + L * S);  // 4 hc S floats after xs
  const float* ch = cf;
  const float* cl = cf + (size_t)L * L;
  auto addr = [&](long long line, int e) -> long long {
    if (cols) {
      const long long f = line / n, col = line % n;
      return f * mn + (long long)e * n + col;
    }
    return line * n + e;
  };
  // Load: coalesced along the line for rows, across lines for columns.
  for (int idx = threadIdx.x; idx < kDctLines * L; idx += kDctThreads) {
    int e, l;
    if (cols) { e = idx / kDctLines; l = idx % kDctLines; }
    else { l = idx / L; e = idx % L; }
    const long long line = l0 + l;
    xs[e * S + l] = line < n_lines ? in[addr(line, e)] : 0.0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kDctThreads / 32;
  auto split = [](double x, float& hi, float& lo) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
  };
  if (!INV) {
    // Sums and differences of mirrored inputs, as hi/lo floats.
    float* esh = fs;
    float* esl = fs + hc * S;
    float* osh = fs + 2 * hc * S;
    float* osl = fs + 3 * hc * S;
    for (int i = warp; i < h; i += nw) {
      const double a = xs[i * S + lane], b = xs[(L - 1 - i) * S + lane];
      split(a + b, esh[i * S + lane], esl[i * S + lane]);
      split(a - b, osh[i * S + lane], osl[i * S + lane]);
    }
    float mid_h = 0.f, mid_l = 0.f;
    if (L & 1) split(xs[h * S + lane], mid_h, mid_l);
    __syncthreads();
    // y[k] into xs (the inputs are no longer needed).
    for (int k = warp; k < L; k += nw) {
      const float* sh = (k & 1) ? osh : esh;
      const float* sl = (k & 1) ? osl : esl;
      const float* ckh = ch + (long long)k * L;
      const float* ckl = cl + (long long)k * L;
      DfAcc acc;
      if (L & 1) acc.add(ckh[h], ckl[h], mid_h, mid_l);
      for (int i = 0; i < h; ++i) acc.add(ckh[i], ckl[i], sh[i * S + lane], sl[i * S + lane]);
      float rh, rl;
      acc.result(rh, rl);
      xs[k * S + lane] = (double)rh + (double)rl;
    }
  } else {
    // The inputs as hi/lo floats.
    float* xh = fs;
    float* xl = fs + L * S;
    for (int idx = threadIdx.x; idx < L * kDctLines; idx += kDctThreads) {
      const int q = (idx / kDctLines) * S + idx % kDctLines;
      split(xs[q], xh[q], xl[q]);
    }
    __syncthreads();
    for (int i = warp; i < hc; i += nw) {
      DfAcc ev, od;
      for (int k = 0; k < L; k += 2) ev.add(ch[(long long)k * L + i], cl[(long long)k * L + i], xh[k * S + lane], xl[k * S + lane]);
      for (int k = 1; k < L; k += 2) od.add(ch[(long long)k * L + i], cl[(long long)k * L + i], xh[k * S + lane], xl[k * S + lane]);
      float eh, el, oh, ol;
      ev.result(eh, el);
      od.result(oh, ol);
      const double e = (double)eh + (double)el, o = (double)oh + (double)ol;
      xs[i * S + lane] = e + o;                          // x[i]
      if (L - 1 - i != i) xs[(L - 1 - i) * S + lane] = e - o;  // x[L-1-i]
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < kDctLines * L; idx += kDctThreads) {
    int e, l;
    if (cols) { e = idx / kDctLines; l = idx % kDctLines; }
    else { l = idx / L; e = idx % L; }
    const long long line = l0 + l;
    if (line < n_lines) out[addr(line, e)] = xs[e * S + l];
  }
}

// One DCT pass over `batch` fields: forward (DCT-II) or inverse (DCT-III)
// along rows (cols = 0, matrix c of size n) or columns (cols = 1, size m).
static void dct_pass(int m, int n, int batch, bool inverse, int cols, const double* c, const float* cf,
                     const double* in, double* out, cudaStream_t stream) {
  const int L = cols ? m : n;
  const long long n_lines = (long long)batch * (cols ? n : m);
  if (L > kDctMaxLen) {
    const long long tot = (long long)m * n * batch;
    const int mode = cols ? (inverse ? 3 : 2) : (inverse ? 1 : 0);
    k_dct_apply<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(m, n, batch, mode, c, in, out);
    return;
  }
  const size_t smem = (size_t)(L + 2 * ((L + 1) / 2)) * (kDctLines + 1) * sizeof(double);
  const unsigned grid = (unsigned)((n_lines + kDctLines - 1) / kDctLines);
  if (inverse) k_dct_lines<true><<<grid, kDctThreads, smem, stream>>>(m, n, batch, cols, cf, in, out);
  else k_dct_lines<false><<<grid, kDctThreads, smem, stream>>>(m, n, batch, cols, cf, in, out);
}

__global__ void k_f2(long long mn, int n_pairs, const double* __restrict__ fd, double* __restrict__ f2,
                     float* __restrict__ f2f) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= mn * n_pairs) return;
  const long long pair = t / mn, e = t % mn;
  const double a = fd[(2 * pair) * mn + e], b = fd[(2 * pair + 1) * mn + e];
  f2[t] = a * a + b * b;
  f2f[t] = (float)(a * a + b * b);
}

static constexpr int kGcvThreads = 512;

// 1/d for d >= 1 from the float32 reciprocal and two Newton steps in float64:
// within an ulp or two of the rounded quotient, at a fraction of the cost of
// a float64 division (float64 throughput on this GPU is low).
PIV_D double rcp_fast(double d) {
  double r = (double)__frcp_rn((float)d);
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

struct GcvEval {
  const double* f2;
  const double* lam2;
  const float* f2f;
  const float* lam2f;
  long long mn;
  double n_finite;
  int n_fields;
};

// GCV score at p (gpu_smoothn.py:353-372, w_mean > 0.9 branch). All threads call.
PIV_D double gcv_score(const GcvEval& g, double p, double* red) {
  const double s = pow(10.0, p);
  double rss = 0.0, tr = 0.0;
  for (long long e = threadIdx.x; e < g.mn; e += blockDim.x) {
    const double gm = rcp_fast(1.0 + s * g.lam2[e]);
    const double d = gm - 1.0;
    rss += g.f2[e] * d * d;
    tr += gm;
  }
  for (int o = 16; o > 0; o >>= 1) {
    rss += __shfl_xor_sync(~0u, rss, o);
    tr += __shfl_xor_sync(~0u, tr, o);
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { red[w] = rss; red[32 + w] = tr; }
  __syncthreads();
  double trss = 0.0, ttr = 0.0;
  for (int k = 0; k < nw; ++k) { trss += red[k]; ttr += red[32 + k]; }
  const double q = 1.0 - ttr / (double)g.mn;
  return trss / g.n_finite / (q * q) / g.n_fields;
}

// Finite-difference gradient as the reference's L-BFGS-B call computes it
// (absolute step 1e-8, backward at the upper bound).
PIV_D double gcv_grad(const GcvEval& g, double p, double f0, double pmax, double* red) {
  const double h = 1e-8;
  if (p + h <= pmax) return (gcv_score(g, p + h, red) - f0) / h;
  return (f0 - gcv_score(g, p - h, red)) / h;
}

// GCV score with float32 terms and float64 sums: 1 - gamma = s l / (1 + s l)
// is formed directly (no cancellation), so every term is a product of
// positive factors within a few float32 ulps; the rounding errors of the
// terms are independent, and their sum over the field stays near 1e-9 of the
// score. s = 10^p is formed once per CTA in float64. Used to rank the scan
// points and for the bounded local search; the gradient test, which divides
// score differences by 1e-8, uses the float64 score.
PIV_D double gcv_score_fast(const GcvEval& g, double p, double* red) {
  if (threadIdx.x == 0) red[64] = pow(10.0, p);
  __syncthreads();
  const float s = (float)red[64];
  float rss = 0.f, tr = 0.f;
  for (long long e = threadIdx.x; e < g.mn; e += blockDim.x) {
    const float sl = s * g.lam2f[e];
    const float d = sl * __frcp_rn(1.0f + sl);  // 1 - gamma
    rss = fmaf(g.f2f[e] * d, d, rss);
    tr += d;
  }
  double drss = rss, dtr = tr;
  for (int o = 16; o > 0; o >>= 1) {
    drss += __shfl_xor_sync(~0u, drss, o);
    dtr += __shfl_xor_sync(~0u, dtr, o);
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { red[w] = drss; red[32 + w] = dtr; }
  __syncthreads();
  double trss = 0.0, ttr = 0.0;
  for (int k = 0; k < nw; ++k) { trss += red[k]; ttr += red[32 + k]; }
  const double q = ttr / (double)g.mn;
  return trss / g.n_finite / (q * q) / g.n_fields;
}

// One CTA per pair. Every thread takes part in the sums of each score; the
// search itself (scan bookkeeping, gradient test, Brent's iteration: scalar
// float64 work) runs in warp 0 alone, which announces each next point as
// s = 10^p in shared memory. Float64 runs at a small fraction of the float32
// rate on this GPU, so the search is not repeated by all 16 warps. The
// operations and their order are those of gcv_score / gcv_score_fast.
__global__ void __launch_bounds__(kGcvThreads)
k_gcv(int m, int n, int n_pairs, const double* __restrict__ f2, const double* __restrict__ lam2,
      const float* __restrict__ f2f, const float* __restrict__ lam2f, double pmin, double pmax,
      double* __restrict__ p_out) {
  __shared__ double red[64];
  __shared__ double sh_s;  // 10^p of the next score
  __shared__ int sh_go;    // warp 0's decision for the next step
  const int pair = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const bool w0 = warp == 0;
  const long long mn = (long long)m * n;
  const double* f2p = f2 + pair * mn;
  const float* f2fp = f2f + pair * mn;
  const double n_finite = (double)mn;
  // Combines the per-warp sums in red[] (valid in warp 0).
  auto combine = [&](double& trss, double& ttr) {
    trss = 0.0;
    ttr = 0.0;
    for (int k = 0; k < nw; ++k) { trss += red[k]; ttr += red[32 + k]; }
  };
  // Scores at the announced point (all threads, after a barrier that follows
  // the announcement); the value is valid in warp 0.
  auto score_fast = [&]() -> double {
    const float s = (float)sh_s;
    float rss = 0.f, tr = 0.f;
    for (long long e = threadIdx.x; e < mn; e += blockDim.x) {
      const float sl = s * lam2f[e];
      const float d = sl * __frcp_rn(1.0f + sl);  // 1 - gamma
      rss = fmaf(f2fp[e] * d, d, rss);
      tr += d;
    }
    double drss = rss, dtr = tr;
    for (int o = 16; o > 0; o >>= 1) {
      drss += __shfl_xor_sync(~0u, drss, o);
      dtr += __shfl_xor_sync(~0u, dtr, o);
    }
    if (lane == 0) { red[warp] = drss; red[32 + warp] = dtr; }
    __syncthreads();
    double f = 0.0;
    if (w0) {
      double trss, ttr;
      combine(trss, ttr);
      const double q = ttr / (double)mn;
      f = trss / n_finite / (q * q) / 2;
    }
    return f;
  };
  auto score = [&]() -> double {
    const double s = sh_s;
    double rss = 0.0, tr = 0.0;
    for (long long e = threadIdx.x; e < mn; e += blockDim.x) {
      const double gm = rcp_fast(1.0 + s * lam2[e]);
      const double d = gm - 1.0;
      rss += f2p[e] * d * d;
      tr += gm;
    }
    for (int o = 16; o > 0; o >>= 1) {
      rss += __shfl_xor_sync(~0u, rss, o);
      tr += __shfl_xor_sync(~0u, tr, o);
    }
    if (lane == 0) { red[warp] = rss; red[32 + warp] = tr; }
    __syncthreads();
    double f = 0.0;
    if (w0) {
      double trss, ttr;
      combine(trss, ttr);
      const double q = 1.0 - ttr / (double)mn;
      f = trss / n_finite / (q * q) / 2;
    }
    return f;
  };
  // Announces p (thread 0) and makes it visible; the barrier also orders the
  // previous score's reads of red[] before the next score's writes.
  auto announce = [&](double p) {
    if (threadIdx.x == 0) sh_s = pow(10.0, p);
    __syncthreads();
  };
  // 10-point scan (gpu_smoothn.py:182-188), ranked with the fast score; the
  // best point is scored in float64 for the gradient test.
  double best_p = pmin, best_f = INFINITY;
  for (int k = 0; k < 10; ++k) {
    const double pk = ((double)k * (1.0 / 9.0)) * (pmax - pmin) + pmin;
    announce(pk);
    const double fk = score_fast();
    if (k == 0 || fk < best_f) { best_f = fk; best_p = pk; }
  }
  double p = best_p;
  announce(p);
  const double f0 = score();
  // Finite-difference gradient as the reference's L-BFGS-B call computes it
  // (absolute step 1e-8, backward at the upper bound).
  const double h = 1e-8;
  const bool fwd = p + h <= pmax;
  announce(fwd ? p + h : p - h);
  const double fh = score();
  if (threadIdx.x == 0) {
    const double g0 = fwd ? (fh - f0) / h : (f0 - fh) / h;
    const double pg = g0 < 0 ? fmax(p - pmax, g0) : fmin(p - pmin, g0);
    sh_go = !(fabs(pg) <= 1e-5);
  }
  announce(p);  // also publishes sh_go
  if (sh_go) {
    // Brent's bounded minimisation on the bracket around the scan point.
    const double step = (pmax - pmin) / 9.0;
    double a = fmax(pmin, p - step), b = fmin(pmax, p + step);
    const double cg = 0.3819660112501051;
    const double fs = score_fast();
    double x = p, w = p, v = p, fx = fs, fw = fs, fv = fs, d = 0.0, e = 0.0;
    for (int it = 0; it < 200; ++it) {
      double u = 0.0;
      if (w0) {
        const double xm = 0.5 * (a + b);
        const double tol1 = 1e-8 * fabs(x) + 1e-10, tol2 = 2.0 * tol1;
        const bool done = fabs(x - xm) <= tol2 - 0.5 * (b - a);
        if (!done) {
          bool golden = true;
          if (fabs(e) > tol1) {
            double r = (x - w) * (fx - fv), q = (x - v) * (fx - fw), pp = (x - v) * q - (x - w) * r;
            q = 2.0 * (q - r);
            if (q > 0) pp = -pp;
            q = fabs(q);
            const double etemp = e;
            e = d;
            if (!(fabs(pp) >= fabs(0.5 * q * etemp) || pp <= q * (a - x) || pp >= q * (b - x))) {
              d = pp / q;
              const double uu = x + d;
              if (uu - a < tol2 || b - uu < tol2) d = xm >= x ? tol1 : -tol1;
              golden = false;
            }
          }
          if (golden) {
            e = (x >= xm) ? a - x : b - x;
            d = cg * e;
          }
          u = fabs(d) >= tol1 ? x + d : x + (d >= 0 ? tol1 : -tol1);
        }
        if (lane == 0) {
          sh_go = !done;
          if (!done) sh_s = pow(10.0, u);
        }
      }
      __syncthreads();
      if (!sh_go) break;
      const double fu = score_fast();
      if (w0) {
        if (fu <= fx) {
          if (u >= x) a = x; else b = x;
          v = w; fv = fw; w = x; fw = fx; x = u; fx = fu;
        } else {
          if (u < x) a = u; else b = u;
          if (fu <= fw || w == x) { v = w; fv = fw; w = u; fw = fu; }
          else if (fu <= fv || v == x || v == w) { v = u; fv = fu; }
        }
      }
    }
    p = x;
    // A minimum within the tolerance of a bound sits on the bound (a projected method lands there).
    if (p - pmin < 1e-9) p = pmin;
    if (pmax - p < 1e-9) p = pmax;
  }
  if (threadIdx.x == 0) p_out[pair] = p;
}

// fd *= gamma(p) for both fields of each pair. Grid: x over the 2 mn
// coefficients of a pair, y over pairs; s = 10^p is formed once per CTA.
__global__ void k_apply_gamma(long long mn, int n_pairs, const double* __restrict__ lam2,
                              const double* __restrict__ p, double fixed_p, double* __restrict__ fd) {
  __shared__ double s_sh;
  const int pair = blockIdx.y;
  if (threadIdx.x == 0) s_sh = pow(10.0, p ? p[pair] : fixed_p);
  __syncthreads();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * mn) return;
  const long long e = t % mn;
  double* f = fd + (long long)pair * 2 * mn + t;
  *f = rcp_fast(1.0 + s_sh * lam2[e]) * *f;
}

__global__ void k_fill(int count, double value, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < count) out[t] = value;
}

static int check(const char* what) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, what);
}

// ---------------------------------------------------------------------------
// Weighted smoothn (a field mask, or fields with non-finite values): Garcia's
// iteration as SmoothnGPU runs it with weights (gpu_smoothn.py:123-231):
// missing values take the value of their nearest finite neighbour
// (replace_non_finite, gpu_smoothn.py:233-251, with scipy's feature-transform
// choice among equidistant neighbours: per column the nearest finite row, the
// lower one on a tie, then the nearest column, the lower one on a tie), the
// start z keeps the low DCT coefficients (get_init_z, gpu_smoothn.py:284-297),
// then z <- rf IDCT2(gamma DCT2(w (f - z) + z)) + (1 - rf) z with rf = 1.75
// until ||z_old - z|| / (||z|| + 1e-6) <= 1e-3 or 100 iterations; with s unset
// the GCV search runs at iterations 1, 2, 4, 8, ... (gpu_smoothn.py:176-193),
// with the w_mean <= 0.9 score refitting the field for every candidate s
// (gpu_smoothn.py:359-368). Output zero inside the mask (gpu_smoothn.py:224-225).
// One CTA per pair does the whole iteration; float64 throughout.
// ---------------------------------------------------------------------------
static constexpr int kSwThreads = 512;

PIV_D double cta_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double t = l < nw ? red[l] : 0.0;
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(~0u, t, o);
  return t;
}

struct DfMats {
  const float *cmh, *cml, *cnh, *cnl;  // [m][m], [n][n] hi and lo parts
};

// 2-D orthonormal DCT-II (inv = false) or DCT-III of one m x n field inside the
// CTA, in the double-float arithmetic of DfAcc. xs: 2 mn floats (the input's
// hi/lo split); tmp: 2 mn floats (the row pass); in and out may not overlap
// tmp or xs.
PIV_D void cta_dct2(const double* in, float* xs, float* tmp, double* out, int m, int n, const DfMats& M, bool inv) {
  const int mn = m * n;
  for (int e = threadIdx.x; e < mn; e += blockDim.x) {
    const double x = in[e];
    const float h = (float)x;
    xs[e] = h;
    xs[mn + e] = (float)(x - (double)h);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < mn; e += blockDim.x) {
    const int i = e / n, l = e % n;
    DfAcc acc;
    for (int j = 0; j < n; ++j) {
      const int ci = inv ? j * n + l : l * n + j;
      acc.add(xs[i * n + j], xs[mn + i * n + j], M.cnh[ci], M.cnl[ci]);
    }
    acc.result(tmp[e], tmp[mn + e]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < mn; e += blockDim.x) {
    const int k = e / n, j = e % n;
    DfAcc acc;
    for (int i = 0; i < m; ++i) {
      const int ci = inv ? i * m + k : k * m + i;
      acc.add(M.cmh[ci], M.cml[ci], tmp[i * n + j], tmp[mn + i * n + j]);
    }
    float h, l;
    acc.result(h, l);
    out[e] = (double)h + (double)l;
  }
  __syncthreads();
}

struct SwCtx {
  int m, n, mn;
  const double* lam2;
  DfMats mats;
  double *f, *z, *t, *fd, *tmp, *w;
  float* xs;  // 2 mn floats: hi/lo split of a DCT input
  double n_finite, w_mean;
  double* red;
};

// GCV score at p (gpu_smoothn.py:353-372). fd: DCT of both fields.
PIV_D double sw_gcv(const SwCtx& c, double p) {
  const double s = pow(10.0, p);
  double rss = 0.0, tr = 0.0;
  if (c.w_mean > 0.9) {
    for (int e = threadIdx.x; e < c.mn; e += blockDim.x) {
      const double gm = rcp_fast(1.0 + s * c.lam2[e]);
      const double d = gm - 1.0;
      rss += (c.fd[e] * c.fd[e] + c.fd[c.mn + e] * c.fd[c.mn + e]) * d * d;
      tr += gm;
    }
  } else {
    for (int e = threadIdx.x; e < c.mn; e += blockDim.x) tr += rcp_fast(1.0 + s * c.lam2[e]);
    for (int fi = 0; fi < 2; ++fi) {
      // f_hat = IDCT2(gamma fd); t holds gamma fd, z is kept.
      for (int e = threadIdx.x; e < c.mn; e += blockDim.x)
        c.t[fi * c.mn + e] = c.fd[fi * c.mn + e] * rcp_fast(1.0 + s * c.lam2[e]);
      __syncthreads();
      cta_dct2(c.t + fi * c.mn, c.xs, reinterpret_cast<float*>(c.tmp), c.tmp + c.mn, c.m, c.n, c.mats, true);
      for (int e = threadIdx.x; e < c.mn; e += blockDim.x) {
        const double fv = c.f[fi * c.mn + e];
        if (isfinite(fv) || c.w[e] > 0) {
          const double d = fv - c.tmp[c.mn + e];
          rss += c.w[e] * d * d;
        }
      }
      __syncthreads();
    }
  }
  rss = cta_sum(rss, c.red);
  tr = cta_sum(tr, c.red);
  const double q = 1.0 - tr / (double)c.mn;
  return rss / c.n_finite / (q * q) / 2.0;
}

// The search of k_gcv (scan on the first call, then the projected-gradient
// stopping test and Brent's bounded minimisation around the start point).
PIV_D double sw_search(const SwCtx& c, double p, bool have_p, double pmin, double pmax) {
  if (!have_p) {
    double best_f = INFINITY;
    for (int k = 0; k < 10; ++k) {
      const double pk = ((double)k * (1.0 / 9.0)) * (pmax - pmin) + pmin;
      const double fk = sw_gcv(c, pk);
      if (k == 0 || fk < best_f) { best_f = fk; p = pk; }
    }
  }
  const double f0 = sw_gcv(c, p);
  const double h = 1e-8;
  const double g0 = p + h <= pmax ? (sw_gcv(c, p + h) - f0) / h : (f0 - sw_gcv(c, p - h)) / h;
  const double pg = g0 < 0 ? fmax(p - pmax, g0) : fmin(p - pmin, g0);
  if (fabs(pg) <= 1e-5) return p;
  const double step = (pmax - pmin) / 9.0;
  double a = fmax(pmin, p - step), b = fmin(pmax, p + step);
  const double cg = 0.3819660112501051;
  double x = p, w = p, v = p, fx = f0, fw = f0, fv = f0, d = 0.0, e = 0.0;
  for (int it = 0; it < 200; ++it) {
    const double xm = 0.5 * (a + b);
    const double tol1 = 1e-11 * fabs(x) + 1e-13, tol2 = 2.0 * tol1;
    if (fabs(x - xm) <= tol2 - 0.5 * (b - a)) break;
    bool golden = true;
    if (fabs(e) > tol1) {
      double r = (x - w) * (fx - fv), q = (x - v) * (fx - fw), pp = (x - v) * q - (x - w) * r;
      q = 2.0 * (q - r);
      if (q > 0) pp = -pp;
      q = fabs(q);
      const double etemp = e;
      e = d;
      if (!(fabs(pp) >= fabs(0.5 * q * etemp) || pp <= q * (a - x) || pp >= q * (b - x))) {
        d = pp / q;
        const double u = x + d;
        if (u - a < tol2 || b - u < tol2) d = xm >= x ? tol1 : -tol1;
        golden = false;
      }
    }
    if (golden) {
      e = (x >= xm) ? a - x : b - x;
      d = cg * e;
    }
    const double u = fabs(d) >= tol1 ? x + d : x + (d >= 0 ? tol1 : -tol1);
    const double fu = sw_gcv(c, u);
    if (fu <= fx) {
      if (u >= x) a = x; else b = x;
      v = w; fv = fw; w = x; fw = fx; x = u; fx = fu;
    } else {
      if (u < x) a = u; else b = u;
      if (fu <= fw || w == x) { v = w; fv = fw; w = u; fw = fu; }
      else if (fu <= fv || v == x || v == w) { v = u; fv = fu; }
    }
  }
  if (x - pmin < 1e-9) x = pmin;
  if (pmax - x < 1e-9) x = pmax;
  return x;
}

__global__ void __launch_bounds__(kSwThreads)
k_smoothn_weighted(int m, int n, const double* u_in, const double* v_in, double* u_out, double* v_out,
                   const uint8_t* __restrict__ mask,
                   double fixed_p, int is_auto, double pmin, double pmax, DfMats mats,
                   const double* __restrict__ lam2, unsigned char* scratch, size_t pair_bytes, double* p_out) {
  __shared__ double red[32];
  __shared__ int s_flag;
  const int pair = blockIdx.x, mn = m * n, tid = threadIdx.x, nt = blockDim.x;
  double* base = reinterpret_cast<double*>(scratch + pair_bytes * pair);
  SwCtx c;
  c.m = m; c.n = n; c.mn = mn; c.mats = mats; c.lam2 = lam2;
  c.f = base; c.z = base + 2 * mn; c.t = base + 4 * mn; c.fd = base + 6 * mn; c.tmp = base + 8 * mn;
  c.w = base + 10 * mn; c.red = red;
  int* near = reinterpret_cast<int*>(base + 11 * mn);
  c.xs = reinterpret_cast<float*>(near + mn);
  float* tmpf = reinterpret_cast<float*>(c.tmp);
  const long long off = (long long)pair * mn;
  // Fields, finite mask and weights.
  double nf = 0.0, ws = 0.0;
  for (int e = tid; e < mn; e += nt) {
    const double a = u_in[off + e], b = v_in[off + e];
    const bool fin = isfinite(a) && isfinite(b);
    c.f[e] = a;
    c.f[mn + e] = b;
    const double wv = (fin && !(mask && mask[e])) ? 1.0 : 0.0;
    c.w[e] = wv;
    nf += fin ? 1.0 : 0.0;
    ws += wv;
  }
  nf = cta_sum(nf, red);
  ws = cta_sum(ws, red);
  c.n_finite = nf;
  c.w_mean = ws / (double)mn;
  const bool weighted = ws != (double)mn;
  // Nearest finite neighbour of the missing points: first the nearest finite
  // row in every column (ties: the lower row), then the nearest column.
  if (nf < (double)mn && nf > 0) {
    for (int col = tid; col < n; col += nt) {
      int last = -1;
      for (int y = 0; y < m; ++y) {
        if (isfinite(c.f[y * n + col]) && isfinite(c.f[mn + y * n + col])) last = y;
        near[y * n + col] = last;
      }
      int next = -1;
      for (int y = m - 1; y >= 0; --y) {
        if (isfinite(c.f[y * n + col]) && isfinite(c.f[mn + y * n + col])) next = y;
        const int up = near[y * n + col];
        int r = up;
        if (up < 0 || (next >= 0 && next - y < y - up)) r = next;
        near[y * n + col] = r;
      }
    }
    __syncthreads();
    for (int e = tid; e < mn; e += nt) {
      if (isfinite(c.f[e]) && isfinite(c.f[mn + e])) continue;
      const int y = e / n, x = e % n;
      long long best = -1;
      int br = 0, bc = 0;
      for (int col = 0; col < n; ++col) {
        const int r = near[y * n + col];
        if (r < 0) continue;
        const long long d = (long long)(col - x) * (col - x) + (long long)(r - y) * (r - y);
        if (best < 0 || d < best) { best = d; br = r; bc = col; }
      }
      c.t[e] = c.f[br * n + bc];
      c.t[mn + e] = c.f[mn + br * n + bc];
    }
    __syncthreads();
    for (int e = tid; e < mn; e += nt) {
      if (isfinite(c.f[e]) && isfinite(c.f[mn + e])) continue;
      c.f[e] = c.t[e];
      c.f[mn + e] = c.t[mn + e];
    }
    __syncthreads();
  }
  // Start: the low DCT coefficients of f (one trailing block cleared), or 0.
  const int n0 = (m + 9) / 10 + 1, n1 = (n + 9) / 10 + 1;
  for (int fi = 0; fi < 2; ++fi) {
    if (weighted) {
      cta_dct2(c.f + fi * mn, c.xs, tmpf, c.t + fi * mn, m, n, mats, false);
      for (int e = tid; e < mn; e += nt)
        if (e / n >= n0 && e % n >= n1) c.t[fi * mn + e] = 0.0;
      __syncthreads();
      cta_dct2(c.t + fi * mn, c.xs, tmpf, c.z + fi * mn, m, n, mats, true);
    } else {
      for (int e = tid; e < mn; e += nt) c.z[fi * mn + e] = 0.0;
    }
  }
  __syncthreads();
  const double rf = weighted ? 1.75 : 1.0;
  double p = fixed_p;
  bool have_p = !is_auto;
  for (int k = 0; k < 100; ++k) {
    for (int e = tid; e < 2 * mn; e += nt) {
      const double wv = c.w[e % mn];
      c.t[e] = wv * (c.f[e] - c.z[e]) + c.z[e];
    }
    __syncthreads();
    for (int fi = 0; fi < 2; ++fi) cta_dct2(c.t + fi * mn, c.xs, tmpf, c.fd + fi * mn, m, n, mats, false);
    if (is_auto && ((k + 1) & k) == 0) {
      p = sw_search(c, p, have_p, pmin, pmax);
      have_p = true;
    }
    const double s = pow(10.0, p);
    double num = 0.0, den = 0.0;
    for (int fi = 0; fi < 2; ++fi) {
      for (int e = tid; e < mn; e += nt) c.t[fi * mn + e] = c.fd[fi * mn + e] * rcp_fast(1.0 + s * lam2[e]);
      __syncthreads();
      cta_dct2(c.t + fi * mn, c.xs, tmpf, c.tmp + mn, m, n, mats, true);
      for (int e = tid; e < mn; e += nt) {
        const double z0 = c.z[fi * mn + e];
        const double z1 = rf * c.tmp[mn + e] + (1.0 - rf) * z0;
        c.z[fi * mn + e] = z1;
        num += (z0 - z1) * (z0 - z1);
        den += z1 * z1;
      }
      __syncthreads();
    }
    num = cta_sum(num, red);
    den = cta_sum(den, red);
    const double tol = weighted ? sqrt(num) / (sqrt(den) + 1e-6) : 0.0;
    if (tid == 0) s_flag = tol <= 1e-3;
    __syncthreads();
    if (s_flag) break;
  }
  for (int e = tid; e < mn; e += nt) {
    const bool in_mask = mask && mask[e];
    u_out[off + e] = in_mask ? 0.0 : c.z[e];
    v_out[off + e] = in_mask ? 0.0 : c.z[mn + e];
  }
  if (tid == 0 && p_out) p_out[pair] = p;
}

static int smoothn_weighted(int m, int n, int n_pairs, const double* u_in, const double* v_in, double* u_out,
                            double* v_out, const uint8_t* field_mask, double s, double* p_out, void* scratch,
                            cudaStream_t stream) {
  const size_t mn = (size_t)m * n;
  char* p = (char*)scratch;
  double* cm = (double*)p; p += align_up((size_t)m * m * 8);
  double* cn = (double*)p; p += align_up((size_t)n * n * 8);
  double* lam2 = (double*)p; p += align_up(mn * 8);
  p += align_up((size_t)n_pairs * 8);
  float* mf = (float*)p; p += weighted_matrix_bytes(m, n);
  const DfMats mats{mf, mf + m * m, mf + 2 * m * m, mf + 2 * m * m + n * n};
  const int bs = 256;
  k_dct_matrix<<<(m * m + bs - 1) / bs, bs, 0, stream>>>(m, cm);
  k_dct_matrix<<<(n * n + bs - 1) / bs, bs, 0, stream>>>(n, cn);
  k_split_f64<<<(m * m + bs - 1) / bs, bs, 0, stream>>>(m * m, cm, const_cast<float*>(mats.cmh),
                                                         const_cast<float*>(mats.cml));
  k_split_f64<<<(n * n + bs - 1) / bs, bs, 0, stream>>>(n * n, cn, const_cast<float*>(mats.cnh),
                                                         const_cast<float*>(mats.cnl));
  k_lambda2<<<(unsigned)((mn + bs - 1) / bs), bs, 0, stream>>>(m, n, lam2);
  const bool is_auto = !(s > 0);
  double pmin = 0, pmax = 0;
  if (is_auto) {
    const double h_min = 1e-3, h_max = 1.0 - h_min;
    const int rank = (m != 1) + (n != 1);
    const double a_max = pow(h_max, 2.0 / rank), a_min = pow(h_min, 2.0 / rank);
    pmin = log10((pow((1.0 + sqrt(1.0 + 8.0 * a_max)) / 4.0 / a_max, 2.0) - 1.0) / 16.0);
    pmax = log10((pow((1.0 + sqrt(1.0 + 8.0 * a_min)) / 4.0 / a_min, 2.0) - 1.0) / 16.0);
  }
  k_smoothn_weighted<<<n_pairs, kSwThreads, 0, stream>>>(m, n, u_in, v_in, u_out, v_out, field_mask,
                                                          is_auto ? 0.0 : log10(s), is_auto ? 1 : 0, pmin, pmax, mats,
                                                          lam2, (unsigned char*)p, weighted_pair_bytes(mn), p_out);
  return check("k_smoothn_weighted");
}

int smoothn(int m, int n, int n_pairs, const double* u_in, const double* v_in, double* u_out, double* v_out,
            const uint8_t* field_mask, double s, double* p_out, void* scratch, cudaStream_t stream) {
  const long long mn = (long long)m * n;
  if (n_pairs == 0 || mn == 0) return PIV_OK;
  if (mn < 2) {
    cudaMemcpyAsync(u_out, u_in, mn * n_pairs * 8, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(v_out, v_in, mn * n_pairs * 8, cudaMemcpyDeviceToDevice, stream);
    return check("smoothn copy");
  }
  if (field_mask) return smoothn_weighted(m, n, n_pairs, u_in, v_in, u_out, v_out, field_mask, s, p_out, scratch, stream);
  SmoothScratch sc = carve(scratch, m, n, n_pairs);
  const int bs = 256;
  k_dct_matrix<<<(m * m + bs - 1) / bs, bs, 0, stream>>>(m, sc.cm);
  k_dct_matrix<<<(n * n + bs - 1) / bs, bs, 0, stream>>>(n, sc.cn);
  k_split_f64<<<(m * m + bs - 1) / bs, bs, 0, stream>>>(m * m, sc.cm, sc.cmf, sc.cmf + m * m);
  k_split_f64<<<(n * n + bs - 1) / bs, bs, 0, stream>>>(n * n, sc.cn, sc.cnf, sc.cnf + n * n);
  k_lambda2<<<(unsigned)((mn + bs - 1) / bs), bs, 0, stream>>>(m, n, sc.lam2, sc.lam2f);
  // Gather u and v as [pair][field][mn] into tmp.
  for (int f = 0; f < 2; ++f) {
    cudaMemcpy2DAsync(sc.tmp + f * mn, 2 * mn * 8, f == 0 ? u_in : v_in, mn * 8, mn * 8, n_pairs,
                      cudaMemcpyDeviceToDevice, stream);
  }
  // Forward DCT-II: rows then columns.
  dct_pass(m, n, 2 * n_pairs, false, 0, sc.cn, sc.cnf, sc.tmp, sc.fd, stream);
  dct_pass(m, n, 2 * n_pairs, false, 1, sc.cm, sc.cmf, sc.fd, sc.tmp, stream);
  int rc = check("smoothn forward dct");
  if (rc) return rc;
  // tmp now holds the DCT coefficients.
  double* pvec = nullptr;
  double fixed_p = 0.0;
  const bool gcv = !(s > 0);
  if (gcv) {
    // p bounds for order 2 (gpu_smoothn.py:320-338), on the host.
    const double h_min = 1e-3, h_max = 1.0 - h_min;
    const int rank = (m != 1) + (n != 1);
    const double a_max = pow(h_max, 2.0 / rank), a_min = pow(h_min, 2.0 / rank);
    const double pmin = log10((pow((1.0 + sqrt(1.0 + 8.0 * a_max)) / 4.0 / a_max, 2.0) - 1.0) / 16.0);
    const double pmax = log10((pow((1.0 + sqrt(1.0 + 8.0 * a_min)) / 4.0 / a_min, 2.0) - 1.0) / 16.0);
    k_f2<<<(unsigned)((mn * n_pairs + bs - 1) / bs), bs, 0, stream>>>(mn, n_pairs, sc.tmp, sc.f2, sc.f2f);
    k_gcv<<<n_pairs, kGcvThreads, 0, stream>>>(m, n, n_pairs, sc.f2, sc.lam2, sc.f2f, sc.lam2f, pmin, pmax, sc.p);
    pvec = sc.p;
    rc = check("k_gcv");
    if (rc) return rc;
  } else {
    fixed_p = log10(s);
  }
  if (n_pairs > 65535) return set_error(PIV_E_UNSUPPORTED, "smoothn: more than 65535 pairs in one call");
  k_apply_gamma<<<dim3((unsigned)((2 * mn + bs - 1) / bs), (unsigned)n_pairs), bs, 0, stream>>>(mn, n_pairs, sc.lam2,
                                                                                               pvec, fixed_p, sc.tmp);
  // Inverse DCT (DCT-III): rows then columns.
  dct_pass(m, n, 2 * n_pairs, true, 0, sc.cn, sc.cnf, sc.tmp, sc.fd, stream);
  dct_pass(m, n, 2 * n_pairs, true, 1, sc.cm, sc.cmf, sc.fd, sc.tmp, stream);
  for (int f = 0; f < 2; ++f) {
    cudaMemcpy2DAsync(f == 0 ? u_out : v_out, mn * 8, sc.tmp + f * mn, 2 * mn * 8, mn * 8, n_pairs,
                      cudaMemcpyDeviceToDevice, stream);
  }
  if (p_out) {
    if (gcv) {
      cudaMemcpyAsync(p_out, sc.p, n_pairs * 8, cudaMemcpyDeviceToDevice, stream);
    } else {
      k_fill<<<(n_pairs + 127) / 128, 128, 0, stream>>>(n_pairs, fixed_p, p_out);
    }
  }
  return check("smoothn");
}

}  // namespace piv

namespace piv {

// ---------------------------------------------------------------------------
// smoothn without device allocation.
//
// Some callers cannot allocate device memory while they run: a host that
// hands this library a fixed memory budget at start-up, a real-time loop that
// must not stall in the allocator, or a framework that owns every device
// allocation itself. piv_smoothn_noalloc serves them with scratch that lives
// in a fixed device array of this file, sized for modest fields. Every GPU
// that loads the library holds the array until the process exits.
// ---------------------------------------------------------------------------
static constexpr size_t kNoAllocScratchBytes = 4u << 20;  // 4 MiB: e.g. 4 pairs of 128 x 128 fields
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch, looked up once per device. In host code
// the array's name is only a host-side stand-in, never a device address.
static void* noalloc_scratch_address(int* rc) {
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    *rc = set_cuda_error(e, "cudaGetDevice");
    return nullptr;
  }
  if (dev < 0 || dev >= 64) {
    *rc = set_error(PIV_E_UNSUPPORTED, "device index %d out of range", dev);
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      *rc = set_cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
      return nullptr;
    }
    addr[dev] = p;
  }
  *rc = PIV_OK;
  return addr[dev];
}

}  // namespace piv

extern "C" int piv_smoothn_noalloc(int m, int n, int n_pairs, double* u, double* v, const uint8_t* field_mask,
                                   double s, double* p_out, void* stream) {
  using namespace piv;
  if (!u || !v) return set_error(PIV_E_ARG, "NULL argument");
  if (m <= 0 || n <= 0 || n_pairs <= 0) return set_error(PIV_E_ARG, "empty field (m=%d, n=%d, pairs=%d)", m, n, n_pairs);
  const size_t need = smoothn_scratch_bytes(m, n, n_pairs);
  if (need > kNoAllocScratchBytes)
    return set_error(PIV_E_ARG,
                     "piv_smoothn_noalloc: %d pair(s) of %d x %d fields need %zu bytes of scratch, more than its "
                     "fixed %zu bytes; use piv_smoothn or fewer/smaller fields",
                     n_pairs, m, n, need, kNoAllocScratchBytes);
  int rc = PIV_OK;
  void* scratch = noalloc_scratch_address(&rc);
  if (!scratch) return rc;
  return smoothn(m, n, n_pairs, u, v, u, v, field_mask, s, p_out, scratch, (cudaStream_t)stream);
}
