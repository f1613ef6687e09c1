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
#include "piv_lbfgsb1.cuh"

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

// Scratch of the unweighted path (no field mask) and of the weighted path.
static size_t smoothn_scratch_bytes_path(int m, int n, int n_pairs, bool weighted_path) {
  const size_t mn = (size_t)m * n;
  const size_t shared = align_up((size_t)m * m * 8) + align_up((size_t)n * n * 8) + align_up(mn * 8) +
                        align_up((size_t)n_pairs * 8);
  if (weighted_path) return shared + weighted_matrix_bytes(m, n) + weighted_pair_bytes(mn) * n_pairs;
  return align_up(2 * mn * n_pairs * 8) * 2 + align_up(mn * n_pairs * 8) + shared + align_up(mn * n_pairs * 4) +
         align_up(mn * 4) + align_up((size_t)m * m * 8) + align_up((size_t)n * n * 8);
}

size_t smoothn_scratch_bytes(int m, int n, int n_pairs) {
  const size_t plain = smoothn_scratch_bytes_path(m, n, n_pairs, false);
  const size_t weighted = smoothn_scratch_bytes_path(m, n, n_pairs, true);
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

// Flags of SmoothnGPU's log messages (gpu_smoothn.py:218-222, 429-439): with
// GCV, the smoothing parameter within 0.1 (in log10) of its lower or else its
// upper bound; the iteration reaching its last allowed step.
PIV_D int smooth_flags(bool is_auto, double p, double pmin, double pmax, bool last_iter) {
  int f = 0;
  if (is_auto) {
    if (fabs(p - pmin) < 0.1) f |= PIV_SMOOTH_S_LOWER;
    else if (fabs(p - pmax) < 0.1) f |= PIV_SMOOTH_S_UPPER;
  }
  if (last_iter) f |= PIV_SMOOTH_MAX_ITERS;
  return f;
}

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

// One CTA per pair. Every thread takes part in the sums of each score; the
// search itself (scan bookkeeping and the L-BFGS-B steps: scalar float64
// work) runs in warp 0 alone, which announces each next point as s = 10^p in
// shared memory. Float64 runs at a small fraction of the float32 rate on this
// GPU, so the search is not repeated by all 16 warps. The fast score (float32
// terms, float64 sums: 1 - gamma = s l / (1 + s l) formed without
// cancellation, each term within a few float32 ulps, the score within ~1e-9)
// only ranks the scan points; the L-BFGS-B evaluations, whose difference
// quotients divide score differences by 1e-8, use the float64 score.
__global__ void __launch_bounds__(kGcvThreads)
k_gcv(int m, int n, int n_pairs, const double* __restrict__ f2, const double* __restrict__ lam2,
      const float* __restrict__ f2f, const float* __restrict__ lam2f, double pmin, double pmax,
      double* __restrict__ p_out, int* __restrict__ flags) {
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
  // Announces p (thread 0) and whether the search goes on, and makes both
  // visible; the barrier also orders the previous score's reads of red[]
  // before the next score's writes.
  auto announce = [&](double p, bool go) {
    if (threadIdx.x == 0) {
      sh_s = pow(10.0, p);
      sh_go = go;
    }
    __syncthreads();
  };
  // 10-point scan (gpu_smoothn.py:182-188), ranked with the fast score; when
  // other points score within 1e-6 of the best, those points are scored
  // again in float64 and the first minimum among them is kept (np.argmin).
  double fast[10];
  double best_f = INFINITY;
  for (int k = 0; k < 10; ++k) {
    const double pk = ((double)k * (1.0 / 9.0)) * (pmax - pmin) + pmin;
    announce(pk, true);
    fast[k] = score_fast();
    if (fast[k] < best_f) best_f = fast[k];
  }
  unsigned near_best = 0;  // scan points within 1e-6 of the best fast score (warp 0)
  for (int k = 0; k < 10; ++k)
    if (fast[k] <= best_f + 1e-6 * fabs(best_f)) near_best |= 1u << k;
  if (threadIdx.x == 0) sh_go = __popc(near_best) > 1 ? (int)near_best : 0;
  __syncthreads();
  const unsigned rescore = (unsigned)sh_go;
  double p0 = pmin;
  if (rescore) {
    double best64 = INFINITY;
    for (int k = 0; k < 10; ++k) {
      if (!((rescore >> k) & 1u)) continue;
      const double pk = ((double)k * (1.0 / 9.0)) * (pmax - pmin) + pmin;
      announce(pk, true);
      const double fk = score();
      if (fk < best64) { best64 = fk; p0 = pk; }
    }
  } else {
    for (int k = 9; k >= 0; --k)
      if (fast[k] == best_f) p0 = ((double)k * (1.0 / 9.0)) * (pmax - pmin) + pmin;
  }
  // L-BFGS-B from the scan point (gpu_smoothn.py:191-193), its scalar state
  // in warp 0; every evaluation is the float64 score at the point and at its
  // forward-difference neighbour.
  Lb1 lb;
  lb_init(lb, p0, pmin, pmax);
  for (int ev = 0; ev < kLbMaxEvals; ++ev) {
    const double xt = lb.xt, xs = lb_fd_point(xt, pmin, pmax);
    announce(xt, !lb.done);
    if (!sh_go) break;
    const double f = score();
    announce(xs, true);
    const double fh = score();
    if (w0) lb_feed(lb, f, (fh - f) / (xs - xt));
  }
  const double p = lb.x;
  if (threadIdx.x == 0) {
    p_out[pair] = p;
    if (flags) flags[pair] = smooth_flags(true, p, pmin, pmax, false);
  }
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

// The search of k_gcv: the 10-point scan on the first call (float64 scores,
// np.argmin's first minimum), then L-BFGS-B from the start point
// (gpu_smoothn.py:179-193). Every thread runs the same scalar steps on the
// same scores (sw_gcv returns the CTA's sums to every thread).
PIV_D double sw_search(const SwCtx& c, double p, bool have_p, double pmin, double pmax) {
  if (!have_p) {
    double best_f = INFINITY;
    for (int k = 0; k < 10; ++k) {
      const double pk = ((double)k * (1.0 / 9.0)) * (pmax - pmin) + pmin;
      const double fk = sw_gcv(c, pk);
      if (k == 0 || fk < best_f) { best_f = fk; p = pk; }
    }
  }
  Lb1 lb;
  lb_init(lb, p, pmin, pmax);
  for (int ev = 0; ev < kLbMaxEvals && !lb.done; ++ev) {
    const double x = lb.xt, xs = lb_fd_point(x, pmin, pmax);
    const double f = sw_gcv(c, x);
    const double fh = sw_gcv(c, xs);
    lb_feed(lb, f, (fh - f) / (xs - x));
  }
  return lb.x;
}

__global__ void __launch_bounds__(kSwThreads)
k_smoothn_weighted(int m, int n, const double* u_in, const double* v_in, double* u_out, double* v_out,
                   const uint8_t* __restrict__ mask,
                   double fixed_p, int is_auto, double pmin, double pmax, DfMats mats,
                   const double* __restrict__ lam2, unsigned char* scratch, size_t pair_bytes, double* p_out,
                   int* flags) {
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
  int k_last = 0;  // index of the last iteration run
  for (int k = 0; k < 100; ++k) {
    k_last = k;
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
  if (tid == 0 && flags) flags[pair] = smooth_flags(is_auto != 0, p, pmin, pmax, k_last == 99);
}

static int smoothn_weighted(int m, int n, int n_pairs, const double* u_in, const double* v_in, double* u_out,
                            double* v_out, const uint8_t* field_mask, double s, double* p_out, void* scratch,
                            cudaStream_t stream, int* flags) {
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
                                                          lam2, (unsigned char*)p, weighted_pair_bytes(mn), p_out,
                                                          flags);
  return check("k_smoothn_weighted");
}

int smoothn(int m, int n, int n_pairs, const double* u_in, const double* v_in, double* u_out, double* v_out,
            const uint8_t* field_mask, double s, double* p_out, void* scratch, cudaStream_t stream, int* flags) {
  const long long mn = (long long)m * n;
  if (n_pairs == 0 || mn == 0) return PIV_OK;
  if (flags && (mn < 2 || (!field_mask && s > 0))) cudaMemsetAsync(flags, 0, sizeof(int) * n_pairs, stream);
  if (mn < 2) {
    cudaMemcpyAsync(u_out, u_in, mn * n_pairs * 8, cudaMemcpyDeviceToDevice, stream);
    cudaMemcpyAsync(v_out, v_in, mn * n_pairs * 8, cudaMemcpyDeviceToDevice, stream);
    return check("smoothn copy");
  }
  if (field_mask)
    return smoothn_weighted(m, n, n_pairs, u_in, v_in, u_out, v_out, field_mask, s, p_out, scratch, stream, flags);
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
    k_gcv<<<n_pairs, kGcvThreads, 0, stream>>>(m, n, n_pairs, sc.f2, sc.lam2, sc.f2f, sc.lam2f, pmin, pmax, sc.p,
                                               flags);
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
// 4 MiB: e.g. 4 pairs of 128 x 128 fields, or with a field mask 2 pairs of
// 127 x 127 (the weighted path keeps more per pair).
static constexpr size_t kNoAllocScratchBytes = 4u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch in the current context. In host code
// the array's name is only a host-side stand-in, never a device address. The
// address is looked up on every call made outside stream capture (so a call
// after a device reset, which reloads the module at a new address, gets the
// new one) and remembered per device for calls made while `stream` is being
// captured, which reuse the address of the device's last uncaptured call.
static void* noalloc_scratch_address(cudaStream_t stream, int* rc) {
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
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) {
    *rc = set_cuda_error(e, "cudaStreamIsCapturing");
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (cap != cudaStreamCaptureStatusNone) {
    if (!addr[dev]) {
      *rc = set_error(PIV_E_ARG,
                      "piv_smoothn_noalloc: the first call on device %d must come before any stream capture", dev);
      return nullptr;
    }
  } else {
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
  // The kernels index with 32-bit products m n, m m and n n and launch one
  // block row per pair: refuse shapes beyond those before sizing the scratch
  // (whose 64-bit byte counts then cannot wrap).
  const long long lim = 1LL << 31;
  if ((long long)m * n >= lim || (long long)m * m >= lim || (long long)n * n >= lim || n_pairs > 65535)
    return set_error(PIV_E_ARG, "piv_smoothn_noalloc: field %d x %d with %d pair(s) is beyond the kernels' limits",
                     m, n, n_pairs);
  const bool weighted = field_mask != nullptr && (long long)m * n >= 2;
  const size_t need = smoothn_scratch_bytes_path(m, n, n_pairs, weighted);
  if (need > kNoAllocScratchBytes)
    return set_error(PIV_E_ARG,
                     "piv_smoothn_noalloc: %d pair(s) of %d x %d %sfields need %zu bytes of scratch, more than its "
                     "fixed %zu bytes; use piv_smoothn or fewer/smaller fields",
                     n_pairs, m, n, weighted ? "masked " : "", need, kNoAllocScratchBytes);
  int rc = PIV_OK;
  void* scratch = noalloc_scratch_address((cudaStream_t)stream, &rc);
  if (!scratch) return rc;
  return smoothn(m, n, n_pairs, u, v, u, v, field_mask, s, p_out, scratch, (cudaStream_t)stream);
}
