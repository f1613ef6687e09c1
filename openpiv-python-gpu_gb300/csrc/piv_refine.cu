// Peak refinement: the float32 correlation values of the subpixel stencil,
// evaluated directly at the lags the correlation engine found.
//
// The fp16-operand tensor-core engine computes every window's correlation map
// to about 6e-4 of the map maximum. That resolves the integer peak (the first
// maximum of the map, gpu_process.py:1248-1254) wherever the two largest
// values are further apart than the engine's tie tolerance (2^-9 of the peak;
// closer windows are flagged as near ties), but the five values of the
// subpixel fit (gpu_process.py:1256-1294) need float32 accuracy. This kernel
// recomputes those five values, c(di, dj) = sum over y, x of
// (a(y, x) - mean a) (b(y + di, x + dj) - mean b) with b zero outside its
// window (the zero-padded, mean-removed windows of gpu_process.py:1201-1246;
// lags without window overlap sum to exactly zero), in float32 from the
// frames, and redoes the fit and the displacement. The result is the float32
// FFT form's up to float32 rounding of the sums, at a cost of 5 ss^2 products
// per window.
//
// Work split: a group of ss / 4 threads per window, each thread four adjacent
// columns; frame b is walked once, row by row, against the three latest rows
// of frame a (refine_window); the window means come from the engine (or are
// summed here), the five sums are reduced over the group by warp shuffles.
#include <math.h>

#include "piv_common.cuh"
#include "piv_corr_common.cuh"
#include "piv_internal.h"

namespace piv {

namespace {

constexpr int kRefineThreads = 256;

// Sum of v over the thread's group of G consecutive lanes (G a power of two,
// at most 32); every lane of the warp must call it.
template <int G, int K>
PIV_D void group_sum(float (&v)[K]) {
  static_assert(G <= 32 && (G & (G - 1)) == 0, "a group is a power-of-two part of a warp");
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// Four adjacent columns per thread: G = ss / 4 threads per window (4, 8 or
// 16), so a window always lies in one warp.
constexpr int kCols = 4;

template <typename P>
PIV_D float px(const P* p) {
  return (float)__ldg(p);
}

// Four adjacent pixels from p; vec: p is aligned for one vector load.
template <typename P>
PIV_D void load4(const P* p, bool vec, float (&v)[4]) {
  if (vec) {
    if constexpr (sizeof(P) == 4) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p));
      v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
    } else if constexpr (sizeof(P) == 2) {
      const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
      v[0] = u16_to_float(q.x & 0xffffu), v[1] = u16_to_float(q.x >> 16), v[2] = u16_to_float(q.y & 0xffffu),
      v[3] = u16_to_float(q.y >> 16);
    } else {
      const unsigned q = __ldg(reinterpret_cast<const unsigned*>(p));
#pragma unroll
      for (int k = 0; k < 4; ++k) v[k] = u16_to_float((q >> (8 * k)) & 0xffu);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = px<P>(p + k);
  }
}

// One window by a group of G threads, thread x taking columns 4x .. 4x + 3 of
// frame a. Frame b is walked row by row: b row r = t + di - 1 (step t) meets
// a row t at lag di - 1, a row t - 1 at lags di and dj -+ 1, and a row t - 2
// at lag di + 1, so each row of either frame is loaded once and the three
// latest rows of a slide along in registers. A thread's six columns of b
// (4x + dj - 1 .. 4x + dj + 4) give the centre column of its four a columns
// and both side columns; columns outside b's window are read at a clamped
// column and weighted by zero (and no mean is removed there), rows outside it
// are left out by the step range. Steps run in chunks of R whose loads are
// issued together.
template <int SS, typename P>
PIV_D void refine_window(const CorrArgs& a, const CorrSeg* seg_s, int n_seg, long long g, bool active, int x) {
  constexpr int G = SS / kCols, HN = SS, N = 2 * SS, R = sizeof(P) == 1 ? 3 : 4;
  int sg = 0;
  long long loc = 0, base = 0;
  bool ok = active;
  const CorrSeg* q = &seg_s[0];
  if (ok) {
    while (sg + 1 < n_seg && g >= seg_s[sg + 1].win0) ++sg;
    q = &seg_s[sg];
    loc = g - q->win0;
    const int li = (int)loc, nw = q->m * q->n;
    const int pair = li / nw, k = li - pair * nw;
    const int wr = k / q->n, wc = k - wr * q->n;
    if (q->win_mask && q->win_mask[k]) ok = false;
    base = pair * (long long)q->height * q->width + (long long)(wr * q->spacing + q->y_offset) * q->width +
           wc * q->spacing + q->x_offset;
    if (ok && !in_bounds(base >= 0 && base + (long long)(SS - 1) * q->width + SS <=
                                           (long long)q->n_pairs * q->height * q->width))
      ok = false;
  }
  // Inactive groups walk the first window of the first segment (in bounds)
  // and write nothing.
  const int width = q->width;
  const int xa0 = kCols * x;
  const P* fa = reinterpret_cast<const P*>(q->frame_a) + (ok ? base : 0);
  const P* fb = reinterpret_cast<const P*>(q->frame_b) + (ok ? base : 0);
  constexpr unsigned VB = kCols * sizeof(P);
  const bool vec = ((reinterpret_cast<uintptr_t>(fa + xa0) | (uintptr_t)width * sizeof(P)) & (VB - 1)) == 0;
  // Window means: written by the engine, or summed here.
  float ma = 0.f, mb = 0.f;
  if (q->win_means) {
    if (ok) {
      ma = q->win_means[2 * loc];
      mb = q->win_means[2 * loc + 1];
    }
  } else {
    const bool vb = ((reinterpret_cast<uintptr_t>(fb + xa0)) & (VB - 1)) == 0 && vec;
    float sums[2] = {0.f, 0.f};
#pragma unroll 4
    for (int y = 0; y < SS; ++y) {
      float va[4], vb4[4];
      load4<P>(fa + y * width + xa0, vec, va);
      load4<P>(fb + y * width + xa0, vb, vb4);
#pragma unroll
      for (int k = 0; k < 4; ++k) sums[0] += va[k], sums[1] += vb4[k];
    }
    group_sum<G, 2>(sums);
    ma = sums[0] / (float)(SS * SS);
    mb = sums[1] / (float)(SS * SS);
  }
  // The engine's integer peak: shifted (i, j), lag (i - N/2, j - N/2).
  int pi_ = HN, pj = HN;
  if (ok) {
    pi_ = q->peak_i[loc];
    pj = q->peak_j[loc];
  }
  const int di = pi_ - HN, dj = pj - HN;
  // The six b columns: clamped read position, weight and removed mean.
  int cb[6];
  float mk[6], nmb[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const int c = xa0 + dj - 1 + j;
    const bool v = (unsigned)c < (unsigned)SS;
    cb[j] = min(max(c, 0), SS - 1);
    mk[j] = v ? 1.f : 0.f;
    nmb[j] = v ? -mb : 0.f;
  }
  auto load_b = [&](const P* row, float (&bv)[6]) {
#pragma unroll
    for (int j = 0; j < 6; ++j) bv[j] = fmaf(px<P>(row + cb[j]), mk[j], nmb[j]);
  };
  auto load_a = [&](const P* row, float (&av)[4]) {
    load4<P>(row + xa0, vec, av);
#pragma unroll
    for (int k = 0; k < 4; ++k) av[k] -= ma;
  };
  float s_c = 0.f, s_d = 0.f, s_u = 0.f, s_l = 0.f, s_r = 0.f;
  auto step = [&](const float (&a0)[4], const float (&a1)[4], const float (&a2)[4], const float (&bv)[6]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      s_d = fmaf(a0[k], bv[k + 1], s_d);
      s_c = fmaf(a1[k], bv[k + 1], s_c);
      s_l = fmaf(a1[k], bv[k], s_l);
      s_r = fmaf(a1[k], bv[k + 2], s_r);
      s_u = fmaf(a2[k], bv[k + 1], s_u);
    }
  };
  // Steps t with b row t + di - 1 inside b's window; a rows t - 1 and t - 2
  // enter as zeros where they are above the window, a row t below it.
  const int t0 = max(0, 1 - di), t1 = min(SS + 2, SS + 1 - di), tm = min(t1, SS);
  float a1[4] = {0.f, 0.f, 0.f, 0.f}, a2[4] = {0.f, 0.f, 0.f, 0.f};
  if (t0 >= 1 && t0 - 1 < SS) load_a(fa + (t0 - 1) * width, a1);
  if (t0 >= 2 && t0 - 2 < SS) load_a(fa + (t0 - 2) * width, a2);
  int t = t0;
  const P* ra = fa + t0 * width;
  const P* rb = fb + (t0 + di - 1) * width;
  for (; t + R <= tm; t += R, ra += R * width, rb += R * width) {
    float av[R][4], bv[R][6];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      load_a(ra + k * width, av[k]);
      load_b(rb + k * width, bv[k]);
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
      step(av[k], a1, a2, bv[k]);
#pragma unroll
      for (int e = 0; e < 4; ++e) a2[e] = a1[e], a1[e] = av[k][e];
    }
  }
  for (; t < t1; ++t, ra += width, rb += width) {
    float a0[4] = {0.f, 0.f, 0.f, 0.f}, bv[6];
    if (t < SS) load_a(ra, a0);
    load_b(rb, bv);
    step(a0, a1, a2, bv);
#pragma unroll
    for (int e = 0; e < 4; ++e) a2[e] = a1[e], a1[e] = a0[e];
  }
  // Stencil sums: c (di, dj), cd (di - 1), cu (di + 1), cl (dj - 1), cr (dj + 1).
  float c5[5] = {s_c, s_d, s_u, s_l, s_r};
  group_sum<G, 5>(c5);
  if (!ok || x != 0 || !in_bounds(loc >= 0 && loc < (long long)q->n_pairs * q->m * q->n)) return;
  float isp = (float)pi_, jsp = (float)pj;
  if (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1)
    subpixel_fit(a.subpixel, pi_, pj, c5[0], c5[1], c5[2], c5[3], c5[4], isp, jsp);
  reinterpret_cast<float*>(q->u)[loc] = sub_rn(jsp, (float)HN);
  reinterpret_cast<float*>(q->v)[loc] = sub_rn(isp, (float)HN);
}

template <int SS, typename P>
__global__ void __launch_bounds__(kRefineThreads, 3) k_refine(CorrArgs a) {
  constexpr int G = SS / kCols, WPB = kRefineThreads / G;
  __shared__ CorrSeg seg_s[kMaxCorrSegs];
  const int n_seg = load_segments(a, seg_s);
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  const int wl = threadIdx.x / G, x = threadIdx.x % G;
  // The loop bound is the same for every thread of the block (group sums).
  for (long long g0 = (long long)blockIdx.x * WPB; g0 < total; g0 += (long long)gridDim.x * WPB) {
    const long long g = g0 + wl;
    refine_window<SS, P>(a, seg_s, n_seg, g, g < total, x);
  }
}

template <int SS>
int launch_refine_ss(const CorrArgs& a, cudaStream_t stream) {
  constexpr int G = SS / kCols, WPB = kRefineThreads / G;
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  long long blocks = (total + WPB - 1) / WPB;
  const long long cap = (long long)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  switch (a.pixel_type) {
    case PIV_PIXEL_U8: k_refine<SS, uint8_t><<<(unsigned)blocks, kRefineThreads, 0, stream>>>(a); break;
    case PIV_PIXEL_U16: k_refine<SS, uint16_t><<<(unsigned)blocks, kRefineThreads, 0, stream>>>(a); break;
    case PIV_PIXEL_F32: k_refine<SS, float><<<(unsigned)blocks, kRefineThreads, 0, stream>>>(a); break;
    default: return set_error(PIV_E_UNSUPPORTED, "peak refinement of float64 frames");
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_refine launch");
}

__global__ void k_compact_ties(const uint8_t* __restrict__ flags, long long windows, int* __restrict__ list,
                               int* __restrict__ count) {
  for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < windows;
       g += (long long)gridDim.x * blockDim.x)
    if (flags[g]) list[atomicAdd(count, 1)] = (int)g;
}

}  // namespace

PIV_DEFINE_BOUNDS_COUNTER(bounds_violations_refine)

int compact_near_ties(const uint8_t* near_tie, long long windows, int* list, int* count, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), stream);
  if (e != cudaSuccess) return set_cuda_error(e, "near-tie list count");
  if (windows == 0) return PIV_OK;
  long long blocks = (windows + 255) / 256;
  if (blocks > (long long)sm_count() * 4) blocks = (long long)sm_count() * 4;
  k_compact_ties<<<(unsigned)blocks, 256, 0, stream>>>(near_tie, windows, list, count);
  e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_compact_ties launch");
}

bool refine_supported(const CorrArgs& a) {
  return a.dtype == PIV_DTYPE_F32 && a.s2n == nullptr && a.ws == a.ss && a.fft_size == 2 * a.ss &&
         (a.ss == 16 || a.ss == 32 || a.ss == 64) && a.pixel_type != PIV_PIXEL_F64;
}

int refine_peaks(const CorrArgs& a, cudaStream_t stream) {
  if (!refine_supported(a)) return set_error(PIV_E_UNSUPPORTED, "peak refinement: unsupported pass");
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  if (total == 0) return PIV_OK;
  if (a.n_segs == 0 && (!a.peak_i || !a.peak_j)) return set_error(PIV_E_ARG, "peak refinement needs the peaks");
  for (int k = 0; k < a.n_segs; ++k)
    if (!a.segs[k].peak_i || !a.segs[k].peak_j) return set_error(PIV_E_ARG, "peak refinement needs the peaks");
  switch (a.ss) {
    case 16: return launch_refine_ss<16>(a, stream);
    case 32: return launch_refine_ss<32>(a, stream);
    default: return launch_refine_ss<64>(a, stream);
  }
}

}  // namespace piv
