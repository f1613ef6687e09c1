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
// Work split: a group of ss / 2 threads per window, each thread two columns
// sliding down the rows in chunks of 8 rows loaded together; the window means
// come from the engine (or are summed here), the five sums are reduced over
// the group by warp shuffles.
#include <math.h>

#include "piv_common.cuh"
#include "piv_corr_common.cuh"
#include "piv_internal.h"

namespace piv {

namespace {

constexpr int kRefineThreads = 256;

// Sum of v over the thread's group of G consecutive threads (G a power of two
// dividing the block); every thread of the block must call it. part: K floats
// per warp of the block.
template <int G, int K>
PIV_D void group_sum(float (&v)[K], float* part) {
  constexpr int L = G < 32 ? G : 32;
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if constexpr (G > 32) {
    const int warp = threadIdx.x >> 5;
    __syncthreads();  // the previous group_sum's reads of part[] are done
    if ((threadIdx.x & 31) == 0)
#pragma unroll
      for (int k = 0; k < K; ++k) part[warp * K + k] = v[k];
    __syncthreads();
    const int w0 = (threadIdx.x / G) * (G / 32);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float s = 0.f;
#pragma unroll
      for (int j = 0; j < G / 32; ++j) s += part[(w0 + j) * K + k];
      v[k] = s;
    }
  }
}

// Threads per window G and columns per thread CPT: two columns per thread
// (8, 16 or 32 threads per window) halve the per-window overhead (window
// decode, means, group sums, fit lanes), and keep a 64-px window in one warp
// (its group sum in shuffles alone).
template <int SS>
struct RefineGroup {
  static constexpr int CPT = 2;
  static constexpr int G = SS / CPT;
};

template <typename P>
PIV_D float px(const P* p) {
  return (float)__ldg(p);
}

// One window by a group of SS threads, thread x taking column x of frame a:
// row y of a meets rows y + di - 1, y + di and y + di + 1 of b at column
// x + dj and row y + di at columns x + dj -+ 1, in chunks of 8 rows whose
// values are all loaded before they are used (the loads of a chunk are in
// flight together; consecutive threads read consecutive columns).
template <int SS, typename P>
PIV_D void refine_window(const CorrArgs& a, const CorrSeg* seg_s, int n_seg, long long g, bool active, int x,
                         float* part) {
  constexpr int CPT = RefineGroup<SS>::CPT, G = RefineGroup<SS>::G, HN = SS, N = 2 * SS;
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
  const int width = q->width;
  const P* fa = reinterpret_cast<const P*>(q->frame_a) + (ok ? base : 0);
  const P* fb = reinterpret_cast<const P*>(q->frame_b) + (ok ? base : 0);
  // Window means: written by the engine, or summed here.
  float ma = 0.f, mb = 0.f;
  if (q->win_means) {
    if (ok) {
      ma = q->win_means[2 * loc];
      mb = q->win_means[2 * loc + 1];
    }
  } else {
    float sums[2] = {0.f, 0.f};
    if (ok)
#pragma unroll 1
      for (int c = 0; c < CPT; ++c)
#pragma unroll 4
        for (int y = 0; y < SS; ++y) {
          sums[0] += px<P>(fa + y * width + x + c * G);
          sums[1] += px<P>(fb + y * width + x + c * G);
        }
    group_sum<G, 2>(sums, part);
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
  // Chunks of R rows: every value of a chunk is loaded before any is used,
  // so that the chunk's loads are in flight together; a row's offset and
  // validity serve its three loads.
  constexpr int R = 8;
  float s_c = 0.f, s_d = 0.f, s_u = 0.f, s_l = 0.f, s_r = 0.f;
#pragma unroll
  for (int c = 0; c < CPT; ++c) {
    const int xa = x + c * G, xb = xa + dj;  // this thread's column of a, and of b
    const bool cm = ok && (unsigned)(xb - 1) < (unsigned)SS, c0 = ok && (unsigned)xb < (unsigned)SS,
               cp = ok && (unsigned)(xb + 1) < (unsigned)SS;
    const P* pb = fb + xb;
#pragma unroll 1
    for (int y0 = 0; y0 < SS; y0 += R) {
      float av[R], bc[R + 2], bl[R], br[R];
      const P* pa = fa + y0 * width + xa;
#pragma unroll
      for (int k = 0; k < R; ++k) av[k] = ok ? px<P>(pa + k * width) : 0.f;
#pragma unroll
      for (int k = 0; k < R + 2; ++k) {  // rows y0 + di - 1 .. y0 + di + R
        const int r = y0 + k + di - 1;
        const bool vr = (unsigned)r < (unsigned)SS;
        const P* row = pb + r * width;
        bc[k] = (vr && c0) ? px<P>(row) - mb : 0.f;
        if (k >= 1 && k <= R) {
          bl[k - 1] = (vr && cm) ? px<P>(row - 1) - mb : 0.f;
          br[k - 1] = (vr && cp) ? px<P>(row + 1) - mb : 0.f;
        }
      }
#pragma unroll
      for (int k = 0; k < R; ++k) {
        const float ap = ok ? av[k] - ma : 0.f;
        s_c = fmaf(ap, bc[k + 1], s_c);
        s_d = fmaf(ap, bc[k], s_d);
        s_u = fmaf(ap, bc[k + 2], s_u);
        s_l = fmaf(ap, bl[k], s_l);
        s_r = fmaf(ap, br[k], s_r);
      }
    }
  }
  // Stencil sums: c (di, dj), cd (di - 1), cu (di + 1), cl (dj - 1), cr (dj + 1).
  float c5[5] = {s_c, s_d, s_u, s_l, s_r};
  group_sum<G, 5>(c5, part);
  if (!ok || x != 0 || !in_bounds(loc >= 0 && loc < (long long)q->n_pairs * q->m * q->n)) return;
  float isp = (float)pi_, jsp = (float)pj;
  if (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1)
    subpixel_fit(a.subpixel, pi_, pj, c5[0], c5[1], c5[2], c5[3], c5[4], isp, jsp);
  reinterpret_cast<float*>(q->u)[loc] = sub_rn(jsp, (float)HN);
  reinterpret_cast<float*>(q->v)[loc] = sub_rn(isp, (float)HN);
}

template <int SS, typename P>
__global__ void __launch_bounds__(kRefineThreads, 3) k_refine(CorrArgs a) {
  constexpr int G = RefineGroup<SS>::G, WPB = kRefineThreads / G;
  __shared__ CorrSeg seg_s[kMaxCorrSegs];
  __shared__ float part[kRefineThreads / 32 * 5];
  const int n_seg = load_segments(a, seg_s);
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  const int wl = threadIdx.x / G, x = threadIdx.x % G;
  // The loop bound is the same for every thread of the block (group sums).
  for (long long g0 = (long long)blockIdx.x * WPB; g0 < total; g0 += (long long)gridDim.x * WPB) {
    const long long g = g0 + wl;
    refine_window<SS, P>(a, seg_s, n_seg, g, g < total, x, part);
  }
}

template <int SS>
int launch_refine_ss(const CorrArgs& a, cudaStream_t stream) {
  constexpr int G = RefineGroup<SS>::G, WPB = kRefineThreads / G;
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
