// Fused window-pair cross-correlation kernel (plain form: in-shared-memory
// FFT), templated on its launch configuration; instantiated for the float
// configurations in piv_correlate.cu and the double ones in
// piv_correlate_f64.cu.
//
// One CTA owns WPC window pairs at a time (persistent loop over tiles). Per
// window pair it: gathers the ss x ss windows of frames A and B, removes their
// means, packs z = a + i b into the centre of an N x N complex buffer (the
// reference's centred zero pad, gpu_process.py:1222-1235), runs one 2-D FFT
// (rows of the non-zero band only, then all columns), forms
// P = conj(A) B with A, B separated from Z by Hermitian symmetry, runs the
// inverse 2-D FFT, scales by 1/N^2 and reads the real part through the
// fftshift index map (gpu_process.py:1218). Lags without window overlap read
// as exact zeros for the peak search and fit. It then finds the first maximum
// in row-major shifted order (gpu_process.py:1248-1254), fits the subpixel
// peak (gpu_process.py:1256-1294), writes the displacement
// (gpu_process.py:1296-1310) and, when asked, the signal-to-noise ratio
// (gpu_process.py:1312-1365).
#pragma once

#include <math.h>
#include <stdio.h>

#include <algorithm>

#include "piv_fft.cuh"
#include "piv_internal.h"
#include "twiddles.h"

namespace piv {

// One launch configuration (tile shape and radix split) of the FFT
// correlation: each length-N line transform runs as R1 x R2 (four-step, R1 = 1:
// one register DFT of N points), WPC window pairs per CTA, NT threads per CTA.
template <int N_, typename T_, int R1_, int R2_, int WPC_, int NT_>
struct FftCfg {
  using T = T_;
  static constexpr int N = N_, R1 = R1_, R2 = R2_, WPC = WPC_, NT = NT_;
  static_assert(R1 * R2 == N, "R1 * R2 must equal N");
  static_assert(NT % 32 == 0 && NT <= 1024, "whole warps, at most 1024 threads");
  static_assert(WPC >= NT / 32 || (NT / 32) % WPC == 0, "windows must split the warps evenly");
};

template <class C>
struct FftLayout {
  using T = typename C::T;
  static constexpr int N = C::N;
  static constexpr int LD = N + 1;                     // padded row length (complex elements)
  static constexpr int WIN = N * LD;                   // complex elements per window
  static constexpr int WPC = C::WPC;
  static constexpr int NT = C::NT;
  static constexpr int NW = NT / 32;
  static constexpr size_t TW_BYTES = 256 * sizeof(Cplx<T>);
  static constexpr int PART = 2 * NW + WPC;            // per-warp / per-slot partial results
  static constexpr size_t RED_BYTES = WPC * sizeof(long long) + PART * (sizeof(T) + sizeof(int)) +
                                      4 * WPC * sizeof(T) + 8 * WPC * sizeof(int);
  static constexpr size_t BUF_BYTES = (size_t)WPC * WIN * sizeof(Cplx<T>);
  static constexpr size_t SMEM_SMALL = TW_BYTES + ((RED_BYTES + 15) / 16) * 16;
  static constexpr bool GLOBAL_BUF = (SMEM_SMALL + BUF_BYTES) > 200 * 1024;
  static constexpr size_t SMEM = GLOBAL_BUF ? SMEM_SMALL : SMEM_SMALL + BUF_BYTES;
};

template <typename T>
PIV_D bool argmax_better(T v1, int i1, T v2, int i2) {
  const bool n1 = is_nan(v1), n2 = is_nan(v2);
  if (n1 != n2) return n1;
  if (n1) return i1 < i2;
  if (v1 != v2) return v1 > v2;
  return i1 < i2;
}

template <typename T>
PIV_D void warp_argmax(T& v, int& i) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    T v2 = __shfl_xor_sync(0xffffffffu, v, off);
    int i2 = __shfl_xor_sync(0xffffffffu, i, off);
    if (argmax_better(v2, i2, v, i)) { v = v2; i = i2; }
  }
}

// warp_argmax that also carries the second-largest value `s` (the largest
// value at any other position): merging (v, i, s) with (v2, i2, s2), the
// loser's best competes with the winner's second.
template <typename T>
PIV_D void warp_argmax2(T& v, int& i, T& s) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const T v2 = __shfl_xor_sync(0xffffffffu, v, off);
    const int i2 = __shfl_xor_sync(0xffffffffu, i, off);
    const T s2 = __shfl_xor_sync(0xffffffffu, s, off);
    if (argmax_better(v2, i2, v, i)) {
      s = s2 > v ? s2 : v;
      v = v2;
      i = i2;
    } else if (v2 > s) {
      s = v2;
    }
  }
}

template <typename T>
PIV_D T warp_sum(T v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// Transform output at shifted position (i, j) (natural buffer position
// (i ^ N/2, j ^ N/2)).
template <int N, typename T>
PIV_D T corr_raw(const Cplx<T>* w, int i, int j) {
  return w[(i ^ (N / 2)) * (N + 1) + (j ^ (N / 2))].x;
}

// Correlation map value at shifted position (i, j). Lags |d| >= ss have no
// window overlap: their exact value is zero while an FFT leaves rounding noise
// of either sign there, so they read as 0. This keeps the peak search and the
// Gaussian fit's positivity test independent of that noise.
template <int N, typename T>
PIV_D T corr_at(const Cplx<T>* w, int i, int j, int ss) {
  const int di = i - N / 2, dj = j - N / 2;
  if (di <= -ss || di >= ss || dj <= -ss || dj >= ss) return (T)0;
  return corr_raw<N, T>(w, i, j);
}

// Block-wide argmax per window over the shifted map, optionally excluding a
// box of half width `box` (wrapped modulo N) around (bi[w], bj[w]). Results in
// out_v[w], out_i[w]; with out_s (part_s then holds one value per warp), also
// the second-largest value out_s[w], the largest at any other position. All
// threads must call.
template <class C, int N = C::N, typename T = typename C::T>
PIV_D void window_argmax(const Cplx<T>* buf, int ss, int box, const int* bi, const int* bj, T* part_v,
                         int* part_i, T* out_v, int* out_i, T* part_s = nullptr, T* out_s = nullptr) {
  using L = FftLayout<C>;
  constexpr int WPC = L::WPC, NW = L::NW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if constexpr (WPC >= NW) {
    for (int w = warp; w < WPC; w += NW) {
      const Cplx<T>* wb = buf + w * L::WIN;
      T bv = -INFINITY, sv = -INFINITY;
      int bidx = 0x7fffffff;
      for (int f = lane; f < N * N; f += 32) {
        const int i = f / N, j = f % N;
        if (box >= 0) {
          int di = (i - bi[w]) & (N - 1), dj = (j - bj[w]) & (N - 1);
          if (di > N / 2) di -= N;
          if (dj > N / 2) dj -= N;
          if (di >= -box && di <= box && dj >= -box && dj <= box) continue;
        }
        T v = corr_at<N, T>(wb, i, j, ss);
        if (argmax_better(v, f, bv, bidx)) { sv = bv; bv = v; bidx = f; }
        else if (v > sv) sv = v;
      }
      if (out_s) warp_argmax2(bv, bidx, sv);
      else warp_argmax(bv, bidx);
      if (lane == 0) {
        out_v[w] = bv;
        out_i[w] = bidx;
        if (out_s) out_s[w] = sv;
      }
    }
    __syncthreads();
  } else {
    constexpr int WPW = NW / WPC;  // warps per window
    const int w = warp / WPW, sub = warp % WPW;
    const Cplx<T>* wb = buf + w * L::WIN;
    constexpr int CHUNK = N * N / WPW;
    T bv = -INFINITY, sv = -INFINITY;
    int bidx = 0x7fffffff;
    for (int f = sub * CHUNK + lane; f < (sub + 1) * CHUNK; f += 32) {
      const int i = f / N, j = f % N;
      if (box >= 0) {
        int di = (i - bi[w]) & (N - 1), dj = (j - bj[w]) & (N - 1);
        if (di > N / 2) di -= N;
        if (dj > N / 2) dj -= N;
        if (di >= -box && di <= box && dj >= -box && dj <= box) continue;
      }
      T v = corr_at<N, T>(wb, i, j, ss);
      if (argmax_better(v, f, bv, bidx)) { sv = bv; bv = v; bidx = f; }
      else if (v > sv) sv = v;
    }
    if (out_s) warp_argmax2(bv, bidx, sv);
    else warp_argmax(bv, bidx);
    if (lane == 0) {
      part_v[warp] = bv;
      part_i[warp] = bidx;
      if (out_s) part_s[warp] = sv;
    }
    __syncthreads();
    if (threadIdx.x < WPC) {
      const int ww = threadIdx.x;
      T v = part_v[ww * WPW];
      int i = part_i[ww * WPW];
      T s2 = out_s ? part_s[ww * WPW] : (T)-INFINITY;
      for (int s = 1; s < WPW; ++s) {
        const T pv = part_v[ww * WPW + s];
        if (argmax_better(pv, part_i[ww * WPW + s], v, i)) {
          if (out_s) s2 = fmax(part_s[ww * WPW + s], v);
          v = pv;
          i = part_i[ww * WPW + s];
        } else if (out_s) {
          s2 = fmax(s2, pv);
        }
      }
      out_v[ww] = v;
      out_i[ww] = i;
      if (out_s) out_s[ww] = s2;
    }
    __syncthreads();
  }
  // A map with every entry excluded keeps index 0 (the reference's argmax of
  // an all -inf map).
  if (threadIdx.x < WPC && out_i[threadIdx.x] == 0x7fffffff) out_i[threadIdx.x] = 0;
  __syncthreads();
}

// Mean of the map values v with v > 0 and, when limit[w] is not NaN, v <= limit[w].
template <class C, int N = C::N, typename T = typename C::T>
PIV_D void window_positive_mean(const Cplx<T>* buf, const T* limit, T* part_v, int* part_i, T* out_mean) {
  using L = FftLayout<C>;
  constexpr int WPC = L::WPC, NW = L::NW;
  constexpr int WPW = WPC >= NW ? 1 : NW / WPC;  // warps per window
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int CHUNK = N * N / WPW;
  for (int slot = warp; slot < WPC * WPW; slot += NW) {
    const int w = slot / WPW, sub = slot % WPW;
    const Cplx<T>* wb = buf + w * L::WIN;
    const T lim = limit[w];
    T s = 0;
    int c = 0;
    for (int f = sub * CHUNK + lane; f < (sub + 1) * CHUNK; f += 32) {
      // Raw transform values, as the reference's estimator sees them.
      const T v = corr_raw<N, T>(wb, f / N, f % N);
      if (v > (T)0 && (is_nan(lim) || !(v > lim))) { s += v; ++c; }
    }
    s = warp_sum(s);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    if (lane == 0) { part_v[slot] = s; part_i[slot] = c; }
  }
  __syncthreads();
  if (threadIdx.x < WPC) {
    const int w = threadIdx.x;
    T s = 0;
    int c = 0;
    for (int k = 0; k < WPW; ++k) { s += part_v[w * WPW + k]; c += part_i[w * WPW + k]; }
    out_mean[w] = c > 0 ? s / (T)c : (T)NAN;
  }
  __syncthreads();
}

template <class C, int N = C::N, typename T = typename C::T>
__global__ void __launch_bounds__(C::NT) k_corr_fft(CorrArgs a, Cplx<T>* gbuf) {
  using L = FftLayout<C>;
  constexpr int R1 = C::R1, R2 = C::R2, WPC = C::WPC, NT = C::NT, NW = L::NW, LD = L::LD;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Cplx<T>* tw = reinterpret_cast<Cplx<T>*>(smem_raw);
  unsigned char* red = smem_raw + L::TW_BYTES;
  long long* win_base = reinterpret_cast<long long*>(red);  // [WPC] element offset of each window's corner
  T* part_v = reinterpret_cast<T*>(red + WPC * sizeof(long long));
  T* win_v = part_v + L::PART;         // 4 * WPC values
  int* part_i = reinterpret_cast<int*>(win_v + 4 * WPC);
  int* win_i = part_i + L::PART;       // 8 * WPC ints
  Cplx<T>* buf = L::GLOBAL_BUF ? gbuf + (size_t)blockIdx.x * WPC * L::WIN
                               : reinterpret_cast<Cplx<T>*>(smem_raw + L::SMEM_SMALL);
  const int tid = threadIdx.x;

  for (int k = tid; k < 256; k += NT) {
    if constexpr (sizeof(T) == 4) {
      float2 w = c_tw256_f[k];
      tw[k] = cmake<T>(w.x, w.y);
    } else {
      double2 w = c_tw256_d[k];
      tw[k] = cmake<T>(w.x, w.y);
    }
  }

  const int ss = a.ss, pad = (N - ss) / 2, sp = a.spacing, nf = a.n;
  const int n_wins = a.m * a.n;
  // A window list selects the windows (slot s -> window win_list[s]).
  const long long total = a.win_list ? (long long)*a.win_count : (long long)a.n_pairs * n_wins;
  const int n_tiles = (int)((total + WPC - 1) / WPC);
  auto win_id = [&](long long slot) -> long long { return a.win_list ? (long long)a.win_list[slot] : slot; };
  const long long frame_elems = (long long)a.height * a.width;
  const int inner0 = (a.ss - a.ws) / 2, inner1 = a.ss - inner0;  // shrink: A's window rows/cols
  const bool normalize = a.normalize || pad != 0;
  const T inv_nn = (T)1 / (T)(N * N);
  T* means = win_v;       // [2*WPC]: mean_a, mean_b
  int* peak = win_i;      // [WPC]: flat peak index
  int* pi = win_i + WPC;  // [WPC]
  int* pj = win_i + 2 * WPC;
  T* pval = win_v + 2 * WPC;  // [WPC]
  int* valid = win_i + 3 * WPC;

  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const long long g0 = (long long)tile * WPC;
    __syncthreads();
    if (tid < WPC) {
      int ok = g0 + tid < total;
      const long long g = ok ? win_id(g0 + tid) : 0;
      long long base = 0;
      if (ok) {
        const int pair = (int)(g / n_wins), k = (int)(g % n_wins);
        if (a.win_mask) ok = a.win_mask[k] == 0;
        base = pair * frame_elems + (long long)((k / nf) * sp + a.y_offset) * a.width + (k % nf) * sp + a.x_offset;
      }
      valid[tid] = ok;
      win_base[tid] = base;
    }
    __syncthreads();

    // Window means (gpu_process.py:1201-1205); shrink: A over its inner window.
    // Pixel loads are specialised on the pixel type outside the loops.
    auto fill = [&](auto tag) {
      using P = decltype(tag);
      const P* fa = reinterpret_cast<const P*>(a.frame_a);
      const P* fb = reinterpret_cast<const P*>(a.frame_b);
      if (normalize) {
        for (int w = 0; w < WPC; ++w) {
          T sa = 0, sb = 0;
          if (valid[w]) {
            const long long base = win_base[w];
            for (int e = tid; e < ss * ss; e += NT) {
              const int r = e / ss, c = e % ss;
              const long long idx = base + (long long)r * a.width + c;
              if (r >= inner0 && r < inner1 && c >= inner0 && c < inner1) sa += (T)__ldg(fa + idx);
              sb += (T)__ldg(fb + idx);
            }
          }
          sa = warp_sum(sa);
          sb = warp_sum(sb);
          if ((tid & 31) == 0) { part_v[tid >> 5] = sa; part_v[NW + (tid >> 5)] = sb; }
          __syncthreads();
          if (tid == 0) {
            T ta = 0, tb = 0;
            for (int q = 0; q < NW; ++q) { ta += part_v[q]; tb += part_v[NW + q]; }
            const int wa = inner1 - inner0;
            means[2 * w] = ta / (T)(wa * wa);
            means[2 * w + 1] = tb / (T)(ss * ss);
          }
          __syncthreads();
        }
      }
      // Fill the N x N buffers: z = (a - mean_a) + i (b - mean_b) in the centre, 0 elsewhere.
      for (int e = tid; e < WPC * N * N; e += NT) {
        const int w = e / (N * N), rc = e % (N * N), r = rc / N - pad, c = rc % N - pad;
        Cplx<T> z = cmake<T>(0, 0);
        if (valid[w] && r >= 0 && r < ss && c >= 0 && c < ss) {
          const long long idx = win_base[w] + (long long)r * a.width + c;
          T va = 0;
          if (r >= inner0 && r < inner1 && c >= inner0 && c < inner1) {
            va = (T)__ldg(fa + idx);
            if (normalize) va = va - means[2 * w];
          }
          T vb = (T)__ldg(fb + idx);
          if (normalize) vb = vb - means[2 * w + 1];
          z = cmake<T>(va, vb);
        }
        buf[w * L::WIN + (rc / N) * LD + (rc % N)] = z;
      }
    };
    switch (a.pixel_type) {
      case PIV_PIXEL_U8: fill(uint8_t{}); break;
      case PIV_PIXEL_U16: fill(uint16_t{}); break;
      case PIV_PIXEL_F32: fill(float{}); break;
      default: fill(double{}); break;
    }
    __syncthreads();

    // Forward 2-D FFT: rows of the non-zero band, then all columns.
    auto row_band = [&](int l) { return (l / ss) * L::WIN + (pad + l % ss) * LD; };
    auto row_all = [&](int l) { return (l / N) * L::WIN + (l % N) * LD; };
    auto col_all = [&](int l) { return (l / N) * L::WIN + (l % N); };
    fft_pass_a<N, R1, R2, false, T>(buf, WPC * ss, row_band, 1, tw, tid, NT);
    __syncthreads();
    if constexpr (R1 > 1) {
      fft_pass_b<N, R1, R2, false, T>(buf, WPC * ss, row_band, 1, tw, tid, NT);
      __syncthreads();
    }
    fft_pass_a<N, R1, R2, false, T>(buf, WPC * N, col_all, LD, tw, tid, NT);
    __syncthreads();
    if constexpr (R1 > 1) {
      fft_pass_b<N, R1, R2, false, T>(buf, WPC * N, col_all, LD, tw, tid, NT);
      __syncthreads();
    }

    // P = conj(A) * B with A = (Z_k + conj(Z_-k)) / 2, B = (Z_k - conj(Z_-k)) / 2i.
    for (int e = tid; e < WPC * N * N; e += NT) {
      const int w = e / (N * N), rc = e % (N * N), pr = rc / N, pc = rc % N;
      const int fr = fft_freq_of_pos<R1, R2>(pr), fc = fft_freq_of_pos<R1, R2>(pc);
      const int qr = fft_pos_of_freq<R1, R2>((N - fr) & (N - 1));
      const int qc = fft_pos_of_freq<R1, R2>((N - fc) & (N - 1));
      const int q = qr * N + qc;
      if (q < rc) continue;
      Cplx<T>* wb = buf + w * L::WIN;
      const Cplx<T> zk = wb[pr * LD + pc];
      const Cplx<T> zm = wb[qr * LD + qc];
      // 2A = zk + conj(zm), 2B = ((zk.y + zm.y), (zm.x - zk.x)) with conj(zm) = (zm.x, -zm.y)
      const T ar = zk.x + zm.x, ai = zk.y - zm.y;
      const T br = zk.y + zm.y, bi = zm.x - zk.x;
      const T q4 = (T)0.25;
      const T pr_ = (ar * br + ai * bi) * q4;
      const T pi_ = (ar * bi - ai * br) * q4;
      wb[pr * LD + pc] = cmake<T>(pr_, pi_);
      if (q != rc) wb[qr * LD + qc] = cmake<T>(pr_, -pi_);
    }
    __syncthreads();

    // Inverse 2-D FFT (columns, then rows) back to natural order.
    if constexpr (R1 > 1) {
      fft_pass_b<N, R1, R2, true, T>(buf, WPC * N, col_all, LD, tw, tid, NT);
      __syncthreads();
    }
    fft_pass_a<N, R1, R2, true, T>(buf, WPC * N, col_all, LD, tw, tid, NT);
    __syncthreads();
    if constexpr (R1 > 1) {
      fft_pass_b<N, R1, R2, true, T>(buf, WPC * N, row_all, 1, tw, tid, NT);
      __syncthreads();
    }
    fft_pass_a<N, R1, R2, true, T>(buf, WPC * N, row_all, 1, tw, tid, NT);
    __syncthreads();
    // Scale by 1/N^2 (irfft2).
    for (int e = tid; e < WPC * N * N; e += NT) {
      const int w = e / (N * N), rc = e % (N * N);
      Cplx<T>& z = buf[w * L::WIN + (rc / N) * LD + (rc % N)];
      z.x = z.x * inv_nn;
    }
    __syncthreads();

    if (a.maps) {
      T* mo = reinterpret_cast<T*>(a.maps);
      for (int e = tid; e < WPC * N * N; e += NT) {
        const int w = e / (N * N), f = e % (N * N);
        if (g0 + w < total) mo[win_id(g0 + w) * N * N + f] = corr_at<N, T>(buf + w * L::WIN, f / N, f % N, ss);
      }
    }

    // First peak (first occurrence in row-major order of the shifted map) and,
    // for the near-tie test, the second-largest value (into the slots of the
    // window means, which the fill no longer needs).
    const bool ties = a.near_tie || a.tie_count;
    T* second = means;
    window_argmax<C>(buf, ss, -1, nullptr, nullptr, part_v, part_i, pval, peak, part_v + NW,
                     ties ? second : nullptr);
    if (tid < WPC) {
      pi[tid] = peak[tid] / N;
      pj[tid] = peak[tid] % N;
    }
    __syncthreads();

    // Subpixel fit and displacement.
    if (tid < WPC && g0 + tid < total) {
      const int w = tid;
      const long long g = win_id(g0 + w);
      const Cplx<T>* wb = buf + w * L::WIN;
      const int i = pi[w], j = pj[w];
      T isp = (T)i, jsp = (T)j;
      if (i > 0 && i < N - 1 && j > 0 && j < N - 1) {
        T c = corr_at<N, T>(wb, i, j, ss);
        T cd = corr_at<N, T>(wb, i - 1, j, ss), cu = corr_at<N, T>(wb, i + 1, j, ss);
        T cl = corr_at<N, T>(wb, i, j - 1, ss), cr = corr_at<N, T>(wb, i, j + 1, ss);
        const T eps = (T)1e-7;
        const T half = (T)0.5, two = (T)2;
        if (a.subpixel == PIV_SUBPIXEL_GAUSSIAN) {
          if (c > 0 && cd > 0 && cu > 0 && cl > 0 && cr > 0) {
            c = log(c); cd = log(cd); cu = log(cu); cl = log(cl); cr = log(cr);
            T di = div_rn(mul_rn(half, sub_rn(cd, cu)), add_rn(add_rn(sub_rn(cd, mul_rn(two, c)), cu), eps));
            T dj = div_rn(mul_rn(half, sub_rn(cl, cr)), add_rn(add_rn(sub_rn(cl, mul_rn(two, c)), cr), eps));
            isp = add_rn((T)i, di);
            jsp = add_rn((T)j, dj);
          }
        } else if (a.subpixel == PIV_SUBPIXEL_PARABOLIC) {
          T di = div_rn(mul_rn(half, sub_rn(cd, cu)), add_rn(add_rn(sub_rn(cd, mul_rn(two, c)), cu), eps));
          T dj = div_rn(mul_rn(half, sub_rn(cl, cr)), add_rn(add_rn(sub_rn(cl, mul_rn(two, c)), cr), eps));
          isp = add_rn((T)i, di);
          jsp = add_rn((T)j, dj);
        } else {
          T di = div_rn(sub_rn(cu, cd), add_rn(add_rn(add_rn(cd, c), cu), eps));
          T dj = div_rn(sub_rn(cr, cl), add_rn(add_rn(add_rn(cl, c), cr), eps));
          isp = add_rn((T)i, di);
          jsp = add_rn((T)j, dj);
        }
      }
      T* uo = reinterpret_cast<T*>(a.u);
      T* vo = reinterpret_cast<T*>(a.v);
      if (valid[w]) {
        uo[g] = sub_rn(jsp, (T)(N / 2));
        vo[g] = sub_rn(isp, (T)(N / 2));
      } else {
        uo[g] = (T)NAN;
        vo[g] = (T)NAN;
      }
      if (a.peak_i) a.peak_i[g] = i;
      if (a.peak_j) a.peak_j[g] = j;
      if (ties) {
        const T best = pval[w], gap = best - second[w];
        const bool tie = valid[w] && !(gap > (T)a.tie_tol * (best < 0 ? -best : best));
        if (a.near_tie) a.near_tie[g] = tie ? 1 : 0;
        if (tie && a.tie_count) atomicAdd(a.tie_count, 1);
      }
    }

    // Signal-to-noise ratio.
    if (a.s2n) {
      T* p2 = win_v + 3 * WPC;  // [WPC]
      if (a.s2n_method == PIV_S2N_PEAK2PEAK) {
        int* peak2 = win_i + 4 * WPC;
        window_argmax<C>(buf, ss, a.s2n_size, pi, pj, part_v, part_i, p2, peak2);
        if (tid < WPC) {
          // The reference reads the second peak value from its masked map: a
          // value inside the excluded box reads -inf.
          const int i2 = peak2[tid] / N, j2 = peak2[tid] % N;
          int di = (i2 - pi[tid]) & (N - 1), dj = (j2 - pj[tid]) & (N - 1);
          if (di > N / 2) di -= N;
          if (dj > N / 2) dj -= N;
          const bool inside = di >= -a.s2n_size && di <= a.s2n_size && dj >= -a.s2n_size && dj <= a.s2n_size;
          p2[tid] = inside ? (T)-INFINITY : corr_at<N, T>(buf + tid * L::WIN, i2, j2, ss);
        }
      } else {
        // peak2mean / peak2energy: mean of the positive map values, excluding
        // values above half the first peak for peak2mean (gpu_process.py:1325-1330).
        T* limit = means;  // the window means are no longer needed
        if (tid < WPC) limit[tid] = a.s2n_method == PIV_S2N_PEAK2MEAN ? (T)0.5 * pval[tid] : (T)NAN;
        __syncthreads();
        window_positive_mean<C>(buf, limit, part_v, part_i, p2);
      }
      __syncthreads();
      if (tid < WPC && g0 + tid < total) {
        const long long g = win_id(g0 + tid);
        const T p1 = pval[tid], q2 = p2[tid];
        T s = 0;
        if (valid[tid]) {
          if (p1 > 0) s = p1 / q2;
          if (q2 <= 0 && p1 > 0) s = (T)INFINITY;
        }
        reinterpret_cast<T*>(a.s2n)[g] = s;
      }
    }
  }
}

// CTAs of a correlation whose buffers live in global memory.
static constexpr int kGlobalBufCtas = 304;

template <class C>
static int launch_corr_fft(const CorrArgs& a, cudaStream_t stream) {
  using L = FftLayout<C>;
  using T = typename C::T;
  const long long total = (long long)a.n_pairs * a.m * a.n;
  if (total == 0) return PIV_OK;
  const int n_tiles = (int)((total + L::WPC - 1) / L::WPC);
  static thread_local int configured_dev = -1;
  static thread_local int per_sm = 1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured_dev != dev) {
    cudaError_t e = cudaFuncSetAttribute(k_corr_fft<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::SMEM);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaFuncSetAttribute(k_corr_fft)");
    per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_corr_fft<C>, L::NT, L::SMEM);
    if (per_sm < 1) per_sm = 1;
    configured_dev = dev;
  }
  int grid = sm_count() * per_sm;
  if (grid > n_tiles) grid = n_tiles;
  Cplx<T>* gbuf = nullptr;
  if (L::GLOBAL_BUF) {
    if (grid > kGlobalBufCtas) grid = kGlobalBufCtas;
    const size_t bytes = (size_t)grid * L::WPC * L::WIN * sizeof(Cplx<T>);
    if (!a.scratch || a.scratch_bytes < bytes)
      return set_error(PIV_E_ARG, "correlation with fft_size %d needs %zu bytes of device scratch", C::N, bytes);
    gbuf = reinterpret_cast<Cplx<T>*>(a.scratch);
  }
  CorrArgs b = a;
  b.tie_tol = sizeof(T) == 8 ? kTieTolF64 : kTieTolF32;
  k_corr_fft<C><<<grid, L::NT, L::SMEM, stream>>>(b, gbuf);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_cuda_error(e, "k_corr_fft launch");
  return PIV_OK;
}

template <class C>
static size_t scratch_for() {
  using L = FftLayout<C>;
  return L::GLOBAL_BUF ? (size_t)kGlobalBufCtas * L::WPC * L::WIN * sizeof(Cplx<typename C::T>) : 0;
}

// Candidate configurations per (N, float type); entry 0 is the default. The
// autotuner times them on a pass's own windows and keeps the fastest. Every
// entry computes the same map up to rounding (the radix split changes the
// order of the sums).
struct FftVariant {
  int r1, r2, wpc, nt;
  int (*launch)(const CorrArgs&, cudaStream_t);
  size_t (*scratch)();
};
#define PIV_FFT_VAR(N, T, R1, R2, WPC, NT) \
  { R1, R2, WPC, NT, launch_corr_fft<FftCfg<N, T, R1, R2, WPC, NT>>, scratch_for<FftCfg<N, T, R1, R2, WPC, NT>> }

template <size_t K>
static const FftVariant* table(const FftVariant (&t)[K], int* count) {
  *count = (int)K;
  return t;
}

}  // namespace piv
