// In-shared-memory power-of-two FFT building blocks.
//
// A length-N line transform is split as N = R1 * R2 (four-step): pass A does
// R2-point DFTs over n2 of x[n1 + R1 n2] and applies the twiddle W_N^(n1 k2);
// pass B does R1-point DFTs over n1. Each small DFT runs in registers. The
// forward transform leaves frequency k2 + R2 k1 at position k1 + R1 k2
// (digit-reversed); the inverse transform reads that order and returns the
// natural order, so a forward/inverse pair never needs a reordering pass. Each
// thread reads and writes the same set of positions within a pass, so passes
// are separated by one __syncthreads() and need no second buffer.
#pragma once

#include <utility>

#include "piv_common.cuh"

namespace piv {

template <int R>
PIV_HD constexpr int bitrev(int i) {
  int r = 0;
  for (int b = 1; b < R; b <<= 1) {
    r = (r << 1) | (i & 1);
    i >>= 1;
  }
  return r;
}

// Radix-2 decimation-in-time DFT of R points held in registers, natural order
// in and out. `tw` is the W_256 table (W_256^k = exp(-2 pi i k/256)); INV uses
// conjugate twiddles and does not scale.
template <int R, typename T, int... I>
PIV_D void bitrev_permute(Cplx<T> (&y)[R], const Cplx<T> (&x)[R], std::integer_sequence<int, I...>) {
  ((y[bitrev<R>(I)] = x[I]), ...);
}

// One radix-2 stage (butterfly span LEN) of the register DFT, then the next.
template <int R, int LEN, bool INV, typename T>
PIV_D void dft_stage(Cplx<T> (&y)[R], const Cplx<T>* __restrict__ tw) {
#pragma unroll
  for (int i = 0; i < R; i += LEN) {
#pragma unroll
    for (int j = 0; j < LEN / 2; ++j) {
      Cplx<T> a = y[i + j];
      Cplx<T> b = y[i + j + LEN / 2];
      if (j != 0) {
        if (LEN >= 4 && j == LEN / 4) {
          // W = -i (forward) or +i (inverse): exact.
          b = INV ? cmake<T>(-b.y, b.x) : cmake<T>(b.y, -b.x);
        } else {
          Cplx<T> w = tw[j * (256 / LEN)];
          if (INV) w.y = -w.y;
          b = cmul(b, w);
        }
      }
      y[i + j] = cadd(a, b);
      y[i + j + LEN / 2] = csub(a, b);
    }
  }
  if constexpr (LEN < R) dft_stage<R, 2 * LEN, INV, T>(y, tw);
}

template <int R, bool INV, typename T>
PIV_D void dft_reg(Cplx<T> (&x)[R], const Cplx<T>* __restrict__ tw) {
  static_assert(R >= 1 && R <= 32 && (R & (R - 1)) == 0, "radix must be a power of two <= 32");
  if constexpr (R > 1) {
    Cplx<T> y[R];
    bitrev_permute<R, T>(y, x, std::make_integer_sequence<int, R>{});
    dft_stage<R, 2, INV, T>(y, tw);
#pragma unroll
    for (int i = 0; i < R; ++i) x[i] = y[i];
  }
}

// W_N^e (or its conjugate) from the W_256 table.
template <int N, bool INV, typename T>
PIV_D Cplx<T> twiddle(const Cplx<T>* __restrict__ tw, int e) {
  Cplx<T> w = tw[(e & (N - 1)) * (256 / N)];
  if (INV) w.y = -w.y;
  return w;
}

// Pass A over n_lines lines. Forward: R2-point DFT then twiddle. Inverse:
// conjugate twiddle then R2-point inverse DFT. line_off(l) gives the offset of
// line l, es the element stride.
template <int N, int R1, int R2, bool INV, typename T, class LineOff>
PIV_D void fft_pass_a(Cplx<T>* buf, int n_lines, LineOff line_off, int es, const Cplx<T>* tw, int tid, int nt) {
  // Line index fastest: a warp's lanes touch 32 lines at the same in-line
  // position (row lines are N+1 elements apart, an odd count, so 8-byte
  // accesses are bank-conflict free; column lines are adjacent).
  for (int it = tid; it < n_lines * R1; it += nt) {
    const int l = it % n_lines;
    const int n1 = it / n_lines;
    Cplx<T>* p = buf + line_off(l) + n1 * es;
    Cplx<T> x[R2];
#pragma unroll
    for (int k = 0; k < R2; ++k) x[k] = p[k * R1 * es];
    if constexpr (INV && R1 > 1) {
#pragma unroll
      for (int k = 1; k < R2; ++k) x[k] = cmul(x[k], twiddle<N, true, T>(tw, n1 * k));
    }
    dft_reg<R2, INV, T>(x, tw);
    if constexpr (!INV && R1 > 1) {
#pragma unroll
      for (int k = 1; k < R2; ++k) x[k] = cmul(x[k], twiddle<N, false, T>(tw, n1 * k));
    }
#pragma unroll
    for (int k = 0; k < R2; ++k) p[k * R1 * es] = x[k];
  }
}

// Pass B over n_lines lines: R1-point DFT over the R1 consecutive positions
// R1*k2 .. R1*k2 + R1 - 1 of each line.
template <int N, int R1, int R2, bool INV, typename T, class LineOff>
PIV_D void fft_pass_b(Cplx<T>* buf, int n_lines, LineOff line_off, int es, const Cplx<T>* tw, int tid, int nt) {
  if constexpr (R1 > 1) {
    for (int it = tid; it < n_lines * R2; it += nt) {
      const int l = it % n_lines;
      const int k2 = it / n_lines;
      Cplx<T>* p = buf + line_off(l) + R1 * k2 * es;
      Cplx<T> x[R1];
#pragma unroll
      for (int k = 0; k < R1; ++k) x[k] = p[k * es];
      dft_reg<R1, INV, T>(x, tw);
#pragma unroll
      for (int k = 0; k < R1; ++k) p[k * es] = x[k];
    }
  }
}

// Frequency held at position p after a forward transform, and the inverse map.
template <int R1, int R2>
PIV_HD int fft_freq_of_pos(int p) { return (p / R1) + R2 * (p % R1); }
template <int R1, int R2>
PIV_HD int fft_pos_of_freq(int f) { return (f / R2) + R1 * (f % R2); }

}  // namespace piv
