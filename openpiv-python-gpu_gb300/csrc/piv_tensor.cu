// Tensor-core (tcgen05) cross-correlation of window pairs: the DFTs of the
// correlation (gpu_process.py:1207-1246) as dense matrix products on the 5th
// generation tensor cores, fp16 operands, fp32 accumulation in TMEM.
//
// Real-input ("packed") DFTs. For a real sequence g of length ss placed at
// offset ss/2 of a zero-padded length N = 2 ss (the reference's default
// n_fft = 2, centred pad), the N real numbers
//   R[0] = Re X(0), R[1] = Re X(N/2), R[2f] = Re X(f), R[2f+1] = Im X(f), 0 < f < N/2
// hold the whole spectrum X (X(N-f) = conj X(f)); F is the N x ss matrix that
// maps g to R. A tile is W = 128/ss window pairs, one 128-row TMEM
// accumulator (one or two threads per TMEM lane for ss 16 / 32, four for the
// warp-specialised 64-px engine further down):
//   stage 1  T = a F^T   rows (w, y),          K = x,  cols packed f_c       (per frame)
//   stage 2  X = T^T F^T rows (tile e|o, w, c), K = y,  cols packed f_r       (per frame)
//            tile e holds the rows k = 2c of T^T (Re T, or the DC column),
//            tile o the rows k = 2c + 1 (Im T, or the Nyquist column), so
//            each thread finds both halves of its complex column in its own lane.
//   product  Q(f_r, c) = conj(A) B for c = 1 .. N/2-1 and all f_r; row c = 0
//            packs the two real-input columns: Q = conj(A0) B0 + i conj(AN) BN.
//            Each frequency pair (g, N - g) is folded into P = Q(g) + Q(N-g)
//            and M = Q(g) - Q(N-g) (stored halved, the 2 in the constants),
//            so that the inverse along f_r needs only cosines and sines of
//            g = 0 .. N/2-1:
//   stage 3  U = Q E / N rows (w, c), two products:  Re U = [Re P | Im M] [C; -S],
//            Im U = [Im P | Re M] [C; S], K = N each, cols r
//   stage 4  c = U E' / N rows (w, r),             K = (Re|Im, c),   cols s
// where E is the inverse DFT along f_r and E' the real inverse along f_c
// (U(r, N-c) = conj U(r, c)). Each frame's window is scaled by a power of two
// 2^e with sum |2^e (a - mean)| <= 2^7, so every spectrum stays below 2^7 and
// every fp16 operand below 2^15; the map is scaled back exactly by
// 2^-(e_a + e_b). The map in TMEM
// (one row per lane) then goes through the same peak search and subpixel fit
// as the FFT engine: first maximum in the fftshift-ed row-major order, lags
// without window overlap read as exact zeros.
#include <cuda_fp16.h>
#include <math.h>

#include <algorithm>

#include "piv_common.cuh"
#include "piv_corr_common.cuh"
#include "piv_internal.h"
#include "piv_tcgen05.cuh"

namespace piv {

// SPLIT: every fp16 operand x is stored as hi = fp16(x) and lo = fp16(x - hi),
// and each product runs as A_hi B_hi + A_hi B_lo + A_lo B_hi into the same
// fp32 accumulator (compensated products): the operands then carry about 22
// bits of mantissa instead of 11. The lo copy of each region sits right after
// its hi copy.
template <int SS, bool SPLIT = false>
struct TcLayout {
  static constexpr int N = 2 * SS;           // DFT size
  static constexpr int HN = N / 2;
  static constexpr int W = 128 / SS;         // window pairs per tile
  static constexpr int TCOLS = 4 * N;        // TMEM columns (stage 2: two frames x two row tiles)
  static constexpr int P = SPLIT ? 2 : 1;    // copies of every operand
  static constexpr int NB1 = N * SS * 2, NB3 = N * HN * 2, NB4 = N * N * 2, NOP = 1024 * SS;
  // Byte offsets in dynamic shared memory (16-byte aligned).
  static constexpr int B1 = 0;                          // F [N][SS] K-major (stages 1 and 2)
  static constexpr int B3 = B1 + P * NB1;               // stage 3: blocks C, -S, S [N][HN] K-major
  static constexpr int B4 = B3 + 3 * P * NB3;           // [N][N] K-major
  // Operand region, rewritten by each phase once the product that read it has
  // completed: A1 2 x [128][SS] K-major; A2 2 x 2 x [128][SS] MN-major; A3
  // [128][2N] K-major; A4 2 x [128][N] MN-major.
  static constexpr int OP = B4 + P * NB4;
  static constexpr int STG = OP + P * NOP;              // next tile's float rows [frame][128][SS], 16-byte chunks swizzled
  static constexpr int NBR = STG + 2 * 128 * SS * 4;    // [W][3][N] floats: map rows pi-1, pi, pi+1 (natural columns)
  static constexpr int END = NBR + W * 3 * N * 4;
  static constexpr int A1_BYTES = 128 * SS * 2;
  static constexpr int A2_BYTES = 128 * SS * 2;
  static constexpr int A4_BYTES = 128 * N * 2;
  static constexpr size_t SMEM = END;
  static constexpr int MIN_BLOCKS = 512 / TCOLS;        // CTAs per SM that the TMEM allows
  static constexpr int CH = SS / 4;                     // 16-byte chunks per staged row
  // Threads per TMEM lane: with two, every phase splits its frames, columns
  // or row tiles between the pair, which doubles the warps an SM holds when
  // the TMEM allows only two CTAs (ss 32) or the shared memory three (the
  // split form of ss 16). The plain ss-16 form keeps one: at four CTAs per SM
  // two threads per lane would have 64 registers each and spill.
  static constexpr int TPL = SS == 32 || SPLIT ? 2 : 1;
  static constexpr int NT = 128 * TPL;
  // CTAs per SM the register budget is compiled for (shared memory limits the
  // split form to 3 CTAs for ss 16 and 1 for ss 32).
  static constexpr int LB_BLOCKS = !SPLIT ? MIN_BLOCKS : (SS == 16 ? 3 : 1);
  // Operand scale: sum |2^e (a - mean)| below 2^(SCALE_BITS + 1).
  static constexpr int SCALE_BITS = SPLIT ? 8 : 6;
};

// Eight fp32 values to fp16 at `off` and, with SPLIT, their fp16 remainders at
// `off` of the lo copy `lo` bytes further on.
template <bool SPLIT>
PIV_D void st8s(unsigned char* base, int lo, uint32_t off, const float* v);

// Swizzled chunk position of chunk c of staged row t: the eight rows a
// quarter-warp reads together hit eight different 16-byte bank groups.
template <int CH>
PIV_D int stg_chunk(int t, int c) {
  return CH >= 8 ? (c ^ (t & 7)) : (c ^ ((t >> 1) & (CH - 1)));
}

PIV_D void cp_async16(uint32_t smem_addr, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr), "l"(gmem) : "memory");
}
// 16 bytes from gmem, or (valid false) 16 zero bytes without a global read.
PIV_D void cp_async16_zfill(uint32_t smem_addr, const void* gmem, bool valid) {
#ifdef PIV_BOUNDS_CHECK
  {
    extern __shared__ __align__(16) unsigned char piv_dyn_smem[];
    unsigned size;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(size));
    const unsigned b = (unsigned)__cvta_generic_to_shared(piv_dyn_smem);
    if (!in_bounds(smem_addr >= b && smem_addr + 16 <= b + size)) return;
  }
#endif
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr), "l"(gmem), "r"(valid ? 16 : 0)
               : "memory");
}
PIV_D void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
PIV_D void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// First maximum of x (lowest index among equal maxima) by a pairwise tree:
// the left operand, which holds the lower indices, wins ties.
template <int N>
PIV_D void first_max(const float (&x)[N], float& best, int& bj) {
  float bv[N / 2];
  int bk[N / 2];
#pragma unroll
  for (int k = 0; k < N / 2; ++k) {
    const bool rgt = x[2 * k + 1] > x[2 * k];
    bv[k] = rgt ? x[2 * k + 1] : x[2 * k];
    bk[k] = rgt ? 2 * k + 1 : 2 * k;
  }
#pragma unroll
  for (int span = N / 4; span > 0; span >>= 1)
#pragma unroll
    for (int k = 0; k < span; ++k) {
      const bool rgt = bv[2 * k + 1] > bv[2 * k];
      bv[k] = rgt ? bv[2 * k + 1] : bv[2 * k];
      bk[k] = rgt ? bk[2 * k + 1] : bk[2 * k];
    }
  best = bv[0];
  bj = bk[0];
}

// Warp-wide first maximum of (best, idx) over the 32 lanes: the largest
// value, ties to the lowest index, in two warp reductions. Values are finite;
// -0 is folded into +0 first, so that equal values have equal integer keys
// (the order-preserving key of a float: its bits, the magnitude bits
// inverted for negative values).
PIV_D void warp_first_max(float& best, int& idx) {
  const int bits = __float_as_int(best + 0.0f);
  const int key = bits ^ ((bits >> 31) & 0x7fffffff);
  const int kmax = __reduce_max_sync(0xffffffffu, key);
  idx = (int)__reduce_min_sync(0xffffffffu, key == kmax ? (unsigned)idx : 0xffffffffu);
  best = __int_as_float(kmax ^ ((kmax >> 31) & 0x7fffffff));
}

// 64-bit key of a candidate peak whose unsigned maximum is the first maximum:
// the value's order-preserving bits (-0 folded into +0) above the inverted
// flat index (a lower index gives a larger key among equal values).
PIV_D unsigned long long peak_key(float best, int idx) {
  const int bits = __float_as_int(best + 0.0f);
  const unsigned k = (unsigned)(bits ^ ((bits >> 31) & 0x7fffffff)) ^ 0x80000000u;
  return ((unsigned long long)k << 32) | (unsigned)~idx;
}
PIV_D int peak_index(unsigned long long key) { return (int)~(unsigned)key; }

// Order-preserving 32-bit key of a float (unsigned comparison of keys orders
// the values; -0 folded into +0) and its inverse.
PIV_D unsigned fkey(float x) {
  const unsigned b = __float_as_uint(x + 0.0f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
PIV_D float fkey_inv(unsigned k) { return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k); }
constexpr unsigned kKeyNegInf = 0x007fffffu;  // fkey(-inf)

// Near-tie test of the windows of a tile, run by the 32 lanes of one warp
// (W windows, 32 / W lanes each): the second-largest map value of window ww
// is the larger of sec_key[ww] (the largest row maximum over the rows other
// than the peak row) and the largest value of the peak row other than the
// peak, read from prow(ww) (natural columns; shifted column j at natural
// column j ^ N/2; lags without window overlap read as zero). Returns, in lane
// l < W, whether window l's top two values are within tol * |peak|.
template <int N, int W, class PeakOf, class RowOf>
PIV_D bool tile_near_ties(int lane, const unsigned* sec_key, float tol, PeakOf peak_of, RowOf row_of) {
  constexpr int HN = N / 2, GL = 32 / W, PER = N / GL;
  static_assert(PER % 4 == 0, "whole float4 chunks per lane");
  const int ww = lane / GL, seg = lane % GL;
  const int pidx = peak_of(ww), pi_ = pidx / N, pj = pidx % N;
  const float* prow = row_of(ww);
  float sec = -INFINITY;
#pragma unroll
  for (int k = 0; k < PER; k += 4) {
    const float4 q4 = *reinterpret_cast<const float4*>(prow + seg * PER + k);
    const float x4[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int j = (seg * PER + k + e) ^ HN;
      const float x = (pi_ == 0 || j == 0) ? 0.f : x4[e];
      if (j != pj) sec = fmaxf(sec, x);
    }
  }
#pragma unroll
  for (int o = 1; o < GL; o <<= 1) sec = fmaxf(sec, __shfl_xor_sync(0xffffffffu, sec, o));
  sec = fmaxf(sec, fkey_inv(sec_key[ww]));
  const float best = (pi_ == 0 || pj == 0) ? 0.f : prow[pj ^ HN];
  const bool tie = !(best - sec > tol * fabsf(best));
  return __shfl_sync(0xffffffffu, tie ? 1 : 0, (lane % W) * GL) != 0;
}

// Byte offset of element (r, k) in a no-swizzle K-major tile with K columns.
PIV_D uint32_t off_k(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
// Byte offset of element (m, k) in a no-swizzle MN-major tile with R rows.
PIV_D uint32_t off_mn(int m, int k, int R) {
  return (uint32_t)((k >> 3) * (R * 16) + (m >> 3) * 128 + (k & 7) * 16 + (m & 7) * 2);
}

// Eight fp32 values -> eight fp16 in one 16-byte store.
PIV_D void st8(unsigned char* base, uint32_t off, const float* v) {
  if (!in_dyn_smem(base + off, 16)) return;
  uint4 q;
  __half2 h0 = __floats2half2_rn(v[0], v[1]), h1 = __floats2half2_rn(v[2], v[3]);
  __half2 h2 = __floats2half2_rn(v[4], v[5]), h3 = __floats2half2_rn(v[6], v[7]);
  q.x = *reinterpret_cast<uint32_t*>(&h0);
  q.y = *reinterpret_cast<uint32_t*>(&h1);
  q.z = *reinterpret_cast<uint32_t*>(&h2);
  q.w = *reinterpret_cast<uint32_t*>(&h3);
  *reinterpret_cast<uint4*>(base + off) = q;
}

PIV_D void sth(unsigned char* base, uint32_t off, float v) {
  if (!in_dyn_smem(base + off, 2)) return;
  *reinterpret_cast<__half*>(base + off) = __float2half_rn(v);
}

template <bool SPLIT>
PIV_D void st8s(unsigned char* base, int lo, uint32_t off, const float* v) {
  st8(base, off, v);
  if (SPLIT) {
    float r[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) r[i] = v[i] - __half2float(__float2half_rn(v[i]));
    st8(base + lo, off, r);
  }
}

template <bool SPLIT>
PIV_D void sths(unsigned char* base, int lo, uint32_t off, float v) {
  if (!in_dyn_smem(base + off, 2) || (SPLIT && !in_dyn_smem(base + lo + off, 2))) return;
  const __half h = __float2half_rn(v);
  *reinterpret_cast<__half*>(base + off) = h;
  if (SPLIT) *reinterpret_cast<__half*>(base + lo + off) = __float2half_rn(v - __half2float(h));
}

// D (+)= A B over `ks_n` k-steps, issued by one elected lane of the calling
// converged warp; with SPLIT also A_hi B_lo and A_lo B_hi (a_lo / b_lo: byte
// distance to the lo copies).
template <bool SPLIT>
PIV_D void mma_chain(uint32_t d, uint32_t a, uint32_t a_lo, uint32_t a_step, uint32_t a_lbo, uint32_t a_sbo,
                     uint32_t b, uint32_t b_lo, uint32_t b_step, uint32_t b_lbo, uint32_t b_sbo, int ks_n,
                     uint32_t id, bool acc_first) {
  for (int ks = 0; ks < ks_n; ++ks)
    tc::mma_f16<true>(d, tc::sdesc(a + ks * a_step, a_lbo, a_sbo), tc::sdesc(b + ks * b_step, b_lbo, b_sbo), id,
                acc_first || ks > 0);
  if (SPLIT) {
    for (int ks = 0; ks < ks_n; ++ks)
      tc::mma_f16<true>(d, tc::sdesc(a + ks * a_step, a_lbo, a_sbo), tc::sdesc(b + b_lo + ks * b_step, b_lbo, b_sbo),
                  id, 1);
    for (int ks = 0; ks < ks_n; ++ks)
      tc::mma_f16<true>(d, tc::sdesc(a + a_lo + ks * a_step, a_lbo, a_sbo), tc::sdesc(b + ks * b_step, b_lbo, b_sbo),
                  id, 1);
  }
}

// 2^e for |e| <= 126.
PIV_D float pow2i(int e) { return __int_as_float((127 + e) << 23); }

// floor(log2(x)) for finite x > 0 from the exponent field: ilogbf for normal x;
// subnormal x gives -127 (the callers clamp the scale exponent anyway).
PIV_D int exp2_floor(float x) { return ((__float_as_int(x) >> 23) & 0xff) - 127; }

// CNT consecutive pixels of one window row as float; the pixel type is
// resolved once, outside the unrolled loads, so that all of them are in flight
// together.
template <typename P, int CNT>
PIV_D void load_row_t(const void* frame, long long off, float (&r)[CNT]) {
  const P* p = reinterpret_cast<const P*>(frame) + off;
#pragma unroll
  for (int x = 0; x < CNT; ++x) r[x] = (float)__ldg(p + x);
}
template <int CNT>
PIV_D void load_row(const void* frame, int pixel_type, long long off, bool ok, float (&r)[CNT]) {
  if (!ok) {
#pragma unroll
    for (int x = 0; x < CNT; ++x) r[x] = 0.f;
    return;
  }
  switch (pixel_type) {
    case PIV_PIXEL_U8: load_row_t<uint8_t>(frame, off, r); break;
    case PIV_PIXEL_U16: load_row_t<uint16_t>(frame, off, r); break;
    case PIV_PIXEL_F32: load_row_t<float>(frame, off, r); break;
    default: load_row_t<double>(frame, off, r); break;
  }
}

static constexpr uint32_t kMaxPolls = 1u << 24;

// Product of one frequency pair: the outputs at f_r = g (r0, i0) and f_r = N - g
// (r1, i1) from the spectra E (even row) and O (odd row) of frames a and b at
// f_r = g. General rows: conj(A) B with A = E_a + i O_a, B = E_b + i O_b; at
// N - g the real-input spectra are conjugated, A' = conj(E_a) + i conj(O_a).
// Row c = 0 (`special`) packs the two real-input columns:
// conj(E_a) E_b + i conj(O_a) O_b, and E_a conj(E_b) + i O_a conj(O_b) at N - g.
struct PairQ {
  float r0, i0, r1, i1;
};
PIV_D PairQ pair_product(float ar, float ai, float orr, float oi, float br, float bi, float pr, float pi,
                         bool special) {
  const float xr = ar - oi, xi = ai + orr, yr = br - pi, yi = bi + pr;        // A, B
  const float xpr = ar + oi, xpi = orr - ai, ypr = br + pi, ypi = pr - bi;    // A', B'
  const float re1 = fmaf(ar, br, ai * bi), im1 = fmaf(ar, bi, -ai * br);     // conj(E_a) E_b
  const float re2 = fmaf(orr, pr, oi * pi), im2 = fmaf(orr, pi, -oi * pr);   // conj(O_a) O_b
  PairQ q;
  q.r0 = special ? re1 - im2 : fmaf(xr, yr, xi * yi);
  q.i0 = special ? im1 + re2 : fmaf(xr, yi, -xi * yr);
  q.r1 = special ? re1 + im2 : fmaf(xpr, ypr, xpi * ypi);
  q.i1 = special ? re2 - im1 : fmaf(xpr, ypi, -xpi * ypr);
  return q;
}

// Half the folded pair: P / 2 and M / 2 with P = Q(g) + Q(N - g) and
// M = Q(g) - Q(N - g) of pair_product's outputs. With u = conj(E_a) E_b +
// conj(O_a) O_b and v = conj(E_a) O_b - conj(O_a) E_b, Q(g) = u + i v and
// Q(N - g) = conj(u) + i conj(v), so P / 2 = Re u + i Re v and
// M / 2 = -Im v + i Im u: eight two-term products, no cancellation of the
// sums A = E_a + i O_a that pair_product forms. Row c = 0 (`special`, the two
// packed real-input columns): P / 2 = Re conj(E_a) E_b + i Re conj(O_a) O_b,
// M / 2 = -Im conj(O_a) O_b + i Im conj(E_a) E_b. Every part is at most
// (|A| |B| + |A'| |B'|) / 2, the bound of one spectrum product.
struct PairPM {
  float pr, pi, mr, mi;
};
PIV_D PairPM pair_fold_half(float ar, float ai, float orr, float oi, float br, float bi, float pr, float pi,
                            bool special) {
  const float t1 = fmaf(ar, br, ai * bi), t3 = fmaf(ar, bi, -ai * br);     // conj(E_a) E_b
  const float t2 = fmaf(orr, pr, oi * pi), t4 = fmaf(orr, pi, -oi * pr);   // conj(O_a) O_b
  const float t5 = fmaf(ar, pr, ai * pi), t7 = fmaf(ar, pi, -ai * pr);     // conj(E_a) O_b
  const float t6 = fmaf(orr, br, oi * bi), t8 = fmaf(orr, bi, -oi * br);   // conj(O_a) E_b
  PairPM o;
  o.pr = special ? t1 : t1 + t2;
  o.pi = special ? t2 : t5 - t6;
  o.mr = special ? -t4 : t8 - t7;
  o.mi = special ? t3 : t3 + t4;
  return o;
}

// Stage-3 operand columns (K = 2N) of one row: [Re P | Im M | Im P | Re M] / 2,
// N/2 columns each; at g = 0 the slots hold Re Q(0), Re Q(N/2), Im Q(0) and
// Im Q(N/2) (the unpaired frequencies), also halved, whose inverse weights
// are 1 and (-1)^r. Value of block k (0: C, 1: -S, 2: S) at output r, column
// g, for cos / sin of 2 pi g r / N scaled by s; the factor 2 restores the
// halved operand (exact: powers of two).
PIV_D float stage3_weight(int blk, int r, int g, float cs, float sn, float s) {
  if (blk == 0) return 2.f * cs;
  if (g == 0) return (r & 1) ? -2.f * s : 2.f * s;
  return blk == 1 ? -2.f * sn : 2.f * sn;
}

// Whether any segment asks for near-tie flags or counts.
PIV_D bool any_tie_output(const CorrSeg* seg_s, int n_seg) {
  bool any = false;
  for (int k = 0; k < n_seg; ++k) any = any || seg_s[k].near_tie != nullptr || seg_s[k].tie_count != nullptr;
  return any;
}

// ASYNC: float32 frames whose window rows start on 16-byte boundaries. The
// next tile's rows are then copied into shared memory with cp.async while the
// current tile runs through its four products; otherwise each tile loads its
// rows from global memory when it starts.
template <int SS, bool ASYNC, bool SPLIT>
__global__ void __launch_bounds__(TcLayout<SS, SPLIT>::NT, TcLayout<SS, SPLIT>::LB_BLOCKS)
    k_corr_tc(CorrArgs a, int* status) {
  using L = TcLayout<SS, SPLIT>;
  constexpr int N = L::N, HN = L::HN, W = L::W, CH = L::CH, TPL = L::TPL, NT = L::NT;
  constexpr int NPART = N / 32;      // warps per window in the epilogue
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  // Per tile slot (three: the tile being correlated, the next one, whose rows
  // are in flight, and the one after, whose corners are being computed).
  __shared__ int sc_e[3][2][W];      // per slot, frame and window: log2 of the operand scale
  __shared__ long long win_base[3][W];
  __shared__ int win_valid[3][W];
  __shared__ long long win_loc[3][W];  // window index within its segment
  __shared__ int win_seg[3][W];
  __shared__ CorrSeg seg_s[kMaxCorrSegs];
  __shared__ float pk_val[W][NPART];
  __shared__ int pk_idx[W][NPART];
  __shared__ unsigned sec_key[W];    // per window: key of the largest row maximum outside the peak row

  const int tid = threadIdx.x;
  const int t = tid & 127;           // TMEM lane (row of the tile) of this thread
  const int half = tid >> 7;         // which of the TPL threads of lane t
  const int warp = tid >> 5, lane = tid & 31;
  const uint32_t lane_sel = (uint32_t)(32 * (warp & 3)) << 16;

  // Constant DFT operands; the twiddles W_N^k = exp(-2 pi i k / N) sit in the
  // operand region until the first tile.
  float* tw_re = reinterpret_cast<float*>(sm + L::OP);
  float* tw_im = tw_re + N;
  for (int k = tid; k < N; k += NT) {
    float sn, cs;
    sincospif(2.0f * (float)k / (float)N, &sn, &cs);
    tw_re[k] = cs;
    tw_im[k] = -sn;
  }
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    abort_s = 0;
  }
  __syncthreads();
  const float inv_n = 1.0f / (float)N;
  const int p0 = SS / 2;
  for (int e = tid; e < N * SS; e += NT) {  // F[k][x]
    const int k = e / SS, x = e % SS, f = k >> 1, q = (f * (x + p0)) % N;
    float v;
    if (k == 0) v = 1.0f;
    else if (k == 1) v = ((x + p0) & 1) ? -1.0f : 1.0f;
    else v = (k & 1) ? tw_im[q] : tw_re[q];
    sths<SPLIT>(sm + L::B1, L::NB1, off_k(k, x, SS), v);
  }
  // The split form keeps the inverse DFTs' 1/N out of B3 and B4 (their lo
  // parts would fall below the fp16 normal range) and scales Q and U instead.
  const float bscale = SPLIT ? 1.0f : inv_n;
  for (int e = tid; e < 3 * N * HN; e += NT) {  // B3 blocks C, -S, S: [r][g]
    const int blk = e / (N * HN), r = (e / HN) % N, g = e % HN;
    const int q = (g * r) % N;
    const float v = stage3_weight(blk, r, g, tw_re[q] * bscale, -tw_im[q] * bscale, bscale);
    sths<SPLIT>(sm + L::B3 + blk * L::P * L::NB3, L::NB3, off_k(r, g, HN), v);
  }
  for (int e = tid; e < N * N; e += NT) {  // B4[s][kappa], kappa = (part, c)
    const int s_ = e / N, kap = e % N, part = kap / HN, c = kap % HN;
    const int q = (c * s_) % N;
    float v;
    if (c == 0) v = part == 0 ? bscale : ((s_ & 1) ? -bscale : bscale);
    else v = part == 0 ? 2.0f * tw_re[q] * bscale : 2.0f * tw_im[q] * bscale;
    sths<SPLIT>(sm + L::B4, L::NB4, off_k(s_, kap, N), v);
  }
  const float oscale = SPLIT ? inv_n : 1.0f;  // applied to Q and U in the split form
  if (warp == 0) tc::tmem_alloc(&tmem_base_s, L::TCOLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base_s;
  // TMEM loads of the CTA's allocation (checked build: columns inside it).
  auto tld = [&](uint32_t addr, float (&v)[16]) {
    if (in_bounds(((addr - tmem) & 0xffffu) + 16 <= (uint32_t)L::TCOLS)) tc::tmem_ld16(addr, v);
  };
  const uint32_t sbase = tc::smem_u32(sm);
  uint32_t phase = 0;

  const int n_seg = load_segments(a, seg_s);
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  const int n_tiles = (int)((total + W - 1) / W);

  // Every thread waits for the last commit itself; a wait that gives up sets
  // abort_s, which all threads read after the next barrier and leave the tile
  // loop together.
  auto wait_mma = [&]() {
    const bool ok = tc::mbar_wait_bounded(&bar, phase, kMaxPolls);
    phase ^= 1u;
    if (!ok) {
      abort_s = 1;
      atomicExch(status, PIV_E_TIMEOUT);
    }
    tc::fence_after_sync();
  };
  // Barrier before an MMA issue; false (for every thread alike) once a wait
  // has given up.
  auto sync_for_mma = [&]() -> bool {
    tc::fence_async_smem();
    tc::fence_before_sync();
    const bool stop = __syncthreads_or(abort_s != 0);
    tc::fence_after_sync();
    return !stop;
  };
  // Corners of window wi of tile `tl` into slot `sl`.
  auto window_setup = [&](int tl, int sl, int wi) {
    const long long g = (long long)tl * W + wi;
    int ok = tl < n_tiles && g < total;
    long long base = 0, loc = 0;
    int sg = 0;
    if (ok) {
      while (sg + 1 < n_seg && g >= seg_s[sg + 1].win0) ++sg;
      const CorrSeg& q = seg_s[sg];
      loc = g - q.win0;
      // 32-bit quotients: a segment holds fewer than 2^31 windows (checked at launch).
      const int li = (int)loc, nw = q.m * q.n;
      const int pair = li / nw, k = li - pair * nw;
      const int wr = k / q.n, wc = k - wr * q.n;
      if (q.win_mask) ok = q.win_mask[k] == 0;
      base = pair * (long long)q.height * q.width + (long long)(wr * q.spacing + q.y_offset) * q.width +
             wc * q.spacing + q.x_offset;
      if (ok && !in_bounds(base >= 0 && base + (long long)(SS - 1) * q.width + SS <=
                                             (long long)q.n_pairs * q.height * q.width))
        ok = 0;
    }
    win_valid[sl][wi] = ok;
    win_base[sl][wi] = base;
    win_loc[sl][wi] = loc;
    win_seg[sl][wi] = sg;
  };
  // Thread (half, t) starts the copies of row t of its frames of the tile in
  // slot `sl`; rows of invalid windows are zero-filled (no global read), so
  // the staging phase reads every row unconditionally.
  auto stage_async = [&](int sl) {
    const int w = t / SS, y = t % SS;
    const bool ok = win_valid[sl][w] != 0;
    const CorrSeg& q = seg_s[win_seg[sl][w]];
    const long long off = ok ? win_base[sl][w] + (long long)y * q.width : 0;
#pragma unroll
    for (int fi = 0; fi < 2 / TPL; ++fi) {
      const int f = TPL == 2 ? half : fi;
      const float* src = reinterpret_cast<const float*>(f == 0 ? q.frame_a : q.frame_b) + off;
      const uint32_t row = sbase + L::STG + (uint32_t)((f * 128 + t) * SS * 4);
#pragma unroll
      for (int c = 0; c < CH; ++c) cp_async16_zfill(row + 16 * stg_chunk<CH>(t, c), src + (ok ? 4 * c : 0), ok);
    }
  };

  if (tid < W) {
    window_setup(blockIdx.x, 0, tid);
    window_setup(blockIdx.x + gridDim.x, 1, tid);
    sec_key[tid] = kKeyNegInf;
  }
  __syncthreads();
  if (ASYNC) {
    stage_async(0);
    cp_async_commit();
  }
  const bool ties = any_tie_output(seg_s, n_seg);
  // Near-tie flag of window `lane` of the current tile (lanes < W of the
  // calling warp; tile_near_ties's result) to the window's outputs.
  int cur_sl = 0;
  long long cur_g0 = 0;
  auto write_near_ties = [&](bool tie) {
    if (lane >= W || cur_g0 + lane >= total) return;
    const CorrSeg& sq = seg_s[win_seg[cur_sl][lane]];
    const long long gl = win_loc[cur_sl][lane];
    tie = tie && win_valid[cur_sl][lane];
    if (!in_bounds(gl >= 0 && gl < (long long)sq.n_pairs * sq.m * sq.n)) return;
    if (sq.near_tie) sq.near_tie[gl] = tie ? 1 : 0;
    if (tie && sq.tie_count) atomicAdd(sq.tie_count, 1);
  };

  int sl = 0;
  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, sl = sl == 2 ? 0 : sl + 1) {
    const int sl1 = sl == 2 ? 0 : sl + 1, sl2 = sl1 == 2 ? 0 : sl1 + 1;
    const long long g0 = (long long)tile * W;
    // No barrier here: warps 0 and 1 may still be finishing the previous
    // tile's near-tie test and fits while the others stage this tile (its
    // rows are the ones each thread copied itself). The stage-1 barrier
    // below waits for all of them.
    if (ASYNC) cp_async_wait_all();
    cur_sl = sl;
    cur_g0 = g0;

    // ---- Staging: thread (half, t = (w, y)) takes row y of window w of its
    // frames (both with one thread per TMEM lane: their reduction chains run
    // side by side, each frame's arithmetic as for a frame alone).
    {
      constexpr int NF = 2 / TPL;
      const int w = t / SS, y = t % SS;
      const bool ok = win_valid[sl][w] != 0;
      float r[NF][SS];
#pragma unroll
      for (int fi = 0; fi < NF; ++fi) {
        const int f = TPL == 2 ? half : fi;
        if (ASYNC) {
          const unsigned char* row = sm + L::STG + (f * 128 + t) * SS * 4;
#pragma unroll
          for (int c = 0; c < CH; ++c) {
            const float4 q4 = *reinterpret_cast<const float4*>(row + 16 * stg_chunk<CH>(t, c));
            r[fi][4 * c] = q4.x;
            r[fi][4 * c + 1] = q4.y;
            r[fi][4 * c + 2] = q4.z;
            r[fi][4 * c + 3] = q4.w;
          }
        } else {
          const CorrSeg& q = seg_s[win_seg[sl][w]];
          load_row(f == 0 ? q.frame_a : q.frame_b, a.pixel_type, win_base[sl][w] + (long long)y * q.width, ok,
                   r[fi]);
        }
      }
      float sum[NF], mean[NF], l[NF];
#pragma unroll
      for (int fi = 0; fi < NF; ++fi) {
        sum[fi] = 0.f;
#pragma unroll
        for (int x = 0; x < SS; ++x) sum[fi] += r[fi][x];
      }
      // Window sums over its SS rows (a window's lanes are contiguous, SS | 32).
#pragma unroll
      for (int o = 1; o < SS; o <<= 1)
#pragma unroll
        for (int fi = 0; fi < NF; ++fi) sum[fi] += __shfl_xor_sync(0xffffffffu, sum[fi], o);
#pragma unroll
      for (int fi = 0; fi < NF; ++fi) {
        mean[fi] = sum[fi] / (float)(SS * SS);
        l[fi] = 0.f;
#pragma unroll
        for (int x = 0; x < SS; ++x) {
          r[fi][x] -= mean[fi];
          l[fi] += fabsf(r[fi][x]);
        }
      }
#pragma unroll
      for (int o = 1; o < SS; o <<= 1)
#pragma unroll
        for (int fi = 0; fi < NF; ++fi) l[fi] += __shfl_xor_sync(0xffffffffu, l[fi], o);
#pragma unroll
      for (int fi = 0; fi < NF; ++fi) {
        const int f = TPL == 2 ? half : fi;
        int e = 0;
        if (l[fi] > 0.f) e = min(120, max(-120, L::SCALE_BITS - exp2_floor(l[fi])));
        const float s = pow2i(e);
#pragma unroll
        for (int x = 0; x < SS; ++x) r[fi][x] *= s;
        if (y == 0) {
          sc_e[sl][f][w] = e;
          const CorrSeg& sq = seg_s[win_seg[sl][w]];
          if (sq.win_means && ok) sq.win_means[2 * win_loc[sl][w] + f] = mean[fi];
        }
#pragma unroll
        for (int x = 0; x < SS; x += 8)
          st8s<SPLIT>(sm + L::OP + f * L::A1_BYTES, L::NOP, off_k(t, x, SS), r[fi] + x);
      }
    }
    if (!sync_for_mma()) break;

    // ---- Stage 1: T = a F^T per frame -> TMEM cols [f N, f N + N).
    if (warp == 0) {  // MMA issue: a converged warp, one elected lane issues
      const uint32_t id = tc::idesc_f16(128, N, 0, 0);
#pragma unroll
      for (int f = 0; f < 2; ++f)
        mma_chain<SPLIT>(tmem + f * N, sbase + L::OP + f * L::A1_BYTES, L::NOP, 256, 128, SS * 16, sbase + L::B1,
                         L::NB1, 256, 128, SS * 16, SS / 16, id, false);
      tc::mma_commit<true>(&bar);
    }
    // The near-tie keys of this tile (the previous tile's test is done).
    if (tid < W) sec_key[tid] = kKeyNegInf;
    wait_mma();

    // ---- Stage 1 -> 2: row (w, y) of T becomes column y of the MN-major rows
    // (w, c) of tile e (k = 2c) and tile o (k = 2c + 1).
    {
      const int w = t / SS, y = t % SS;
      // The thread's columns as chunks of 16 (frame-major); chunk k + 1 is
      // loaded while chunk k is converted.
      constexpr int K = (2 / TPL) * N / 16;
      auto col_src = [&](int k) -> uint32_t {
        const int cs = 16 * k, f = TPL == 2 ? half : cs / N;
        return tmem + lane_sel + f * N + cs % N;
      };
      auto put = [&](int k, const float (&vals)[16]) {
        const int cs = 16 * k, f = TPL == 2 ? half : cs / N, c0 = (cs % N) / 2;
#pragma unroll
        for (int rt = 0; rt < 2; ++rt) {
          float v8[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) v8[j] = vals[2 * j + rt];
          st8s<SPLIT>(sm + L::OP + (f * 2 + rt) * L::A2_BYTES, L::NOP, off_mn(w * HN + c0, y, 128), v8);
        }
      };
      float b0[16], b1[16];
      tld(col_src(0), b0);
      tc::tmem_ld_wait();
      tc::reg_fence(b0);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        if (k + 1 < K) tld(col_src(k + 1), (k & 1) ? b0 : b1);
        put(k, (k & 1) ? b1 : b0);
        if (k + 1 < K) {
          tc::tmem_ld_wait();
          if (k & 1) tc::reg_fence(b0);
          else tc::reg_fence(b1);
        }
      }
    }
    if (!sync_for_mma()) break;

    // ---- Stage 2: X = T^T F^T for tiles e, o and frames a, b -> TMEM cols [rt 2N + f N, +N).
    if (warp == 0) {  // MMA issue: a converged warp, one elected lane issues
      const uint32_t id = tc::idesc_f16(128, N, 1, 0);
#pragma unroll
      for (int rt = 0; rt < 2; ++rt)
#pragma unroll
        for (int f = 0; f < 2; ++f)
          mma_chain<SPLIT>(tmem + rt * 2 * N + f * N, sbase + L::OP + (f * 2 + rt) * L::A2_BYTES, L::NOP, 32 * 128,
                           128 * 16, 128, sbase + L::B1, L::NB1, 256, 128, SS * 16, SS / 16, id, false);
      tc::mma_commit<true>(&bar);
    }
    // The next tile's rows land while this tile runs (issued after the MMAs,
    // so that the issuing thread's copies do not hold up the product). Not
    // before this tile's stage-1 barrier: warp 2 writes slot sl1's corners
    // during the previous tile's fits, and that barrier is what orders them
    // before these reads.
    if (ASYNC) {
      stage_async(sl1);
      cp_async_commit();
    }
    wait_mma();

    // ---- Product: thread (w, c) forms row c of the stage-3 operand,
    // [Re P | Im M | Im P | Re M] / 2 of the folded pairs (g, N - g); at g = 0
    // Re Q(0), Re Q(N/2), Im Q(0), Im Q(N/2), halved.
    {
      const bool special = (t % HN) == 0;
      unsigned char* dst = sm + L::OP;
#pragma unroll
      for (int gi = 0; gi < HN / TPL; gi += 8) {
        const int g0 = half * (HN / TPL) + gi;
        float ea[16], eb[16], oa[16], ob[16];
        tld(tmem + lane_sel + 0 * N + 2 * g0, ea);
        tld(tmem + lane_sel + 1 * N + 2 * g0, eb);
        tld(tmem + lane_sel + 2 * N + 2 * g0, oa);
        tld(tmem + lane_sel + 3 * N + 2 * g0, ob);
        tc::tmem_ld_wait();
        tc::reg_fence(ea); tc::reg_fence(eb); tc::reg_fence(oa); tc::reg_fence(ob);
        float rp[8], im[8], ip[8], rm[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          PairPM o;
          if (g0 + i == 0) {
            // f_r = 0 and f_r = N/2: real spectra R[0] and R[1], not folded (halved).
            const PairQ q0 = pair_product(ea[0], 0.f, oa[0], 0.f, eb[0], 0.f, ob[0], 0.f, special);
            const PairQ q1 = pair_product(ea[1], 0.f, oa[1], 0.f, eb[1], 0.f, ob[1], 0.f, special);
            o.pr = 0.5f * q0.r0; o.mi = 0.5f * q1.r0; o.pi = 0.5f * q0.i0; o.mr = 0.5f * q1.i0;
          } else {
            o = pair_fold_half(ea[2 * i], ea[2 * i + 1], oa[2 * i], oa[2 * i + 1], eb[2 * i], eb[2 * i + 1],
                               ob[2 * i], ob[2 * i + 1], special);
          }
          rp[i] = o.pr * oscale; im[i] = o.mi * oscale; ip[i] = o.pi * oscale; rm[i] = o.mr * oscale;
        }
        st8s<SPLIT>(dst, L::NOP, off_k(t, 0 * HN + g0, 2 * N), rp);
        st8s<SPLIT>(dst, L::NOP, off_k(t, 1 * HN + g0, 2 * N), im);
        st8s<SPLIT>(dst, L::NOP, off_k(t, 2 * HN + g0, 2 * N), ip);
        st8s<SPLIT>(dst, L::NOP, off_k(t, 3 * HN + g0, 2 * N), rm);
      }
    }
    if (!sync_for_mma()) break;

    // ---- Stage 3: Re U = [Re P | Im M] [C; -S] -> TMEM cols [0, N),
    // Im U = [Im P | Re M] [C; S] -> cols [N, 2N).
    if (warp == 0) {  // MMA issue: a converged warp, one elected lane issues
      const uint32_t id = tc::idesc_f16(128, N, 0, 0);
#pragma unroll
      for (int part = 0; part < 2; ++part)
#pragma unroll
        for (int kb = 0; kb < 2; ++kb)
          mma_chain<SPLIT>(tmem + part * N, sbase + L::OP + (part * N + kb * HN) * 16, L::NOP, 256, 128, 2 * N * 16,
                           sbase + L::B3 + (kb == 0 ? 0 : 1 + part) * L::P * L::NB3, L::NB3, 256, 128, HN * 16,
                           HN / 16, id, kb > 0);
      tc::mma_commit<true>(&bar);
    }
    wait_mma();

    // ---- Stage 3 -> 4: row (w, c) of U becomes columns (Re|Im, c) of the MN-major rows (w, r).
    {
      const int w = t / HN, c = t % HN;
#pragma unroll
      for (int pi = 0; pi < 2 / TPL; ++pi) {
        const int part = TPL == 2 ? half : pi;
        float v[N];
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16)
          tld(tmem + lane_sel + part * N + c0, *reinterpret_cast<float(*)[16]>(v + c0));
        tc::tmem_ld_wait();
        tc::reg_fence(v);
        if (SPLIT) {
#pragma unroll
          for (int r0 = 0; r0 < N; ++r0) v[r0] *= oscale;
        }
#pragma unroll
        for (int r0 = 0; r0 < N; r0 += 8) {
          const int m = w * N + r0;
          st8s<SPLIT>(sm + L::OP + (m >> 7) * L::A4_BYTES, L::NOP, off_mn(m & 127, part * HN + c, 128), v + r0);
        }
      }
    }
    if (!sync_for_mma()) break;

    // ---- Stage 4: c = U E' / N -> TMEM cols [rt N, rt N + N).
    if (warp == 0) {  // MMA issue: a converged warp, one elected lane issues
      const uint32_t id = tc::idesc_f16(128, N, 1, 0);
#pragma unroll
      for (int rt = 0; rt < 2; ++rt)
        mma_chain<SPLIT>(tmem + rt * N, sbase + L::OP + rt * L::A4_BYTES, L::NOP, 32 * 128, 128 * 16, 128,
                         sbase + L::B4, L::NB4, 256, 128, N * 16, N / 16, id, false);
      tc::mma_commit<true>(&bar);
    }
    wait_mma();

    // ---- Epilogue. Row rt*128 + tid of the tile is map row r of window w
    // (scaled by 2^(e_a + e_b)); shifted row index i = r ^ N/2, shifted
    // column j = s ^ N/2. Lags without window overlap (i = 0 or j = 0) are 0.
    float* nbrow = reinterpret_cast<float*>(sm + L::NBR);  // [W][3][N]: rows pi-1, pi, pi+1 (natural columns)
    // Subpixel fit and outputs of window ww with flat peak index pidx (its
    // neighbour rows in nbrow).
    auto finish = [&](int ww, int pidx) {
      const int pi_ = pidx / N, pj = pidx % N;
      float isp = (float)pi_, jsp = (float)pj;
      if (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1) {
        const int ue = -sc_e[sl][0][ww] - sc_e[sl][1][ww];
        // Shifted (i, j) -> stored row slot i - pi + 1, natural column j ^ N/2.
        // x 2^ue as two exact power-of-two products (|ue| <= 240; each factor is a normal float).
        const float s1 = pow2i(ue >> 1), s2 = pow2i(ue - (ue >> 1));
        auto at = [&](int i, int j) -> float {
          return (i == 0 || j == 0) ? 0.f : nbrow[(ww * 3 + (i - pi_ + 1)) * N + (j ^ HN)] * s1 * s2;
        };
        subpixel_fit(a.subpixel, pi_, pj, at(pi_, pj), at(pi_ - 1, pj), at(pi_ + 1, pj), at(pi_, pj - 1),
                     at(pi_, pj + 1), isp, jsp);
      }
      const CorrSeg& sq = seg_s[win_seg[sl][ww]];
      const long long gl = win_loc[sl][ww];
      float* uo = reinterpret_cast<float*>(sq.u);
      float* vo = reinterpret_cast<float*>(sq.v);
      if (!in_bounds(gl >= 0 && gl < (long long)sq.n_pairs * sq.m * sq.n)) return;
      if (win_valid[sl][ww]) {
        uo[gl] = sub_rn(jsp, (float)HN);
        vo[gl] = sub_rn(isp, (float)HN);
      } else {
        uo[gl] = NAN;
        vo[gl] = NAN;
      }
      if (sq.peak_i) sq.peak_i[gl] = pi_;
      if (sq.peak_j) sq.peak_j[gl] = pj;
    };
    auto peak_row = [&](int ww) { return nbrow + (ww * 3 + 1) * N; };
    bool stop = false;
    if constexpr (N == 32 && TPL == 1) {
      // One window per warp and row tile (N = 32 rows): the warp finds its
      // window's peak by shuffles and the lanes of the rows next to it store
      // them at once (no second TMEM pass); then one barrier, and W lanes fit.
#pragma unroll
      for (int rt = 0; rt < 2; ++rt) {
        const int m = rt * 128 + t, w = m / N, r = m % N, i = r ^ HN;
        float v[N];
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16)
          tld(tmem + lane_sel + rt * N + c0, *reinterpret_cast<float(*)[16]>(v + c0));
        tc::tmem_ld_wait();
        tc::reg_fence(v);
        float rowc[N];
#pragma unroll
        for (int j = 0; j < N; ++j) rowc[j] = j == 0 ? 0.f : v[j ^ HN];
        float best;
        int bj;
        first_max<N>(rowc, best, bj);
        int idx = i * N + bj;
        if (i == 0) { best = 0.f; idx = 0; }
        const float rbest = best;
        warp_first_max(best, idx);
        if (a.maps && g0 + w < total) {
          const int ue = -sc_e[sl][0][w] - sc_e[sl][1][w];
          float* mo = reinterpret_cast<float*>(a.maps) + (g0 + w) * N * N + (long long)i * N;
#pragma unroll
          for (int j = 0; j < N; ++j) mo[j] = i == 0 ? 0.f : ldexpf(rowc[j], ue);
        }
        const int pi_ = idx / N, pj = idx % N;
        if (ties) {  // the window's rows are this warp's: its largest row maximum outside the peak row
          const unsigned k = __reduce_max_sync(0xffffffffu, i == pi_ ? kKeyNegInf : fkey(rbest));
          if (lane == 0) sec_key[w] = k;
        }
        if ((ties && i == pi_) || (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1 && i >= pi_ - 1 && i <= pi_ + 1)) {
          float4* dst = reinterpret_cast<float4*>(nbrow + (w * 3 + (i - pi_ + 1)) * N);
          if (in_dyn_smem(dst, N * 4))
#pragma unroll
            for (int c4 = 0; c4 < N / 4; ++c4)
              dst[c4] = make_float4(v[4 * c4], v[4 * c4 + 1], v[4 * c4 + 2], v[4 * c4 + 3]);
        }
        if (lane == 0) pk_idx[w][0] = idx;
      }
      // The peaks and neighbour rows are in shared memory (the map's TMEM
      // columns are read); the abort decision is the same for every thread.
      tc::fence_before_sync();
      stop = __syncthreads_or(abort_s != 0);
      // The near-tie flags in warp 1 while warp 0 fits.
      if (ties && warp == 1)
        write_near_ties(tile_near_ties<N, W>(lane, sec_key, a.tie_tol, [&](int ww) { return pk_idx[ww][0]; },
                                             peak_row));
      if (tid < W && g0 + tid < total) finish(tid, pk_idx[tid][0]);
      if (warp == 2 && lane < W) window_setup(tile + 2 * gridDim.x, sl2, lane);
    } else {
      float rbest[2 / TPL];  // this thread's row maxima
#pragma unroll
      for (int ri = 0; ri < 2 / TPL; ++ri) {
        const int rt = TPL == 2 ? half : ri;
        const int m = rt * 128 + t, w = m / N, r = m % N, i = r ^ HN;
        float v[N];
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16)
          tld(tmem + lane_sel + rt * N + c0, *reinterpret_cast<float(*)[16]>(v + c0));
        tc::tmem_ld_wait();
        tc::reg_fence(v);
        float rowc[N];
#pragma unroll
        for (int j = 0; j < N; ++j) rowc[j] = j == 0 ? 0.f : v[j ^ HN];
        float best;
        int bj;
        first_max<N>(rowc, best, bj);
        int idx = i * N + bj;
        if (i == 0) { best = 0.f; idx = 0; }
        rbest[ri] = best;
        warp_first_max(best, idx);
        if (lane == 0) {
          pk_val[w][r / 32] = best;
          pk_idx[w][r / 32] = idx;
        }
        if (a.maps && g0 + w < total) {
          const int ue = -sc_e[sl][0][w] - sc_e[sl][1][w];
          float* mo = reinterpret_cast<float*>(a.maps) + (g0 + w) * N * N + (long long)i * N;
#pragma unroll
          for (int j = 0; j < N; ++j) mo[j] = i == 0 ? 0.f : ldexpf(rowc[j], ue);
        }
      }
      __syncthreads();
      // First maximum of window w over its NPART warp partials (each thread
      // that needs it combines them itself: no further barrier).
      auto window_peak = [&](int w) -> int {
        float v = pk_val[w][0];
        int idx = pk_idx[w][0];
#pragma unroll
        for (int p = 1; p < NPART; ++p)
          if (pk_val[w][p] > v || (pk_val[w][p] == v && pk_idx[w][p] < idx)) {
            v = pk_val[w][p];
            idx = pk_idx[w][p];
          }
        return idx;
      };
      // The rows next to the peak go to shared memory for the five-point fit.
#pragma unroll
      for (int ri = 0; ri < 2 / TPL; ++ri) {
        const int rt = TPL == 2 ? half : ri;
        const int m = rt * 128 + t, w = m / N, r = m % N, i = r ^ HN;
        const int pidx = window_peak(w), pi_ = pidx / N, pj = pidx % N;
        if (ties) {  // the warp's largest row maximum outside the peak row (a warp's rows share a window)
          const unsigned k = __reduce_max_sync(0xffffffffu, i == pi_ ? kKeyNegInf : fkey(rbest[ri]));
          if (lane == 0) atomicMax(&sec_key[w], k);
        }
        const bool mine = (ties && i == pi_) ||
                          (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1 && i >= pi_ - 1 && i <= pi_ + 1);
        if (__any_sync(0xffffffffu, mine)) {
          float v[N];
#pragma unroll
          for (int c0 = 0; c0 < N; c0 += 16)
            tld(tmem + lane_sel + rt * N + c0, *reinterpret_cast<float(*)[16]>(v + c0));
          tc::tmem_ld_wait();
          tc::reg_fence(v);
          if (mine) {
            float4* dst = reinterpret_cast<float4*>(nbrow + (w * 3 + (i - pi_ + 1)) * N);
            if (in_dyn_smem(dst, N * 4))
#pragma unroll
              for (int c4 = 0; c4 < N / 4; ++c4)
                dst[c4] = make_float4(v[4 * c4], v[4 * c4 + 1], v[4 * c4 + 2], v[4 * c4 + 3]);
          }
        }
      }
      // The peaks and neighbour rows are in shared memory (the map's TMEM
      // columns are read); the abort decision is the same for every thread.
      tc::fence_before_sync();
      stop = __syncthreads_or(abort_s != 0);
      // The near-tie flags in warp 1 while warp 0 fits.
      if (ties && warp == 1) write_near_ties(tile_near_ties<N, W>(lane, sec_key, a.tie_tol, window_peak, peak_row));
      if (tid < W && g0 + tid < total) finish(tid, window_peak(tid));
      if (warp == 2 && lane < W) window_setup(tile + 2 * gridDim.x, sl2, lane);
    }
    // No barrier: the other warps go on to stage the next tile while warps 0
    // and 1 finish this one and warp 2 sets up the corners of the tile after
    // the next (slot sl2, last read by the previous tile) with its integer
    // divisions off the path of the MMAs; the next tile's stage-1 barrier
    // waits for all of them.
    if (stop) break;
  }
  if (ASYNC) cp_async_wait_all();
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, L::TCOLS);
}

// ---------------------------------------------------------------------------
// 64-pixel windows (N = 128), warp-specialised and pipelined over tiles. One
// CTA per SM with 16 compute warps (512 threads, four per TMEM lane; warp w
// reads lanes 32 (w % 4); each phase splits its columns or frames between
// the four), one MMA warp and one fit warp. The MMA warp issues each product
// as soon as the compute warps have written its operand (one arrival per
// compute warp on that operand's "ready" mbarrier) and commits it to the
// product's own mbarrier, so the tensor core and the compute warps work on
// different phases at the same time: the window statistics of tile i + 1
// are formed while stage 2 of tile i runs, the product of the first half of
// stage 2 (f_r columns 0-63) while the second half is computed, and the
// first half of stage 3 while the second half of the product is formed;
// tile i + 1 is staged while stage 4 of tile i runs, and the map of tile i
// is searched while stage 1 of tile i + 1 runs. The fit warp runs the
// near-tie test and the subpixel fits of tile i (from the peak keys and the
// three map rows around each peak, which the compute warps leave in a
// buffer of their own) while tile i + 1 is correlated, so the compute warps
// go from the peak search straight on to the next tile.
//   TMEM: stage 1 -> columns [256, 512); stage 2 half 0 -> [0, 256), half 1
//   -> [256, 512); stages 3 and 4 -> [0, 256).
//   Shared memory (216,064 bytes): constants F (16 KB), C / -S / S (48 KB) and E'
//   (32 KB); the stage-1 operands (32 KB, then the first half of the stage-3
//   operand); a 64 KB region for the stage-2 operands, then the second half
//   of the stage-3 operand and the stage-4 operands; the next tile's 8-bit
//   rows (16 KB); the peak-neighbour rows (3 KB).
// ---------------------------------------------------------------------------
struct Tc64 {
  static constexpr int SS = 64, N = 128, HN = 64, W = 2, TCOLS = 512;
  // Compute warps, their threads, all threads (with the MMA warp and the fit warp).
  static constexpr int NCW = 16, NC = 32 * NCW, NT = NC + 64;
  static constexpr int NB3 = N * HN * 2;
  static constexpr int B1 = 0;                      // F [N][SS] K-major
  static constexpr int B3 = B1 + N * SS * 2;        // stage 3: blocks C, -S, S (/ N) [N][HN] K-major
  static constexpr int B4 = B3 + 3 * NB3;           // [N][N] K-major, K = (part, c)
  static constexpr int A1 = B4 + N * N * 2;         // 2 x [128][SS] K-major; then stage-3 operand half 0
  static constexpr int OP = A1 + 2 * 128 * SS * 2;  // 64 KB operand region
  static constexpr int STG = OP + 65536;            // next tile's 8-bit rows [frame][w][y][64 B], chunks swizzled
  static constexpr int NBR = STG + 2 * W * SS * SS; // [W][3][N] floats: map rows pi-1, pi, pi+1 (natural columns)
  static constexpr int END = NBR + W * 3 * N * 4;
  static constexpr int A1_BYTES = 128 * SS * 2;     // per frame, K-major [128][SS]
  static constexpr int A2_BYTES = 128 * SS * 2;     // per (frame, tile), MN-major [128][SS]
  static constexpr int A4_BYTES = 128 * N * 2;      // per tile, MN-major [128][N]
  static constexpr int QH = 128;                    // columns of one half of the stage-3 operand (K-major)
  static constexpr uint32_t T_S1 = 256;             // TMEM column of the stage-1 outputs
  static constexpr size_t SMEM = END;
};

// Swizzled 16-byte chunk k (0..3) of staged 8-bit row t.
PIV_D int stg64_chunk(int t, int k) { return k ^ ((t >> 1) & 3); }

// ASYNC: 8-bit frames whose window rows start on 16-byte boundaries; the next
// tile's rows are copied with cp.async while the current tile runs.
// Registers: the 18 warps are spread over the SM's four sub-partitions (16K
// registers each), five on each of the first two, so a thread may hold at
// most 96.
template <bool ASYNC>
__global__ void __maxnreg__(96) k_corr_tc64(CorrArgs a, int* status) {
  using L = Tc64;
  constexpr int SS = L::SS, N = L::N, HN = L::HN, W = L::W;
  extern __shared__ __align__(16) unsigned char sm[];
  // Completion of each product (committed by the MMA warp) and readiness of
  // each operand (one arrival per compute warp). Each completes once per tile.
  enum { kS1, kS2a, kS2b, kS3, kS4, kNDone };
  enum { kRA1, kRA2, kRQa, kRQ, kRA4, kNReady };
  __shared__ uint64_t done_bar[kNDone], ready_bar[kNReady];
  // The neighbour rows and peak keys of a tile are written (one arrival per
  // compute warp) / have been read by its fits (fit warp). Each completes
  // once per tile.
  __shared__ uint64_t nbr_full, nbr_empty;
  __shared__ uint32_t tmem_base_s;
  __shared__ int abort_s;
  __shared__ float red[2][2][W][4];  // sums, then absolute deviations: per frame and window, the four row groups' partials
  // Per tile slot (four: the tile whose fits are pending, the tile being
  // correlated, the next one, whose rows are in flight, and the one after,
  // whose corners are being computed); slot = local tile count % 4.
  __shared__ int sc_e[4][2][W];      // per frame and window: log2 of the operand scale
  __shared__ float mean_s[4][2][W];  // per frame and window: the window mean
  __shared__ long long win_base[4][W];
  __shared__ int win_valid[4][W];
  __shared__ long long win_loc[4][W];  // window index within its segment
  __shared__ int win_seg[4][W];
  __shared__ CorrSeg seg_s[kMaxCorrSegs];
  // Per window, for the current tile and the one whose fits are pending
  // (local tile count % 2): the running first maximum (peak_key) and the key
  // of the largest half-row maximum outside the peak row.
  __shared__ unsigned long long pk_key[2][W];
  __shared__ unsigned sec_key[2][W];

  const int tid = threadIdx.x;
  const int q = tid >> 7, t = tid & 127;
  const int warp = tid >> 5, lane = tid & 31;
  const uint32_t lane_sel = (uint32_t)(32 * (warp & 3)) << 16;

  float* tw_re = reinterpret_cast<float*>(sm + L::OP);
  float* tw_im = tw_re + N;
  for (int k = tid; k < N; k += L::NT) {
    float sn, cs;
    sincospif(2.0f * (float)k / (float)N, &sn, &cs);
    tw_re[k] = cs;
    tw_im[k] = -sn;
  }
  if (tid == 0) {
    for (int k = 0; k < kNDone; ++k) tc::mbar_init(&done_bar[k], 1);
    for (int k = 0; k < kNReady; ++k) tc::mbar_init(&ready_bar[k], L::NCW);
    tc::mbar_init(&nbr_full, L::NCW);
    tc::mbar_init(&nbr_empty, 1);
    abort_s = 0;
  }
  __syncthreads();
  const float inv_n = 1.0f / (float)N;
  const int p0 = SS / 2;
  for (int e = tid; e < N * SS; e += L::NT) {  // F[k][x]
    const int k = e / SS, x = e % SS, f = k >> 1, qq = (f * (x + p0)) % N;
    float v;
    if (k == 0) v = 1.0f;
    else if (k == 1) v = ((x + p0) & 1) ? -1.0f : 1.0f;
    else v = (k & 1) ? tw_im[qq] : tw_re[qq];
    sth(sm + L::B1, off_k(k, x, SS), v);
  }
  for (int e = tid; e < 3 * N * HN; e += L::NT) {  // B3 blocks C, -S, S: [r][g]
    const int blk = e / (N * HN), r = (e / HN) % N, g = e % HN;
    const int qq = (g * r) % N;
    sth(sm + L::B3 + blk * L::NB3, off_k(r, g, HN),
        stage3_weight(blk, r, g, tw_re[qq] * inv_n, -tw_im[qq] * inv_n, inv_n));
  }
  for (int e = tid; e < N * N; e += L::NT) {  // B4[s][kappa = (part, c)]
    const int s_ = e / N, kap = e % N, part = kap / HN, c = kap % HN;
    const int qq = (c * s_) % N;
    float v;
    if (c == 0) v = part == 0 ? inv_n : ((s_ & 1) ? -inv_n : inv_n);
    else v = part == 0 ? 2.0f * tw_re[qq] * inv_n : 2.0f * tw_im[qq] * inv_n;
    sth(sm + L::B4, off_k(s_, kap, N), v);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base_s, L::TCOLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base_s;
  const uint32_t sbase = tc::smem_u32(sm);

  const int n_seg = load_segments(a, seg_s);
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  const int n_tiles = (int)((total + W - 1) / W);
  const int first = blockIdx.x, stride = gridDim.x;
  const bool ties = any_tie_output(seg_s, n_seg);
  float* nbrow = reinterpret_cast<float*>(sm + L::NBR);  // [W][3][N]: rows pi-1, pi, pi+1 (natural columns)

  // Corners, validity and segment of window wi of tile tl, into slot sl.
  auto window_setup = [&](int tl, int sl, int wi) {
    const long long g = (long long)tl * W + wi;
    int ok = tl < n_tiles && g < total;
    long long base = 0, loc = 0;
    int sg = 0;
    if (ok) {
      while (sg + 1 < n_seg && g >= seg_s[sg + 1].win0) ++sg;
      const CorrSeg& sq = seg_s[sg];
      loc = g - sq.win0;
      // 32-bit quotients: a segment holds fewer than 2^31 windows (checked at launch).
      const int li = (int)loc, nw = sq.m * sq.n;
      const int pair = li / nw, k = li - pair * nw;
      const int wr = k / sq.n, wc = k - wr * sq.n;
      if (sq.win_mask) ok = sq.win_mask[k] == 0;
      base = pair * (long long)sq.height * sq.width + (long long)(wr * sq.spacing + sq.y_offset) * sq.width +
             wc * sq.spacing + sq.x_offset;
      if (ok && !in_bounds(base >= 0 && base + (long long)(SS - 1) * sq.width + SS <=
                                            (long long)sq.n_pairs * sq.height * sq.width))
        ok = 0;
    }
    win_valid[sl][wi] = ok;
    win_base[sl][wi] = base;
    win_loc[sl][wi] = loc;
    win_seg[sl][wi] = sg;
  };
  uint32_t ph_full = 0u;
  // Near-tie flags and subpixel fits of tile `tl` (local tile count `it`), run
  // by the fit warp: every lane waits for the tile's neighbour rows, the warp
  // runs the near-tie test, lanes < W fit one window each and set up the
  // windows of tile tl + 4 strides, then lane 0 hands the rows back. False
  // when the wait gave up.
  auto fit_tile = [&](int tl, int it) -> bool {
    const bool got = __all_sync(0xffffffffu, tc::mbar_wait_bounded(&nbr_full, ph_full, kMaxPolls));
    ph_full ^= 1u;
    if (!got) {
      if (lane == 0) {
        abort_s = 1;
        atomicExch(status, PIV_E_TIMEOUT);
      }
      return false;
    }
    const int sl = it & 3, kb = it & 1;
    const long long g0 = (long long)tl * W;
    const bool mine = lane < W && g0 + lane < total;
    const CorrSeg& sq = seg_s[win_seg[sl][mine ? lane : 0]];
    const long long gl = win_loc[sl][mine ? lane : 0];
    const bool gl_ok = mine && in_bounds(gl >= 0 && gl < (long long)sq.n_pairs * sq.m * sq.n);
    if (ties) {
      const bool tie = tile_near_ties<N, W>(lane, sec_key[kb], a.tie_tol,
                                            [&](int ww) { return peak_index(pk_key[kb][ww]); },
                                            [&](int ww) { return nbrow + (ww * 3 + 1) * N; }) &&
                       mine && win_valid[sl][lane];
      if (gl_ok) {
        if (sq.near_tie) sq.near_tie[gl] = tie ? 1 : 0;
        if (tie && sq.tie_count) atomicAdd(sq.tie_count, 1);
      }
    }
    if (gl_ok) {
      const int ww = lane;
      const int pidx = peak_index(pk_key[kb][ww]), pi_ = pidx / N, pj = pidx % N;
      float isp = (float)pi_, jsp = (float)pj;
      if (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1) {
        const int ue = -sc_e[sl][0][ww] - sc_e[sl][1][ww];
        const float s1 = pow2i(ue >> 1), s2 = pow2i(ue - (ue >> 1));
        auto at = [&](int ii, int j) -> float {
          return (ii == 0 || j == 0) ? 0.f : nbrow[(ww * 3 + (ii - pi_ + 1)) * N + (j ^ HN)] * s1 * s2;
        };
        subpixel_fit(a.subpixel, pi_, pj, at(pi_, pj), at(pi_ - 1, pj), at(pi_ + 1, pj), at(pi_, pj - 1),
                     at(pi_, pj + 1), isp, jsp);
      }
      float* uo = reinterpret_cast<float*>(sq.u);
      float* vo = reinterpret_cast<float*>(sq.v);
      if (win_valid[sl][ww]) {
        uo[gl] = sub_rn(jsp, (float)HN);
        vo[gl] = sub_rn(isp, (float)HN);
      } else {
        uo[gl] = NAN;
        vo[gl] = NAN;
      }
      if (sq.peak_i) sq.peak_i[gl] = pi_;
      if (sq.peak_j) sq.peak_j[gl] = pj;
    }
    // The corners of the tile four strides on, into this tile's slot (its
    // fits are done): the compute warps use them from tile it + 3 on (the
    // copy of its rows), after waiting for these fits in the epilogue of
    // tile it + 1.
    if (lane < W) window_setup(tl + 4 * stride, it & 3, lane);
    __syncwarp();
    if (lane == 0) tc::mbar_arrive(&nbr_empty);
    return true;
  };
  if (warp == L::NCW) {
    // ---- MMA warp: lane 0 waits for each operand, then the converged warp
    // issues the product (one elected lane; the descriptor arithmetic stays
    // on the uniform datapath) and commits it; a wait that gives up stops
    // the warp (the compute warps' own waits then give up as well).
    uint32_t ph[kNReady] = {0u, 0u, 0u, 0u, 0u};
    auto ready = [&](int k) -> bool {
      bool ok = true;
      if (lane == 0) {
        ok = tc::mbar_wait_bounded(&ready_bar[k], ph[k], kMaxPolls);
        if (!ok) {
          abort_s = 1;
          atomicExch(status, PIV_E_TIMEOUT);
        }
      }
      ph[k] ^= 1u;
      ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
      tc::fence_after_sync();
      return ok;
    };
    // Stage 1: T = a F^T per frame -> TMEM cols [T_S1 + f N, + N).
    auto stage1 = [&]() {
      const uint32_t id = tc::idesc_f16(128, N, 0, 0);
#pragma unroll
      for (int f = 0; f < 2; ++f)
#pragma unroll
        for (int ks = 0; ks < SS / 16; ++ks)
          tc::mma_f16<true>(tmem + L::T_S1 + f * N,
                            tc::sdesc(sbase + L::A1 + f * L::A1_BYTES + ks * 256, 128, SS * 16),
                            tc::sdesc(sbase + L::B1 + ks * 256, 128, SS * 16), id, ks > 0);
      tc::mma_commit<true>(&done_bar[kS1]);
      __syncwarp();
    };
    if (first < n_tiles && ready(kRA1)) {
      stage1();
      for (int tile = first; tile < n_tiles; tile += stride) {
        // Stage 2 in two halves of f_r: X = T^T F^T, packed columns [64 h, 64 h + 64)
        // of spectrum (rt, f) -> TMEM cols [256 h + (2 rt + f) 64, + 64).
        if (!ready(kRA2)) break;
        {
          const uint32_t id = tc::idesc_f16(128, HN, 1, 0);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
#pragma unroll
            for (int rt = 0; rt < 2; ++rt)
#pragma unroll
              for (int f = 0; f < 2; ++f)
#pragma unroll
                for (int ks = 0; ks < SS / 16; ++ks)
                  tc::mma_f16<true>(
                      tmem + 256 * h + (rt * 2 + f) * HN,
                      tc::sdesc(sbase + L::OP + (f * 2 + rt) * L::A2_BYTES + ks * 32 * 128, 128 * 16, 128),
                      tc::sdesc(sbase + L::B1 + h * 8 * SS * 16 + ks * 256, 128, SS * 16), id, ks > 0);
            tc::mma_commit<true>(&done_bar[h == 0 ? kS2a : kS2b]);
          }
        }
        __syncwarp();
        // Stage 3: Re U = [Re P | Im M] [C; -S] -> cols [0, N); Im U = [Im P | Re M] [C; S]
        // -> cols [N, 2N). Block b4 of the operand (Re P, Im M, Im P, Re M), g in
        // [16 s, 16 s + 16), sits in half s / 2 at column 32 b4 + 16 (s % 2). The
        // K steps of operand half hh (g in [32 hh, 32 hh + 32)) go as soon as the
        // compute warps have written that half.
        {
          const uint32_t id = tc::idesc_f16(128, N, 0, 0);
          bool ok = true;
#pragma unroll
          for (int hh = 0; hh < 2 && ok; ++hh) {
            ok = ready(hh == 0 ? kRQa : kRQ);
            if (!ok) break;
#pragma unroll
            for (int part = 0; part < 2; ++part)
#pragma unroll
              for (int kb = 0; kb < 2; ++kb)
#pragma unroll
                for (int s = 2 * hh; s < 2 * hh + 2; ++s) {
                  const int b4 = 2 * part + kb;
                  tc::mma_f16<true>(
                      tmem + part * N,
                      tc::sdesc(sbase + (hh == 0 ? L::A1 : L::OP) + (32 * b4 + 16 * (s & 1)) * 16, 128, L::QH * 16),
                      tc::sdesc(sbase + L::B3 + (kb == 0 ? 0 : 1 + part) * L::NB3 + s * 256, 128, HN * 16), id,
                      (kb | s) != 0);
                }
          }
          if (!ok) break;
          tc::mma_commit<true>(&done_bar[kS3]);
        }
        __syncwarp();
        // Stage 4: c = U E' / N -> TMEM cols [rt N, rt N + N).
        if (!ready(kRA4)) break;
        {
          const uint32_t id = tc::idesc_f16(128, N, 1, 0);
#pragma unroll
          for (int rt = 0; rt < 2; ++rt)
#pragma unroll
            for (int ks = 0; ks < N / 16; ++ks)
              tc::mma_f16<true>(tmem + rt * N,
                                tc::sdesc(sbase + L::OP + rt * L::A4_BYTES + ks * 32 * 128, 128 * 16, 128),
                                tc::sdesc(sbase + L::B4 + ks * 256, 128, N * 16), id, ks > 0);
          tc::mma_commit<true>(&done_bar[kS4]);
        }
        __syncwarp();
        if (tile + stride < n_tiles) {
          if (!ready(kRA1)) break;
          stage1();
        }
      }
    }
  } else if (warp == L::NCW + 1) {
    // ---- Fit warp: the near-tie test and the subpixel fits of each tile,
    // once the compute warps have left its neighbour rows and peak keys.
    for (int tile = first, it = 0; tile < n_tiles; tile += stride, ++it)
      if (!fit_tile(tile, it)) break;
  } else {
    // ---- Compute warps (512 threads).
    // TMEM loads of the CTA's allocation (checked build: columns inside it).
    auto tld = [&](uint32_t addr, float (&v)[16]) {
      if (in_bounds(((addr - tmem) & 0xffffu) + 16 <= (uint32_t)L::TCOLS)) tc::tmem_ld16(addr, v);
    };
    auto cw_sync = []() { asm volatile("bar.sync 1, %0;" ::"n"(L::NC) : "memory"); };
    // Barrier of the compute warps that also ORs `p` over them: every thread
    // gets the same answer (a flag read by each thread separately could
    // change between the reads when the MMA warp sets it).
    auto cw_sync_or = [](bool p) -> bool {
      int r;
      asm volatile(
          "{\n"
          ".reg .pred a, b;\n"
          "setp.ne.s32 a, %1, 0;\n"
          "bar.red.or.pred b, 1, %2, a;\n"
          "selp.s32 %0, 1, 0, b;\n"
          "}\n"
          : "=r"(r)
          : "r"((int)p), "n"(L::NC)
          : "memory");
      return r != 0;
    };
    uint32_t ph[kNDone] = {0u, 0u, 0u, 0u, 0u};
    uint32_t ph_empty = 0u;
    // Every thread waits for the product itself; a wait that gives up sets
    // abort_s, which the compute warps read through the barrier reduction
    // after the peak search.
    auto done = [&](int k) {
      const bool ok = tc::mbar_wait_bounded(&done_bar[k], ph[k], kMaxPolls);
      ph[k] ^= 1u;
      if (!ok) {
        abort_s = 1;
        atomicExch(status, PIV_E_TIMEOUT);
      }
      tc::fence_after_sync();
    };
    // This warp's operand writes (and its TMEM loads) are complete.
    auto signal = [&](int k) {
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&ready_bar[k]);
    };
    // Thread (q, t) copies chunks 2h, 2h + 1 of row t of frame f: the bytes it
    // stages itself; rows of invalid windows are zero-filled (no global read).
    auto stage_async = [&](int sl) {
      const int f = q & 1, h = q >> 1, w = t >> 6, y = t & 63;
      const bool ok = win_valid[sl][w] != 0;
      const CorrSeg& sq = seg_s[win_seg[sl][w]];
      const uint8_t* src = reinterpret_cast<const uint8_t*>(f == 0 ? sq.frame_a : sq.frame_b) +
                           (ok ? win_base[sl][w] + (long long)y * sq.width + 16 * 2 * h : 0);
      const uint32_t row = sbase + L::STG + (uint32_t)((f * 128 + t) * SS);
#pragma unroll
      for (int c = 0; c < 2; ++c)
        cp_async16_zfill(row + 16 * stg64_chunk(t, 2 * h + c), src + (ok ? 16 * c : 0), ok);
    };
    // Half h = q >> 1 of row y of window w of frame f = q & 1 of the tile in
    // slot sl, as floats (thread (q, t), w = t >> 6, y = t & 63).
    auto load_half_row = [&](int sl, float (&r)[32]) {
      const int f = q & 1, h = q >> 1, w = t >> 6, y = t & 63;
      if (ASYNC) {
        const unsigned char* row = sm + L::STG + (f * 128 + t) * SS;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const uint4 q4 = *reinterpret_cast<const uint4*>(row + 16 * stg64_chunk(t, 2 * h + c));
          const uint32_t wds[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
          for (int k = 0; k < 16; ++k) r[16 * c + k] = u8_to_float(wds[k >> 2], k & 3);
        }
      } else {
        const CorrSeg& sq = seg_s[win_seg[sl][w]];
        load_row(f == 0 ? sq.frame_a : sq.frame_b, a.pixel_type, win_base[sl][w] + (long long)y * sq.width + 32 * h,
                 win_valid[sl][w] != 0, r);
      }
    };
    // Window statistics of the tile in slot sl: mean and operand scale
    // exponent per frame and window (sum |2^e (a - mean)| <= 2^7), formed
    // while the previous tile's stage 2 is on the tensor cores.
    auto stage_stats = [&](int sl) {
      const int f = q & 1, h = q >> 1, w = t >> 6, y = t & 63, grp = h * 2 + ((t >> 5) & 1);
      float r[32];
      load_half_row(sl, r);
      float sum = 0.f;
#pragma unroll
      for (int x = 0; x < 32; ++x) sum += r[x];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      if (lane == 0) red[0][f][w][grp] = sum;
      cw_sync();
      const float mean = (red[0][f][w][0] + red[0][f][w][1] + red[0][f][w][2] + red[0][f][w][3]) / (float)(SS * SS);
      float l = 0.f;
#pragma unroll
      for (int x = 0; x < 32; ++x) l += fabsf(r[x] - mean);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
      if (lane == 0) red[1][f][w][grp] = l;
      cw_sync();
      if (h == 0 && y == 0) {
        const float l1 = red[1][f][w][0] + red[1][f][w][1] + red[1][f][w][2] + red[1][f][w][3];
        int e = 0;
        if (l1 > 0.f) e = min(120, max(-120, 6 - exp2_floor(l1)));
        sc_e[sl][f][w] = e;
        mean_s[sl][f][w] = mean;
        const CorrSeg& sq = seg_s[win_seg[sl][w]];
        if (sq.win_means && win_valid[sl][w]) sq.win_means[2 * win_loc[sl][w] + f] = mean;
      }
      // Every thread's stage_tile reads them (nothing else orders the two).
      cw_sync();
    };
    // Staging of the tile in slot sl (statistics known) -> stage-1 operands:
    // (a - mean) 2^e as fp16, no reductions or barriers on this path.
    auto stage_tile = [&](int sl) {
      const int f = q & 1, h = q >> 1, w = t >> 6;
      float r[32];
      load_half_row(sl, r);
      const float mean = mean_s[sl][f][w], s = pow2i(sc_e[sl][f][w]);
#pragma unroll
      for (int x = 0; x < 32; ++x) r[x] = (r[x] - mean) * s;
#pragma unroll
      for (int x = 0; x < 32; x += 8) st8(sm + L::A1 + f * L::A1_BYTES, off_k(t, 32 * h + x, SS), r + x);
    };

    if (tid < W)
      for (int k = 0; k < 4; ++k) window_setup(first + k * stride, k, tid);
    cw_sync();
    if (first < n_tiles) {
      if (ASYNC) {
        stage_async(0);
        cp_async_commit();
        cp_async_wait_all();
      }
      stage_stats(0);
      stage_tile(0);
      signal(kRA1);
      if (ASYNC && first + stride < n_tiles) {
        stage_async(1);  // the next tile's rows land while this tile runs
        cp_async_commit();
      }
    }

    int it = 0;  // local tile count
    for (int tile = first; tile < n_tiles; tile += stride, ++it) {
      const long long g0 = (long long)tile * W;
      const int sl = it & 3, sl1 = (it + 1) & 3, kb = it & 1;
      const bool has_next = tile + stride < n_tiles;
      // The fits of tile it - 2 (same keys) have finished: this thread waited
      // for them before writing the neighbour rows of tile it - 1.
      if (tid < W) {
        pk_key[kb][tid] = 0ull;
        sec_key[kb][tid] = kKeyNegInf;
      }

      // ---- Stage 1 -> 2: thread (q, t) moves packed columns [64 h, 64 h + 64) of frame f.
      done(kS1);
      {
        const int f = q & 1, h = q >> 1, w = t >> 6, y = t & 63;
        float v[64];
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16)
          tld(tmem + lane_sel + L::T_S1 + f * N + 64 * h + c0, *reinterpret_cast<float(*)[16]>(v + c0));
        tc::tmem_ld_wait();
        tc::reg_fence(v);
#pragma unroll
        for (int rt = 0; rt < 2; ++rt) {
          unsigned char* dst = sm + L::OP + (f * 2 + rt) * L::A2_BYTES;
#pragma unroll
          for (int c0 = 0; c0 < 32; c0 += 8) {
            float v8[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v8[j] = v[2 * (c0 + j) + rt];
            st8(dst, off_mn(w * HN + 32 * h + c0, y, 128), v8);
          }
        }
      }
      signal(kRA2);
      // The next tile's window statistics while stage 2 runs (its rows were
      // copied during the previous tile).
      if (has_next) {
        if (ASYNC) cp_async_wait_all();
        stage_stats(sl1);
      }

      // ---- Product, per half hh of f_r: thread (q, t) folds g in [32 hh + 8 q, + 8)
      // of row c = t % HN of window t / HN into half hh of the stage-3 operand
      // (K-major [128][128], block b4 at column 32 b4).
      {
        const bool special = (t % HN) == 0;
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
          done(hh == 0 ? kS2a : kS2b);
          const int g0 = 32 * hh + 8 * q;
          const uint32_t src = tmem + lane_sel + 256 * hh + 16 * q;
          float ea[16], eb[16], oa[16], ob[16];
          tld(src + 0 * HN, ea);
          tld(src + 1 * HN, eb);
          tld(src + 2 * HN, oa);
          tld(src + 3 * HN, ob);
          tc::tmem_ld_wait();
          tc::reg_fence(ea); tc::reg_fence(eb); tc::reg_fence(oa); tc::reg_fence(ob);
          float rp[8], im[8], ip[8], rm[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            PairPM o;
            if (i == 0 && g0 == 0) {  // f_r = 0 and N/2, not folded (halved)
              const PairQ q0 = pair_product(ea[0], 0.f, oa[0], 0.f, eb[0], 0.f, ob[0], 0.f, special);
              const PairQ q1 = pair_product(ea[1], 0.f, oa[1], 0.f, eb[1], 0.f, ob[1], 0.f, special);
              o.pr = 0.5f * q0.r0; o.mi = 0.5f * q1.r0; o.pi = 0.5f * q0.i0; o.mr = 0.5f * q1.i0;
            } else {
              o = pair_fold_half(ea[2 * i], ea[2 * i + 1], oa[2 * i], oa[2 * i + 1], eb[2 * i], eb[2 * i + 1],
                                 ob[2 * i], ob[2 * i + 1], special);
            }
            rp[i] = o.pr; im[i] = o.mi; ip[i] = o.pi; rm[i] = o.mr;
          }
          unsigned char* dst = sm + (hh == 0 ? L::A1 : L::OP);
          st8(dst, off_k(t, 0 * 32 + 8 * q, L::QH), rp);
          st8(dst, off_k(t, 1 * 32 + 8 * q, L::QH), im);
          st8(dst, off_k(t, 2 * 32 + 8 * q, L::QH), ip);
          st8(dst, off_k(t, 3 * 32 + 8 * q, L::QH), rm);
          signal(hh == 0 ? kRQa : kRQ);
        }
      }

      // ---- Stage 3 -> 4: thread (q, t) moves r in [64 rh, 64 rh + 64) of part q & 1 of row (w, c).
      done(kS3);
      {
        const int part = q & 1, rh = q >> 1, w = t / HN, c = t % HN;
        float v[64];
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16)
          tld(tmem + lane_sel + part * N + 64 * rh + c0, *reinterpret_cast<float(*)[16]>(v + c0));
        tc::tmem_ld_wait();
        tc::reg_fence(v);
#pragma unroll
        for (int r0 = 0; r0 < 64; r0 += 8) {
          const int m = w * N + 64 * rh + r0;
          st8(sm + L::OP + (m >> 7) * L::A4_BYTES, off_mn(m & 127, part * HN + c, 128), v + r0);
        }
      }
      signal(kRA4);

      // ---- The next tile's staging while stage 4 runs; then the copy of the
      // rows of the tile after it (each thread copies the bytes it reads).
      if (has_next) {
        stage_tile(sl1);
        signal(kRA1);
        if (ASYNC && tile + 2 * stride < n_tiles) {
          stage_async((it + 2) & 3);
          cp_async_commit();
        }
      }

      // ---- Epilogue: thread (q, t) holds shifted columns [64 ch, 64 ch + 64) of
      // map row t of window w = q & 1 (row index i = t ^ N/2).
      done(kS4);
      const int w = q & 1, ch = q >> 1, i = t ^ HN;
      const int s0 = ch == 0 ? HN : 0;  // natural column of shifted column 64 ch
      float hbest;  // maximum of this thread's half row
      {
        float v[64];
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16)
          tld(tmem + lane_sel + w * N + s0 + c0, *reinterpret_cast<float(*)[16]>(v + c0));
        tc::tmem_ld_wait();
        tc::reg_fence(v);
        if (ch == 0) v[0] = 0.f;  // shifted column 0: no window overlap
        float best;
        int bk;
        first_max<64>(v, best, bk);
        int idx = i * N + 64 * ch + bk;
        if (i == 0) { best = 0.f; idx = 64 * ch; }  // shifted row 0: no window overlap
        hbest = best;
        warp_first_max(best, idx);
        if (lane == 0) atomicMax(&pk_key[kb][w], peak_key(best, idx));
        if (a.maps && g0 + w < total) {
          const int ue = -sc_e[sl][0][w] - sc_e[sl][1][w];
          float* mo = reinterpret_cast<float*>(a.maps) + (g0 + w) * N * N + (long long)i * N + 64 * ch;
#pragma unroll
          for (int k = 0; k < 64; ++k) mo[k] = i == 0 ? 0.f : ldexpf(v[k], ue);
        }
      }
      // Every warp's candidate is in the peak keys; the abort decision is the
      // same for every compute thread (the fit warp's wait for this tile's
      // rows then gives up by itself).
      if (cw_sync_or(abort_s != 0)) break;
      {
        const int pidx = peak_index(pk_key[kb][w]), pi_ = pidx / N, pj = pidx % N;
        if (ties) {  // the warp's largest half-row maximum outside the peak row (a warp's rows share a window)
          const unsigned k = __reduce_max_sync(0xffffffffu, i == pi_ ? kKeyNegInf : fkey(hbest));
          if (lane == 0) atomicMax(&sec_key[kb][w], k);
        }
        const bool mine = (ties && i == pi_) ||
                          (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1 && i >= pi_ - 1 && i <= pi_ + 1);
        // The fit warp has run the fits of the previous tile (it has read the rows).
        if (it > 0) {
          const bool ok = tc::mbar_wait_bounded(&nbr_empty, ph_empty, kMaxPolls);
          ph_empty ^= 1u;
          if (!ok) {
            abort_s = 1;
            atomicExch(status, PIV_E_TIMEOUT);
          }
        }
        if (__any_sync(0xffffffffu, mine)) {
          float v[64];
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += 16)
            tld(tmem + lane_sel + w * N + s0 + c0, *reinterpret_cast<float(*)[16]>(v + c0));
          tc::tmem_ld_wait();
          tc::reg_fence(v);
          if (mine) {
            float4* dst = reinterpret_cast<float4*>(nbrow + (w * 3 + (i - pi_ + 1)) * N + s0);
            if (in_dyn_smem(dst, 64 * 4))
#pragma unroll
              for (int c4 = 0; c4 < 16; ++c4)
                dst[c4] = make_float4(v[4 * c4], v[4 * c4 + 1], v[4 * c4 + 2], v[4 * c4 + 3]);
          }
        }
      }
      // This warp's neighbour rows and near-tie key are written: the fit warp
      // runs the fits once all sixteen warps have arrived, while this tile's
      // successor is correlated. (The map's TMEM columns are read before
      // this warp's stage-2 arrival of the next tile, which the stage-2
      // product waits for.)
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&nbr_full);
    }
    if (ASYNC) cp_async_wait_all();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, L::TCOLS);
}

#define PIV_TRY_TC(expr)             \
  do {                               \
    const int _rc = (expr);          \
    if (_rc != PIV_OK) return _rc;   \
  } while (0)

template <bool ASYNC>
static int launch_tc64_t(const CorrArgs& a, cudaStream_t stream) {
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  const int n_tiles = (int)((total + Tc64::W - 1) / Tc64::W);
  static thread_local int configured_dev = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured_dev != dev) {
    cudaError_t e =
        cudaFuncSetAttribute(k_corr_tc64<ASYNC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Tc64::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_corr_tc64<ASYNC>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaFuncSetAttribute(k_corr_tc64)");
    configured_dev = dev;
  }
  int grid = sm_count();
  if (grid > n_tiles) grid = n_tiles;
  CorrArgs b = a;
  b.tie_tol = kTieTolF16;
  k_corr_tc64<ASYNC><<<grid, Tc64::NT, Tc64::SMEM, stream>>>(b, a.status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_corr_tc64 launch");
}

// Rows of 8-bit frames start on 16-byte boundaries (asynchronous staging of
// the 64-px engine).
static bool rows_aligned(const void* fa, const void* fb, int width, int x_offset, int spacing, int px) {
  return ((uintptr_t)fa % 16) == 0 && ((uintptr_t)fb % 16) == 0 && width % px == 0 && x_offset % px == 0 &&
         spacing % px == 0;
}

// Every geometry of the launch satisfies rows_aligned with px pixels per 16 bytes.
static bool all_rows_aligned(const CorrArgs& a, int px) {
  if (a.n_segs <= 0) return rows_aligned(a.frame_a, a.frame_b, a.width, a.x_offset, a.spacing, px);
  for (int k = 0; k < a.n_segs; ++k) {
    const CorrSeg& q = a.segs[k];
    if (!rows_aligned(q.frame_a, q.frame_b, q.width, q.x_offset, q.spacing, px)) return false;
  }
  return true;
}

static bool tc64_aligned(const CorrArgs& a) { return a.pixel_type == PIV_PIXEL_U8 && all_rows_aligned(a, 16); }

// Rows of float frames start on 16-byte boundaries (asynchronous staging of
// the 16/32-px engine).
static bool tc_aligned(const CorrArgs& a) { return a.pixel_type == PIV_PIXEL_F32 && all_rows_aligned(a, 4); }

// One bounded wait on an mbarrier that no arrival completes: the primitive
// behind every tcgen05 completion wait of the correlation kernels, run until
// it gives up. Writes the status word the kernels would set.
__global__ void k_wait_probe(uint32_t max_polls, int* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  const bool ok = tc::mbar_wait_bounded(&bar, 0, max_polls);
  if (threadIdx.x == 0) *status = ok ? PIV_OK : PIV_E_TIMEOUT;
}

int bounded_wait_probe(uint32_t max_polls, int* status_dev, cudaStream_t stream) {
  k_wait_probe<<<1, 32, 0, stream>>>(max_polls, status_dev);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_wait_probe launch");
}

bool correlate_tensor_supported(const CorrArgs& a, int dft_mode) {
  if (dft_mode != PIV_DFT_TENSOR && dft_mode != PIV_DFT_TENSOR_SPLIT && dft_mode != PIV_DFT_TENSOR_REFINED)
    return false;
  // The refined form, and the split form's 64-px passes (which take the
  // refined path: the split engine's operands do not fit beside 64-px
  // constants), need the refinement.
  if ((dft_mode == PIV_DFT_TENSOR_REFINED || (dft_mode == PIV_DFT_TENSOR_SPLIT && a.ss == 64)) &&
      !refine_supported(a))
    return false;
  if (a.n_segs < 0 || a.n_segs > kMaxCorrSegs) return false;
  if (a.n_segs == 0 && (long long)a.n_pairs * a.m * a.n >= (1LL << 31)) return false;
  for (int k = 0; k < a.n_segs; ++k)
    if ((long long)a.segs[k].n_pairs * a.segs[k].m * a.segs[k].n >= (1LL << 31)) return false;
  return a.dtype == PIV_DTYPE_F32 && a.s2n == nullptr && a.ws == a.ss && a.fft_size == 2 * a.ss &&
         (a.ss == 16 || a.ss == 32 || a.ss == 64);
}

// Resident CTAs per SM the 16/32-px engine allows (TMEM, registers, shared
// memory), and the device limits the shared-memory padding is computed from:
// the occupancy API does not know about TMEM, so a launch pads its dynamic
// shared memory until no more than the chosen number of CTAs fits on an SM.
struct TcLaunch {
  int max_per_sm = 0;
  size_t static_smem = 0;
  int smem_sm = 0, smem_optin = 0, resv = 0;
};

template <int SS, bool ASYNC, bool SPLIT>
static int tc_launch_config(TcLaunch& out) {
  using L = TcLayout<SS, SPLIT>;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k_corr_tc<SS, ASYNC, SPLIT>);
  if (e != cudaSuccess) return set_cuda_error(e, "cudaFuncGetAttributes(k_corr_tc)");
  int smem_sm = 0, smem_optin = 0, resv = 0, regs_sm = 0;
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
  const size_t per_cta = L::SMEM + fa.sharedSizeBytes + resv;
  int per_sm = 512 / L::TCOLS;
  const int by_smem = (int)(smem_sm / per_cta);
  const int regs_cta = ((fa.numRegs * 32 + 255) / 256) * 256 * (L::NT / 32);
  const int by_regs = regs_cta > 0 ? regs_sm / regs_cta : per_sm;
  per_sm = std::min(per_sm, std::min(by_smem, by_regs));
  if (per_sm < 1) return set_error(PIV_E_UNSUPPORTED, "tensor correlation does not fit on an SM");
  e = cudaFuncSetAttribute(k_corr_tc<SS, ASYNC, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(smem_optin - fa.sharedSizeBytes));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_corr_tc<SS, ASYNC, SPLIT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return set_cuda_error(e, "cudaFuncSetAttribute(k_corr_tc)");
  out.max_per_sm = per_sm;
  out.static_smem = fa.sharedSizeBytes;
  out.smem_sm = smem_sm;
  out.smem_optin = smem_optin;
  out.resv = resv;
  return PIV_OK;
}

// Dynamic shared memory that makes exactly k CTAs resident per SM.
static size_t tc_smem_for(const TcLaunch& c, int k, size_t need) {
  size_t smem = (size_t)c.smem_sm / k - c.static_smem - c.resv;
  smem = std::min(smem, (size_t)c.smem_optin - c.static_smem);
  smem = std::max(smem, need) & ~(size_t)15;
  return smem < need ? need : smem;
}

template <int SS, bool ASYNC, bool SPLIT>
static int tc_config_cached(TcLaunch*& cfg) {
  static thread_local int configured_dev = -1;
  static thread_local TcLaunch c;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured_dev != dev) {
    const int rc = tc_launch_config<SS, ASYNC, SPLIT>(c);
    if (rc != PIV_OK) return rc;
    configured_dev = dev;
  }
  cfg = &c;
  return PIV_OK;
}

// per_sm <= 0: as many CTAs per SM as fit.
template <int SS, bool ASYNC, bool SPLIT>
static int launch_tc_t(const CorrArgs& a, int per_sm, cudaStream_t stream) {
  using L = TcLayout<SS, SPLIT>;
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  const int n_tiles = (int)((total + L::W - 1) / L::W);
  TcLaunch* cfg = nullptr;
  PIV_TRY_TC((tc_config_cached<SS, ASYNC, SPLIT>(cfg)));
  const int k = per_sm <= 0 || per_sm > cfg->max_per_sm ? cfg->max_per_sm : per_sm;
  int grid = sm_count() * k;
  if (grid > n_tiles) grid = n_tiles;
  CorrArgs b = a;
  b.tie_tol = SPLIT ? kTieTolF32 : kTieTolF16;
  k_corr_tc<SS, ASYNC, SPLIT><<<grid, L::NT, tc_smem_for(*cfg, k, L::SMEM), stream>>>(b, a.status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_corr_tc launch");
}

template <int SS, bool SPLIT>
static int max_per_sm(bool async, int* out) {
  TcLaunch* cfg = nullptr;
  const int rc = async ? tc_config_cached<SS, true, SPLIT>(cfg) : tc_config_cached<SS, false, SPLIT>(cfg);
  *out = rc == PIV_OK ? cfg->max_per_sm : 0;
  return rc;
}

// Launch variants of a tensor pass. The 16/32-px engine: variant v runs
// (max_per_sm - v / S) CTAs per SM with asynchronous staging when S = 2 and v
// is even (S = 2 when the rows allow asynchronous staging, else 1). The
// 64-px engine: one CTA per SM; variant 1 loads synchronously. Variant 0 is
// the default; all variants give identical results.
int correlate_tensor_variant_count(const CorrArgs& a, int dft_mode) {
  if (!correlate_tensor_supported(a, dft_mode)) return 0;
  if (a.ss == 64) return tc64_aligned(a) ? 2 : 1;
  const bool al = tc_aligned(a);
  const bool split = dft_mode == PIV_DFT_TENSOR_SPLIT;
  int m = 0;
  if (a.ss == 16) split ? max_per_sm<16, true>(al, &m) : max_per_sm<16, false>(al, &m);
  else split ? max_per_sm<32, true>(al, &m) : max_per_sm<32, false>(al, &m);
  return m * (al ? 2 : 1);
}

int correlate_tensor_variant_describe(const CorrArgs& a, int dft_mode, int variant, int* per_sm, int* async) {
  const int n = correlate_tensor_variant_count(a, dft_mode);
  if (variant < 0 || variant >= n) return PIV_E_ARG;
  if (a.ss == 64) {
    *per_sm = 1;
    *async = tc64_aligned(a) && variant == 0;
    return PIV_OK;
  }
  const int S = tc_aligned(a) ? 2 : 1;
  *per_sm = n / S - variant / S;
  *async = S == 2 && variant % 2 == 0;
  return PIV_OK;
}

static int correlate_tensor_maps(const CorrArgs& a, int dft_mode, int variant, cudaStream_t stream);

// The refined form: the fp16 engine's maps give the integer peaks, then the
// subpixel stencil is recomputed in float32 (refine_peaks). Windows whose two
// largest fp16 values are within the fp16 tie tolerance (their fp16 peak may
// not be the float32 map's first maximum) are correlated again by the float32
// FFT engine, when the caller gives a list buffer; the near-tie flags and
// counts are then those of the FFT engine on those windows.
int correlate_tensor(const CorrArgs& a, int dft_mode, int variant, cudaStream_t stream) {
  if (!correlate_tensor_supported(a, dft_mode))
    return set_error(PIV_E_UNSUPPORTED, "tensor correlation: unsupported pass");
  const bool refined = dft_mode == PIV_DFT_TENSOR_REFINED || (dft_mode == PIV_DFT_TENSOR_SPLIT && a.ss == 64);
  if (!refined) return correlate_tensor_maps(a, dft_mode, variant, stream);
  const int n = a.n_segs > 0 ? a.n_segs : 1;
  bool rerun = true;
  for (int k = 0; k < n; ++k) {
    const CorrSeg* q = a.n_segs > 0 ? &a.segs[k] : nullptr;
    rerun = rerun && (q ? q->near_tie && q->tie_list && q->tie_list_count
                        : a.near_tie && a.tie_list && a.tie_list_count);
  }
  CorrArgs m = a;  // with a re-run, the fp16 pass flags its near ties but counts none
  if (rerun) {
    m.tie_count = nullptr;
    for (int k = 0; k < a.n_segs; ++k) m.segs[k].tie_count = nullptr;
  }
  int rc = correlate_tensor_maps(m, PIV_DFT_TENSOR, variant, stream);
  if (rc == PIV_OK) rc = refine_peaks(m, stream);
  for (int k = 0; rerun && rc == PIV_OK && k < n; ++k) {
    CorrArgs f = a;  // one frame geometry at a time
    f.n_segs = 0;
    if (a.n_segs > 0) {
      const CorrSeg& q = a.segs[k];
      f.frame_a = q.frame_a; f.frame_b = q.frame_b; f.u = q.u; f.v = q.v; f.peak_i = q.peak_i; f.peak_j = q.peak_j;
      f.win_mask = q.win_mask; f.near_tie = q.near_tie; f.tie_count = q.tie_count; f.tie_list = q.tie_list;
      f.tie_list_count = q.tie_list_count; f.height = q.height; f.width = q.width; f.spacing = q.spacing;
      f.m = q.m; f.n = q.n; f.x_offset = q.x_offset; f.y_offset = q.y_offset; f.n_pairs = q.n_pairs;
    }
    rc = compact_near_ties(f.near_tie, (long long)f.n_pairs * f.m * f.n, f.tie_list, f.tie_list_count, stream);
    f.win_list = f.tie_list;
    f.win_count = f.tie_list_count;
    if (rc == PIV_OK) rc = correlate_fft(f, 0, stream);
  }
  return rc;
}

static int correlate_tensor_maps(const CorrArgs& a, int dft_mode, int variant, cudaStream_t stream) {
  const long long total = a.n_segs > 0 ? a.seg_windows : (long long)a.n_pairs * a.m * a.n;
  if (total == 0) return PIV_OK;
  if (!a.status) return set_error(PIV_E_ARG, "tensor correlation needs a device status word");
  if (a.ss == 64) {
    const bool async = tc64_aligned(a) && variant <= 0;
    return async ? launch_tc64_t<true>(a, stream) : launch_tc64_t<false>(a, stream);
  }
  int per_sm = 0, async = tc_aligned(a);
  if (variant > 0 && correlate_tensor_variant_describe(a, dft_mode, variant, &per_sm, &async) != PIV_OK) {
    per_sm = 0;
    async = tc_aligned(a);
  }
  const bool split = dft_mode == PIV_DFT_TENSOR_SPLIT;
  if (a.ss == 16) {
    if (split) return async ? launch_tc_t<16, true, true>(a, per_sm, stream) : launch_tc_t<16, false, true>(a, per_sm, stream);
    return async ? launch_tc_t<16, true, false>(a, per_sm, stream) : launch_tc_t<16, false, false>(a, per_sm, stream);
  }
  if (split) return async ? launch_tc_t<32, true, true>(a, per_sm, stream) : launch_tc_t<32, false, true>(a, per_sm, stream);
  return async ? launch_tc_t<32, true, false>(a, per_sm, stream) : launch_tc_t<32, false, false>(a, per_sm, stream);
}

PIV_DEFINE_BOUNDS_COUNTER(bounds_violations_tensor)

}  // namespace piv
