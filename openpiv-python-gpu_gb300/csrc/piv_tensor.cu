// Tensor-core (tcgen05) cross-correlation of window pairs: the DFTs of the
// correlation (gpu_process.py:1207-1246) as dense matrix products on the 5th
// generation tensor cores, fp16 operands, fp32 accumulation in TMEM.
//
// A CTA of 256 threads owns a tile of W = 128/ss window pairs; threads t and
// t + 128 share TMEM lane t and split every phase in two natural halves
// (frame a / frame b, or row tile 0 / row tile 1). With N = 2 ss (the reference's default n_fft = 2, centred zero
// pad of ss/2):
//   stage 1  T = a G^T             rows (w, y),   K = x,             cols (Re|Im, f_c)
//   stage 2  A = G T               rows (w, f_c), K = (Re|Im, y),    cols (Re|Im, f_r)
//   product  P = s_w conj(A) B     in registers (fp32), s_w a power of two
//   stage 3  U = P E / N           rows (w, f_c), K = (Re|Im, f_r),  cols (Re|Im, r)
//   stage 4  c = Re(U E^T) / N     rows (w, r),   K = (Re|Im, f_c),  cols s
// G = exp(-2 pi i f (x + ss/2)/N) folds the zero pad into the forward matrices,
// E = exp(+2 pi i f r / N). Between stages a warp reads its accumulator lanes
// (tcgen05.ld), converts to fp16 and writes the next stage's operand tile to
// shared memory (K-major or MN-major, no swizzle). s_w = 2^(14 - ceil(log2(
// sum|a| * sum|b|))) keeps |P| below 2^14, inside fp16 range, and the two 1/N
// factors keep U and c there too; c is scaled back exactly. The map in TMEM
// (one row per lane) then goes through the same peak search and subpixel fit
// as the FFT engine: first maximum in the fftshift-ed row-major order, lags
// without window overlap read as exact zeros.
#include <cuda_fp16.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "piv_common.cuh"
#include "piv_internal.h"
#include "piv_tcgen05.cuh"

namespace piv {

template <int SS>
struct TcLayout {
  static constexpr int N = 2 * SS;          // DFT size
  static constexpr int W = 128 / SS;        // window pairs per tile
  static constexpr int TCOLS = 8 * N;       // TMEM columns (stage 2 holds A and B of both row tiles)
  // fp16 operand tiles (bytes).
  static constexpr int B1 = 0;                             // [2N][SS]   K-major
  static constexpr int B2 = B1 + 2 * N * SS * 2;           // [2N][2SS]  K-major
  static constexpr int B3 = B2 + 2 * N * 2 * SS * 2;       // [2N][2N]   K-major
  static constexpr int B4 = B3 + 2 * N * 2 * N * 2;        // [N][2N]    K-major
  static constexpr int A1 = B4 + N * 2 * N * 2;            // 2 x [128][SS] K-major (frames a, b)
  static constexpr int A2 = A1 + 2 * 128 * SS * 2;         // 2 frames x 2 row tiles x [128][2SS] MN-major; reused as A4
  static constexpr int A3 = A2 + 2 * 2 * 128 * 2 * SS * 2; // 2 row tiles x [128][2N] K-major
  static constexpr int END = A3 + 2 * 128 * 2 * N * 2;
  static constexpr int A2_TILE = 128 * 2 * SS * 2;         // bytes of one A2 row tile
  static constexpr int A4_TILE = 128 * 2 * N * 2;          // bytes of one A4 row tile (in the A2 region)
  static constexpr int A3_TILE = 128 * 2 * N * 2;
  static constexpr size_t SMEM = END + 1024;               // + alignment slack
};

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
  *reinterpret_cast<__half*>(base + off) = __float2half_rn(v);
}

static constexpr uint32_t kMaxPolls = 1u << 24;

template <int SS>
struct TcThreads {
  static constexpr int NT = 256;                  // two threads per TMEM lane
  static constexpr int MIN_BLOCKS = SS == 16 ? 2 : 1;
};

template <int SS>
__global__ void __launch_bounds__(256, TcThreads<SS>::MIN_BLOCKS) k_corr_tc(CorrArgs a, int* status) {
  using L = TcLayout<SS>;
  constexpr int N = L::N, W = L::W, H = N / 2;
  constexpr int NT = TcThreads<SS>::NT;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base_s;
  __shared__ float tw_re[N], tw_im[N];
  __shared__ float l1[2][W];         // sum |a - mean| and sum |b - mean| per window
  __shared__ float sc_exp[W];        // log2 of the product scale per window
  __shared__ long long win_base[W];
  __shared__ int win_valid[W];
  __shared__ float pk_val[W][2];     // per window: best value of each 32-row part
  __shared__ int pk_idx[W][2];
  __shared__ float nb[W][5];         // c, cd, cu, cl, cr

  const int tid = threadIdx.x;
  const int half = tid >> 7;         // frame (staging, stage 1 -> 2) or row tile (later phases)
  const int t = tid & 127;           // TMEM lane of this thread
  const int warp = tid >> 5, lane = tid & 31;
  const uint32_t lane_sel = (uint32_t)(32 * (warp & 3)) << 16;

  // Twiddles W_N^k = exp(-2 pi i k / N).
  for (int k = tid; k < N; k += NT) {
    float sn, cs;
    sincospif(2.0f * (float)k / (float)N, &sn, &cs);
    tw_re[k] = cs;
    tw_im[k] = -sn;
  }
  if (tid == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  // Constant DFT operands.
  const float inv_n = 1.0f / (float)N;
  const int pad = SS / 2;
  for (int e = tid; e < 2 * N * SS; e += NT) {  // B1[n][x]
    const int n = e / SS, x = e % SS, f = n % N, q = (f * (x + pad)) % N;
    sth(sm + L::B1, off_k(n, x, SS), n < N ? tw_re[q] : tw_im[q]);
  }
  for (int e = tid; e < 2 * N * 2 * SS; e += NT) {  // B2[n][k]
    const int n = e / (2 * SS), k = e % (2 * SS), fr = n % N, y = k % SS, part = k / SS;
    const int q = (fr * (y + pad)) % N;
    const float gr = tw_re[q], gi = tw_im[q];
    const float v = n < N ? (part == 0 ? gr : -gi) : (part == 0 ? gi : gr);
    sth(sm + L::B2, off_k(n, k, 2 * SS), v);
  }
  for (int e = tid; e < 2 * N * 2 * N; e += NT) {  // B3[n][k], E = conj(W)/N
    const int n = e / (2 * N), k = e % (2 * N), r = n % N, fr = k % N;
    const int q = (fr * r) % N;
    const float er = tw_re[q] * inv_n, ei = -tw_im[q] * inv_n;
    const float v = n < N ? (k < N ? er : -ei) : (k < N ? ei : er);
    sth(sm + L::B3, off_k(n, k, 2 * N), v);
  }
  for (int e = tid; e < N * 2 * N; e += NT) {  // B4[s][k]: Re(U e^{+i theta}) / N
    const int sidx = e / (2 * N), k = e % (2 * N), fc = k % N;
    const int q = (fc * sidx) % N;
    const float v = k < N ? tw_re[q] * inv_n : tw_im[q] * inv_n;
    sth(sm + L::B4, off_k(sidx, k, 2 * N), v);
  }
  if (warp == 0) tc::tmem_alloc(&tmem_base_s, L::TCOLS);
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base_s;
  const uint32_t sbase = tc::smem_u32(sm);
  uint32_t phase = 0;

  const int sp = a.spacing, nf = a.n;
  const int n_wins = a.m * a.n;
  const long long total = (long long)a.n_pairs * n_wins;
  const int n_tiles = (int)((total + W - 1) / W);
  const long long frame_elems = (long long)a.height * a.width;

  // Waits for the last commit; on timeout every thread leaves the tile loop.
  auto wait_mma = [&]() -> bool {
    bool ok = tc::mbar_wait_bounded(&bar, phase, kMaxPolls);
    phase ^= 1u;
    ok = __syncthreads_and(ok);
    if (!ok && tid == 0) atomicExch(status, PIV_E_TIMEOUT);
    tc::fence_after_sync();
    return ok;
  };
  auto sync_for_mma = [&]() {
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  };

  for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const long long g0 = (long long)tile * W;
    if (tid < W) {
      const long long g = g0 + tid;
      int ok = g < total;
      long long base = 0;
      if (ok) {
        const int pair = (int)(g / n_wins), k = (int)(g % n_wins);
        if (a.win_mask) ok = a.win_mask[k] == 0;
        base = pair * frame_elems + (long long)((k / nf) * sp + a.y_offset) * a.width + (k % nf) * sp + a.x_offset;
      }
      win_valid[tid] = ok;
      win_base[tid] = base;
    }
    __syncthreads();

    // ---- Staging: thread (half, t): frame `half`, row t = (w, y) of the tile.
    {
      const int w = t / SS, y = t % SS;
      const bool ok = win_valid[w] != 0;
      const void* frame = half == 0 ? a.frame_a : a.frame_b;
      float r[SS];
      float sum = 0.f;
      const long long rowoff = win_base[w] + (long long)y * a.width;
#pragma unroll
      for (int x = 0; x < SS; ++x) {
        r[x] = ok ? load_pixel<float>(frame, a.pixel_type, rowoff + x) : 0.f;
        sum += r[x];
      }
      // Window sum over its SS rows (a window's lanes are contiguous, SS | 32).
#pragma unroll
      for (int o = 1; o < SS && o < 32; o <<= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
      const float mean = sum / (float)(SS * SS);
      float l = 0.f;
#pragma unroll
      for (int x = 0; x < SS; ++x) {
        r[x] -= mean;
        l += fabsf(r[x]);
      }
#pragma unroll
      for (int o = 1; o < SS && o < 32; o <<= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
      if (y == 0) l1[half][w] = l;
#pragma unroll
      for (int x = 0; x < SS; x += 8) st8(sm + L::A1 + half * 128 * SS * 2, off_k(t, x, SS), r + x);
    }
    sync_for_mma();
    if (tid < W) {
      const float prod = l1[0][tid] * l1[1][tid];
      sc_exp[tid] = prod > 0.f ? (float)(14 - (int)ceilf(log2f(prod))) : 0.f;
    }

    // ---- Stage 1: T = a G^T for a and b -> TMEM cols [0, 2N) and [2N, 4N).
    if (tid == 0) {
      const uint32_t id = tc::idesc_f16(128, 2 * N, 0, 0);
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        for (int ks = 0; ks < SS / 16; ++ks) {
          const uint64_t ad = tc::sdesc(sbase + L::A1 + f * 128 * SS * 2 + ks * 256, 128, SS * 16);
          const uint64_t bd = tc::sdesc(sbase + L::B1 + ks * 256, 128, SS * 16);
          tc::mma_f16(tmem + f * 2 * N, ad, bd, id, ks > 0);
        }
      }
      tc::mma_commit(&bar);
    }
    if (!wait_mma()) break;

    // ---- Stage 1 -> 2: frame `half`: T rows (w, y) become MN-major rows (w, f_c), K = (Re|Im, y).
    {
      const int w = t / SS, y = t % SS;
      unsigned char* dst = sm + L::A2 + half * 2 * L::A2_TILE;
      float v[2 * N];
#pragma unroll
      for (int c0 = 0; c0 < 2 * N; c0 += 16)
        tc::tmem_ld16(tmem + lane_sel + half * 2 * N + c0, *reinterpret_cast<float(*)[16]>(v + c0));
      tc::tmem_ld_wait();
#pragma unroll
      for (int c0 = 0; c0 < 2 * N; c0 += 8) {
        const int k = (c0 / N) * SS + y;   // Re rows then Im rows of K
        const int m = w * N + (c0 % N);    // global operand row
        st8(dst + (m >> 7) * L::A2_TILE, off_mn(m & 127, k, 128), v + c0);
      }
    }
    sync_for_mma();

    // ---- Stage 2: A = G T for a, b and both row tiles -> TMEM cols [f*4N + rt*2N, +2N).
    if (tid == 0) {
      const uint32_t id = tc::idesc_f16(128, 2 * N, 1, 0);
      for (int f = 0; f < 2; ++f)
        for (int rt = 0; rt < 2; ++rt)
          for (int ks = 0; ks < 2 * SS / 16; ++ks) {
            const uint64_t ad = tc::sdesc(sbase + L::A2 + (f * 2 + rt) * L::A2_TILE + ks * 32 * 128, 128 * 16, 128);
            const uint64_t bd = tc::sdesc(sbase + L::B2 + ks * 256, 128, 2 * SS * 16);
            tc::mma_f16(tmem + f * 4 * N + rt * 2 * N, ad, bd, id, ks > 0);
          }
      tc::mma_commit(&bar);
    }
    if (!wait_mma()) break;

    // ---- Product (row tile `half`): P = s_w conj(A) B, K-major rows (w, f_c), K = (Re|Im, f_r).
    {
      const int rt = half, m = rt * 128 + t, w = m / N;
      const float sc = exp2f(sc_exp[w]);
      unsigned char* dst = sm + L::A3 + rt * L::A3_TILE;
#pragma unroll
      for (int c0 = 0; c0 < N; c0 += 16) {
        float ar[16], ai[16], br[16], bi[16];
        tc::tmem_ld16(tmem + lane_sel + rt * 2 * N + c0, ar);
        tc::tmem_ld16(tmem + lane_sel + rt * 2 * N + N + c0, ai);
        tc::tmem_ld16(tmem + lane_sel + 4 * N + rt * 2 * N + c0, br);
        tc::tmem_ld16(tmem + lane_sel + 4 * N + rt * 2 * N + N + c0, bi);
        tc::tmem_ld_wait();
        float pr[16], pi[16];
#pragma unroll
        for (int h = 0; h < 16; ++h) {
          pr[h] = (ar[h] * br[h] + ai[h] * bi[h]) * sc;
          pi[h] = (ar[h] * bi[h] - ai[h] * br[h]) * sc;
        }
#pragma unroll
        for (int h = 0; h < 16; h += 8) {
          st8(dst, off_k(t, c0 + h, 2 * N), pr + h);
          st8(dst, off_k(t, N + c0 + h, 2 * N), pi + h);
        }
      }
    }
    sync_for_mma();

    // ---- Stage 3: U = P E / N -> TMEM cols [rt*2N, +2N).
    if (tid == 0) {
      const uint32_t id = tc::idesc_f16(128, 2 * N, 0, 0);
      for (int rt = 0; rt < 2; ++rt)
        for (int ks = 0; ks < 2 * N / 16; ++ks) {
          const uint64_t ad = tc::sdesc(sbase + L::A3 + rt * L::A3_TILE + ks * 256, 128, 2 * N * 16);
          const uint64_t bd = tc::sdesc(sbase + L::B3 + ks * 256, 128, 2 * N * 16);
          tc::mma_f16(tmem + rt * 2 * N, ad, bd, id, ks > 0);
        }
      tc::mma_commit(&bar);
    }
    if (!wait_mma()) break;

    // ---- Stage 3 -> 4 (row tile `half`): rows (w, f_c) of U become MN-major rows (w, r), K = (Re|Im, f_c).
    {
      const int rt = half, m = rt * 128 + t, w = m / N, fc = m % N;
      unsigned char* dst = sm + L::A2;
      float v[2 * N];
#pragma unroll
      for (int c0 = 0; c0 < 2 * N; c0 += 16)
        tc::tmem_ld16(tmem + lane_sel + rt * 2 * N + c0, *reinterpret_cast<float(*)[16]>(v + c0));
      tc::tmem_ld_wait();
#pragma unroll
      for (int c0 = 0; c0 < 2 * N; c0 += 8) {
        const int k = (c0 / N) * N + fc;
        const int mo = w * N + (c0 % N);
        st8(dst + (mo >> 7) * L::A4_TILE, off_mn(mo & 127, k, 128), v + c0);
      }
    }
    sync_for_mma();

    // ---- Stage 4: c = Re(U E^T) / N -> TMEM cols [rt*N, +N).
    if (tid == 0) {
      const uint32_t id = tc::idesc_f16(128, N, 1, 0);
      for (int rt = 0; rt < 2; ++rt)
        for (int ks = 0; ks < 2 * N / 16; ++ks) {
          const uint64_t ad = tc::sdesc(sbase + L::A2 + rt * L::A4_TILE + ks * 32 * 128, 128 * 16, 128);
          const uint64_t bd = tc::sdesc(sbase + L::B4 + ks * 256, 128, 2 * N * 16);
          tc::mma_f16(tmem + rt * N, ad, bd, id, ks > 0);
        }
      tc::mma_commit(&bar);
    }
    if (!wait_mma()) break;

    // ---- Epilogue (row tile `half`): this thread holds map row r of window w.
    const int rt = half, m = rt * 128 + t, w = m / N, r = m % N, i = r ^ H;
    float rowc[N];
    {
      const float unscale = exp2f(-sc_exp[w]);
      float v[N];
#pragma unroll
      for (int c0 = 0; c0 < N; c0 += 16)
        tc::tmem_ld16(tmem + lane_sel + rt * N + c0, *reinterpret_cast<float(*)[16]>(v + c0));
      tc::tmem_ld_wait();
#pragma unroll
      for (int sc = 0; sc < N; ++sc) {
        const int j = sc ^ H;
        const int di = i - H, dj = j - H;
        const bool zero_lag = di <= -SS || di >= SS || dj <= -SS || dj >= SS;
        rowc[j] = zero_lag ? 0.f : v[sc] * unscale;
      }
    }
    {
      // Row maximum (first in column order), then the window maximum (first in
      // row-major order of the shifted map) over the window's rows.
      float v = rowc[0];
      int bj = 0;
#pragma unroll
      for (int j = 1; j < N; ++j)
        if (rowc[j] > v) { v = rowc[j]; bj = j; }
      int idx = i * N + bj;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
        if (v2 > v || (v2 == v && i2 < idx)) { v = v2; idx = i2; }
      }
      if (lane == 0) {
        const int part = r / 32;  // a window spans N / 32 warps
        pk_val[w][part] = v;
        pk_idx[w][part] = idx;
        if (N == 32) { pk_val[w][1] = -INFINITY; pk_idx[w][1] = 0x7fffffff; }
      }
    }
    __syncthreads();
    if (tid < W) {
      float v = pk_val[tid][0];
      int idx = pk_idx[tid][0];
      if (pk_val[tid][1] > v || (pk_val[tid][1] == v && pk_idx[tid][1] < idx)) idx = pk_idx[tid][1];
      pk_idx[tid][0] = idx;
    }
    __syncthreads();
    {
      // Neighbours of the peak: rows i-1, i, i+1 at column j, and j-1, j+1 of row i.
      const int pidx = pk_idx[w][0], pi_ = pidx / N, pj = pidx % N;
      if (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1 && i >= pi_ - 1 && i <= pi_ + 1) {
        // Masked sums keep the row in registers (an indexed read would move it
        // to local memory); exactly one term of each sum is non-zero.
        float vc = 0.f, vl = 0.f, vr = 0.f;
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const float x = rowc[j];
          vc = fmaf(j == pj ? 1.f : 0.f, x, vc);
          vl = fmaf(j == pj - 1 ? 1.f : 0.f, x, vl);
          vr = fmaf(j == pj + 1 ? 1.f : 0.f, x, vr);
        }
        if (i == pi_) {
          nb[w][0] = vc;
          nb[w][3] = vl;
          nb[w][4] = vr;
        } else if (i == pi_ - 1) {
          nb[w][1] = vc;
        } else {
          nb[w][2] = vc;
        }
      }
    }
    if (a.maps && g0 + w < total) {
      float* mo = reinterpret_cast<float*>(a.maps) + (g0 + w) * N * N + (long long)i * N;
#pragma unroll
      for (int j = 0; j < N; ++j) mo[j] = rowc[j];
    }
    __syncthreads();
    if (tid < W && g0 + tid < total) {
      const int ww = tid;
      const long long g = g0 + ww;
      const int pidx = pk_idx[ww][0], pi_ = pidx / N, pj = pidx % N;
      float isp = (float)pi_, jsp = (float)pj;
      if (pi_ > 0 && pi_ < N - 1 && pj > 0 && pj < N - 1) {
        float c = nb[ww][0], cd = nb[ww][1], cu = nb[ww][2], cl = nb[ww][3], cr = nb[ww][4];
        const float eps = 1e-7f;
        if (a.subpixel == PIV_SUBPIXEL_GAUSSIAN) {
          if (c > 0 && cd > 0 && cu > 0 && cl > 0 && cr > 0) {
            c = logf(c); cd = logf(cd); cu = logf(cu); cl = logf(cl); cr = logf(cr);
            isp = add_rn((float)pi_, div_rn(mul_rn(0.5f, sub_rn(cd, cu)), add_rn(add_rn(sub_rn(cd, mul_rn(2.f, c)), cu), eps)));
            jsp = add_rn((float)pj, div_rn(mul_rn(0.5f, sub_rn(cl, cr)), add_rn(add_rn(sub_rn(cl, mul_rn(2.f, c)), cr), eps)));
          }
        } else if (a.subpixel == PIV_SUBPIXEL_PARABOLIC) {
          isp = add_rn((float)pi_, div_rn(mul_rn(0.5f, sub_rn(cd, cu)), add_rn(add_rn(sub_rn(cd, mul_rn(2.f, c)), cu), eps)));
          jsp = add_rn((float)pj, div_rn(mul_rn(0.5f, sub_rn(cl, cr)), add_rn(add_rn(sub_rn(cl, mul_rn(2.f, c)), cr), eps)));
        } else {
          isp = add_rn((float)pi_, div_rn(sub_rn(cu, cd), add_rn(add_rn(add_rn(cd, c), cu), eps)));
          jsp = add_rn((float)pj, div_rn(sub_rn(cr, cl), add_rn(add_rn(add_rn(cl, c), cr), eps)));
        }
      }
      float* uo = reinterpret_cast<float*>(a.u);
      float* vo = reinterpret_cast<float*>(a.v);
      if (win_valid[ww]) {
        uo[g] = sub_rn(jsp, (float)H);
        vo[g] = sub_rn(isp, (float)H);
      } else {
        uo[g] = NAN;
        vo[g] = NAN;
      }
      if (a.peak_i) a.peak_i[g] = pi_;
      if (a.peak_j) a.peak_j[g] = pj;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, L::TCOLS);
}

bool correlate_tensor_supported(const CorrArgs& a) {
  return a.dtype == PIV_DTYPE_F32 && a.s2n == nullptr && a.ws == a.ss && a.fft_size == 2 * a.ss &&
         (a.ss == 16 || a.ss == 32);
}

template <int SS>
static int launch_tc(const CorrArgs& a, cudaStream_t stream) {
  using L = TcLayout<SS>;
  const long long total = (long long)a.n_pairs * a.m * a.n;
  if (total == 0) return PIV_OK;
  const int n_tiles = (int)((total + L::W - 1) / L::W);
  constexpr int NT = TcThreads<SS>::NT;
  static thread_local int configured_dev = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (configured_dev != dev) {
    cudaError_t e = cudaFuncSetAttribute(k_corr_tc<SS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_corr_tc<SS>, cudaFuncAttributePreferredSharedMemoryCarveout,
                               cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return set_cuda_error(e, "cudaFuncSetAttribute(k_corr_tc)");
    configured_dev = dev;
  }
  // At most 512 TMEM columns per SM in flight: CTAs per SM = min(occupancy, 512 / TCOLS).
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_corr_tc<SS>, NT, L::SMEM);
  const int tmem_limit = 512 / L::TCOLS;
  if (getenv("PIV_DEBUG_LAUNCH")) {
    cudaFuncAttributes fa;
    cudaFuncGetAttributes(&fa, k_corr_tc<SS>);
    int smem_sm = 0, smem_blk = 0, regs_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&smem_blk, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    fprintf(stderr, "k_corr_tc<%d>: occupancy %d/SM, tmem limit %d, regs %d, static smem %zu, dyn smem %zu, "
            "max dyn %d, smem/SM %d, smem/block %d, regs/SM %d\n", SS, per_sm, tmem_limit, fa.numRegs,
            fa.sharedSizeBytes, (size_t)L::SMEM, fa.maxDynamicSharedSizeBytes, smem_sm, smem_blk, regs_sm);
  }
  if (per_sm > tmem_limit) per_sm = tmem_limit;
  if (per_sm < 1) return set_error(PIV_E_UNSUPPORTED, "tensor correlation does not fit on an SM");
  int grid = sm_count() * per_sm;
  if (grid > n_tiles) grid = n_tiles;
  if (!a.status) return set_error(PIV_E_ARG, "tensor correlation needs a device status word");
  k_corr_tc<SS><<<grid, NT, L::SMEM, stream>>>(a, a.status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_corr_tc launch");
}

int correlate_tensor(const CorrArgs& a, cudaStream_t stream) {
  if (!correlate_tensor_supported(a)) return set_error(PIV_E_UNSUPPORTED, "tensor correlation: unsupported pass");
  return a.ss == 16 ? launch_tc<16>(a, stream) : launch_tc<32>(a, stream);
}

}  // namespace piv
