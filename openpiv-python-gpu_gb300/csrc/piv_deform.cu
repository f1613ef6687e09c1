// Predictor interpolation and frame deformation.
//
// * regrid: the previous pass's field onto the new grid (interpolate_displacement,
//   gpu_process.py:730-742);
// * deform: the predictor onto every pixel and the deformed frames
//   (deform_frame + interpolate_frame, gpu_process.py:1149-1192, 1461-1547), with
//   the reference's bilinear kernel or this project's cubic B-spline sampling.
//   The per-pixel predictor is evaluated in float32 (the reference uses
//   float64 and casts to float32; float64 throughput on this GPU is a small
//   fraction of float32);
// * spline_prefilter: cubic B-spline coefficients (mirror boundary) for the cubic path.
//
// Both interpolations of the predictor restate RegularGridInterpolator(...,
// bounds_error=False, fill_value=None) on the reference's uniform grids:
// interval index clamped to [0, n-2], weights from the unclamped normalised
// distance. The field-to-field regrid runs in float64 as separate IEEE
// operations in the order the host oracle uses.
#include <math.h>

#include <algorithm>

#include "piv_common.cuh"
#include "piv_internal.h"

namespace piv {

// Coordinate of grid index k along one axis: k * spacing + ss / 2 + offset
// (gpu_process.py:944-945), exact in float32 and float64.
PIV_D double grid_coord(int k, int spacing, int ss, int offset) {
  return (double)k * spacing + ss * 0.5 + offset;
}

// searchsorted(grid, q, 'right') - 1 clamped to [0, len-2] on a uniform grid.
PIV_D int grid_interval(double q, double g0, int spacing, int len) {
  double t = floor((q - g0) / spacing);
  int i = t < 0 ? 0 : (t > len - 2 ? len - 2 : (int)t);
  return i < 0 ? 0 : i;
}

struct GridAxis {
  double g0;
  int spacing, len;
};

PIV_HD GridAxis axis_x(const piv_geometry& g) {
  return GridAxis{(double)g.search_size * 0.5 + g.x_offset, g.spacing, g.n};
}
PIV_HD GridAxis axis_y(const piv_geometry& g) {
  return GridAxis{(double)g.search_size * 0.5 + g.y_offset, g.spacing, g.m};
}

// RegularGridInterpolator's linear rule in float64, one separate IEEE
// operation at a time in the host oracle's order. One CTA per (destination
// row, group of pairs): the column weights of the row are computed once into
// shared memory and reused for every pair, so the per-point work is four
// loads and the bilinear sum.
static constexpr int kRegridPairGroups = 8;
static constexpr int kRegridMaxCols = 4096;

__global__ void __launch_bounds__(128) k_regrid(piv_geometry src, piv_geometry dst, int n_pairs,
                                                const double* __restrict__ u_src, const double* __restrict__ v_src,
                                                double* __restrict__ u_dst, double* __restrict__ v_dst) {
  __shared__ int s_ix[kRegridMaxCols];
  __shared__ double s_tx[kRegridMaxCols];
  const int i = blockIdx.x;
  const GridAxis ay = axis_y(src), ax = axis_x(src);
  for (int j = threadIdx.x; j < dst.n; j += blockDim.x) {
    const double xq = grid_coord(j, dst.spacing, dst.search_size, dst.x_offset);
    const int ix = grid_interval(xq, ax.g0, ax.spacing, ax.len);
    const double x0 = ax.g0 + (double)ix * ax.spacing, x1 = ax.g0 + (double)(ix + 1) * ax.spacing;
    s_ix[j] = ix;
    s_tx[j] = __ddiv_rn(__dsub_rn(xq, x0), __dsub_rn(x1, x0));
  }
  const double yq = grid_coord(i, dst.spacing, dst.search_size, dst.y_offset);
  const int iy = grid_interval(yq, ay.g0, ay.spacing, ay.len);
  const double y0 = ay.g0 + (double)iy * ay.spacing, y1 = ay.g0 + (double)(iy + 1) * ay.spacing;
  const double ty = __ddiv_rn(__dsub_rn(yq, y0), __dsub_rn(y1, y0));
  const double oy = __dsub_rn(1.0, ty);
  __syncthreads();
  const bool degenerate = ay.len < 2 || ax.len < 2;
  const int n = src.n;
  const long long src_sz = (long long)src.m * src.n, dst_sz = (long long)dst.m * dst.n;
  for (int pair = blockIdx.y; pair < n_pairs; pair += gridDim.y) {
    const double* us = u_src + pair * src_sz;
    const double* vs = v_src + pair * src_sz;
    const long long o = pair * dst_sz + (long long)i * dst.n;
    for (int j = threadIdx.x; j < dst.n; j += blockDim.x) {
      const int ix = s_ix[j];
      if (degenerate) {
        const int jy = ay.len < 2 ? 0 : iy, jx = ax.len < 2 ? 0 : ix;
        u_dst[o + j] = us[jy * n + jx];
        v_dst[o + j] = vs[jy * n + jx];
        continue;
      }
      const double tx = s_tx[j], ox = __dsub_rn(1.0, tx);
      const int k00 = iy * n + ix;
#pragma unroll
      for (int f = 0; f < 2; ++f) {
        const double* v = f == 0 ? us : vs;
        const double v00 = v[k00], v01 = v[k00 + 1], v10 = v[k00 + n], v11 = v[k00 + n + 1];
        const double t1 = __dmul_rn(__dmul_rn(v00, oy), ox);
        const double t2 = __dmul_rn(__dmul_rn(v01, oy), tx);
        const double t3 = __dmul_rn(__dmul_rn(v10, ty), ox);
        const double t4 = __dmul_rn(__dmul_rn(v11, ty), tx);
        (f == 0 ? u_dst : v_dst)[o + j] = __dadd_rn(__dadd_rn(__dadd_rn(t1, t2), t3), t4);
      }
    }
  }
}

int regrid(const piv_geometry& src, const piv_geometry& dst, int n_pairs, const double* u_src, const double* v_src,
           double* u_dst, double* v_dst, cudaStream_t stream) {
  if ((long long)dst.m * dst.n * n_pairs == 0) return PIV_OK;
  if (dst.n > kRegridMaxCols) return set_error(PIV_E_UNSUPPORTED, "regrid: more than %d field columns", kRegridMaxCols);
  if (dst.m > 2147483647 || n_pairs < 1) return set_error(PIV_E_ARG, "regrid: bad field size");
  const dim3 grid((unsigned)dst.m, (unsigned)std::min(n_pairs, kRegridPairGroups));
  k_regrid<<<grid, 128, 0, stream>>>(src, dst, n_pairs, u_src, v_src, u_dst, v_dst);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_regrid launch");
}

// The reference's bilinear kernel (gpu_process.py:1528-1546) in T: clamped base
// index, unclamped weights. The base index is floorf of the coordinate as a
// float (the reference calls floorf in both precisions).
template <typename T>
PIV_D T sample_bilinear(const void* frame, int pixel_type, long long base, int W, int H, T xi, T yi) {
  int xl = (int)floorf((float)xi);
  int yu = (int)floorf((float)yi);
  if (yu < 0) yu = 0; else if (yu > H - 2) yu = H - 2;
  if (xl < 0) xl = 0; else if (xl > W - 2) xl = W - 2;
  const int yd = yu + 1, xr = xl + 1;
  const T ful = load_pixel<T>(frame, pixel_type, base + (long long)yu * W + xl);
  const T fur = load_pixel<T>(frame, pixel_type, base + (long long)yu * W + xr);
  const T fdl = load_pixel<T>(frame, pixel_type, base + (long long)yd * W + xl);
  const T fdr = load_pixel<T>(frame, pixel_type, base + (long long)yd * W + xr);
  const T a1 = sub_rn(yi, (T)yu), a2 = sub_rn((T)yd, yi);
  const T b1 = sub_rn((T)xr, xi), b2 = sub_rn(xi, (T)xl);
  T r = mul_rn(mul_rn(a1, b1), fdl);
  r = add_rn(r, mul_rn(mul_rn(a1, b2), fdr));
  r = add_rn(r, mul_rn(mul_rn(a2, b1), ful));
  r = add_rn(r, mul_rn(mul_rn(a2, b2), fur));
  return r;
}

// Mirror index for taps in [-(n-1), 2(n-1)] (sample coordinates are clamped
// into the frame, so taps stay within one reflection).
PIV_D int mirror_index(int i, int n) {
  if (n == 1) return 0;
  i = i < 0 ? -i : i;
  return i < n ? i : 2 * (n - 1) - i;
}

PIV_D void bspline3_weights(float t, float* w) {
  const float t2 = t * t, t3 = t2 * t, u = 1.0f - t;
  w[0] = u * u * u * (1.0f / 6.0f);
  w[1] = (2.0f / 3.0f) - t2 + 0.5f * t3;
  w[2] = (2.0f / 3.0f) - u * u + 0.5f * u * u * u;
  w[3] = t3 * (1.0f / 6.0f);
}

// Cubic B-spline sample at clamped (yi, xi) whose 4 x 4 support crosses an
// edge: mirror taps. Kept out of line so that the interior path below stays a
// short branch.
__device__ __noinline__ float sample_cubic_edge(const float* __restrict__ coef, int W, int H, float xi, float yi) {
  const float fx = floorf(xi), fy = floorf(yi);
  float wx[4], wy[4];
  bspline3_weights(xi - fx, wx);
  bspline3_weights(yi - fy, wy);
  const int x0 = (int)fx - 1, y0 = (int)fy - 1;
  int cx[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) cx[c] = mirror_index(x0 + c, W);
  float acc = 0.0f;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float* row = coef + mirror_index(y0 + r, H) * W;
    float s = wx[0] * __ldg(row + cx[0]);
    s = fmaf(wx[1], __ldg(row + cx[1]), s);
    s = fmaf(wx[2], __ldg(row + cx[2]), s);
    s = fmaf(wx[3], __ldg(row + cx[3]), s);
    acc = fmaf(wy[r], s, acc);
  }
  return acc;
}

// Cubic B-spline sample of the coefficient frame at (yi, xi) clamped into the
// frame. Taps inside the frame are read directly; the mirror rule is only
// evaluated for samples whose 4 x 4 support crosses an edge.
PIV_D float sample_cubic(const float* __restrict__ coef, int W, int H, float xi, float yi) {
  xi = fminf(fmaxf(xi, 0.0f), (float)(W - 1));
  yi = fminf(fmaxf(yi, 0.0f), (float)(H - 1));
  const float fx = floorf(xi), fy = floorf(yi);
  const int x0 = (int)fx - 1, y0 = (int)fy - 1;
  if (x0 < 0 || x0 + 3 >= W || y0 < 0 || y0 + 3 >= H) return sample_cubic_edge(coef, W, H, xi, yi);
  float wx[4], wy[4];
  bspline3_weights(xi - fx, wx);
  bspline3_weights(yi - fy, wy);
  const float* p = coef + (y0 * W + x0);
  float acc = 0.0f;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float* row = p + r * W;
    float s = wx[0] * __ldg(row);
    s = fmaf(wx[1], __ldg(row + 1), s);
    s = fmaf(wx[2], __ldg(row + 2), s);
    s = fmaf(wx[3], __ldg(row + 3), s);
    acc = fmaf(wy[r], s, acc);
  }
  return acc;
}

// Cubic B-spline sample of a padded coefficient frame (origin of the frame at
// coef, row stride S = W + 4, mirrored 2-pixel border): a sample clamped into
// the frame has all 16 taps inside the padded buffer.
PIV_D float sample_cubic_padded(const float* __restrict__ coef, int S, int W, int H, float xi, float yi) {
  xi = fminf(fmaxf(xi, 0.0f), (float)(W - 1));
  yi = fminf(fmaxf(yi, 0.0f), (float)(H - 1));
  const float fx = floorf(xi), fy = floorf(yi);
  const int x0 = (int)fx - 1, y0 = (int)fy - 1;
  float w[4], v[4];
  bspline3_weights(xi - fx, w);
  bspline3_weights(yi - fy, v);
  const float* p = coef + (y0 * S + x0);
  float acc = 0.0f;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float* row = p + r * S;
    float s = w[0] * __ldg(row);
    s = fmaf(w[1], __ldg(row + 1), s);
    s = fmaf(w[2], __ldg(row + 2), s);
    s = fmaf(w[3], __ldg(row + 3), s);
    acc = fmaf(v[r], s, acc);
  }
  return acc;
}

// Predictor weight of one axis at integer pixel coordinate q on the uniform
// grid g_k = k*sp + ss/2 + off: interval index clamped to [0, len-2], weight
// from the unclamped distance. Works in doubled integer coordinates so that
// odd search sizes (half-integer grid points) stay exact.
struct AxisWeight {
  int i;
  float t;
};
// Per-launch constants of one axis: q -> d2 = 2 q - c0, interval i = floor(d2 / sp2).
struct AxisMap {
  int c0, sp2, len;
  float inv_sp2;
};
PIV_HD AxisMap axis_map(int ss, int off, int sp, int len) {
  return AxisMap{ss + 2 * off, 2 * sp, len, 1.0f / (float)(2 * sp)};
}
PIV_D AxisWeight axis_weight(int q, const AxisMap& a) {
  const int d2 = 2 * q - a.c0;
  // floor(d2 / sp2) from the float quotient, corrected to the exact integer.
  int i = (int)floorf((float)d2 * a.inv_sp2);
  if (i * a.sp2 > d2) --i;
  else if ((i + 1) * a.sp2 <= d2) ++i;
  i = i < 0 ? 0 : (i > a.len - 2 ? a.len - 2 : i);
  if (a.len < 2) i = 0;
  const float t = a.len < 2 ? 0.0f : (float)(d2 - i * a.sp2) * a.inv_sp2;
  return AxisWeight{i, t};
}
PIV_D AxisWeight axis_weight(int q, int ss, int off, int sp, int len) {
  return axis_weight(q, axis_map(ss, off, sp, len));
}

static constexpr int kDeformThreads = 256;
static constexpr int kDeformRows = 8;                       // image rows per CTA
// Field columns / rows one CTA can touch (spacing >= 1).
static constexpr int kDeformMaxCols = kDeformThreads + 2;
static constexpr int kDeformMaxGridRows = kDeformRows + 1;

// One thread per pixel column of an 8-row x 256-pixel block; each thread
// handles the block's eight rows. The predictor (float32; the reference
// evaluates it in float64 and casts to the frame type, a difference of one or
// two float32 ulps) is staged as the field rows and columns the block touches
// and interpolated along y, then x. Frame A is sampled at x + up*dta and frame
// B at x + up*dtb.
// Launch grid: x over row segments, y over blocks of rows, z over pairs.
template <typename T>
__global__ void __launch_bounds__(kDeformThreads) k_deform(DeformArgs a, AxisMap ax, AxisMap ay, T dta, T dtb,
                                                           int do_a, int do_b) {
  __shared__ float su[kDeformMaxGridRows][kDeformMaxCols], sv[kDeformMaxGridRows][kDeformMaxCols];
  __shared__ int s_klo, s_khi;
  const piv_geometry& g = a.geom;
  const int H = g.height, W = g.width;
  const int j0 = blockIdx.x * kDeformThreads;
  const int j = j0 + threadIdx.x;
  const int i0 = blockIdx.y * kDeformRows, pair = blockIdx.z;
  const int i_last = min(i0 + kDeformRows, H) - 1;
  const int r_lo = axis_weight(i0, ay).i;
  const int r_hi = min(axis_weight(i_last, ay).i + 1, g.m - 1);
  const AxisWeight wx = axis_weight(min(j, W - 1), ax);
  if (threadIdx.x == 0) s_klo = axis_weight(j0, ax).i;
  if (threadIdx.x == kDeformThreads - 1 || j == W - 1) s_khi = min(wx.i + 1, g.n - 1);
  __syncthreads();
  const int k_lo = s_klo, k_hi = s_khi;
  const int nc = k_hi - k_lo + 1, nr = r_hi - r_lo + 1;
  const long long fo = (long long)pair * g.m * g.n;
  for (int e = threadIdx.x; e < nr * nc; e += kDeformThreads) {
    const int r = e / nc, c = e % nc;
    const long long q = fo + (long long)(r_lo + r) * g.n + k_lo + c;
    su[r][c] = (float)__ldg(a.up + q);
    sv[r][c] = (float)__ldg(a.vp + q);
  }
  __syncthreads();
  if (j >= W) return;
  const long long base = (long long)pair * H * W;
  T* out_a = reinterpret_cast<T*>(a.out_a) + base;
  T* out_b = reinterpret_cast<T*>(a.out_b) + base;
  // Coefficient frames of the pair (origin of the frame, row stride cs).
  const int cpad = a.coef_pad, cs = W + 2 * cpad;
  const long long cbase = (long long)pair * (H + 2 * cpad) * cs + (long long)cpad * cs + cpad;
  const float* cfa = a.coef_a ? a.coef_a + cbase : nullptr;
  const float* cfb = a.coef_b ? a.coef_b + cbase : nullptr;
  const int c0 = wx.i - k_lo, c1 = (g.n < 2 ? wx.i : wx.i + 1) - k_lo;
  const T x = (T)j;
#pragma unroll 1
  for (int rr = 0; rr < kDeformRows; ++rr) {
    const int i = i0 + rr;
    if (i > i_last) break;
    const int p = i * W + j;
    if (a.frame_mask && a.frame_mask[p]) {
      out_a[p] = (T)0;
      out_b[p] = (T)0;
      continue;
    }
    const AxisWeight wy = axis_weight(i, ay);
    const int y0r = wy.i - r_lo, y1r = (g.m < 2 ? wy.i : wy.i + 1) - r_lo;
    const float u0 = fmaf(wy.t, su[y1r][c0] - su[y0r][c0], su[y0r][c0]);
    const float u1 = fmaf(wy.t, su[y1r][c1] - su[y0r][c1], su[y0r][c1]);
    const float v0 = fmaf(wy.t, sv[y1r][c0] - sv[y0r][c0], sv[y0r][c0]);
    const float v1 = fmaf(wy.t, sv[y1r][c1] - sv[y0r][c1], sv[y0r][c1]);
    const T up = (T)fmaf(wx.t, u1 - u0, u0);
    const T vp = (T)fmaf(wx.t, v1 - v0, v0);
    const T y = (T)i;
    // Both samples are formed before either store, so that the loads of the
    // second frame need not wait behind the first frame's store.
    T ra, rb;
    if (do_a) {
      const T xi = add_rn(x, mul_rn(up, dta)), yi = add_rn(y, mul_rn(vp, dta));
      ra = a.order != 3 ? sample_bilinear<T>(a.frames_a, a.pixel_type, base, W, H, xi, yi)
           : a.coef_pad ? (T)sample_cubic_padded(cfa, cs, W, H, (float)xi, (float)yi)
                        : (T)sample_cubic(cfa, W, H, (float)xi, (float)yi);
    } else {
      ra = load_pixel<T>(a.frames_a, a.pixel_type, base + p);
    }
    if (do_b) {
      const T xi = add_rn(x, mul_rn(up, dtb)), yi = add_rn(y, mul_rn(vp, dtb));
      rb = a.order != 3 ? sample_bilinear<T>(a.frames_b, a.pixel_type, base, W, H, xi, yi)
           : a.coef_pad ? (T)sample_cubic_padded(cfb, cs, W, H, (float)xi, (float)yi)
                        : (T)sample_cubic(cfb, W, H, (float)xi, (float)yi);
    } else {
      rb = load_pixel<T>(a.frames_b, a.pixel_type, base + p);
    }
    out_a[p] = ra;
    out_b[p] = rb;
  }
}

// Cubic B-spline weights with the partition of the taps shared: u = 1 - t.
PIV_D void bspline3_weights_fast(float t, float& w0, float& w1, float& w2, float& w3) {
  const float t2 = t * t, t3 = t2 * t, u = 1.0f - t, u2 = u * u, u3 = u2 * u;
  w0 = u3 * (1.0f / 6.0f);
  w1 = fmaf(0.5f, t3, (2.0f / 3.0f) - t2);
  w2 = fmaf(0.5f, u3, (2.0f / 3.0f) - u2);
  w3 = t3 * (1.0f / 6.0f);
}

// sample_cubic with 32-bit indexing of one frame's coefficients (H W < 2^31).
PIV_D float sample_cubic32(const float* __restrict__ coef, int W, int H, float xi, float yi) {
  xi = fminf(fmaxf(xi, 0.0f), (float)(W - 1));
  yi = fminf(fmaxf(yi, 0.0f), (float)(H - 1));
  const float fx = floorf(xi), fy = floorf(yi);
  const int x0 = (int)fx - 1, y0 = (int)fy - 1;
  if ((unsigned)x0 > (unsigned)(W - 4) || (unsigned)y0 > (unsigned)(H - 4))
    return sample_cubic_edge(coef, W, H, xi, yi);
  float wx0, wx1, wx2, wx3, wy0, wy1, wy2, wy3;
  bspline3_weights_fast(xi - fx, wx0, wx1, wx2, wx3);
  bspline3_weights_fast(yi - fy, wy0, wy1, wy2, wy3);
  const float* r0 = coef + (y0 * W + x0);
  const float* r1 = r0 + W;
  const float* r2 = r1 + W;
  const float* r3 = r2 + W;
  float s0 = wx0 * __ldg(r0), s1 = wx0 * __ldg(r1), s2 = wx0 * __ldg(r2), s3 = wx0 * __ldg(r3);
  s0 = fmaf(wx1, __ldg(r0 + 1), s0); s1 = fmaf(wx1, __ldg(r1 + 1), s1);
  s2 = fmaf(wx1, __ldg(r2 + 1), s2); s3 = fmaf(wx1, __ldg(r3 + 1), s3);
  s0 = fmaf(wx2, __ldg(r0 + 2), s0); s1 = fmaf(wx2, __ldg(r1 + 2), s1);
  s2 = fmaf(wx2, __ldg(r2 + 2), s2); s3 = fmaf(wx2, __ldg(r3 + 2), s3);
  s0 = fmaf(wx3, __ldg(r0 + 3), s0); s1 = fmaf(wx3, __ldg(r1 + 3), s1);
  s2 = fmaf(wx3, __ldg(r2 + 3), s2); s3 = fmaf(wx3, __ldg(r3 + 3), s3);
  return fmaf(wy3, s3, fmaf(wy2, s2, fmaf(wy1, s1, wy0 * s0)));
}

// sample_cubic32 on a padded coefficient frame (row stride S): no edge case.
PIV_D float sample_cubic32p(const float* __restrict__ coef, int S, int W, int H, float xi, float yi) {
  xi = fminf(fmaxf(xi, 0.0f), (float)(W - 1));
  yi = fminf(fmaxf(yi, 0.0f), (float)(H - 1));
  const float fx = floorf(xi), fy = floorf(yi);
  const int x0 = (int)fx - 1, y0 = (int)fy - 1;
  float wx0, wx1, wx2, wx3, wy0, wy1, wy2, wy3;
  bspline3_weights_fast(xi - fx, wx0, wx1, wx2, wx3);
  bspline3_weights_fast(yi - fy, wy0, wy1, wy2, wy3);
  const float* r0 = coef + (y0 * S + x0);
  const float* r1 = r0 + S;
  const float* r2 = r1 + S;
  const float* r3 = r2 + S;
  float s0 = wx0 * __ldg(r0), s1 = wx0 * __ldg(r1), s2 = wx0 * __ldg(r2), s3 = wx0 * __ldg(r3);
  s0 = fmaf(wx1, __ldg(r0 + 1), s0); s1 = fmaf(wx1, __ldg(r1 + 1), s1);
  s2 = fmaf(wx1, __ldg(r2 + 1), s2); s3 = fmaf(wx1, __ldg(r3 + 1), s3);
  s0 = fmaf(wx2, __ldg(r0 + 2), s0); s1 = fmaf(wx2, __ldg(r1 + 2), s1);
  s2 = fmaf(wx2, __ldg(r2 + 2), s2); s3 = fmaf(wx2, __ldg(r3 + 2), s3);
  s0 = fmaf(wx3, __ldg(r0 + 3), s0); s1 = fmaf(wx3, __ldg(r1 + 3), s1);
  s2 = fmaf(wx3, __ldg(r2 + 3), s2); s3 = fmaf(wx3, __ldg(r3 + 3), s3);
  return fmaf(wy3, s3, fmaf(wy2, s2, fmaf(wy1, s1, wy0 * s0)));
}

// k_deform for the common case: float32 fields, cubic B-spline sampling of
// both frames (0 < deforming_par < 1). The row weights of the block's rows
// are computed once per CTA; pixel offsets are 32-bit.
template <bool PADDED>
__global__ void __launch_bounds__(kDeformThreads) k_deform_cubic(DeformArgs a, AxisMap ax, AxisMap ay, float dta,
                                                                 float dtb) {
  __shared__ float su[kDeformMaxGridRows][kDeformMaxCols], sv[kDeformMaxGridRows][kDeformMaxCols];
  __shared__ int s_klo, s_khi;
  __shared__ int s_y0[kDeformRows], s_y1[kDeformRows];
  __shared__ float s_ty[kDeformRows];
  const piv_geometry& g = a.geom;
  const int H = g.height, W = g.width;
  const int j0 = blockIdx.x * kDeformThreads;
  const int j = j0 + threadIdx.x;
  const int i0 = blockIdx.y * kDeformRows, pair = blockIdx.z;
  const int i_last = min(i0 + kDeformRows, H) - 1;
  const int r_lo = axis_weight(i0, ay).i;
  const int r_hi = min(axis_weight(i_last, ay).i + 1, g.m - 1);
  const AxisWeight wx = axis_weight(min(j, W - 1), ax);
  if (threadIdx.x == 0) s_klo = axis_weight(j0, ax).i;
  if (threadIdx.x == kDeformThreads - 1 || j == W - 1) s_khi = min(wx.i + 1, g.n - 1);
  if (threadIdx.x < kDeformRows) {
    const AxisWeight wy = axis_weight(min(i0 + (int)threadIdx.x, H - 1), ay);
    s_y0[threadIdx.x] = wy.i - r_lo;
    s_y1[threadIdx.x] = (g.m < 2 ? wy.i : wy.i + 1) - r_lo;
    s_ty[threadIdx.x] = wy.t;
  }
  __syncthreads();
  const int k_lo = s_klo, k_hi = s_khi;
  const int nc = k_hi - k_lo + 1, nr = r_hi - r_lo + 1;
  const long long fo = (long long)pair * g.m * g.n;
  for (int e = threadIdx.x; e < nr * nc; e += kDeformThreads) {
    const int r = e / nc, c = e % nc;
    const long long q = fo + (long long)(r_lo + r) * g.n + k_lo + c;
    su[r][c] = (float)__ldg(a.up + q);
    sv[r][c] = (float)__ldg(a.vp + q);
  }
  __syncthreads();
  if (j >= W) return;
  const long long base = (long long)pair * H * W;
  const int cs = PADDED ? W + 2 * kCoefPad : W;
  const long long cbase = PADDED ? (long long)pair * (H + 2 * kCoefPad) * cs + (long long)kCoefPad * cs + kCoefPad
                                 : base;
  const float* ca = a.coef_a + cbase;
  const float* cb = a.coef_b + cbase;
  float* out_a = reinterpret_cast<float*>(a.out_a) + base;
  float* out_b = reinterpret_cast<float*>(a.out_b) + base;
  const uint8_t* mask = a.frame_mask;
  const int c0 = wx.i - k_lo, c1 = (g.n < 2 ? wx.i : wx.i + 1) - k_lo;
  const float x = (float)j;
  // Unrolled: the row index, its shared-memory slots and the output offsets
  // become constants of each copy (2.6% faster than a rolled loop).
#pragma unroll
  for (int rr = 0; rr < kDeformRows; ++rr) {
    const int i = i0 + rr;
    if (i > i_last) break;
    const int p = i * W + j;
    if (mask && mask[p]) {
      out_a[p] = 0.f;
      out_b[p] = 0.f;
      continue;
    }
    const int y0r = s_y0[rr], y1r = s_y1[rr];
    const float ty = s_ty[rr];
    const float u0 = fmaf(ty, su[y1r][c0] - su[y0r][c0], su[y0r][c0]);
    const float u1 = fmaf(ty, su[y1r][c1] - su[y0r][c1], su[y0r][c1]);
    const float v0 = fmaf(ty, sv[y1r][c0] - sv[y0r][c0], sv[y0r][c0]);
    const float v1 = fmaf(ty, sv[y1r][c1] - sv[y0r][c1], sv[y0r][c1]);
    const float up = fmaf(wx.t, u1 - u0, u0);
    const float vp = fmaf(wx.t, v1 - v0, v0);
    const float y = (float)i;
    const float xa = add_rn(x, mul_rn(up, dta)), ya = add_rn(y, mul_rn(vp, dta));
    const float xb = add_rn(x, mul_rn(up, dtb)), yb = add_rn(y, mul_rn(vp, dtb));
    const float ra = PADDED ? sample_cubic32p(ca, cs, W, H, xa, ya) : sample_cubic32(ca, W, H, xa, ya);
    const float rb = PADDED ? sample_cubic32p(cb, cs, W, H, xb, yb) : sample_cubic32(cb, W, H, xb, yb);
    out_a[p] = ra;
    out_b[p] = rb;
  }
}

int deform(const DeformArgs& a, cudaStream_t stream) {
  const long long total = (long long)a.geom.height * a.geom.width * a.n_pairs;
  if (total == 0) return PIV_OK;
  if (a.order == 3 && (!a.coef_a || !a.coef_b))
    return set_error(PIV_E_ARG, "cubic deformation needs spline coefficient frames");
  if (a.coef_pad != 0 && a.coef_pad != kCoefPad) return set_error(PIV_E_ARG, "coef_pad must be 0 or %d", kCoefPad);
  if (a.geom.spacing < 1) return set_error(PIV_E_ARG, "deformation: spacing must be >= 1");
  const double dp = a.deforming_par;
  double dta = 0, dtb = 0;
  int do_a = 0, do_b = 0;
  if (dp > 0 && dp < 1) { dta = dp - 1; dtb = dp; do_a = do_b = 1; }
  else if (dp == 1) { dtb = 1; do_b = 1; }
  else { dta = -1; do_a = 1; }
  if (a.n_pairs > 65535) return set_error(PIV_E_UNSUPPORTED, "deformation grid limit (pairs <= 65535)");
  const dim3 grid((unsigned)((a.geom.width + kDeformThreads - 1) / kDeformThreads),
                  (unsigned)((a.geom.height + kDeformRows - 1) / kDeformRows), (unsigned)a.n_pairs);
  if ((long long)a.geom.height * a.geom.width > 2147483647LL)
    return set_error(PIV_E_UNSUPPORTED, "deformation: frames above 2^31 pixels");
  const AxisMap ax = axis_map(a.geom.search_size, a.geom.x_offset, a.geom.spacing, a.geom.n);
  const AxisMap ay = axis_map(a.geom.search_size, a.geom.y_offset, a.geom.spacing, a.geom.m);
  if (a.dtype == PIV_DTYPE_F64)
    k_deform<double><<<grid, kDeformThreads, 0, stream>>>(a, ax, ay, dta, dtb, do_a, do_b);
  else if (a.order == 3 && do_a && do_b && a.coef_pad)
    k_deform_cubic<true><<<grid, kDeformThreads, 0, stream>>>(a, ax, ay, (float)dta, (float)dtb);
  else if (a.order == 3 && do_a && do_b)
    k_deform_cubic<false><<<grid, kDeformThreads, 0, stream>>>(a, ax, ay, (float)dta, (float)dtb);
  else
    k_deform<float><<<grid, kDeformThreads, 0, stream>>>(a, ax, ay, (float)dta, (float)dtb, do_a, do_b);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_deform launch");
}

// ---------------------------------------------------------------------------
// Cubic B-spline prefilter, mirror boundary. The exact prefilter (inverse of
// the sampled cubic B-spline, one pole z = sqrt(3) - 2, gain 6 per axis) is
// the symmetric filter h[k] = sqrt(3) z^|k| applied to the mirror-extended
// frame. Each CTA filters a 64 x 64 output tile from a 12-pixel mirrored halo
// in shared memory with the causal / anti-causal recursions
//   c+[k] = s[k] + z c+[k-1],   c-[k] = z (c-[k+1] - c+[k]),   c = 6 c-
// started from zero 12 samples before the first value that is kept: the
// start-up error is below |z|^12 / (1 - |z|) < 2e-7 of the signal, under
// float32 rounding of the recursion itself. Each line (a region row, then a
// tile column) is split between two threads: the first keeps outputs
// [12, 44) from recursions over samples [0, 56), the second outputs [44, 76)
// from samples [32, 88), so that both recursions start 12 samples outside
// the half they keep.
// ---------------------------------------------------------------------------
static constexpr int kPfK = 12;
static constexpr int kPfT = 64;                    // output tile edge
static constexpr int kPfR = kPfT + 2 * kPfK;       // region edge (a multiple of 8)
static_assert(kPfR % 8 == 0, "the recursions run in chunks of eight");
// Row stride: a multiple of four floats (16-byte rows for vector access) whose
// rows fall on distinct banks for eight consecutive rows (92 = 28 mod 32), and
// consecutive columns on consecutive banks.
static constexpr int kPfS = kPfR + 4;
static constexpr int kPfL = kPfT / 2 + 2 * kPfK;   // samples of a half line's recursions (56)
static constexpr int kPfNT = 2 * kPfR + 16;        // threads: two per region row, in whole warps
static_assert(kPfNT % 32 == 0 && kPfL % 4 == 0, "prefilter launch shape");
static constexpr float kPole = -0.26794919243112270f;  // sqrt(3) - 2

// Mirror ('d c b | a b c d | c b a') index for any integer q.
PIV_D int mirror_any(int q, int n) {
  if (n == 1) return 0;
  const int p = 2 * n - 2;
  q %= p;
  if (q < 0) q += p;
  return q < n ? q : p - q;
}

// Causal then anti-causal recursion over a half line v[0, kPfL) (both started
// from zero); v[kPfK, kPfL) then holds c-.
PIV_D void half_line(float (&v)[kPfL]) {
  const float z = kPole;
  float c = 0.f;
#pragma unroll
  for (int k = 0; k < kPfL; ++k) {
    c = fmaf(z, c, v[k]);
    v[k] = c;
  }
  float d = 0.f;
#pragma unroll
  for (int k = kPfL - 1; k >= kPfK; --k) {
    d = z * (d - v[k]);
    v[k] = d;
  }
}

template <typename P>
__global__ void __launch_bounds__(kPfNT) k_prefilter(int H, int W, const P* __restrict__ in, float* __restrict__ out,
                                                     int pad) {
  __shared__ __align__(16) float reg[kPfR * kPfS];
  const int x0 = blockIdx.x * kPfT, y0 = blockIdx.y * kPfT;
  const long long fbase = (long long)blockIdx.z * H * W;
  const P* src = in + fbase;
  const int t = threadIdx.x;
  const bool interior = x0 >= kPfK && y0 >= kPfK && x0 + kPfT + kPfK <= W && y0 + kPfT + kPfK <= H;
  if (sizeof(P) == 1 && interior && (W & 3) == 0 && ((uintptr_t)in & 3) == 0) {
    // 8-bit frames away from the edges: the region's rows start on 4-byte
    // boundaries (x0 - 12 is a multiple of 4). Thread t < 176 converts word
    // column t % 22 of region rows t / 22, t / 22 + 8, ...: its addresses
    // advance by a fixed stride, all of its loads in flight together.
    constexpr int kWords = kPfR / 4, kGroups = kPfNT / kWords, kIters = (kPfR + kGroups - 1) / kGroups;
    if (t < kWords * kGroups) {
      const int wc = t % kWords, r0 = t / kWords;
      const long long wstep = (long long)kGroups * (W / 4);
      const uint32_t* wsrc =
          reinterpret_cast<const uint32_t*>(src + (long long)(y0 - kPfK + r0) * W + (x0 - kPfK)) + wc;
      float* dst = reg + r0 * kPfS + 4 * wc;
      uint32_t wv[kIters];
#pragma unroll
      for (int k = 0; k < kIters; ++k) wv[k] = r0 + kGroups * k < kPfR ? __ldg(wsrc + k * wstep) : 0u;
#pragma unroll
      for (int k = 0; k < kIters; ++k)
        if (r0 + kGroups * k < kPfR) {
          const uint32_t w = wv[k];
          *reinterpret_cast<float4*>(dst + k * kGroups * kPfS) =
              make_float4(u8_to_float(w, 0), u8_to_float(w, 1), u8_to_float(w, 2), u8_to_float(w, 3));
        }
    }
  } else if (t < 2 * kPfR) {
    // Any pixel type, mirrored edges: thread t holds region column t % 88 (its
    // mirrored frame column found once) and walks half of the region's rows.
    const int rc = t % kPfR, r0 = (t / kPfR) * (kPfR / 2);
    int gx = x0 - kPfK + rc;
    if (gx < 0 || gx >= W) gx = mirror_any(gx, W);
    const P* col = src + gx;
#pragma unroll 4
    for (int r = r0; r < r0 + kPfR / 2; ++r) {
      int gy = y0 - kPfK + r;
      if (gy < 0 || gy >= H) gy = mirror_any(gy, H);
      reg[r * kPfS + rc] = pixel_to_float<P>(__ldg(col + (long long)gy * W));
    }
  }
  __syncthreads();
  // Along x: thread t < 176 takes half t / 88 of region row t % 88; every
  // thread reads its samples before any writes its outputs back in place.
  float v[kPfL];
  const int xr = t % kPfR, xs = (t / kPfR) * (kPfR - kPfL);
  if (t < 2 * kPfR) {
    const float4* rp = reinterpret_cast<const float4*>(reg + xr * kPfS + xs);
#pragma unroll
    for (int q = 0; q < kPfL / 4; ++q) {
      const float4 u = rp[q];
      v[4 * q] = u.x; v[4 * q + 1] = u.y; v[4 * q + 2] = u.z; v[4 * q + 3] = u.w;
    }
    half_line(v);
  }
  __syncthreads();
  if (t < 2 * kPfR) {
    float4* wp = reinterpret_cast<float4*>(reg + xr * kPfS + xs + kPfK);
#pragma unroll
    for (int q = 0; q < kPfT / 8; ++q)
      wp[q] = make_float4(v[kPfK + 4 * q], v[kPfK + 4 * q + 1], v[kPfK + 4 * q + 2], v[kPfK + 4 * q + 3]);
  }
  __syncthreads();
  // Along y: thread t < 128 takes half t / 64 of tile column t % 64; writes
  // its 32 rows of the tile with the gain 6 * 6.
  if (t < 2 * kPfT) {
    const int tc = t % kPfT, ys = (t / kPfT) * (kPfR - kPfL), col = kPfK + tc;
#pragma unroll
    for (int k = 0; k < kPfL; ++k) v[k] = reg[(ys + k) * kPfS + col];
    half_line(v);
    const int gx = x0 + tc, os = W + 2 * pad;
    if (gx < W) {
      float* dst = out + (long long)blockIdx.z * (H + 2 * pad) * os + (long long)pad * os + pad + gx;
#pragma unroll
      for (int k = kPfK; k < kPfK + kPfT / 2; ++k) {
        const int gy = y0 + ys + k - kPfK;
        if (gy < H) dst[(long long)gy * os] = 36.0f * v[k];
      }
    }
  }
}

// The 2-pixel border of padded coefficient frames: border element (y, x) of
// the frame holds coefficient (mirror(y), mirror(x)), as the unpadded
// sampler's mirror rule reads it. Grid: x over the border elements, y over
// frames.
__global__ void k_coef_border(int H, int W, float* __restrict__ coef) {
  const int S = W + 2 * kCoefPad, HP = H + 2 * kCoefPad;
  const int n_border = S * HP - H * W;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_border) return;
  float* f = coef + (long long)blockIdx.y * HP * S;
  // Border elements: the 2 * kCoefPad full rows first, then the side columns.
  int y, x;
  const int top = 2 * kCoefPad * S;
  if (t < top) {
    const int r = t / S;
    y = r < kCoefPad ? r - kCoefPad : H + (r - kCoefPad);
    x = t % S - kCoefPad;
  } else {
    const int q = t - top, r = q / (2 * kCoefPad), c = q % (2 * kCoefPad);
    y = r;
    x = c < kCoefPad ? c - kCoefPad : W + (c - kCoefPad);
  }
  const int my = mirror_any(y, H), mx = mirror_any(x, W);  // mirror_index's value wherever that is in range
  f[(long long)(y + kCoefPad) * S + x + kCoefPad] = f[(long long)(my + kCoefPad) * S + mx + kCoefPad];
}

int spline_prefilter(int H, int W, int n_frames, const void* frames, int pixel_type, float* coef,
                     cudaStream_t stream, int pad) {
  if ((long long)H * W * n_frames == 0) return PIV_OK;
  if (n_frames > 65535) return set_error(PIV_E_UNSUPPORTED, "spline prefilter: more than 65535 frames");
  if (pad != 0 && pad != kCoefPad) return set_error(PIV_E_ARG, "spline prefilter: pad must be 0 or %d", kCoefPad);
  const dim3 grid((unsigned)((W + kPfT - 1) / kPfT), (unsigned)((H + kPfT - 1) / kPfT), (unsigned)n_frames);
  switch (pixel_type) {
    case PIV_PIXEL_U8: k_prefilter<<<grid, kPfNT, 0, stream>>>(H, W, (const uint8_t*)frames, coef, pad); break;
    case PIV_PIXEL_U16: k_prefilter<<<grid, kPfNT, 0, stream>>>(H, W, (const uint16_t*)frames, coef, pad); break;
    case PIV_PIXEL_F32: k_prefilter<<<grid, kPfNT, 0, stream>>>(H, W, (const float*)frames, coef, pad); break;
    default: k_prefilter<<<grid, kPfNT, 0, stream>>>(H, W, (const double*)frames, coef, pad); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_cuda_error(e, "k_prefilter launch");
  if (pad) {
    const int n_border = (W + 2 * kCoefPad) * (H + 2 * kCoefPad) - H * W;
    k_coef_border<<<dim3((unsigned)((n_border + 255) / 256), (unsigned)n_frames), 256, 0, stream>>>(H, W, coef);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(e, "k_coef_border launch");
  }
  return PIV_OK;
}

}  // namespace piv
