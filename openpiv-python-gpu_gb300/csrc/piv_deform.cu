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

PIV_D double grid_interp(const double* v, int n, const GridAxis& ay, const GridAxis& ax, double yq, double xq) {
  const int iy = grid_interval(yq, ay.g0, ay.spacing, ay.len);
  const int ix = grid_interval(xq, ax.g0, ax.spacing, ax.len);
  const double y0 = ay.g0 + (double)iy * ay.spacing, y1 = ay.g0 + (double)(iy + 1) * ay.spacing;
  const double x0 = ax.g0 + (double)ix * ax.spacing, x1 = ax.g0 + (double)(ix + 1) * ax.spacing;
  if (ay.len < 2 || ax.len < 2) {
    // Degenerate one-point axis: constant along it.
    const int jy = ay.len < 2 ? 0 : iy, jx = ax.len < 2 ? 0 : ix;
    return v[jy * n + jx];
  }
  const double ty = __ddiv_rn(__dsub_rn(yq, y0), __dsub_rn(y1, y0));
  const double tx = __ddiv_rn(__dsub_rn(xq, x0), __dsub_rn(x1, x0));
  const double v00 = v[iy * n + ix], v01 = v[iy * n + ix + 1];
  const double v10 = v[(iy + 1) * n + ix], v11 = v[(iy + 1) * n + ix + 1];
  const double oy = __dsub_rn(1.0, ty), ox = __dsub_rn(1.0, tx);
  const double t1 = __dmul_rn(__dmul_rn(v00, oy), ox);
  const double t2 = __dmul_rn(__dmul_rn(v01, oy), tx);
  const double t3 = __dmul_rn(__dmul_rn(v10, ty), ox);
  const double t4 = __dmul_rn(__dmul_rn(v11, ty), tx);
  return __dadd_rn(__dadd_rn(__dadd_rn(t1, t2), t3), t4);
}

PIV_HD GridAxis axis_x(const piv_geometry& g) {
  return GridAxis{(double)g.search_size * 0.5 + g.x_offset, g.spacing, g.n};
}
PIV_HD GridAxis axis_y(const piv_geometry& g) {
  return GridAxis{(double)g.search_size * 0.5 + g.y_offset, g.spacing, g.m};
}

__global__ void k_regrid(piv_geometry src, piv_geometry dst, int n_pairs, const double* __restrict__ u_src,
                         const double* __restrict__ v_src, double* __restrict__ u_dst, double* __restrict__ v_dst) {
  const long long npts = (long long)dst.m * dst.n;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npts * n_pairs) return;
  const int pair = (int)(t / npts);
  const int k = (int)(t % npts);
  const int i = k / dst.n, j = k % dst.n;
  const double yq = grid_coord(i, dst.spacing, dst.search_size, dst.y_offset);
  const double xq = grid_coord(j, dst.spacing, dst.search_size, dst.x_offset);
  const GridAxis ay = axis_y(src), ax = axis_x(src);
  const long long so = (long long)pair * src.m * src.n;
  u_dst[t] = grid_interp(u_src + so, src.n, ay, ax, yq, xq);
  v_dst[t] = grid_interp(v_src + so, src.n, ay, ax, yq, xq);
}

int regrid(const piv_geometry& src, const piv_geometry& dst, int n_pairs, const double* u_src, const double* v_src,
           double* u_dst, double* v_dst, cudaStream_t stream) {
  const long long total = (long long)dst.m * dst.n * n_pairs;
  if (total == 0) return PIV_OK;
  const int bs = 256;
  k_regrid<<<(unsigned)((total + bs - 1) / bs), bs, 0, stream>>>(src, dst, n_pairs, u_src, v_src, u_dst, v_dst);
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

// Cubic B-spline sample of the coefficient frame at (yi, xi) clamped into the frame.
PIV_D float sample_cubic(const float* __restrict__ coef, int W, int H, float xi, float yi) {
  xi = fminf(fmaxf(xi, 0.0f), (float)(W - 1));
  yi = fminf(fmaxf(yi, 0.0f), (float)(H - 1));
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
    const float* row = coef + (long long)mirror_index(y0 + r, H) * W;
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < 4; ++c) s += wx[c] * __ldg(row + cx[c]);
    acc += wy[r] * s;
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
PIV_D AxisWeight axis_weight(int q, int ss, int off, int sp, int len) {
  const int d2 = 2 * q - (ss + 2 * off), sp2 = 2 * sp;
  int i = d2 >= 0 ? d2 / sp2 : -((-d2 + sp2 - 1) / sp2);  // floor division
  i = i < 0 ? 0 : (i > len - 2 ? len - 2 : i);
  if (len < 2) i = 0;
  const float t = len < 2 ? 0.0f : (float)(d2 - i * sp2) / (float)sp2;
  return AxisWeight{i, t};
}

// Bilinear predictor value from four float64 field values, in float32.
PIV_D float lerp2(const double* v, int n, const AxisWeight& wy, const AxisWeight& wx, int my, int nx) {
  const int iy1 = my < 2 ? wy.i : wy.i + 1, ix1 = nx < 2 ? wx.i : wx.i + 1;
  const float v00 = (float)__ldg(v + wy.i * n + wx.i), v01 = (float)__ldg(v + wy.i * n + ix1);
  const float v10 = (float)__ldg(v + iy1 * n + wx.i), v11 = (float)__ldg(v + iy1 * n + ix1);
  const float top = fmaf(wx.t, v01 - v00, v00);
  const float bot = fmaf(wx.t, v11 - v10, v10);
  return fmaf(wy.t, bot - top, top);
}

// One thread per pixel: predictor at the pixel (float32; the reference
// evaluates it in float64 and casts to the frame type, a difference of one or
// two float32 ulps), then frame A sampled at x + up*dta and frame B at
// x + up*dtb.
// Launch grid: x over the columns of a row, y over rows, z over pairs.
template <typename T>
__global__ void k_deform(DeformArgs a, T dta, T dtb, int do_a, int do_b) {
  const piv_geometry& g = a.geom;
  const int H = g.height, W = g.width;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= W) return;
  const int i = blockIdx.y, pair = blockIdx.z;
  const long long npix = (long long)H * W;
  const long long p = (long long)i * W + j;
  const long long base = (long long)pair * npix;
  const long long t = base + p;
  T* out_a = reinterpret_cast<T*>(a.out_a);
  T* out_b = reinterpret_cast<T*>(a.out_b);
  if (a.frame_mask && a.frame_mask[p]) {
    out_a[t] = (T)0;
    out_b[t] = (T)0;
    return;
  }
  const AxisWeight wy = axis_weight(i, g.search_size, g.y_offset, g.spacing, g.m);
  const AxisWeight wx = axis_weight(j, g.search_size, g.x_offset, g.spacing, g.n);
  const long long fo = (long long)pair * g.m * g.n;
  const T x = (T)j, y = (T)i;
  const T up = (T)lerp2(a.up + fo, g.n, wy, wx, g.m, g.n);
  const T vp = (T)lerp2(a.vp + fo, g.n, wy, wx, g.m, g.n);
  if (do_a) {
    const T xi = add_rn(x, mul_rn(up, dta)), yi = add_rn(y, mul_rn(vp, dta));
    out_a[t] = a.order == 3 ? (T)sample_cubic(a.coef_a + base, W, H, (float)xi, (float)yi)
                            : sample_bilinear<T>(a.frames_a, a.pixel_type, base, W, H, xi, yi);
  } else {
    out_a[t] = load_pixel<T>(a.frames_a, a.pixel_type, t);
  }
  if (do_b) {
    const T xi = add_rn(x, mul_rn(up, dtb)), yi = add_rn(y, mul_rn(vp, dtb));
    out_b[t] = a.order == 3 ? (T)sample_cubic(a.coef_b + base, W, H, (float)xi, (float)yi)
                            : sample_bilinear<T>(a.frames_b, a.pixel_type, base, W, H, xi, yi);
  } else {
    out_b[t] = load_pixel<T>(a.frames_b, a.pixel_type, t);
  }
}

int deform(const DeformArgs& a, cudaStream_t stream) {
  const long long total = (long long)a.geom.height * a.geom.width * a.n_pairs;
  if (total == 0) return PIV_OK;
  if (a.order == 3 && (!a.coef_a || !a.coef_b))
    return set_error(PIV_E_ARG, "cubic deformation needs spline coefficient frames");
  const double dp = a.deforming_par;
  double dta = 0, dtb = 0;
  int do_a = 0, do_b = 0;
  if (dp > 0 && dp < 1) { dta = dp - 1; dtb = dp; do_a = do_b = 1; }
  else if (dp == 1) { dtb = 1; do_b = 1; }
  else { dta = -1; do_a = 1; }
  if (a.geom.height > 65535 || a.n_pairs > 65535)
    return set_error(PIV_E_UNSUPPORTED, "deformation grid limit (height and pairs <= 65535)");
  const int bs = 256;
  const dim3 grid((unsigned)((a.geom.width + bs - 1) / bs), (unsigned)a.geom.height, (unsigned)a.n_pairs);
  if (a.dtype == PIV_DTYPE_F64)
    k_deform<double><<<grid, bs, 0, stream>>>(a, dta, dtb, do_a, do_b);
  else
    k_deform<float><<<grid, bs, 0, stream>>>(a, (float)dta, (float)dtb, do_a, do_b);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_deform launch");
}

// ---------------------------------------------------------------------------
// Cubic B-spline prefilter (one pole z = sqrt(3) - 2, gain 6 per axis),
// mirror boundary, axis 0 then axis 1.
// ---------------------------------------------------------------------------
static constexpr float kPole = -0.26794919243112270f;  // sqrt(3) - 2
static constexpr int kHorizon = 24;                     // |z|^24 < 2e-14

// Causal initial value for the mirror boundary over n samples read by get(k).
template <class Get>
PIV_D float causal_init_mirror(Get get, int n) {
  const float z = kPole;
  if (n == 1) return get(0);
  if (n > kHorizon) {
    float zk = 1.0f, s = 0.0f;
    for (int k = 0; k < kHorizon; ++k) { s += zk * get(k); zk *= z; }
    return s;
  }
  // Exact sum over the mirrored sequence.
  const float zn = powf(z, (float)(n - 1));
  float s = get(0) + zn * get(n - 1);
  float zk = z;
  const float z2n = zn * zn;
  for (int k = 1; k < n - 1; ++k) {
    s += (zk + z2n / zk) * get(k);
    zk *= z;
  }
  return s / (1.0f - z2n);
}

// Column pass (axis 0): one thread per (frame, column); reads `in` of pixel
// type (or float when in_f is set), writes out.
__global__ void k_prefilter_cols(int H, int W, int n_frames, const void* in, int pixel_type, float* out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n_frames * W) return;
  const int f = (int)(t / W), x = (int)(t % W);
  const long long base = (long long)f * H * W + x;
  const float z = kPole, gain = 6.0f;
  auto get = [&](int k) { return gain * load_pixel<float>(in, pixel_type, base + (long long)k * W); };
  float c = causal_init_mirror(get, H);
  out[base] = c;
  for (int k = 1; k < H; ++k) {
    c = get(k) + z * c;
    out[base + (long long)k * W] = c;
  }
  if (H == 1) return;
  const float cm2 = out[base + (long long)(H - 2) * W];
  float a = (z / (z * z - 1.0f)) * (c + z * cm2);
  out[base + (long long)(H - 1) * W] = a;
  for (int k = H - 2; k >= 0; --k) {
    a = z * (a - out[base + (long long)k * W]);
    out[base + (long long)k * W] = a;
  }
}

// Row pass (axis 1), in place on `io`: a warp filters 32 rows, staging 32 x 32
// tiles through shared memory so global accesses stay coalesced.
__global__ void k_prefilter_rows(int H, int W, int n_frames, float* io) {
  __shared__ float tile[4][32][33];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long row0 = ((long long)blockIdx.x * 4 + warp) * 32;  // global row index over all frames
  const long long n_rows = (long long)n_frames * H;
  if (row0 >= n_rows) return;
  float(*tl)[33] = tile[warp];
  const float z = kPole, gain = 6.0f;
  const long long my_row = row0 + lane;
  const bool active = my_row < n_rows;
  float* rowp = io + (active ? my_row : row0) * W;
  const int n_chunks = (W + 31) / 32;
  // Causal pass.
  float c = 0.0f;
  for (int ch = 0; ch < n_chunks; ++ch) {
    const int x0 = ch * 32;
    for (int r = 0; r < 32; ++r) {
      const long long gr = row0 + r;
      tl[r][lane] = (gr < n_rows && x0 + lane < W) ? io[gr * W + x0 + lane] * gain : 0.0f;
    }
    __syncwarp();
    if (active) {
      int k0 = 0;
      if (ch == 0) {
        auto get = [&](int k) { return k < 32 ? tl[lane][k] : rowp[k] * gain; };
        c = causal_init_mirror(get, W);
        tl[lane][0] = c;
        k0 = 1;
      }
      for (int k = k0; k < 32 && x0 + k < W; ++k) {
        c = tl[lane][k] + z * c;
        tl[lane][k] = c;
      }
    }
    __syncwarp();
    for (int r = 0; r < 32; ++r) {
      const long long gr = row0 + r;
      if (gr < n_rows && x0 + lane < W) io[gr * W + x0 + lane] = tl[r][lane];
    }
    __syncwarp();
  }
  if (W == 1) return;
  // Anti-causal pass.
  float a = 0.0f;
  for (int ch = n_chunks - 1; ch >= 0; --ch) {
    const int x0 = ch * 32;
    for (int r = 0; r < 32; ++r) {
      const long long gr = row0 + r;
      tl[r][lane] = (gr < n_rows && x0 + lane < W) ? io[gr * W + x0 + lane] : 0.0f;
    }
    __syncwarp();
    if (active) {
      int k = (ch == n_chunks - 1) ? (W - 1 - x0) : 31;
      if (ch == n_chunks - 1) {
        const float cl = tl[lane][k];
        const float cm2 = k >= 1 ? tl[lane][k - 1] : rowp[W - 2];
        a = (z / (z * z - 1.0f)) * (cl + z * cm2);
        tl[lane][k] = a;
        --k;
      }
      for (; k >= 0; --k) {
        a = z * (a - tl[lane][k]);
        tl[lane][k] = a;
      }
    }
    __syncwarp();
    for (int r = 0; r < 32; ++r) {
      const long long gr = row0 + r;
      if (gr < n_rows && x0 + lane < W) io[gr * W + x0 + lane] = tl[r][lane];
    }
    __syncwarp();
  }
}

int spline_prefilter(int H, int W, int n_frames, const void* frames, int pixel_type, float* coef,
                     cudaStream_t stream) {
  if ((long long)H * W * n_frames == 0) return PIV_OK;
  const int bs = 128;
  const long long ncols = (long long)n_frames * W;
  k_prefilter_cols<<<(unsigned)((ncols + bs - 1) / bs), bs, 0, stream>>>(H, W, n_frames, frames, pixel_type, coef);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_cuda_error(e, "k_prefilter_cols launch");
  const long long nrows = (long long)n_frames * H;
  const long long nblocks = (nrows + 127) / 128;
  k_prefilter_rows<<<(unsigned)nblocks, 128, 0, stream>>>(H, W, n_frames, coef);
  e = cudaGetLastError();
  return e == cudaSuccess ? PIV_OK : set_cuda_error(e, "k_prefilter_rows launch");
}

}  // namespace piv
