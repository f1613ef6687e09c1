// Helpers shared by the tensor-core correlation engines and the peak
// refinement: the subpixel fit of the reference and the segment table of a
// multi-geometry correlation launch.
#pragma once

#include "piv_common.cuh"
#include "piv_internal.h"

namespace piv {

// Subpixel peak (gpu_process.py:1256-1294) from the five map values.
PIV_D void subpixel_fit(int subpixel, int pi_, int pj, float c, float cd, float cu, float cl, float cr, float& isp,
                        float& jsp) {
  const float eps = 1e-7f;
  isp = (float)pi_;
  jsp = (float)pj;
  if (subpixel == PIV_SUBPIXEL_GAUSSIAN) {
    if (c > 0 && cd > 0 && cu > 0 && cl > 0 && cr > 0) {
      c = logf(c); cd = logf(cd); cu = logf(cu); cl = logf(cl); cr = logf(cr);
      isp = add_rn((float)pi_, div_rn(mul_rn(0.5f, sub_rn(cd, cu)), add_rn(add_rn(sub_rn(cd, mul_rn(2.f, c)), cu), eps)));
      jsp = add_rn((float)pj, div_rn(mul_rn(0.5f, sub_rn(cl, cr)), add_rn(add_rn(sub_rn(cl, mul_rn(2.f, c)), cr), eps)));
    }
  } else if (subpixel == PIV_SUBPIXEL_PARABOLIC) {
    isp = add_rn((float)pi_, div_rn(mul_rn(0.5f, sub_rn(cd, cu)), add_rn(add_rn(sub_rn(cd, mul_rn(2.f, c)), cu), eps)));
    jsp = add_rn((float)pj, div_rn(mul_rn(0.5f, sub_rn(cl, cr)), add_rn(add_rn(sub_rn(cl, mul_rn(2.f, c)), cr), eps)));
  } else {
    isp = add_rn((float)pi_, div_rn(sub_rn(cu, cd), add_rn(add_rn(add_rn(cd, c), cu), eps)));
    jsp = add_rn((float)pj, div_rn(sub_rn(cr, cl), add_rn(add_rn(add_rn(cl, c), cr), eps)));
  }
}

// The launch's segment table in shared memory (one segment built from the
// single geometry of `a` when a.n_segs == 0); returns the segment count. All
// threads call it; it ends with a barrier.
PIV_D int load_segments(const CorrArgs& a, CorrSeg* seg_s) {
  const int n = a.n_segs > 0 ? a.n_segs : 1;
  if ((int)threadIdx.x < n) {
    CorrSeg q;
    if (a.n_segs > 0) {
#pragma unroll
      for (int k = 0; k < kMaxCorrSegs; ++k)  // static indices keep the table in parameter space
        if (k == (int)threadIdx.x) q = a.segs[k];
    } else {
      q.frame_a = a.frame_a;
      q.frame_b = a.frame_b;
      q.u = a.u;
      q.v = a.v;
      q.peak_i = a.peak_i;
      q.peak_j = a.peak_j;
      q.win_mask = a.win_mask;
      q.near_tie = a.near_tie;
      q.tie_count = a.tie_count;
      q.tie_list = a.tie_list;
      q.tie_list_count = a.tie_list_count;
      q.win_means = a.win_means;
      q.win0 = 0;
      q.height = a.height;
      q.width = a.width;
      q.spacing = a.spacing;
      q.m = a.m;
      q.n = a.n;
      q.x_offset = a.x_offset;
      q.y_offset = a.y_offset;
      q.n_pairs = a.n_pairs;
    }
    seg_s[threadIdx.x] = q;
  }
  __syncthreads();
  return n;
}

}  // namespace piv
