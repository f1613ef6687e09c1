// L-BFGS-B for one bounded variable, as a reverse-communication state
// machine: the search smoothn's GCV step runs to choose p = log10(s)
// (gpu_smoothn.py:191-193 calls scipy.optimize.fmin_l_bfgs_b(gcv, [p0],
// approx_grad=True, factr=10, bounds=[(p_min, p_max)])).
//
// Restated from the published algorithm (Byrd, Lu, Nocedal & Zhu 1995, with
// the line search of More & Thuente 1994) for n = 1, with SciPy's settings:
// pgtol 1e-5, relative-reduction tolerance factr * machine epsilon, at most
// 20 evaluations per line search, line-search constants ftol 1e-3, gtol 0.9,
// xtol 0.1, and the gradient by forward differences with absolute step 1e-8
// (backward where the forward point leaves the box), divided by the
// representable step. With one variable the limited-memory matrix is the
// latest secant slope theta = y y / y s, the generalized Cauchy point is the
// Newton point -g / theta or the bound it crosses first, and the subspace
// minimisation leaves it unchanged. The caller evaluates f at lb.xt and at
// lb_fd_point(lb.xt), passes f and the difference quotient to lb_feed, and
// repeats until lb.done; lb.x is then the result.
#pragma once

#include <math.h>

#include "piv_common.cuh"

namespace piv {

constexpr double kLbEps = 2.220446049250313e-16;  // float64 machine epsilon
constexpr int kLbMaxEvals = 200;                  // evaluations (f and its difference quotient) per search

// More-Thuente line search on phi(stp) = f(x + stp d), phi'(0) < 0.
struct LbLine {
  bool brackt;
  int stage;
  double finit, ginit, gtest, width, width1;
  double stx, fx, gx, sty, fy, gy, stmin, stmax, stpmin, stpmax;
};

PIV_HD void lb_line_init(LbLine& s, double f, double g, double stp, double stpmin, double stpmax) {
  s.brackt = false;
  s.stage = 1;
  s.finit = f;
  s.ginit = g;
  s.gtest = 1e-3 * g;
  s.width = stpmax - stpmin;
  s.width1 = s.width / 0.5;
  s.stx = 0.0; s.fx = f; s.gx = g;
  s.sty = 0.0; s.fy = f; s.gy = g;
  s.stmin = 0.0;
  s.stmax = stp + 4.0 * stp;
  s.stpmin = stpmin;
  s.stpmax = stpmax;
}

// The safeguarded step (the four cases of More and Thuente); updates the
// bracket (stx, sty) and returns the next trial step.
PIV_HD double lb_dcstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double stp, double fp,
                       double dp, bool& brackt, double stpmin, double stpmax) {
  const double sgnd = dp * (dx / fabs(dx));
  double stpf;
  if (fp > fx) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
    double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp < stx) gamma = -gamma;
    const double p = (gamma - dx) + theta, q = ((gamma - dx) + gamma) + dp, r = p / q;
    const double stpc = stx + r * (stp - stx);
    const double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx);
    stpf = fabs(stpc - stx) < fabs(stpq - stx) ? stpc : stpc + (stpq - stpc) / 2.0;
    brackt = true;
  } else if (sgnd < 0.0) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
    double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dx, r = p / q;
    const double stpc = stp + r * (stx - stp);
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    stpf = fabs(stpc - stp) > fabs(stpq - stp) ? stpc : stpq;
    brackt = true;
  } else if (fabs(dp) < fabs(dx)) {
    const double theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp;
    const double s = fmax(fmax(fabs(theta), fabs(dx)), fabs(dp));
    double gamma = s * sqrt(fmax(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
    if (stp > stx) gamma = -gamma;
    const double p = (gamma - dp) + theta, q = (gamma + (dx - dp)) + gamma, r = p / q;
    double stpc;
    if (r < 0.0 && gamma != 0.0) stpc = stp + r * (stx - stp);
    else if (stp > stx) stpc = stpmax;
    else stpc = stpmin;
    const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
    if (brackt) {
      stpf = fabs(stpc - stp) < fabs(stpq - stp) ? stpc : stpq;
      if (stp > stx) stpf = fmin(stp + 0.66 * (sty - stp), stpf);
      else stpf = fmax(stp + 0.66 * (sty - stp), stpf);
    } else {
      stpf = fabs(stpc - stp) > fabs(stpq - stp) ? stpc : stpq;
      stpf = fmin(stpmax, stpf);
      stpf = fmax(stpmin, stpf);
    }
  } else {
    if (brackt) {
      const double theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp;
      const double s = fmax(fmax(fabs(theta), fabs(dy)), fabs(dp));
      double gamma = s * sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
      if (stp > sty) gamma = -gamma;
      const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dy, r = p / q;
      stpf = stp + r * (sty - stp);
    } else if (stp > stx) {
      stpf = stpmax;
    } else {
      stpf = stpmin;
    }
  }
  if (fp > fx) {
    sty = stp; fy = fp; dy = dp;
  } else {
    if (sgnd < 0.0) { sty = stx; fy = fx; dy = dx; }
    stx = stp; fx = fp; dx = dp;
  }
  return stpf;
}

// One line-search step at stp with phi = f, phi' = g. Returns 0 when the
// search asks for phi at the new *stp, 1 when it ends at stp (converged, or a
// warning that no further progress is possible).
PIV_HD int lb_line_step(LbLine& s, double& stp, double f, double g) {
  const double ftest = s.finit + stp * s.gtest;
  if (s.stage == 1 && f <= ftest && g >= 0.0) s.stage = 2;
  bool end = false;
  if (s.brackt && (stp <= s.stmin || stp >= s.stmax)) end = true;
  if (s.brackt && s.stmax - s.stmin <= 0.1 * s.stmax) end = true;
  if (stp == s.stpmax && f <= ftest && g <= s.gtest) end = true;
  if (stp == s.stpmin && (f > ftest || g >= s.gtest)) end = true;
  if (f <= ftest && fabs(g) <= 0.9 * (-s.ginit)) end = true;
  if (end) return 1;
  const double gt = s.gtest;
  if (s.stage == 1 && f <= s.fx && f > ftest) {
    double fxm = s.fx - s.stx * gt, fym = s.fy - s.sty * gt, gxm = s.gx - gt, gym = s.gy - gt;
    stp = lb_dcstep(s.stx, fxm, gxm, s.sty, fym, gym, stp, f - stp * gt, g - gt, s.brackt, s.stmin, s.stmax);
    s.fx = fxm + s.stx * gt;
    s.fy = fym + s.sty * gt;
    s.gx = gxm + gt;
    s.gy = gym + gt;
  } else {
    stp = lb_dcstep(s.stx, s.fx, s.gx, s.sty, s.fy, s.gy, stp, f, g, s.brackt, s.stmin, s.stmax);
  }
  if (s.brackt) {
    if (fabs(s.sty - s.stx) >= 0.66 * s.width1) stp = s.stx + 0.5 * (s.sty - s.stx);
    s.width1 = s.width;
    s.width = fabs(s.sty - s.stx);
  }
  if (s.brackt) {
    s.stmin = fmin(s.stx, s.sty);
    s.stmax = fmax(s.stx, s.sty);
  } else {
    s.stmin = stp + 1.1 * (stp - s.stx);
    s.stmax = stp + 4.0 * (stp - s.stx);
  }
  stp = fmax(stp, s.stpmin);
  stp = fmin(stp, s.stpmax);
  if ((s.brackt && (stp <= s.stmin || stp >= s.stmax)) || (s.brackt && s.stmax - s.stmin <= 0.1 * s.stmax))
    stp = s.stx;
  return 0;
}

struct Lb1 {
  double lo, hi;
  double x, f, g;        // current iterate
  double xt;             // the point whose f and difference quotient are requested
  double theta;          // limited-memory matrix (scalar)
  bool have_pairs, started, done;
  int it, nfev, evals;
  double x_old, f_old, g_old, z, d, stp, gdold;
  LbLine ls;
};

// The point of the forward difference at x (backward where x + 1e-8 leaves
// the box; the fallbacks of a zero or oversized step as SciPy's
// approx_derivative has them).
PIV_HD double lb_fd_point(double x, double lo, double hi) {
  double step = 1e-8;
  if ((x + step) - x == 0.0) step = 1.4901161193847656e-08 * (x >= 0.0 ? 1.0 : -1.0) * fmax(1.0, fabs(x));
  const double xs = x + step;
  if (xs < lo || xs > hi) {
    if (fabs(step) <= fmax(x - lo, hi - x)) step = -step;
    else if (hi - x >= x - lo) step = hi - x;
    else step = -(x - lo);
  }
  return x + step;
}

PIV_HD double lb_projg(double x, double g, double lo, double hi) {
  return g < 0.0 ? fabs(fmax(x - hi, g)) : fabs(fmin(x - lo, g));
}

PIV_HD void lb_init(Lb1& s, double x0, double lo, double hi) {
  s.lo = lo;
  s.hi = hi;
  s.x = fmin(fmax(x0, lo), hi);
  s.xt = s.x;
  s.theta = 1.0;
  s.have_pairs = false;
  s.started = false;
  s.done = false;
  s.it = 0;
  s.nfev = 0;
  s.evals = 0;
}

// Starts an iteration at the current iterate: Cauchy point z, direction d,
// the line search's first trial point. Ends the search (done, x unchanged)
// when d is not a descent direction and there is no memory to drop.
PIV_HD void lb_start_iteration(Lb1& s) {
  for (int attempt = 0; attempt < 2; ++attempt) {
    const double g = s.g, x = s.x;
    const double bound = g < 0.0 ? s.hi : s.lo;
    const double tb = g < 0.0 ? (x - s.hi) / g : (x - s.lo) / g;
    const double f1 = -g * g;
    const double f2 = -s.theta * f1;
    const double dtm = -f1 / f2;
    double z;
    if ((g < 0.0 && x >= s.hi) || (g > 0.0 && x <= s.lo)) z = x;
    else if (dtm < tb) z = x + dtm * (-g);
    else z = bound;
    const double d = z - x;
    double stpmx = 1.0;
    if (s.it != 0) {
      stpmx = 1e10;
      if (d < 0.0) {
        const double a2 = s.lo - x;
        if (a2 >= 0.0) stpmx = 0.0;
        else if (d * stpmx < a2) stpmx = a2 / d;
      } else if (d > 0.0) {
        const double a2 = s.hi - x;
        if (a2 <= 0.0) stpmx = 0.0;
        else if (d * stpmx > a2) stpmx = a2 / d;
      }
    }
    s.z = z;
    s.d = d;
    s.stp = 1.0;
    s.x_old = x;
    s.f_old = s.f;
    s.g_old = g;
    s.gdold = g * d;
    s.nfev = 0;
    if (s.gdold < 0.0) {
      lb_line_init(s.ls, s.f, s.gdold, s.stp, 0.0, stpmx);
      s.xt = z;
      return;
    }
    // Not a descent direction: drop the memory and retry once, else stop.
    if (!s.have_pairs) break;
    s.theta = 1.0;
    s.have_pairs = false;
  }
  s.done = true;
}

// Feeds f and the difference quotient g at s.xt; sets the next s.xt or done.
PIV_HD void lb_feed(Lb1& s, double f, double g) {
  if (++s.evals >= kLbMaxEvals) {  // bounded: keep the best accepted iterate
    s.done = true;
    return;
  }
  if (!s.started) {
    s.started = true;
    s.x = s.xt;
    s.f = f;
    s.g = g;
    if (lb_projg(s.x, s.g, s.lo, s.hi) <= 1e-5) {
      s.done = true;
      return;
    }
    lb_start_iteration(s);
    return;
  }
  ++s.nfev;
  double stp = s.stp;
  const int end = lb_line_step(s.ls, stp, f, g * s.d);
  if (!end) {
    if (s.nfev >= 20) {  // line search failed: back to the last iterate
      if (!s.have_pairs) {
        s.done = true;
        return;
      }
      s.theta = 1.0;
      s.have_pairs = false;
      lb_start_iteration(s);
      return;
    }
    s.stp = stp;
    s.xt = stp == 1.0 ? s.z : stp * s.d + s.x_old;
    return;
  }
  // Accepted: the new iterate.
  s.x = s.xt;
  s.f = f;
  s.g = g;
  ++s.it;
  if (lb_projg(s.x, s.g, s.lo, s.hi) <= 1e-5 ||
      (s.f_old - s.f) <= 10.0 * kLbEps * fmax(fmax(fabs(s.f_old), fabs(s.f)), 1.0)) {
    s.done = true;
    return;
  }
  const double y = s.g - s.g_old;
  const double rr = y * y, gd_new = s.g * s.d;
  double dr, ddum;
  if (s.stp == 1.0) {
    dr = gd_new - s.gdold;
    ddum = -s.gdold;
  } else {
    dr = (gd_new - s.gdold) * s.stp;
    ddum = -s.gdold * s.stp;
  }
  if (dr > kLbEps * ddum) {
    s.theta = rr / dr;
    s.have_pairs = true;
  }
  lb_start_iteration(s);
}

}  // namespace piv
