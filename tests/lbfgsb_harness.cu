// Host-side harness of the device L-BFGS-B search (csrc/piv_lbfgsb1.cuh), for
// the CPU tests: the same state machine compiled for the host and driven by a
// callback, so that its steps can be compared with oracle/lbfgsb_1d.py and
// SciPy without a GPU.
#include "../openpiv-python-gpu_gb300/csrc/piv_lbfgsb1.cuh"

extern "C" double lb1_minimize(double (*fun)(double), double x0, double lo, double hi, int* n_evals) {
  piv::Lb1 s;
  piv::lb_init(s, x0, lo, hi);
  int evals = 0;
  for (int ev = 0; ev < piv::kLbMaxEvals && !s.done; ++ev) {
    const double x = s.xt, xs = piv::lb_fd_point(x, lo, hi);
    const double f = fun(x);
    const double fh = fun(xs);
    evals += 2;
    piv::lb_feed(s, f, (fh - f) / (xs - x));
  }
  if (n_evals) *n_evals = evals;
  return s.x;
}
