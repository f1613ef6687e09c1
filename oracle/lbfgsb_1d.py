"""L-BFGS-B for one bounded variable: the search the reference's smoothn runs
to choose its smoothing parameter (test infrastructure: the specification the
device search in csrc/piv_smoothn.cu follows, checked here against SciPy).

The reference calls ``scipy.optimize.fmin_l_bfgs_b(gcv, [p0], fprime=None,
factr=10, approx_grad=True, bounds=[(p_min, p_max)])``
(openpiv_gpu/gpu_smoothn.py:191-193). SciPy is not vendored by the reference
(no pinned version); its L-BFGS-B is the published algorithm of

* R. H. Byrd, P. Lu, J. Nocedal, C. Zhu, "A limited memory algorithm for
  bound constrained optimization", SIAM J. Sci. Comput. 16 (1995), with the
  line search of
* J. J. More, D. J. Thuente, "Line search algorithms with guaranteed
  sufficient decrease", ACM TOMS 20 (1994),

with SciPy's defaults: memory m = 10, pgtol = 1e-5, factr * machine epsilon as
the relative-reduction tolerance, at most 20 function evaluations per line
search, line-search constants ftol = 1e-3, gtol = 0.9, xtol = 0.1, and the
gradient by forward differences with absolute step 1e-8 (backward where the
forward point leaves the box), divided by the representable step.

With one variable the limited-memory matrix is the latest secant slope
B = y s / s s = y y / y s (every BFGS update of a scalar discards its history),
the generalized Cauchy point is the minimiser of the quadratic model along
the projected steepest-descent path (the Newton point, or the bound it
crosses first), and the subspace minimisation leaves it unchanged.
"""

from math import sqrt

EPSMCH = 2.220446049250313e-16


def fd_point(x, lo, hi, h=1e-8):
    """The point of the forward difference at x with absolute step h:
    backward where x + h leaves [lo, hi] (with the fallbacks of SciPy's
    approx_derivative for a zero or an oversized step). The quotient is
    (f(fd_point) - f(x)) / (fd_point - x), over the representable step."""
    step = h
    if (x + step) - x == 0.0:
        step = EPSMCH ** 0.5 * (1.0 if x >= 0 else -1.0) * max(1.0, abs(x))
    xs = x + step
    if xs < lo or xs > hi:
        if abs(step) <= max(x - lo, hi - x):
            step = -step
        elif hi - x >= x - lo:
            step = hi - x
        else:
            step = -(x - lo)
    return x + step


def _dcstep(stx, fx, dx, sty, fy, dy, stp, fp, dp, brackt, stpmin, stpmax):
    """Safeguarded step of the More-Thuente line search (their four cases)."""
    sgnd = dp * (dx / abs(dx))
    if fp > fx:  # case 1: higher value, minimum bracketed
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp < stx:
            gamma = -gamma
        p = (gamma - dx) + theta
        q = ((gamma - dx) + gamma) + dp
        r = p / q
        stpc = stx + r * (stp - stx)
        stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx)
        stpf = stpc if abs(stpc - stx) < abs(stpq - stx) else stpc + (stpq - stpc) / 2.0
        brackt = True
    elif sgnd < 0.0:  # case 2: lower value, derivatives of opposite sign
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = ((gamma - dp) + gamma) + dx
        r = p / q
        stpc = stp + r * (stx - stp)
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
        brackt = True
    elif abs(dp) < abs(dx):  # case 3: same sign, derivative magnitude decreases
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * sqrt(max(0.0, (theta / s) ** 2 - (dx / s) * (dp / s)))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = (gamma + (dx - dp)) + gamma
        r = p / q
        if r < 0.0 and gamma != 0.0:
            stpc = stp + r * (stx - stp)
        elif stp > stx:
            stpc = stpmax
        else:
            stpc = stpmin
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        if brackt:
            stpf = stpc if abs(stpc - stp) < abs(stpq - stp) else stpq
            if stp > stx:
                stpf = min(stp + 0.66 * (sty - stp), stpf)
            else:
                stpf = max(stp + 0.66 * (sty - stp), stpf)
        else:
            stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
            stpf = min(stpmax, stpf)
            stpf = max(stpmin, stpf)
    else:  # case 4: same sign, derivative magnitude does not decrease
        if brackt:
            theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp
            s = max(abs(theta), abs(dy), abs(dp))
            gamma = s * sqrt((theta / s) ** 2 - (dy / s) * (dp / s))
            if stp > sty:
                gamma = -gamma
            p = (gamma - dp) + theta
            q = ((gamma - dp) + gamma) + dy
            r = p / q
            stpf = stp + r * (sty - stp)
        elif stp > stx:
            stpf = stpmax
        else:
            stpf = stpmin
    if fp > fx:
        sty, fy, dy = stp, fp, dp
    else:
        if sgnd < 0.0:
            sty, fy, dy = stx, fx, dx
        stx, fx, dx = stp, fp, dp
    return stx, fx, dx, sty, fy, dy, stpf, brackt


class _LineSearch:
    """The More-Thuente search on phi(stp) = f(x + stp d) with phi'(0) < 0."""

    FTOL, GTOL, XTOL, XTRAPL, XTRAPU = 1e-3, 0.9, 0.1, 1.1, 4.0

    def __init__(self, f, g, stp, stpmin, stpmax):
        self.brackt = False
        self.stage = 1
        self.finit, self.ginit = f, g
        self.gtest = self.FTOL * g
        self.width = stpmax - stpmin
        self.width1 = self.width / 0.5
        self.stx, self.fx, self.gx = 0.0, f, g
        self.sty, self.fy, self.gy = 0.0, f, g
        self.stmin, self.stmax = 0.0, stp + self.XTRAPU * stp
        self.stpmin, self.stpmax = stpmin, stpmax

    def step(self, stp, f, g):
        """Returns (status, next stp); status 'FG' asks for phi at the next
        stp, 'CONV' or 'WARN' ends the search at stp."""
        ftest = self.finit + stp * self.gtest
        if self.stage == 1 and f <= ftest and g >= 0.0:
            self.stage = 2
        status = "FG"
        if self.brackt and (stp <= self.stmin or stp >= self.stmax):
            status = "WARN"
        if self.brackt and self.stmax - self.stmin <= self.XTOL * self.stmax:
            status = "WARN"
        if stp == self.stpmax and f <= ftest and g <= self.gtest:
            status = "WARN"
        if stp == self.stpmin and (f > ftest or g >= self.gtest):
            status = "WARN"
        if f <= ftest and abs(g) <= self.GTOL * (-self.ginit):
            status = "CONV"
        if status != "FG":
            return status, stp
        gt = self.gtest
        if self.stage == 1 and f <= self.fx and f > ftest:
            stx, fxm, gxm, sty, fym, gym, stp, self.brackt = _dcstep(
                self.stx, self.fx - self.stx * gt, self.gx - gt, self.sty, self.fy - self.sty * gt, self.gy - gt,
                stp, f - stp * gt, g - gt, self.brackt, self.stmin, self.stmax)
            self.stx, self.sty = stx, sty
            self.fx, self.fy = fxm + stx * gt, fym + sty * gt
            self.gx, self.gy = gxm + gt, gym + gt
        else:
            (self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, self.brackt) = _dcstep(
                self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, f, g, self.brackt, self.stmin,
                self.stmax)
        if self.brackt:
            if abs(self.sty - self.stx) >= 0.66 * self.width1:
                stp = self.stx + 0.5 * (self.sty - self.stx)
            self.width1 = self.width
            self.width = abs(self.sty - self.stx)
        if self.brackt:
            self.stmin, self.stmax = min(self.stx, self.sty), max(self.stx, self.sty)
        else:
            self.stmin = stp + self.XTRAPL * (stp - self.stx)
            self.stmax = stp + self.XTRAPU * (stp - self.stx)
        stp = max(stp, self.stpmin)
        stp = min(stp, self.stpmax)
        if (self.brackt and (stp <= self.stmin or stp >= self.stmax)) or \
                (self.brackt and self.stmax - self.stmin <= self.XTOL * self.stmax):
            stp = self.stx
        return "FG", stp


def _projected_gradient(x, g, lo, hi):
    if g < 0.0:
        return abs(max(x - hi, g))
    return abs(min(x - lo, g))


class Lb1:
    """Reverse-communication form (the device search has the same steps):
    evaluate f at ``xt`` and the difference quotient there, ``feed`` them,
    repeat until ``done``; ``x`` is then the result."""

    MAX_EVALS = 200

    def __init__(self, x0, lo, hi):
        self.lo, self.hi = lo, hi
        self.x = min(max(x0, lo), hi)
        self.xt = self.x
        self.theta = 1.0  # the limited-memory matrix (a scalar: the latest secant slope)
        self.have_pairs = self.started = self.done = False
        self.it = self.nfev = self.evals = 0

    def _start_iteration(self):
        for _ in range(2):
            g, x = self.g, self.x
            bound = self.hi if g < 0.0 else self.lo
            tb = (x - self.hi) / g if g < 0.0 else (x - self.lo) / g
            f1 = -g * g
            f2 = -self.theta * f1
            dtm = -f1 / f2
            if (g < 0.0 and x >= self.hi) or (g > 0.0 and x <= self.lo):
                z = x
            elif dtm < tb:
                z = x + dtm * (-g)
            else:
                z = bound
            d = z - x
            stpmx = 1.0
            if self.it != 0:
                stpmx = 1e10
                if d < 0.0:
                    a2 = self.lo - x
                    if a2 >= 0.0:
                        stpmx = 0.0
                    elif d * stpmx < a2:
                        stpmx = a2 / d
                elif d > 0.0:
                    a2 = self.hi - x
                    if a2 <= 0.0:
                        stpmx = 0.0
                    elif d * stpmx > a2:
                        stpmx = a2 / d
            self.z, self.d, self.stp = z, d, 1.0
            self.x_old, self.f_old, self.g_old = x, self.f, g
            self.gdold = g * d
            self.nfev = 0
            if self.gdold < 0.0:
                self.ls = _LineSearch(self.f, self.gdold, self.stp, 0.0, stpmx)
                self.xt = z
                return
            if not self.have_pairs:  # not a descent direction and no memory to drop
                break
            self.theta, self.have_pairs = 1.0, False
        self.done = True

    def feed(self, f, g):
        self.evals += 1
        if self.evals >= self.MAX_EVALS:
            self.done = True
            return
        if not self.started:
            self.started = True
            self.x, self.f, self.g = self.xt, f, g
            if _projected_gradient(self.x, self.g, self.lo, self.hi) <= 1e-5:
                self.done = True
                return
            self._start_iteration()
            return
        self.nfev += 1
        status, stp = self.ls.step(self.stp, f, g * self.d)
        if status == "FG":
            if self.nfev >= 20:  # line search failed: back to the last iterate
                if not self.have_pairs:
                    self.done = True
                    return
                self.theta, self.have_pairs = 1.0, False
                self._start_iteration()
                return
            self.stp = stp
            self.xt = self.z if stp == 1.0 else stp * self.d + self.x_old
            return
        self.x, self.f, self.g = self.xt, f, g
        self.it += 1
        if _projected_gradient(self.x, self.g, self.lo, self.hi) <= 1e-5 or \
                (self.f_old - self.f) <= 10.0 * EPSMCH * max(max(abs(self.f_old), abs(self.f)), 1.0):
            self.done = True
            return
        y = self.g - self.g_old
        rr, gd_new = y * y, self.g * self.d
        if self.stp == 1.0:
            dr, ddum = gd_new - self.gdold, -self.gdold
        else:
            dr, ddum = (gd_new - self.gdold) * self.stp, -self.gdold * self.stp
        if dr > EPSMCH * ddum:
            self.theta, self.have_pairs = rr / dr, True
        self._start_iteration()


def lbfgsb_1d(fun, x0, lo, hi, trace=None):
    """Minimises fun over [lo, hi] from x0 as SciPy's fmin_l_bfgs_b does with
    approx_grad=True (factr 10, pgtol 1e-5); returns the final x. ``trace``
    (a list) receives every point at which f and its difference quotient are
    evaluated."""
    s = Lb1(x0, lo, hi)
    while not s.done:
        x = s.xt
        f = fun(x)
        xs = fd_point(x, lo, hi)
        if trace is not None:
            trace.append(x)
        s.feed(f, (fun(xs) - f) / (xs - x))
    return s.x
