"""CPU restatement of the occupation optimiser's minimiser -- test infrastructure.

The reference minimises the occupation energy over gamma with
``scipy.optimize.minimize(calcocce, gamma, jac=calcoccg, method="CG")``
(``pynof/minimization.py:77-97``; ``p.occupation_optimizer = "CG"``,
``pynof/parameters.py:96``).  scipy is a dependency the reference does not pin
(``pyproject.toml:15``); this module restates the published algorithm of its
CG method as scipy 1.18 runs it, the step-by-step oracle of the device
optimiser:

* nonlinear conjugate gradients, Polak-Ribiere with the "+" restart
  (beta = max(0, g1.(g1 - g0) / g0.g0)), with the sufficient-descent check of
  Gilbert & Nocedal (SIAM J. Optim. 2 (1992) 21-42) on every accepted step
  (p1.g1 <= -0.01 g1.g1 unless ||g1||_inf <= gtol);
* the first trial step of each line search from the previous decrease,
  alpha1 = min(1, 2.02 (f0 - f_prev) / phi'(0)) (1 when that is negative),
  with f_prev = f0 + ||g0||_2 / 2 before the first iteration;
* the line search of More & Thuente (ACM TOMS 20 (1994) 286-307): strong Wolfe
  conditions with ftol c1 = 1e-4, gtol c2 = 0.4, xtol 1e-14, steps in
  [1e-100, 1e100], at most 100 calls; the safeguarded cubic / quadratic step
  of the paper's four cases; the modified function in the first stage;
* stop when ||g||_inf <= gtol (1e-5) or after 200 nv iterations.

scipy falls back to a second line search (Nocedal & Wright's zoom) when this
one fails or its step does not give sufficient descent, and stops when that
fails too.  Here, as on the device, a failed search restarts from steepest
descent once (when the direction was not already -g) and otherwise stops at
the current point: the two agree whenever the first line search succeeds,
which ``tests/test_occ_cg_cpu.py`` checks against scipy itself.

Only ``tests/`` may import this module.
"""
from __future__ import annotations

import math

import numpy as np

XTRAPL, XTRAPU, P5, P66 = 1.1, 4.0, 0.5, 0.66


def _sqrt(v):
    """Square root that gives NaN below zero (the search then fails), as
    scipy's dcstep does with numpy's sqrt."""
    return math.sqrt(v) if v >= 0.0 else float("nan")


def dcstep(stx, fx, dx, sty, fy, dy, stp, fp, dp, brackt, stpmin, stpmax):
    """One safeguarded step of More & Thuente (section 4 of the paper):
    returns (stx, fx, dx, sty, fy, dy, stp, brackt)."""
    sgnd = dp * (dx / abs(dx))
    if fp > fx:
        # case 1: a higher function value; the minimum is bracketed
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * _sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp < stx:
            gamma = -gamma
        p = (gamma - dx) + theta
        q = ((gamma - dx) + gamma) + dp
        r = p / q
        stpc = stx + r * (stp - stx)
        stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx)
        stpf = stpc if abs(stpc - stx) < abs(stpq - stx) else stpc + (stpq - stpc) / 2.0
        brackt = True
    elif sgnd < 0.0:
        # case 2: lower value, derivatives of opposite sign; bracketed
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * _sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = ((gamma - dp) + gamma) + dx
        r = p / q
        stpc = stp + r * (stx - stp)
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
        brackt = True
    elif abs(dp) < abs(dx):
        # case 3: lower value, same sign, the derivative's magnitude decreases
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * _sqrt(max(0.0, (theta / s) ** 2 - (dx / s) * (dp / s)))
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
                stpf = min(stp + P66 * (sty - stp), stpf)
            else:
                stpf = max(stp + P66 * (sty - stp), stpf)
        else:
            stpf = stpc if abs(stpc - stp) > abs(stpq - stp) else stpq
            stpf = min(stpmax, stpf)
            stpf = max(stpmin, stpf)
    else:
        # case 4: lower value, same sign, the derivative does not decrease
        if brackt:
            theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp
            s = max(abs(theta), abs(dy), abs(dp))
            gamma = s * _sqrt((theta / s) ** 2 - (dy / s) * (dp / s))
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


class LineSearch:
    """More & Thuente's search in reverse communication: ``start`` takes
    phi(0), phi'(0) and the first trial step, ``step`` takes phi, phi' at the
    current trial step; both return ("FG", next step), ("CONV", step) or
    ("FAIL", None)."""

    def __init__(self, ftol=1e-4, gtol=0.4, xtol=1e-14, stpmin=1e-100, stpmax=1e100, maxcalls=100):
        self.ftol, self.gtol, self.xtol, self.stpmin, self.stpmax = ftol, gtol, xtol, stpmin, stpmax
        self.maxcalls = maxcalls

    def start(self, stp, f, g):
        self.calls = 1
        if stp < self.stpmin or stp > self.stpmax or g >= 0.0:
            return "FAIL", None
        self.brackt = False
        self.stage = 1
        self.finit, self.ginit = f, g
        self.gtest = self.ftol * g
        self.width = self.stpmax - self.stpmin
        self.width1 = self.width / P5
        self.stx, self.fx, self.gx = 0.0, f, g
        self.sty, self.fy, self.gy = 0.0, f, g
        self.stmin = 0.0
        self.stmax = stp + XTRAPU * stp
        self.stp = stp
        return self._next("FG", stp)

    def _next(self, task, stp):
        if task == "FG":
            if not math.isfinite(stp):
                return "FAIL", None
            if self.calls >= self.maxcalls:
                return "FAIL", None
        return task, stp

    def step(self, f, g):
        self.calls += 1
        stp = self.stp
        ftest = self.finit + stp * self.gtest
        if self.stage == 1 and f <= ftest and g >= 0.0:
            self.stage = 2
        warn = (self.brackt and (stp <= self.stmin or stp >= self.stmax)) or \
               (self.brackt and self.stmax - self.stmin <= self.xtol * self.stmax) or \
               (stp == self.stpmax and f <= ftest and g <= self.gtest) or \
               (stp == self.stpmin and (f > ftest or g >= self.gtest))
        if f <= ftest and abs(g) <= self.gtol * (-self.ginit):
            return "CONV", stp
        if warn:
            return "FAIL", None
        if self.stage == 1 and f <= self.fx and f > ftest:
            # the modified function psi(a) = phi(a) - phi(0) - ftol phi'(0) a
            fm, fxm, fym = f - stp * self.gtest, self.fx - self.stx * self.gtest, self.fy - self.sty * self.gtest
            gm, gxm, gym = g - self.gtest, self.gx - self.gtest, self.gy - self.gtest
            self.stx, fxm, gxm, self.sty, fym, gym, stp, self.brackt = dcstep(
                self.stx, fxm, gxm, self.sty, fym, gym, stp, fm, gm, self.brackt, self.stmin, self.stmax)
            self.fx, self.fy = fxm + self.stx * self.gtest, fym + self.sty * self.gtest
            self.gx, self.gy = gxm + self.gtest, gym + self.gtest
        else:
            self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, self.brackt = dcstep(
                self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, f, g, self.brackt, self.stmin,
                self.stmax)
        if self.brackt:
            if abs(self.sty - self.stx) >= P66 * self.width1:
                stp = self.stx + P5 * (self.sty - self.stx)
            self.width1 = self.width
            self.width = abs(self.sty - self.stx)
            self.stmin, self.stmax = min(self.stx, self.sty), max(self.stx, self.sty)
        else:
            self.stmin = stp + XTRAPL * (stp - self.stx)
            self.stmax = stp + XTRAPU * (stp - self.stx)
        stp = min(max(stp, self.stpmin), self.stpmax)
        if (self.brackt and (stp <= self.stmin or stp >= self.stmax)) or \
           (self.brackt and self.stmax - self.stmin <= self.xtol * self.stmax):
            stp = self.stx
        self.stp = stp
        return self._next("FG", stp)


def minimize_cg(fg, x0, gtol=1e-5, maxiter=None, c1=1e-4, c2=0.4):
    """Minimise f over x from x0; ``fg(x)`` returns (f, g).  Returns
    (x, f, iterations, evaluations, success)."""
    x = np.array(x0, dtype=np.float64).ravel()
    maxiter = 200 * x.size if maxiter is None else maxiter
    f, g = fg(x)
    nev = 1
    f_prev = f + np.linalg.norm(g) / 2.0
    p = -g
    gnorm = np.max(np.abs(g)) if g.size else 0.0
    k = 0
    success = True
    restarted = False
    while gnorm > gtol and k < maxiter:
        delta = np.dot(g, g)
        d0 = np.dot(g, p)
        alpha1 = 1.0
        if d0 != 0.0:
            alpha1 = min(1.0, 1.01 * 2 * (f - f_prev) / d0)
            if alpha1 < 0.0:
                alpha1 = 1.0
        ls = LineSearch(c1, c2)
        task, stp = ls.start(alpha1, f, d0)
        f1 = g1 = None
        while task == "FG":
            f1, g1 = fg(x + stp * p)
            nev += 1
            task, stp = ls.step(f1, np.dot(g1, p))
        accepted = False
        if task == "CONV":
            x1 = x + stp * p
            beta = max(0.0, np.dot(g1 - g, g1) / delta)
            p1 = -g1 + beta * p
            gn1 = np.max(np.abs(g1))
            if gn1 <= gtol or np.dot(p1, g1) <= -0.01 * np.dot(g1, g1):
                accepted = True
        if not accepted:
            if restarted or np.array_equal(p, -g):
                success = False
                break
            p = -g  # steepest descent, once
            restarted = True
            continue
        restarted = False
        f_prev, f = f, f1
        x, g, p, gnorm = x1, g1, p1, gn1
        k += 1
    return x, f, k, nev, success and gnorm <= gtol
