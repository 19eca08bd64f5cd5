"""Limited-memory BFGS with a restartable state, for the weight training.

The reference trains with L-BFGS-B 3.0 (lib/Lbfgsb.3.0, Byrd, Lu, Nocedal
and Zhu; opt_init_bfgs / opt_bfgs_weights, src/optimize.f90:1600-1609,
1721-1771) with m = 20 correction pairs and no bounds, one iteration per
epoch, and saves the optimiser's workspace to `train.restart`
(opt_save_state_bfgs, optimize.f90:1636-1652) so that a later run resumes
the same iteration sequence.  That file is the Fortran routine's own work
arrays.  Here the optimiser is written out: without bounds L-BFGS-B's
step is the limited-memory quasi-Newton step (the two-loop recursion of
Nocedal and Wright, Numerical Optimization, Alg. 7.4, with the same
s'y/y'y scaling), followed by a line search for the strong Wolfe
conditions (sufficient decrease 1e-3 and curvature 0.9, the constants of
L-BFGS-B's line search) by bracketing and zooming with cubic
interpolation (Alg. 3.5 and 3.6).  Its whole state -- point, value,
gradient, correction pairs, counters -- is saved to and loaded from a
restart file, so an interrupted training resumes on the same trajectory.
"""
import numpy as np

__all__ = ["LBFGS"]

FTOL = 1e-3     # sufficient decrease
GTOL = 0.9      # curvature
MAX_EVALS = 20  # function evaluations per line search


class LBFGS:
    """Minimise ``fg(x) -> (f, g)``."""

    def __init__(self, fg, x0=None, m=20, state=None):
        self.fg = fg
        self.m = int(m)
        if state is not None:
            self._set_state(state)
            return
        self.x = np.array(x0, dtype=np.float64)
        self.f, self.g = self._eval(self.x)
        self.S, self.Y = [], []
        self.k = 0
        self.nfev = 1

    def _eval(self, x):
        f, g = self.fg(x)
        return float(f), np.array(g, dtype=np.float64)

    # ---------------------------------------------------------------- state
    def state(self):
        n = self.x.size
        S = np.array(self.S).reshape(-1, n)
        Y = np.array(self.Y).reshape(-1, n)
        return {"method": "lbfgs", "m": self.m, "n": n, "x": self.x.copy(), "f": self.f,
                "g": self.g.copy(), "S": S, "Y": Y, "k": self.k, "nfev": self.nfev}

    def _set_state(self, st):
        if str(st["method"]) != "lbfgs" or int(st["m"]) != self.m:
            raise ValueError("incompatible restart state")
        self.x = np.array(st["x"], dtype=np.float64)
        self.f = float(st["f"])
        self.g = np.array(st["g"], dtype=np.float64)
        self.S = [np.array(v) for v in np.asarray(st["S"])]
        self.Y = [np.array(v) for v in np.asarray(st["Y"])]
        self.k = int(st["k"])
        self.nfev = int(st["nfev"])

    def save(self, path):
        with open(path, "wb") as fh:
            np.savez(fh, **self.state())

    @classmethod
    def load(cls, fg, path, m=20):
        with np.load(path, allow_pickle=False) as z:
            st = {k: z[k] for k in z.files}
        if int(st["n"]) != st["x"].size:
            raise ValueError("corrupt restart state")
        return cls(fg, m=m, state=st)

    # ----------------------------------------------------------- iteration
    def direction(self):
        q = -self.g.copy()
        alpha = []
        for s, y in zip(reversed(self.S), reversed(self.Y)):
            rho = 1.0 / (y @ s)
            a = rho * (s @ q)
            alpha.append((rho, a))
            q -= a * y
        if self.S:
            s, y = self.S[-1], self.Y[-1]
            q *= (s @ y) / (y @ y)
        for (s, y), (rho, a) in zip(zip(self.S, self.Y), reversed(alpha)):
            b = rho * (y @ q)
            q += (a - b) * s
        return q

    def step(self):
        """One iteration; returns False when no progress is possible."""
        d = self.direction()
        dg0 = d @ self.g
        if not dg0 < 0.0:       # not a descent direction: drop the memory
            self.S, self.Y = [], []
            d = -self.g
            dg0 = d @ self.g
            if not dg0 < 0.0:
                return False
        # first iteration: unit step in x (L-BFGS-B starts with 1/||d||)
        stp0 = min(1.0, 1.0 / np.linalg.norm(d)) if not self.S else 1.0
        res = self._line_search(d, dg0, stp0)
        if res is None:
            return False
        stp, f1, g1 = res
        s = stp * d
        y = g1 - self.g
        if s @ y > np.finfo(float).eps * (y @ y):
            self.S.append(s)
            self.Y.append(y)
            if len(self.S) > self.m:
                self.S.pop(0)
                self.Y.pop(0)
        self.x = self.x + s
        self.f, self.g = f1, g1
        self.k += 1
        return True

    def _phi(self, d, stp):
        f, g = self._eval(self.x + stp * d)
        self.nfev += 1
        return f, g, g @ d

    def _line_search(self, d, dg0, stp):
        f0 = self.f
        lo = (0.0, f0, dg0, self.g)
        prev = lo
        for it in range(MAX_EVALS):
            f, g, dg = self._phi(d, stp)
            if f > f0 + FTOL * stp * dg0 or (it > 0 and f >= prev[1]):
                return self._zoom(d, dg0, prev, (stp, f, dg, g))
            if abs(dg) <= -GTOL * dg0:
                return stp, f, g
            if dg >= 0.0:
                return self._zoom(d, dg0, (stp, f, dg, g), prev)
            prev = (stp, f, dg, g)
            stp *= 4.0
        return None

    def _zoom(self, d, dg0, lo, hi):
        f0 = self.f
        for _ in range(MAX_EVALS):
            stp = _cubic_min(lo, hi)
            f, g, dg = self._phi(d, stp)
            if f > f0 + FTOL * stp * dg0 or f >= lo[1]:
                hi = (stp, f, dg, g)
            else:
                if abs(dg) <= -GTOL * dg0:
                    return stp, f, g
                if dg * (hi[0] - lo[0]) >= 0.0:
                    hi = lo
                lo = (stp, f, dg, g)
            if abs(hi[0] - lo[0]) <= 1e-12 * max(1.0, abs(lo[0])):
                break
        # no Wolfe point: accept the best decrease found, if any
        if lo[0] > 0.0 and lo[1] < f0:
            return lo[0], lo[1], lo[3]
        return None


def _cubic_min(a, b):
    """Minimiser of the cubic through (stp, f, f') at a and b, kept inside
    the bracket (bisection when the cubic has no interior minimum)."""
    x0, f0, d0 = a[0], a[1], a[2]
    x1, f1, d1 = b[0], b[1], b[2]
    lo, hi = min(x0, x1), max(x0, x1)
    d_1 = d0 + d1 - 3.0 * (f0 - f1) / (x0 - x1)
    rad = d_1 * d_1 - d0 * d1
    if rad >= 0.0:
        d_2 = np.copysign(np.sqrt(rad), x1 - x0)
        den = d1 - d0 + 2.0 * d_2
        if den != 0.0:
            x = x1 - (x1 - x0) * (d1 + d_2 - d_1) / den
            w = hi - lo
            if lo + 0.1 * w <= x <= hi - 0.1 * w:
                return x
    return 0.5 * (lo + hi)
