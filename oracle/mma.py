"""Method of Moving Asymptotes, restated in numpy -- TEST INFRASTRUCTURE ONLY (the oracle of the device MMA).

Follows pyMOTO's MMA (pymoto/common/mma.py, v2.0.1): the asymptote adaptation of MMA.step (:96-168), the
convex separable approximation of mmasub (:170-234, versions MMA1987 / MMA2007 / GCMMA) and the primal-dual
interior-point Newton method of subsolv (:236-474), with the same update formulas, step-length rule, line
search and epsilon schedule.  Pinned against pyMOTO's own MMA steps (tests/golden/mma_mbb.npz).
"""
import numpy as np


class MMAOracle:
    """State of one MMA run over n variables with m >= 1 constraints (a dummy one when unconstrained)."""

    def __init__(self, n, m_resp, xmin=0.0, xmax=1.0, move=0.1, mmaversion="MMA2007", a0=1.0, epsimin=1e-10,
                 cCoef=1e3, albefa=0.1, asyinit=0.5, asyincr=1.2, asydecr=0.7, asybound=10.0, a=None, c=None):
        self.n = n
        self.xmin = np.broadcast_to(np.asarray(xmin, dtype=float), (n,)).copy()
        self.xmax = np.broadcast_to(np.asarray(xmax, dtype=float), (n,)).copy()
        self.move = move
        self.version = mmaversion.lower()
        self.a0, self.epsimin = a0, epsimin
        self.albefa, self.asyincr, self.asydecr, self.asybound = albefa, asyincr, asydecr, asybound
        self.dx = self.xmax - self.xmin
        self.offset = asyinit * np.ones(n)
        self.xold1 = self.xold2 = None
        self.m = max(1, m_resp - 1)
        self.a = np.zeros(self.m) if a is None else np.asarray(a, dtype=float)
        self.c = np.full(self.m, cCoef, dtype=float) if c is None else np.asarray(c, dtype=float)
        self.d = np.ones(self.m)
        self.low = self.upp = self.gest = self.dk = None
        self.stats = {}

    def adapt_asymptotes(self, x):
        """Offsets grow where the last two steps kept their sign and shrink where they alternated
        (mma.py:110-126)."""
        if self.xold1 is not None and self.xold2 is not None:
            trend = (x - self.xold1) * (self.xold1 - self.xold2)
            self.offset[trend > 0] *= self.asyincr
            self.offset[trend < 0] *= self.asydecr
            self.offset = np.clip(self.offset, 1 / (self.asybound ** 2), self.asybound)

    def step(self, x, g, dg, rho=1e-5):
        """One MMA (not GCMMA) step from responses g (m_resp,) and sensitivities dg (m_resp, n)."""
        self.adapt_asymptotes(x)
        xnew = self.mmasub(x, np.asarray(g, dtype=float), np.atleast_2d(dg), rho)
        self.xold2, self.xold1 = self.xold1, x.copy()
        return xnew

    def approximation(self, xval, g, dg, rho):
        """Asymptotes, move limits and the coefficients P, Q, rhs of the separable approximation (mma.py:170-212)."""
        if g.size == 1:   # unconstrained: dummy constraint -1 with zero sensitivities (mma.py:172-175)
            g = np.hstack((g, -1.0))
            dg = np.vstack((dg, np.zeros(self.n)))
        shift = self.offset * self.dx
        low, upp = xval - shift, xval + shift
        alfa = np.maximum(np.maximum(low + self.albefa * shift, xval - self.move * self.dx), self.xmin)
        beta = np.minimum(np.minimum(upp - self.albefa * shift, xval + self.move * self.dx), self.xmax)
        dgp, dgm = np.maximum(dg, 0), np.maximum(-dg, 0)
        sq = shift ** 2
        if "1987" in self.version:
            P, Q = sq * dgp, sq * dgm
        elif "2007" in self.version:
            P = sq * (1.001 * dgp + 0.001 * dgm + rho / self.dx)
            Q = sq * (0.001 * dgp + 1.001 * dgm + rho / self.dx)
        elif "gcmma" in self.version:
            r = np.maximum(np.asarray(rho, dtype=float)[:, None], 1e-6)
            P = sq * (1.001 * dgp + 0.001 * dgm + r / self.dx)
            Q = sq * (0.001 * dgp + 1.001 * dgm + r / self.dx)
        else:
            raise ValueError("unknown MMA version")
        rhs = P @ (1 / shift) + Q @ (1 / shift) - g
        return g, low, upp, alfa, beta, P, Q, rhs

    def mmasub(self, xval, g, dg, rho=1e-5):
        unconstrained = g.size == 1
        g, low, upp, alfa, beta, P, Q, rhs = self.approximation(xval, g, dg, rho)
        self.low, self.upp = low, upp
        eps = self.epsimin * np.sqrt(self.m + self.n)
        xm = subsolv(eps, low, upp, alfa, beta, P, Q, self.a0, self.a, rhs[1:], self.c, self.d, xval, self.stats)
        self.gest = np.sum(P / (upp - xm) + Q / (xm - low), axis=1) - rhs
        if unconstrained:
            self.gest = self.gest[[0]]
        self.dk = np.sum((upp - low) * (xm - xval) ** 2 / ((upp - xm) * (xm - low) * self.dx))
        return xm


def _residual(x, y, z, lam, xsi, eta, mu, zet, s, low, upp, alfa, beta, P0, Q0, P1, Q1, a0, a, b, c, d, epsi):
    """Squared KKT residuals of the perturbed subproblem (mma.py:302-325)."""
    ux1, xl1 = upp - x, x - low
    plam, qlam = P0 + lam @ P1, Q0 + lam @ Q1
    gvec = P1 @ (1 / ux1) + Q1 @ (1 / xl1)
    dpsidx = plam / (ux1 ** 2) - qlam / (xl1 ** 2)
    r = np.concatenate([dpsidx - xsi + eta, c + d * y - mu - lam, [a0 - zet - a @ lam], gvec - a * z - y + s - b,
                        xsi * (x - alfa) - epsi, eta * (beta - x) - epsi, mu * y - epsi, [zet * z - epsi],
                        lam * s - epsi])
    return r ** 2


def subsolv(epsimin, low, upp, alfa, beta, P, Q, a0, a, b, c, d, x0, stats=None):
    """Primal-dual Newton solution of the MMA subproblem (mma.py:236-474): epsilon 1, 0.1, ... down to epsimin,
    Newton steps while the largest squared residual exceeds (0.9 epsilon)^2 (at most 400), each with the
    fraction-to-boundary step 1/max(1.01 ratios, 1) halved until the residual norm decreases (at most 400)."""
    n, m = len(alfa), len(a)
    maxit = 400
    x = np.clip(x0, alfa + 1e-10, beta - 1e-10)
    y, z, lam, s = np.ones(m), 1.0, np.ones(m), np.ones(m)
    xsi, eta = np.maximum(1.0 / (x - alfa), 1), np.maximum(1.0 / (beta - x), 1)
    mu, zet = np.maximum(1, 0.5 * c), 1.0
    P0, Q0, P1, Q1 = P[0], Q[0], P[1:], Q[1:]
    epsi, outer, newton, trials = 1.0, 0, 0, 0
    while epsi > epsimin:
        outer += 1
        r2 = _residual(x, y, z, lam, xsi, eta, mu, zet, s, low, upp, alfa, beta, P0, Q0, P1, Q1, a0, a, b, c, d,
                       epsi)
        rnorm, rmax = r2.sum(), r2.max()
        it = 0
        while rmax > (0.9 * epsi) ** 2 and it < maxit:
            it += 1
            newton += 1
            ux1, xl1 = upp - x, x - low
            ux2, xl2 = ux1 ** 2, xl1 ** 2
            uxinv1, xlinv1, uxinv2, xlinv2 = 1.0 / ux1, 1.0 / xl1, 1.0 / ux2, 1.0 / xl2
            plam, qlam = P0 + lam @ P1, Q0 + lam @ Q1
            gvec = P1 @ uxinv1 + Q1 @ xlinv1
            GG = P1 * uxinv2 - Q1 * xlinv2
            dpsidx = plam / ux2 - qlam / xl2
            delx = dpsidx - epsi / (x - alfa) + epsi / (beta - x)
            dely = c + d * y - lam - epsi / y
            delz = a0 - a @ lam - epsi / z
            dellam = gvec - a * z - y - b + epsi / lam
            diagx = 2 * (plam / (ux1 * ux2) + qlam / (xl1 * xl2)) + xsi / (x - alfa) + eta / (beta - x)
            diagy = d + mu / y
            diaglamyi = s / lam + 1.0 / diagy
            AA = np.empty((m + 1, m + 1))
            AA[:-1, :-1] = np.diag(diaglamyi) + (GG / diagx) @ GG.T
            AA[-1, :-1] = AA[:-1, -1] = a
            AA[-1, -1] = -zet / z
            bb = np.append(dellam + dely / diagy - GG @ (delx / diagx), delz)
            sol = np.linalg.solve(AA, bb)
            dlam, dz = sol[:m], sol[m]
            dx = -delx / diagx - (dlam @ GG) / diagx
            dy = -dely / diagy + dlam / diagy
            dxsi = -xsi + epsi / (x - alfa) - (xsi * dx) / (x - alfa)
            deta = -eta + epsi / (beta - x) + (eta * dx) / (beta - x)
            dmu = -mu + epsi / y - (mu * dy) / y
            dzet = -zet + epsi / z - zet * dz / z
            ds = -s + epsi / lam - (s * dlam) / lam
            stmxx = max(-1.01 * np.min(dy / y), -1.01 * dz / z, -1.01 * np.min(dlam / lam),
                        -1.01 * np.min(dxsi / xsi), -1.01 * np.min(deta / eta), -1.01 * np.min(dmu / mu),
                        -1.01 * dzet / zet, -1.01 * np.min(ds / s))
            stmalfa = -1.01 * np.min(dx / (x - alfa))
            stmbeta = 1.01 * np.max(dx / (beta - x))
            steg = 1.0 / max(stmalfa, stmbeta, stmxx, 1.0)
            old = (x.copy(), y.copy(), z, lam.copy(), xsi.copy(), eta.copy(), mu.copy(), zet, s.copy())
            for _ in range(maxit):
                trials += 1
                x = old[0] + steg * dx
                y = old[1] + steg * dy
                z = old[2] + steg * dz
                lam = old[3] + steg * dlam
                xsi = old[4] + steg * dxsi
                eta = old[5] + steg * deta
                mu = old[6] + steg * dmu
                zet = old[7] + steg * dzet
                s = old[8] + steg * ds
                r2 = _residual(x, y, z, lam, xsi, eta, mu, zet, s, low, upp, alfa, beta, P0, Q0, P1, Q1, a0, a, b,
                               c, d, epsi)
                if r2.sum() < rnorm:
                    break
                steg /= 2
            rnorm, rmax = r2.sum(), r2.max()
        epsi /= 10
    if stats is not None:
        stats.update(outer=outer, newton=newton, trials=trials)
    return x
