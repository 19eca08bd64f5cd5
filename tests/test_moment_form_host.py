"""The moment form of the angular Chebyshev terms, checked on the host.

The FP32 descriptor and adjoint kernels (aenet_gb300/csrc/k_cheb_mom.cuh)
evaluate the reference's angular pair sum (sfb_angular,
src/ext/sfbasis.f90:797-858)

    G_n = sum_{a<b} w_a w_b T_n(x(u_a . u_b))

as power spectra of per-atom harmonic moments.  This module restates the
kernels' arithmetic in numpy -- the Legendre table of capi.cpp
(legendre_table), the harmonic recurrences with the same constants and
component order, the closed-form gradient of the adjoint -- and checks it
against the pair sum itself: values to FP64 rounding in both angular
domains and for every instantiated order, gradients against central
differences, and the FP32 error the mixed path inherits.
"""
import math

import numpy as np
import pytest

SFB_PI = 3.14159265358979


def legendre_table(a_N, legacy, D=7):
    """q[n][l] with T_n(x(c)) = sum_l q[n][l] P_l(c): monomial coefficients
    of both families, peeled from the top degree (capi.cpp)."""
    al, be = (2.0 / SFB_PI, -1.0) if legacy else (1.0, 0.0)
    Tn = np.zeros((D, D))
    Pl = np.zeros((D, D))
    Tn[0, 0] = 1.0
    Tn[1, 0], Tn[1, 1] = be, al
    for k in range(1, D - 1):
        Tn[k + 1] = 2.0 * be * Tn[k] - Tn[k - 1]
        Tn[k + 1, 1:] += 2.0 * al * Tn[k, :-1]
    Pl[0, 0] = 1.0
    Pl[1, 1] = 1.0
    for k in range(1, D - 1):
        Pl[k + 1] = -k * Pl[k - 1]
        Pl[k + 1, 1:] += (2.0 * k + 1.0) * Pl[k, :-1]
        Pl[k + 1] /= k + 1.0
    q = np.zeros((D, D))
    for n in range(a_N):
        rem = Tn[n].copy()
        for l in range(n, -1, -1):
            c = rem[l] / Pl[l, l]
            q[n, l] = c
            rem[: l + 1] -= c * Pl[l, : l + 1]
    return q


def mom_consts(D=7):
    qmm = [1.0 if m == 0 else math.sqrt(2.0 / math.factorial(2 * m)) * _dfact(2 * m - 1)
           for m in range(D)]
    a1 = [math.sqrt(2.0 * m + 1.0) for m in range(D)]
    a = np.zeros((D, D))
    b = np.zeros((D, D))
    kap = np.zeros((D, D))
    for m in range(D):
        for l in range(m, D):
            if l >= m + 2:
                a[l, m] = (2.0 * l - 1.0) / math.sqrt((l - m) * (l + m))
                b[l, m] = math.sqrt((l + m - 1) * (l - m - 1) / ((l - m) * (l + m)))
            kap[l, m] = math.sqrt(0.5 * l * (l + 1)) if m == 0 else math.sqrt((l - m) * (l + m + 1))
    return qmm, a1, a, b, kap


def _dfact(n):
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


C = mom_consts()


def harmonics(u, L, dt=np.float64):
    """Y[k] for the kernel's l-major component order."""
    qmm, a1, a, b, _ = C
    x, y, z = (dt(v) for v in u)
    Y = np.zeros((L + 1) ** 2, dtype=dt)
    cm, sm = dt(1), dt(0)
    for m in range(L + 1):
        if m > 0:
            cm, sm = x * cm - y * sm, x * sm + y * cm
        q1 = q2 = dt(0)
        for l in range(m, L + 1):
            if l == m:
                q = dt(qmm[m])
            elif l == m + 1:
                q = dt(a1[m]) * z * q1
            else:
                q = dt(a[l, m]) * z * q1 - dt(b[l, m]) * q2
            q2, q1 = q1, q
            if m == 0:
                Y[l * l] = q
            else:
                k = l * l + 2 * m - 1
                Y[k], Y[k + 1] = q * cm, q * sm
    return Y


def gradient(u, s, D0, D1, L):
    """F = sum C_k Y_k(u), C = D0 + s D1, and the gradient of its
    polynomial extension (the adjoint's closed form)."""
    qmm, a1, a, b, kap = C
    x, y, z = u
    cp, sp = [1.0], [0.0]
    for m in range(1, L + 1):
        cp.append(x * cp[m - 1] - y * sp[m - 1])
        sp.append(x * sp[m - 1] + y * cp[m - 1])
    Ep = [0.0] * (L + 1)
    F = px = py = pz = 0.0
    for m in range(L + 1):
        gam = dl = q1 = q2 = 0.0
        for l in range(m, L + 1):
            if l == m:
                q = qmm[m]
            elif l == m + 1:
                q = a1[m] * z * q1
            else:
                q = a[l, m] * z * q1 - b[l, m] * q2
            q2, q1 = q1, q
            if m == 0:
                Cv = D0[l * l] + s * D1[l * l]
                F += Cv * q
                Ep[l] = kap[l, 0] * Cv
            else:
                k = l * l + 2 * m - 1
                Cc, Cs = D0[k] + s * D1[k], D0[k + 1] + s * D1[k + 1]
                gam += q * Cc
                dl += q * Cs
                pz += Ep[l] * q
                if l > m:
                    Ep[l] = kap[l, m] * (Cc * cp[m] + Cs * sp[m])
        if m > 0:
            F += gam * cp[m] + dl * sp[m]
            px += m * (gam * cp[m - 1] + dl * sp[m - 1])
            py += m * (dl * cp[m - 1] - gam * sp[m - 1])
    return F, np.array([px, py, pz])


def cheb(x, A):
    T = [1.0, x]
    for _ in range(2, A):
        T.append(2.0 * x * T[-1] - T[-2])
    return np.array(T[:A])


def fc(d, rc):
    return 0.5 * (np.cos(SFB_PI / rc * d) + 1.0)


def dfc(d, rc):
    return -0.5 * (SFB_PI / rc) * np.sin(SFB_PI / rc * d)


def pair_sum(R, spin, A, legacy, rc):
    """The reference's angular block: plain and spin-weighted."""
    d = np.linalg.norm(R, axis=1)
    u = R / d[:, None]
    w = fc(d, rc)
    G0, G1 = np.zeros(A), np.zeros(A)
    for p in range(len(d)):
        for k in range(p + 1, len(d)):
            c = float(u[p] @ u[k])
            x = (2.0 * c - SFB_PI) / SFB_PI if legacy else c
            t = cheb(x, A) * w[p] * w[k]
            G0 += t
            G1 += spin[p] * spin[k] * t
    return G0, G1


def moment_form(R, spin, A, legacy, rc, dt=np.float64):
    L = A - 1
    q = legendre_table(A, legacy)[:A, :A].astype(dt)
    d = np.sqrt((R.astype(dt) ** 2).sum(1))
    u = R.astype(dt) / d[:, None]
    w = fc(d, dt(rc)).astype(dt)
    M0 = np.zeros(A * A, dtype=dt)
    M1 = np.zeros(A * A, dtype=dt)
    for p in range(len(d)):
        Y = harmonics(u[p], L, dt)
        M0 += w[p] * Y
        M1 += (w[p] * dt(spin[p])) * Y
    W0 = (w * w).sum(dtype=dt)
    W1 = ((w * spin.astype(dt)) ** 2).sum(dtype=dt)
    p0 = np.array([(M0[l * l:(l + 1) ** 2] ** 2).sum(dtype=dt) for l in range(A)], dtype=dt)
    p1 = np.array([(M1[l * l:(l + 1) ** 2] ** 2).sum(dtype=dt) for l in range(A)], dtype=dt)
    t1 = q.sum(1)
    return dt(0.5) * (q @ p0 - t1 * W0), dt(0.5) * (q @ p1 - t1 * W1), M0, M1


def environment(seed, n=24, rc=4.0):
    rng = np.random.default_rng(seed)
    R = rng.normal(size=(n, 3))
    R *= (rng.uniform(0.9, rc * 0.999, n) / np.linalg.norm(R, axis=1))[:, None]
    spin = rng.choice([-1.0, 0.0, 1.0], n)
    return R, spin


@pytest.mark.parametrize("legacy", [False, True])
def test_legendre_table_reproduces_the_angular_basis(legacy):
    c = np.linspace(-1.0, 1.0, 41)
    for A in range(1, 8):
        q = legendre_table(A, legacy)
        x = (2.0 * c - SFB_PI) / SFB_PI if legacy else c
        for n in range(A):
            lhs = np.array([cheb(v, n + 1)[n] for v in x])
            rhs = sum(q[n, l] * np.polynomial.legendre.Legendre.basis(l)(c) for l in range(n + 1))
            np.testing.assert_allclose(rhs, lhs, rtol=0, atol=1e-12 * max(1.0, np.abs(lhs).max()))


def test_addition_theorem_of_the_harmonics():
    rng = np.random.default_rng(5)
    for _ in range(20):
        u, v = rng.normal(size=(2, 3))
        u /= np.linalg.norm(u)
        v /= np.linalg.norm(v)
        Yu, Yv = harmonics(u, 6), harmonics(v, 6)
        for l in range(7):
            sl = slice(l * l, (l + 1) ** 2)
            Pl = np.polynomial.legendre.Legendre.basis(l)(u @ v)
            assert abs(Yu[sl] @ Yv[sl] - Pl) < 1e-13


@pytest.mark.parametrize("legacy", [False, True])
@pytest.mark.parametrize("A", [1, 3, 5, 7])
def test_moment_form_equals_the_pair_sum(legacy, A):
    for seed in range(3):
        R, spin = environment(seed)
        G0, G1 = pair_sum(R, spin, A, legacy, 4.0)
        H0, H1, _, _ = moment_form(R, spin, A, legacy, 4.0)
        scale = max(1.0, np.abs(G0).max())
        assert np.abs(H0 - G0).max() < 1e-12 * scale
        assert np.abs(H1 - G1).max() < 1e-12 * scale


@pytest.mark.parametrize("legacy", [False, True])
def test_moment_form_in_fp32(legacy):
    """What the mixed path inherits: FP32 moments against FP64 pair sums."""
    for seed in range(3):
        R, spin = environment(seed, n=30)
        G0, G1 = pair_sum(R, spin, 5, legacy, 4.0)
        H0, H1, _, _ = moment_form(R, spin, 5, legacy, 4.0, dt=np.float32)
        scale = max(1.0, np.abs(G0).max())
        assert np.abs(H0 - G0).max() < 2e-6 * scale
        assert np.abs(H1 - G1).max() < 2e-6 * scale


@pytest.mark.parametrize("legacy", [False, True])
def test_adjoint_gradient_matches_finite_differences(legacy):
    A, rc = 5, 4.0
    R, spin = environment(11, n=14)
    rng = np.random.default_rng(2)
    g0, g1 = rng.normal(size=A), rng.normal(size=A)

    def energy(Rx):
        G0, G1 = pair_sum(Rx, spin, A, legacy, rc)
        return g0 @ G0 + g1 @ G1

    q = legendre_table(A, legacy)[:A, :A]
    _, _, M0, M1 = moment_form(R, spin, A, legacy, rc)
    B0, B1 = g0 @ q, g1 @ q
    tau0, tau1 = B0.sum(), B1.sum()
    D0, D1 = np.zeros(A * A), np.zeros(A * A)
    for l in range(A):
        sl = slice(l * l, (l + 1) ** 2)
        D0[sl], D1[sl] = B0[l] * M0[sl], B1[l] * M1[sl]
    for p in range(len(R)):
        d = np.linalg.norm(R[p])
        u = R[p] / d
        F, grad = gradient(u, spin[p], D0, D1, A - 1)
        wd = fc(d, rc) / d
        cu = dfc(d, rc) * (F - (tau0 + tau1 * spin[p] ** 2) * fc(d, rc)) - wd * (u @ grad)
        g = cu * u + wd * grad
        fd = np.zeros(3)
        for c in range(3):
            h = 1e-6
            Rp, Rm = R.copy(), R.copy()
            Rp[p, c] += h
            Rm[p, c] -= h
            fd[c] = (energy(Rp) - energy(Rm)) / (2 * h)
        np.testing.assert_allclose(g, fd, rtol=0, atol=2e-7 * max(1.0, np.abs(fd).max()))
