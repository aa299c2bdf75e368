"""Wilson-chain coefficients for z-averaged and arbitrary-DOS baths: the
host-side input generator of independFiles/zAverage (Campo and Oliveira,
Phys. Rev. B 72, 104432 (2005)).  It only feeds the hoppings t_n (and the
site energies) of add_bath_site; nothing here runs on the GPU.

Both generators run the Lanczos tridiagonalisation of the discretised
conduction band from the impurity-coupled state f_0, in multiple precision
(mpmath), as the reference does with MPFR (1000 digits there):

* flat_band_tn (hoppingElement.cpp:8-106): the flat band, z-shifted
  logarithmic mesh with 2 x (hcmax + 1) levels; returns t_n Lambda^(n/2).
* dos_tn (zAverage.hpp:11-195): an arbitrary density of states rho(e) on
  [-D, D]; each interval I_j of the z-shifted mesh becomes one level
  E_j = int rho / int rho/e (trapezoid rule, 100 points, as quadrature.hpp
  trapiziodal) with weight int rho; returns (t_n Lambda^(n/2), e_n Lambda^(n/2)).

The Lanczos vectors are not re-orthogonalised (the reference relies on its
precision); `digits` sets the working precision here.
"""
import mpmath


def _onsite(lam, z, i):
    """Level i of the flat-band mesh (hoppingElement.cpp:8-14)."""
    k = abs(i)
    if k == 0:
        return (1 - mpmath.power(lam, -z)) / (z * mpmath.log(lam))
    return (1 - 1 / lam) * mpmath.power(lam, 1 - k - z) / mpmath.log(lam)


def flat_band_tn(z, lam, nmax=80, hcmax=10, digits=1000):
    """t_n Lambda^(n/2), n = 0 .. nmax, of the flat band at shift z
    (hoppingElement.cpp calcTn).  Only the first 2 hcmax + 1 values are
    meaningful: the mesh has 2 (hcmax + 1) levels, and the recurrence runs
    past the Krylov space as the reference's does."""
    with mpmath.workdps(digits):
        lam, z = mpmath.mpf(lam), mpmath.mpf(z)
        h = [-_onsite(lam, z, i) for i in range(hcmax + 1)] + [_onsite(lam, z, i) for i in range(hcmax, -1, -1)]
        w0 = mpmath.sqrt(0.5 * (1 - mpmath.power(lam, -z)))
        v0 = [w0] + [mpmath.sqrt(0.5 * (1 - 1 / lam) * mpmath.power(lam, 1 - i - z)) for i in range(1, hcmax + 1)]
        v0 += [mpmath.sqrt(0.5 * (1 - 1 / lam) * mpmath.power(lam, 1 - i - z)) for i in range(hcmax, 0, -1)] + [w0]
        a = mpmath.fsum(hi * x * x for hi, x in zip(h, v0))
        v1 = [x * (hi - a) for hi, x in zip(h, v0)]
        nrm = mpmath.sqrt(mpmath.fsum(x * x for x in v1))
        v1 = [x / nrm for x in v1]
        tn = [nrm]
        prev, cur = v0, v1
        for _ in range(nmax):
            a1 = mpmath.fsum(hi * x * x for hi, x in zip(h, cur))
            a2 = mpmath.fsum(hi * x * y for hi, x, y in zip(h, cur, prev))
            nxt = [x * (hi - a1) - a2 * y for hi, x, y in zip(h, cur, prev)]
            nrm = mpmath.sqrt(mpmath.fsum(x * x for x in nxt))
            nxt = [x / nrm for x in nxt]
            tn.append(nrm)
            prev, cur = cur, nxt
        return [float(t * mpmath.power(lam, 0.5 * i)) for i, t in enumerate(tn)]


def _trapezoid(f, lo, hi, n=100):
    """quadrature.hpp trapiziodal: n left-point samples times the step."""
    dx = (hi - lo) / n
    return dx * mpmath.fsum(f(lo + i * dx) for i in range(n))


def dos_tn(dos, z=1.0, lam=3.0, nitr=80, bandwidth=1.0, energy_points=60, digits=1000):
    """(t_n Lambda^(n/2), e_n Lambda^(n/2)) of a bath with density of states
    `dos` (a function of an mpmath number, zero outside [-D, D]) on the
    z-shifted logarithmic mesh +-D Lambda^(2 - i - z), i = 2 .. energy_points - 1
    (zAverage.hpp: setlogmess, setFirstVector, setNextVector, solve).  The
    reference's mesh has 10000 points; for 80 sites the intervals past the
    first few dozen no longer change a double (60 points reproduce the
    reference's pseudogap coefficients to 1e-16).  The precision may not be
    lowered much: the unorthogonalised recursion at 200 digits already
    departs from the reference after 40 sites."""
    with mpmath.workdps(digits):
        lam, z, D = mpmath.mpf(lam), mpmath.mpf(z), mpmath.mpf(bandwidth)
        mesh = {1: D, -1: -D}
        for i in range(2, energy_points):
            mesh[i] = D * mpmath.power(lam, 2 - i - z)
            mesh[-i] = -D * mpmath.power(lam, 2 - i - z)
        by_x = lambda x: dos(x) / x  # noqa: E731
        h, v0 = [], []
        for i in range(-energy_points + 1, -1):  # negative energies, innermost first
            lo, hi = mesh[i], mesh[i + 1]
            num = _trapezoid(dos, lo, hi)
            h.append(num / _trapezoid(by_x, lo, hi))
            v0.append(mpmath.sqrt(abs(num)))
        for i in range(1, energy_points - 1):  # positive energies, outermost first
            lo, hi = mesh[i + 1], mesh[i]
            num = _trapezoid(dos, lo, hi)
            h.append(num / _trapezoid(by_x, lo, hi))
            v0.append(mpmath.sqrt(abs(num)))
        nrm = mpmath.sqrt(mpmath.fsum(x * x for x in v0))
        v0 = [x / nrm for x in v0]
        en, tn = [], []
        a = mpmath.fsum(hi * x * x for hi, x in zip(h, v0))
        en.append(a)
        cur = [hi * x - a * x for hi, x in zip(h, v0)]
        nrm = mpmath.sqrt(mpmath.fsum(x * x for x in cur))
        tn.append(nrm)
        cur = [x / nrm for x in cur]
        prev = v0
        for _ in range(nitr):
            a = mpmath.fsum(hi * x * x for hi, x in zip(h, cur))
            a2 = mpmath.fsum(hi * x * y for hi, x, y in zip(h, cur, prev))
            en.append(a)
            nxt = [hi * x - a * x - a2 * y for hi, x, y in zip(h, cur, prev)]
            nrm = mpmath.sqrt(mpmath.fsum(x * x for x in nxt))
            tn.append(nrm)
            prev, cur = cur, [x / nrm for x in nxt]
        sc = [mpmath.power(lam, 0.5 * i) for i in range(len(tn))]
        return [float(t * s) for t, s in zip(tn, sc)], [float(e * s) for e, s in zip(en, sc)]


def pseudogap_dos(r):
    """|e|^r on |e| < 1 (independFiles/zAverage/pseudogap.cpp:15-21)."""
    def f(x):
        return mpmath.power(abs(x), r) if abs(x) < 1 else mpmath.mpf(0)
    return f
