"""Parity criteria shared by the CPU (oracle vs reference) and GPU (engine vs
oracle) tests.

FP64 round-off is amplified by the RG flow: a perturbation introduced at site
m grows like Lambda^((N-m)/2) by site N (relevant directions scale with
Lambda^(1/2) per site in iteration units).  Two FP64 LAPACK runs of the
reference differ by 1.9e-10 at site 39 of the Nkeep=512 SIAM flow (1 vs 8
threads), and the numpy restatement differs from the reference by 3e-9
there.  The eigenvalue tolerance is therefore
    tol(N) = max(1e-10, 1e-14 * Lambda^(N/2))
absolute, in the iteration's own (rescaled) energy units: 1e-10 up to the
point where the reference's own FP64 noise floor exceeds it.
"""
import numpy as np


def eig_tol(N, lam, floor=1e-10, eps=1e-14):
    return max(floor, eps * lam ** (N / 2.0))


def clusters(E, tol=1e-9):
    """Group sorted indices of E into runs of (near-)equal values."""
    order = np.argsort(E, kind="stable")
    out, cur = [], [order[0]] if len(order) else []
    for a, b in zip(order[:-1], order[1:]):
        if abs(E[b] - E[a]) <= tol * max(1.0, abs(E[a])):
            cur.append(b)
        else:
            out.append(cur)
            cur = [b]
    if cur:
        out.append(cur)
    return out


def degenerate_weights(F, Ei, Ej, tol=1e-9):
    """Basis-invariant content of an operator block: sum of |<a|O|b>|^2 over
    each pair of degenerate multiplets (rows of Ei x columns of Ej), keyed by
    the multiplets' energies."""
    ci, cj = clusters(np.asarray(Ei), tol), clusters(np.asarray(Ej), tol)
    W = np.zeros((len(ci), len(cj)))
    F2 = np.asarray(F) ** 2
    for a, ra in enumerate(ci):
        for b, rb in enumerate(cj):
            W[a, b] = F2[np.ix_(ra, rb)].sum()
    return W
