"""Host-side site models: the inputs of the NRG iteration.

These are tiny (4-16 state) Hilbert spaces built once per run on the host,
restating the reference's model builders:

* ``fermion_basis``  - models/fermionBasis.hpp:49-82, 122-140, 230-317, 397-419
* ``spinhalf``       - models/spinhalf.hpp:81-124
* ``spinhalf_kondo`` - models/spinhalfKondo.hpp:28-166
* ``two_channel``    - src/models/twoChannel.cpp:12-45
* ``spinhalf_sc``, ``sc_bath`` - models/spinhalfSC.hpp:26-125 (S_z-only sectors,
  pairing bath refreshed per site)
* ``d_dag_chi``      - the d-dagger-chi operators of examples/fdmSpectrumSiam/main.cpp:40-60

A :class:`Site` carries exactly what ``nrgcore`` reads from a model
(nrgcore.hpp:44-53, 68-70): the sector quantum numbers (``get_basis``), the
eigenvalues per sector (``get_eigenvaluesQ``), the fermion parity per sector
(``get_chi_Q``) and the block-sparse creation operators (``f_dag_operator``).
"""
from dataclasses import dataclass, field
from typing import Dict, List, Tuple

import numpy as np

CHARGE_ONLY, SPIN_ONLY, CHARGE_AND_SPIN = 0, 1, 2


@dataclass
class Site:
    qnums: List[Tuple[int, ...]]
    energies: List[np.ndarray]
    chi: np.ndarray
    fdag: List[Dict[Tuple[int, int], np.ndarray]]
    extra: Dict[str, object] = field(default_factory=dict)

    @property
    def dims(self):
        return [len(e) for e in self.energies]

    def with_ops(self, fdag):
        """Same site with a different creation-operator list (e.g. duplicated)."""
        return Site(self.qnums, self.energies, self.chi, list(fdag), dict(self.extra))


def _jordan_wigner(dof):
    """f-dagger of each orbital: I^(dof-1-i) (x) [[0,0],[1,0]] (x) sz^i
    (fermionBasis.hpp:397-419; qmatrix::krDot is the standard Kronecker product)."""
    fdag = np.array([[0.0, 0.0], [1.0, 0.0]])
    sz = np.array([[1.0, 0.0], [0.0, -1.0]])
    ops = []
    for i in range(dof):
        prev = np.ones((1, 1))
        for _ in range(dof - i - 1):
            prev = np.kron(np.eye(2), prev)
        nxt = np.ones((1, 1))
        for _ in range(i):
            nxt = np.kron(sz, nxt)
        ops.append(np.kron(prev, np.kron(fdag, nxt)))
    return ops


class FermionBasis:
    """Occupation basis, quantum numbers and block structure of ``dof`` orbitals."""

    def __init__(self, dof, symmetry=CHARGE_AND_SPIN, occupations=None):
        self.raw_fdag = _jordan_wigner(dof)
        if occupations is None:
            occupations = [np.diag(f @ f.T).copy() for f in self.raw_fdag]
        self.occ = occupations
        nstates = len(occupations[0])
        if symmetry == CHARGE_ONLY:
            q = [(int(sum(o[s] for o in occupations)),) for s in range(nstates)]
        elif symmetry == SPIN_ONLY:
            q = [(int(sum(occupations[j][s] for j in range(len(occupations)) if j % 2 == 0)
                      - sum(occupations[j][s] for j in range(len(occupations)) if j % 2 == 1)),)
                 for s in range(nstates)]
        else:
            q = [(int(sum(occupations[j][s] for j in range(len(occupations)) if j % 2 == 0)),
                  int(sum(occupations[j][s] for j in range(len(occupations)) if j % 2 == 1)))
                 for s in range(nstates)]
        self.state_q = q
        # blocks in order of first appearance, members ascending
        # (fermionBasis.hpp:230-268)
        self.qnums, self.blocks = [], []
        seen = {}
        for s, qs in enumerate(q):
            if qs not in seen:
                seen[qs] = len(self.qnums)
                self.qnums.append(qs)
                self.blocks.append([])
            self.blocks[seen[qs]].append(s)

    def block_operators(self, mats):
        """Split full-space operators into sector blocks, keeping only blocks
        with a nonzero entry (fermionBasis.hpp:291-318)."""
        out = []
        for m in mats:
            d = {}
            for i, bi in enumerate(self.blocks):
                for j, bj in enumerate(self.blocks):
                    sub = m[np.ix_(bi, bj)]
                    if np.abs(sub).sum() > 0:
                        d[(i, j)] = sub.copy()
            out.append(d)
        return out

    def block_diag(self, h):
        if np.abs(h - h.T).sum() > 1e-10:
            raise ValueError("Hamiltonian is not Hermitian")
        return [h[np.ix_(b, b)].copy() for b in self.blocks]


def _chi(qnums):
    return np.array([(-1.0) ** sum(q) for q in qnums])


def spinhalf(eps, U, h=0.0):
    """Spin-1/2 Anderson impurity / Wilson site (spinhalf.hpp:81-124).
    The f-dagger blocks are left in the occupation basis, exactly as the
    reference does (all four sectors are one-dimensional)."""
    fb = FermionBasis(2, CHARGE_AND_SPIN)
    fu, fd = fb.raw_fdag
    nu, nd = fu @ fu.T, fd @ fd.T
    H = (nu + nd) * eps + (nu - nd) * h + (nu @ nd) * U
    energies = [np.linalg.eigvalsh(b) for b in fb.block_diag(H)]
    return Site(list(fb.qnums), energies, _chi(fb.qnums), fb.block_operators(fb.raw_fdag),
                {"basis": fb})


def spinhalf_kondo(J, S=0.5):
    """Kondo impurity already coupled to Wilson site 0 (spinhalfKondo.hpp:28-166);
    f-dagger is rotated into the eigenbasis of each sector."""
    sd = int(round(2 * S + 1))
    Sz = np.zeros((sd, sd))
    Sp = np.zeros((sd, sd))
    for i in range(sd):
        m = -S + i
        Sz[i, i] = m
        if i != sd - 1:
            Sp[i, i + 1] = np.sqrt(S * (S + 1.0) - m * (m + 1))
    Sm = Sp.T
    Sx = (Sp + Sm) * 0.5
    Sy = (Sp - Sm) * 0.5
    fb = FermionBasis(2, CHARGE_AND_SPIN)
    cu, cd = fb.raw_fdag
    wx = (cu @ cd.T + cd @ cu.T) * 0.5
    wy = (cd @ cu.T - cu @ cd.T) * 0.5
    wz = (cu @ cu.T - cd @ cd.T) * 0.5
    wn = cu @ cu.T + cd @ cd.T
    H = (np.kron(Sz, wz) + np.kron(Sx, wx) - np.kron(Sy, wy)) * J
    I4, I2 = np.eye(4), np.eye(sd)
    spinSz = np.kron(Sz, I4)
    wz2, wn2 = np.kron(I2, wz), np.kron(I2, wn)
    cu2, cd2 = np.kron(I2, cu), np.kron(I2, cd)
    n = spinSz.shape[0]
    occ = [np.diag((np.eye(n) + spinSz * 2.0) * 0.5).copy(),
           np.diag((np.eye(n) - spinSz * 2.0) * 0.5).copy(),
           np.diag((wn2 + wz2 * 2.0) * 0.5).copy(),
           np.diag((wn2 - wz2 * 2.0) * 0.5).copy()]
    # block structure from the four pseudo-occupations (spinhalfKondo.hpp:104-124)
    q = [(int(occ[0][s] + occ[2][s]), int(occ[1][s] + occ[3][s])) for s in range(n)]
    qnums, blocks, seen = [], [], {}
    for s, qs in enumerate(q):
        if qs not in seen:
            seen[qs] = len(qnums)
            qnums.append(qs)
            blocks.append([])
        blocks[seen[qs]].append(s)
    energies, vecs = [], []
    for b in blocks:
        hb = H[np.ix_(b, b)]
        w, v = np.linalg.eigh(hb)
        energies.append(w)
        vecs.append(v)
    fdag = []
    for m in (cu2, cd2):
        d = {}
        for i, bi in enumerate(blocks):
            for j, bj in enumerate(blocks):
                sub = m[np.ix_(bi, bj)]
                if np.abs(sub).sum() > 0:
                    d[(i, j)] = vecs[i].T @ sub @ vecs[j]
        fdag.append(d)
    return Site(qnums, energies, _chi(qnums), fdag)


def _rotated_site(fb, H):
    """Sector eigenvalues of H and the f-dagger blocks rotated into the
    sector eigenbases, U_i^T f U_j (spinhalfSC.hpp:57-84)."""
    energies, vecs = [], []
    for b in fb.block_diag(H):
        w, v = np.linalg.eigh(b)
        energies.append(w)
        vecs.append(v)
    fdag = []
    for d in fb.block_operators(fb.raw_fdag):
        fdag.append({(i, j): vecs[i].T @ m @ vecs[j] for (i, j), m in d.items()})
    return Site(list(fb.qnums), energies, _chi(fb.qnums), fdag, {"basis": fb})


def spinhalf_sc(eps, U, h=0.0):
    """Spin-1/2 site with S_z as its only quantum number, for baths with a
    pairing term (models/spinhalfSC.hpp:26-85): H = eps n + h (n_up - n_down)
    + U n_up n_down, sectors S_z = 0, +1, -1, f-dagger in the sector
    eigenbasis."""
    fb = FermionBasis(2, SPIN_ONLY)
    fu, fd = fb.raw_fdag
    nu, nd = fu @ fu.T, fd @ fd.T
    return _rotated_site(fb, (nu + nd) * eps + (nu - nd) * h + (nu @ nd) * U)


def sc_bath(delta):
    """spinhalfSC::addSCDelta (spinhalfSC.hpp:87-125): the site Hamiltonian
    replaced by the s-wave pairing delta (c_up c_down + c_down^+ c_up^+);
    a Wilson site of a superconducting bath, refreshed every site
    (nrgcore.hpp:68-70)."""
    fb = FermionBasis(2, SPIN_ONLY)
    fu, fd = fb.raw_fdag
    return _rotated_site(fb, (fu.T @ fd.T + fd @ fu) * delta)


def two_channel():
    """Two-channel Wilson site: 4 orbitals, (N_up, N_down) sectors, zero
    on-site energy (src/models/twoChannel.cpp:12-45)."""
    fb = FermionBasis(4, CHARGE_AND_SPIN)
    H = np.zeros((16, 16))
    energies = [np.linalg.eigvalsh(b) for b in fb.block_diag(H)]
    return Site(list(fb.qnums), energies, _chi(fb.qnums), fb.block_operators(fb.raw_fdag),
                {"basis": fb})


def duplicate_ops(site, times=2):
    """Impurity f-dagger list repeated for a multi-channel bath
    (examples/twoChannelSiam/main.cpp:24-25)."""
    return site.with_ops(list(site.fdag) * times)


def d_dag_chi():
    """d_sigma-dagger times the impurity parity chi = (-1)^N in the spinhalf
    sector basis (examples/fdmSpectrumSiam/main.cpp:40-60)."""
    fb = FermionBasis(2, CHARGE_AND_SPIN)
    f = fb.raw_fdag
    nt = sum(x @ x.T for x in f)
    chi = np.diag([(-1.0) ** nt[i, i] for i in range(nt.shape[0])])
    return fb.block_operators([x @ chi for x in f])


def n_d():
    """Impurity occupancy n_d = sum_sigma d_sigma-dagger d_sigma in the
    spinhalf sector basis (block diagonal), built as the reference's
    fermionBasis::get_block_operators of the raw occupancy matrix
    (models/fermionBasis.hpp:292-330)."""
    fb = FermionBasis(2, CHARGE_AND_SPIN)
    f = fb.raw_fdag
    return fb.block_operators([sum(x @ x.T for x in f)])


def hopping(site, lam):
    """Wilson-chain hopping t_n (examples/rgflowSIAM/main.cpp:5-10)."""
    return (0.5 * (1.0 + 1.0 / lam) * (1.0 - lam ** (-site - 1))
            / np.sqrt((1.0 - lam ** (-2.0 * site - 1)) * (1.0 - lam ** (-2.0 * site - 3))))
