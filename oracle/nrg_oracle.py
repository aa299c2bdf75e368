"""CPU oracle: numpy restatement of the reference's NRG hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only to check
the engine's results (or as the timed CPU baseline); the product path never
calls it.

Parity is pinned two ways: against the golden vectors the reference shipped
(examples/entropyKondo/resultsJ0.250000.h5 and resultsZero.h5: per-iteration
eigenvalues, entropy, specific heat) and against outputs of the reference
itself compiled here (oracle/build_ref.sh), committed as fixtures under
tests/golden/.

Each function cites the reference lines it restates.  Arithmetic follows the
reference: FP64 throughout, LAPACK ``syevd`` (numpy.linalg.eigh) for the block
eigensolve, dense products for the rotations.  The only liberties taken are
ones that cannot change any published value: empty coupling terms are skipped
and the sparse f-dagger embedding T (nrgcore.hpp:446-465) is applied as row
slices instead of a dense matrix product.
"""
import math

import numpy as np

ERRORBAR_IN_ENERGY = 1e-8          # nrgcore.hpp:338
FDM_ENERGY_PTS = 100000            # fdmSpectrum.hpp:351
FDM_MAX_ENERGY = 10.0              # fdmSpectrum.hpp:352
FDM_MIN_ENERGY = 1e-10             # fdmSpectrum.hpp:353
FDM_DELE = (FDM_ENERGY_PTS - 1.0) / math.log(FDM_MAX_ENERGY / FDM_MIN_ENERGY)  # :354
FDM_ENERGY_ERRORBAR = 1e-5         # fdmSpectrum.hpp:363
FDM_WEIGHT_ERRORBAR = 1e-20        # fdmSpectrum.hpp:343


class NrgOracle:
    """Restatement of ``nrgcore<Imp,Bath>`` (nrgcore/include/nrgcore/nrgcore.hpp)."""

    def __init__(self, impurity, bath, nkeep=1024):
        self.imp = impurity
        self.bath = bath
        if len(impurity.fdag) != len(bath.fdag):            # test() :117-134
            raise RuntimeError("f_dag_operator.size is different on model and impurity!")
        self.set_parameters(nkeep)
        self.all_eigenvalue = np.zeros(0)
        self.relativeGroundStateEnergy = []
        self.kept = []                 # sizes of eigenvaluesQ_kept_indices (prefixes)
        self.eigenvaluesQ = []
        self.pre_sysmQ = []
        self.current_sysmQ = []
        self.coupled = []              # coupled_nQ_index
        self.U = []                    # current_hamiltonQ (eigenvectors after diag)
        self.H = []                    # assembled Hamiltonians (kept for parity tests)
        self.pre_fdag = []

    def set_parameters(self, n=1024):                       # :336-342
        self.no_of_kept_states = n
        self.max_kept_states = n
        self.nrg_iterations_cnt = 0
        self.nrg_iterations_min = 0

    # -- a1 --------------------------------------------------------------
    def create_next_basis(self):                             # :238-261
        nb = len(self.bath.qnums)
        self.current_sysmQ, self.coupled = [], []
        where = {}
        for i, q in enumerate(self.pre_sysmQ):
            for j, qb in enumerate(self.bath.qnums):
                tm = tuple(a + b for a, b in zip(q, qb))
                if tm in where:
                    self.coupled[where[tm]].append(i * nb + j)
                else:
                    where[tm] = len(self.current_sysmQ)
                    self.current_sysmQ.append(tm)
                    self.coupled.append([i * nb + j])
        # per sector: list of (ii, bb, offset, k, d)
        self.sub = []
        self.sub_of = {}
        for s, lindex in enumerate(self.coupled):
            off, lst = 0, []
            for kidx in lindex:
                ii, bb = divmod(kidx, nb)
                k, d = self.kept[ii], len(self.bath.energies[bb])
                lst.append((ii, bb, off, k, d))
                self.sub_of[(ii, bb)] = (s, off)
                off += k * d
            self.sub.append(lst)

    # -- a2 --------------------------------------------------------------
    def create_next_hamiltonians(self, t, rescale):          # :146-230
        if len(t) != len(self.pre_fdag):
            raise RuntimeError("t_hopping %d =! pre_fdag_oparator %d" % (len(t), len(self.pre_fdag)))
        Eb, fb, chi = self.bath.energies, self.bath.fdag, self.bath.chi
        self.H = []
        for lst in self.sub:
            n = sum(k * d for (_, _, _, k, d) in lst)
            h = np.zeros((n, n))
            for (ii, bb, off, k, d) in lst:                  # diagonal :179-185
                for il in range(d):
                    idx = off + il * k + np.arange(k)
                    h[idx, idx] = self.eigenvaluesQ[ii][:k] * rescale + Eb[bb][il]
            for (ii, bb, off, k, d) in lst:                  # hopping :186-224
                for (iip, bbp, offp, kp, dp) in lst:
                    for ip in range(len(self.pre_fdag)):
                        F = self.pre_fdag[ip].get((ii, iip))
                        B = fb[ip].get((bbp, bb))
                        if F is None or B is None or k == 0 or kp == 0:
                            continue
                        aa = np.kron(B.T, F[:k, :kp]) * chi[bbp] * t[ip]
                        h[off:off + k * d, offp:offp + kp * dp] += aa
                        h[offp:offp + kp * dp, off:off + k * d] += aa.T
            self.H.append(h)

    # -- a3 --------------------------------------------------------------
    def diagonalise(self):                                   # :85-89, qmatrix.hpp:375-404
        self.eigenvaluesQ, self.U = [], []
        for h in self.H:
            if h.shape[0] == 0:
                self.eigenvaluesQ.append(np.zeros(0))
                self.U.append(np.zeros((0, 0)))
                continue
            w, v = np.linalg.eigh(h)
            self.eigenvaluesQ.append(w)
            self.U.append(v)

    # -- a4 --------------------------------------------------------------
    def set_current_fdag_operator(self, full=True):          # :401-477
        """f-dagger rotated into the new eigenbasis, U_i^T T_ij U_j.  With
        ``full`` the whole n_i x n_j block is formed (what the reference
        stores); otherwise only the kept-kept part the next site reads."""
        fb = self.bath.fdag
        new = []
        for ip in range(len(fb)):
            acc = {}
            for (bb, bbp), B in fb[ip].items():
                for ii, k in enumerate(self.kept):
                    if (ii, bb) not in self.sub_of or (ii, bbp) not in self.sub_of:
                        continue
                    i, off = self.sub_of[(ii, bb)]
                    j, offp = self.sub_of[(ii, bbp)]
                    if (i, j) not in acc:
                        acc[(i, j)] = np.zeros((self.U[i].shape[0], self.U[j].shape[0]))
                    if k == 0:
                        continue
                    Ui, Uj = self.U[i], self.U[j]
                    for il in range(B.shape[0]):
                        for ilp in range(B.shape[1]):
                            v = B[il, ilp]
                            if v == 0.0:
                                continue
                            ra = off + il * k
                            rb = offp + ilp * k
                            acc[(i, j)] += v * (Ui[ra:ra + k, :].T @ Uj[rb:rb + k, :])
            new.append(acc)
        self.pre_fdag = new

    # -- a5 --------------------------------------------------------------
    def discard_higher_energies(self):                       # :269-327
        allv = np.sort(np.concatenate([np.asarray(e, float) for e in self.eigenvaluesQ]))
        self.all_eigenvalue = allv
        en_min = allv[0]
        if allv.size <= self.max_kept_states:
            self.kept = [len(e) for e in self.eigenvaluesQ]
        else:
            thr = allv[self.max_kept_states]
            self.kept = [int(np.count_nonzero(np.asarray(e) < thr + ERRORBAR_IN_ENERGY))
                         for e in self.eigenvaluesQ]
        self.no_of_kept_states = sum(self.kept)
        if self.no_of_kept_states <= self.max_kept_states:
            self.nrg_iterations_min = self.nrg_iterations_cnt
        else:
            self.relativeGroundStateEnergy.append(en_min)
            self.eigenvaluesQ = [np.asarray(e) - en_min for e in self.eigenvaluesQ]

    # -- public API --------------------------------------------------------
    def add_bath_site(self, t, rescale, full_fdag=True):     # :65-97
        if self.nrg_iterations_cnt == 0:
            self.eigenvaluesQ = [np.array(e, float) for e in self.imp.energies]
            self.pre_sysmQ = [tuple(q) for q in self.imp.qnums]
            self.pre_fdag = [dict(d) for d in self.imp.fdag]
            self.discard_higher_energies()
        self.create_next_basis()
        self.create_next_hamiltonians(list(t), rescale)
        self.diagonalise()
        self.set_current_fdag_operator(full=full_fdag)

    def update_internal_state(self):                         # :105-109
        self.nrg_iterations_cnt += 1
        self.prev_kept = list(self.kept)
        self.discard_higher_energies()
        self.pre_sysmQ = self.current_sysmQ

    def checkHigherEnergyDiscarded(self):                    # :384-386
        return self.no_of_kept_states >= self.max_kept_states

    # -- a6 --------------------------------------------------------------
    def update_system_operator(self, ops):                   # sysOperator.hpp:36-133
        """Rotate user operators (given in the previous basis) into the current
        eigenbasis: (O_prev (x) 1_bath) embedded, then U_i^T c U_j."""
        new = []
        for op in ops:
            acc = {}
            for (ii, iip), O in op.items():
                k, kp = self.kept[ii], self.kept[iip]
                for bb in range(len(self.bath.qnums)):
                    if (ii, bb) not in self.sub_of or (iip, bb) not in self.sub_of:
                        continue
                    i, off = self.sub_of[(ii, bb)]
                    j, offp = self.sub_of[(iip, bb)]
                    if (i, j) not in acc:
                        acc[(i, j)] = np.zeros((self.U[i].shape[0], self.U[j].shape[0]))
                    if k == 0 or kp == 0:
                        continue
                    Ui, Uj = self.U[i], self.U[j]
                    Ok = O[:k, :kp]
                    for il in range(len(self.bath.energies[bb])):
                        ra, rb = off + il * k, offp + il * kp
                        acc[(i, j)] += Ui[ra:ra + k, :].T @ (Ok @ Uj[rb:rb + kp, :])
            new.append(acc)
        return new

    def snapshot(self, ops=None):
        """In-memory stand-in for NrgData::saveCurrentData/saveqOperator
        (nrgData.hpp:134-205): the public members the backward pass reloads."""
        return {
            "U": self.U, "eigenvaluesQ": [np.array(e) for e in self.eigenvaluesQ],
            "kept": list(self.kept), "current_sysmQ": list(self.current_sysmQ),
            "pre_sysmQ": list(self.pre_sysmQ), "coupled": [list(c) for c in self.coupled],
            "sub": self.sub, "ops": ops,
        }


class FdmSpectrumOracle:
    """Restatement of fdmSpectrum (dynamics/fdmSpectrum.hpp): T = 0 as the
    reference runs it, or at a finite temperature when `shell_weights` is
    given -- per calc_spectrum call (backward order) the Boltzmann weights of
    that shell's discarded states in FdmThermoOracle.shell_weights layout,
    placed on the diagonal as fdmBackwardIteration::setRhoZero(tBoltzmannFactor)
    does (dynamics/fdmBackwardIteration.hpp:207-239).  `static` accumulates
    rhoDotStaticOperators (:166-199) over the shells: Tr(O_ii rho_i) with the
    kept x kept part of O zeroed, per operator."""

    def __init__(self, nops, shell_weights=None):
        self.last = True                                     # setup :44-48
        self.cur_kept = None
        self.prev_kept = None
        self.reduced = []
        self.pos = np.zeros((nops, FDM_ENERGY_PTS))          # setOperator :306-314
        self.neg = np.zeros((nops, FDM_ENERGY_PTS))
        self.shell_weights = shell_weights
        self.ncalc = 0
        self.static = np.zeros(nops)

    def calc_spectrum(self, snap, scale):                    # :55-63
        nsec = len(snap["current_sysmQ"])
        if self.cur_kept is None:                            # setCurrentIndex :289-298
            self.cur_kept = [0] * nsec
        else:
            self.cur_kept = self.prev_kept
        self.prev_kept = list(snap["kept"])
        E = snap["eigenvaluesQ"]
        rho = []                                             # setRhoZero :165-199
        if self.shell_weights is not None:                   # setRhoZero(tBoltzmannFactor)
            w, o = self.shell_weights[self.ncalc], 0
            for i in range(nsec):
                n, kc = len(E[i]), self.cur_kept[i]
                m = np.zeros((n, n))
                m[np.arange(kc, n), np.arange(kc, n)] = w[o:o + n - kc]
                o += n - kc
                if self.reduced and kc:
                    m[:kc, :kc] = self.reduced[i][:kc, :kc]
                rho.append(m)
        elif self.last:                                      # setLocalPartitionFunction :122-155
            egs = 0.0
            for e in E:
                if len(e):
                    egs = min(egs, float(np.min(e)))
            z = sum(int(np.count_nonzero(np.abs(e - egs) < FDM_ENERGY_ERRORBAR)) for e in E)
            self.boltz = [np.where(np.abs(e - egs) < FDM_ENERGY_ERRORBAR, 1.0 / z, 0.0) for e in E]
        for i in range(nsec if self.shell_weights is None else 0):
            n = len(E[i])
            m = np.zeros((n, n))
            if self.last:
                m[np.arange(n), np.arange(n)] = self.boltz[i]
            if self.reduced:
                kc = self.cur_kept[i]
                m[:kc, :kc] = self.reduced[i][:kc, :kc]
            rho.append(m)
        ops = snap["ops"]
        for ip, op in enumerate(ops):                        # rhoDotStaticOperators :166-199
            for (i, j), O in op.items():
                if i != j or O.size == 0:
                    continue
                O = O.copy()
                kc = self.cur_kept[i]
                O[:kc, :kc] = 0.0
                self.static[ip] += float(np.sum(O * rho[i].T))
        # rhoDotOperators :207-277
        for ip, op in enumerate(ops):
            for (i, j), B in op.items():
                if B.size == 0:
                    continue
                A = B.T.copy()
                A[:self.cur_kept[j], :self.cur_kept[i]] = 0.0
                rhoA = B @ rho[j]
                ARho = rho[i] @ B
                aa = rhoA * A.T
                bv = ARho * A.T
                de = np.abs(scale * (E[i][:, None] - E[j][None, :]))
                idx = (np.log(1.0 + de / FDM_MIN_ENERGY) * FDM_DELE).astype(np.int64)
                ok = (idx >= 0) & (idx < FDM_ENERGY_PTS)
                ma = ok & (np.abs(aa) > FDM_WEIGHT_ERRORBAR)
                mb = ok & (np.abs(bv) > FDM_WEIGHT_ERRORBAR)
                np.add.at(self.pos[ip], idx[ma], np.abs(aa[ma]))
                np.add.at(self.neg[ip], idx[mb], np.abs(bv[mb]))
        # setReduceDensityMatrix :71-114
        kept_prev = snap["kept"]
        self.reduced = [np.zeros((k, k)) for k in kept_prev]
        for i in range(nsec):
            U = snap["U"][i]
            if U.size == 0:
                continue
            r = U @ rho[i] @ U.T
            for (ii, bb, off, k, d) in snap["sub"][i]:
                if k == 0:
                    continue
                acc = np.zeros((k, k))
                for il in range(d):
                    a = off + il * k
                    acc += r[a:a + k, a:a + k]
                self.reduced[ii] += acc
        self.last = False
        self.ncalc += 1

    @staticmethod
    def energy_points():                                     # saveFinalData :322-337
        return FDM_MIN_ENERGY * np.exp(np.arange(FDM_ENERGY_PTS) / FDM_DELE)


def broaden(weights, energies, omegas, b):
    """Log-Gaussian broadening of examples/fdmSpectrumSiam/spec.py:27-44
    (without its pi*Gamma display factor):
    A(w) = (1/w) sum_i w_i exp(-(ln(w/e_i)/b - b/4)^2) / (b sqrt(pi))."""
    pre = 1.0 / (b * math.sqrt(math.pi))
    out = np.zeros(len(omegas))
    nz = weights != 0
    w, e = weights[nz], energies[nz]
    for k, x in enumerate(omegas):
        out[k] = (1.0 / x) * np.sum(w * np.exp(-np.power(-b * 0.25 + np.log(x / e) / b, 2)))
    return out * pre


class FdmThermoOracle:
    """Restatement of fdmThermodynamics (static/fdmThermodynamics.hpp)."""

    def __init__(self, nrg_iterations, bath_dimension, temps):   # :26-38
        self.nmax = nrg_iterations
        self.bathdim = bath_dimension
        self.T = np.asarray(temps, float)
        self.cur_kept = None
        self.prev_kept = None
        self.disc, self.allv = [], []
        self.qval = []

    def calc(self, snap, scale, sysops=None):                 # :42-89
        """One shell (backward order).  sysops: the system operators of
        this shell ({(i, j): block} per operator, setSystemOperator :37-39);
        the diagonal elements of their (i, i) blocks on the discarded states
        are kept (:63-88)."""
        if self.cur_kept is None:                             # setCurrentKeptIndex :91-100
            self.cur_kept = [0] * len(snap["current_sysmQ"])
        else:
            self.cur_kept = self.prev_kept
        self.prev_kept = list(snap["kept"])
        E = snap["eigenvaluesQ"]
        self.disc.append(np.concatenate([np.asarray(E[i][self.cur_kept[i]:]) * scale
                                         for i in range(len(E))] or [np.zeros(0)]))
        self.allv.append(np.concatenate([np.asarray(e) * scale for e in E]))
        if sysops is not None:
            q = []
            for op in sysops:
                v = np.zeros(self.disc[-1].size)
                o = 0
                for i in range(len(E)):
                    nd = len(E[i]) - self.cur_kept[i]
                    B = op.get((i, i))
                    if B is not None and B.size:
                        v[o:o + nd] = np.diag(B)[self.cur_kept[i]:]
                    o += nd
                q.append(v)
            self.qval.append(q)

    def _shells(self):
        """Discarded energies relative to each shell's ground state and the
        one-step corrected shell ground-state energies (:114-140)."""
        nsh = len(self.allv)
        gs = np.zeros(nsh)
        disc = [d.copy() for d in self.disc]
        for it in range(nsh):
            r = float(np.min(self.allv[it]))
            disc[it] = disc[it] - r
            gs[it] = r
        for it in range(nsh - 1):                             # one-step correction :133-135
            gs[it] += gs[it + 1]
        return disc, gs - gs[0]

    @staticmethod
    def _rexp(x):                                             # regulateExp :240-249
        return np.exp(np.clip(x, -100.0, 100.0))

    def _weights(self, disc, gs, kbt):
        """w_m (normalised), Z'_m and the partition sum at one temperature
        (:159-175)."""
        nsh = len(disc)
        cnt = self.nmax
        wm = np.zeros(nsh)
        zp = np.zeros(nsh)
        for i in range(nsh):
            pref = float(self.bathdim) ** (self.nmax - cnt)
            zi = float(np.sum(self._rexp((gs[i] - disc[i]) / kbt)))
            cnt -= 1
            wm[i] = zi * pref
            zp[i] = zi
        lpart = float(np.sum(wm))
        return wm / lpart, zp, lpart

    def shell_weights(self, kbt):
        """Boltzmann weight of every discarded state of every shell at
        temperature kbt, w_m exp((E0_m - E)/T) / Z'_m (the weights the
        thermodynamic averages use, :183-218), in the layout of `disc`:
        the form fdmBackwardIteration::setRhoZero(tBoltzmannFactor)
        (dynamics/fdmBackwardIteration.hpp:207-239) takes per shell."""
        disc, gs = self._shells()
        wm, zp, _ = self._weights(disc, gs, kbt)
        return [wm[i] * self._rexp((gs[i] - disc[i]) / kbt) / zp[i] if disc[i].size else np.zeros(0)
                for i in range(len(disc))]

    def final(self):                                          # saveFinalData :101-236
        disc, gs = self._shells()
        nsh = len(disc)
        ent = np.zeros(len(self.T))
        cv = np.zeros(len(self.T))
        nq = len(self.qval[0]) if self.qval else 0
        self.opexp = np.zeros((nq, len(self.T)))
        for itm, kbt in enumerate(self.T):
            wm, zp, lpart = self._weights(disc, gs, kbt)
            eav = esq = 0.0
            for i in range(nsh):
                if disc[i].size == 0:
                    continue
                blm = self._rexp((gs[i] - disc[i]) / kbt) / zp[i]
                x = disc[i] - gs[i]
                eav += float(np.sum(x * wm[i] * blm))
                esq += float(np.sum(x * x * wm[i] * blm))
                for iq in range(nq):                          # qsysOPeratorExpValue :200-218
                    self.opexp[iq, itm] += float(np.sum(self.qval[i][iq] * wm[i] * blm))
            ent[itm] = math.log(lpart) + eav / kbt
            cv[itm] = (esq - eav * eav) / (kbt * kbt)
        return ent, cv


def temperature_grid(points=200, tmin=1e-10, tmax=2.0):
    """Log temperature grid of examples/entropySIAM/main.cpp:68-76."""
    d = (points - 1.0) / math.log(tmax / tmin)
    return tmin * np.exp(np.arange(points) / d)


def siam_run(imp, bath, nkeep, nsites, lam, V=None, kondo=False, track_ops=None,
             fdm=False, thermo=False, full_fdag=True, record_h=False, fdm_T=None, sysop_index=None):
    """Drive the oracle the way the reference's example mains do.  Returns a
    dict with per-iteration eigenvalues, kept counts and (optionally) FDM and
    thermodynamic results.  fdm_T: the FDM spectrum at that temperature
    (shell Boltzmann weights from the thermodynamics pass) instead of T = 0;
    sysop_index: tracked operators handed to the thermodynamics as system
    operators (their <O>(T) in res["opexp"])."""
    from nrgplusplus_gb300.models import hopping
    nops = len(imp.fdag)
    n = NrgOracle(imp, bath, nkeep)
    ops = track_ops
    res = {"eig": [], "kept": [], "dims": [], "H": [], "snaps": {}}
    min_it = 0
    if not kondo:
        n.add_bath_site([V] * nops, 1.0, full_fdag=full_fdag)
        if ops is not None:
            ops = n.update_system_operator(ops)
        n.update_internal_state()
        res["eigV"] = n.all_eigenvalue.copy()
    for it in range(nsites):
        r = math.sqrt(lam) if (kondo or it > 0) else 1.0
        n.add_bath_site([hopping(it, lam)] * nops, r, full_fdag=full_fdag)
        if record_h:
            res["H"].append([h.copy() for h in n.H])
        if ops is not None:
            ops = n.update_system_operator(ops)
        if fdm or thermo:
            if n.checkHigherEnergyDiscarded():
                res["snaps"][n.nrg_iterations_cnt] = n.snapshot(ops)
            else:
                min_it += 1
        n.update_internal_state()
        res["eig"].append(n.all_eigenvalue.copy())
        res["kept"].append(list(n.kept))
        res["dims"].append([len(e) for e in n.eigenvaluesQ])
    res["min_it"] = min_it
    res["nrg"] = n
    def thermo_pass(temps):
        th = FdmThermoOracle(n.nrg_iterations_cnt, sum(len(e) for e in bath.energies), temps)
        cnt = n.nrg_iterations_cnt
        lo = min_it + (1 if kondo else 0)
        for it in range(nsites, lo, -1):
            cnt -= 1
            snap = res["snaps"][cnt]
            sys = None if sysop_index is None else [snap["ops"][k] for k in sysop_index]
            th.calc(snap, lam ** (-(1.0 * it - 1.0) / 2.0), sys)
        return th

    if fdm:
        weights = None
        if fdm_T is not None:
            if kondo:
                raise ValueError("finite-T FDM: the thermodynamic shells of a Kondo run start one later")
            weights = thermo_pass([fdm_T]).shell_weights(fdm_T)
        f = FdmSpectrumOracle(len(ops), weights)
        cnt = n.nrg_iterations_cnt
        for it in range(nsites, min_it, -1):
            cnt -= 1
            f.calc_spectrum(res["snaps"][cnt], lam ** (-(it - 1.0) / 2.0))
        res["pos"], res["neg"] = f.pos, f.neg
        res["static"] = f.static
    if thermo:
        th = thermo_pass(temperature_grid())
        res["entropy"], res["cv"] = th.final()
        res["opexp"] = th.opexp
    return res
