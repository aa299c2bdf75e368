"""The thermodynamics kernel's single-pass form against the reference's
two-pass form (CPU).

fdmThermodynamics::saveFinalData (fdmThermodynamics.hpp:101-236), restated by
the oracle, first sums each shell's partition function Z_i and then, in a
second pass, the shell-weighted Boltzmann probabilities times x = E - E_gs
and x^2.  k_thermo (nrgplusplus_gb300/csrc/k_fdm.cu) evaluates every
Boltzmann factor e once and keeps per shell Z_i = sum e, M1_i = sum x e,
M2_i = sum x^2 e; with d_i = bathdim^i and L = sum_i d_i Z_i it takes
<E> = sum_i d_i M1_i / L and <E^2> = sum_i d_i M2_i / L.  This checks the
identity on shell data of the shape an NRG run produces (energies spreading
over many decades, empty shells, the clamp of regulateExp in play)."""
import math

import numpy as np

from oracle.nrg_oracle import FdmThermoOracle, temperature_grid


def _single_pass(th):
    nsh = len(th.allv)
    gs = np.array([float(np.min(a)) for a in th.allv])
    disc = [d - g for d, g in zip(th.disc, gs)]
    for it in range(nsh - 1):  # the reference's one-step correction
        gs[it] += gs[it + 1]
    gs = gs - gs[0]
    ent, cv = np.zeros(len(th.T)), np.zeros(len(th.T))
    for k, kbt in enumerate(th.T):
        z = m1 = m2 = lpart = 0.0
        for i in range(nsh):
            x = disc[i] - gs[i]
            e = np.exp(np.clip(-x / kbt, -100.0, 100.0))
            d = float(th.bathdim) ** i
            lpart += d * float(np.sum(e))
            m1 += d * float(np.sum(x * e))
            m2 += d * float(np.sum(x * x * e))
        eav, esq = m1 / lpart, m2 / lpart
        ent[k] = math.log(lpart) + eav / kbt
        cv[k] = (esq - eav * eav) / (kbt * kbt)
    return ent, cv


def test_single_pass_moments_equal_the_two_pass_form():
    rng = np.random.default_rng(12)
    nsh, lam = 40, 2.0
    th = FdmThermoOracle(nsh, 4, temperature_grid())
    for n in range(nsh):
        # shell n of the backward pass (the last site first): energies of the
        # iteration above its ground state, times the shell's energy scale
        scale = lam ** (-(nsh - 1 - n) / 2.0)
        kept_e = np.sort(rng.exponential(1.0, 300)) * scale
        disc_e = kept_e[-1] + np.sort(rng.exponential(3.0, 0 if n == 7 else 900)) * scale
        allv = np.concatenate([kept_e, disc_e])
        th.disc.append(allv if n == 0 else disc_e)  # the last site discards every state
        th.allv.append(allv)
    ent_ref, cv_ref = th.final()
    ent, cv = _single_pass(th)
    assert np.all(np.isfinite(ent_ref)) and np.all(np.isfinite(cv_ref))
    assert 0.0 < ent_ref.max() < nsh * math.log(4.0) + 10  # a physical entropy range
    np.testing.assert_allclose(ent, ent_ref, rtol=1e-11, atol=1e-12)
    np.testing.assert_allclose(cv, cv_ref, rtol=1e-9, atol=1e-10)
