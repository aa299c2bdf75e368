// Backward-pass kernels: FDM spectral binning, reduced density matrix trace,
// log-Gaussian broadening and the thermodynamic sums.
#include "nrg_internal.h"

namespace nrg {
namespace {

constexpr double kFdmMinEnergy = 1e-10;      // fdmSpectrum.hpp:353
constexpr double kFdmWeightErrorbar = 1e-20;  // fdmSpectrum.hpp:343

// Spectral weights of one (op, i, j) pair (fdmSpectrum::rhoDotOperators,
// fdmSpectrum.hpp:207-277):
//   A = B^T with the kept x kept part zeroed
//   w+ = |(B rho_j)(v,v') A(v',v)|,  w- = |(rho_i B)(v,v') A(v',v)|
//   bin = int(ln(1 + |s (E_i[v] - E_j[v'])| / 1e-10) * delE)
// Weights above 1e-20 in bins [0, npts) are added to the op's histograms.
__global__ void k_fdm_bin(const FdmPair *__restrict__ pairs, int npairs, double delE, int npts) {
  const int64_t chunk = blockIdx.x;
  int lo = 0, hi = npairs - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (pairs[mid].chunk0 <= chunk) lo = mid; else hi = mid - 1;
  }
  const FdmPair P = pairs[lo];
  const int64_t nel = int64_t(P.ni) * P.nj;
  const int64_t e = (chunk - P.chunk0) * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  const int iv = int(e / P.nj), ivp = int(e - int64_t(iv) * P.nj);
  if (iv < P.kci && ivp < P.kcj) return;  // kept-kept part of A is zero
  const double a = P.B[e];
  const double aa = P.rhoA[e] * a;
  const double bv = P.ARho[e] * a;
  const int bin = int(log(1 + (fabs(P.scale * (P.Ei[iv] - P.Ej[ivp])) / kFdmMinEnergy)) * delE);
  if (bin < npts && bin >= 0) {
    if (fabs(aa) > kFdmWeightErrorbar) atomicAdd(P.pos + bin, fabs(aa));
    if (fabs(bv) > kFdmWeightErrorbar) atomicAdd(P.neg + bin, fabs(bv));
  }
}

// One shell's density-matrix blocks, written whole (no separate zeroing):
// the reduced density matrix of the later shell in the kept x kept corner,
// the Boltzmann weights on the diagonal of the last shell, zero elsewhere
// (fdmSpectrum::setRhoZero, fdmSpectrum.hpp:165-199).
__global__ void k_rho_init(const RhoTask *__restrict__ tasks, int ntasks) {
  const int64_t chunk = blockIdx.x;
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].chunk0 <= chunk) lo = mid; else hi = mid - 1;
  }
  const RhoTask T = tasks[lo];
  const int64_t e = (chunk - T.chunk0) * blockDim.x + threadIdx.x;
  if (e >= int64_t(T.n) * T.n) return;
  const int r = int(e / T.n), c = int(e - int64_t(r) * T.n);
  double v = 0.0;
  if (T.red && r < T.kc && c < T.kc) v = T.red[int64_t(r) * T.kc + c];
  else if (T.diag && r == c) v = T.diag[r];
  T.rho[e] = v;
}

// reducedRho[ii](it,it') = sum over the sub-blocks (ii, bb) of every block
// (in the reference's sector order) and the bath index il of
// rho(off + it + k il, off + it' + k il)
// (fdmSpectrum::setReduceDensityMatrix, fdmSpectrum.hpp:87-113).
// One CTA row (blockIdx.y) per output matrix; each element sums its inputs
// in list order and is written once.
__global__ void k_partial_trace(const TraceTask *__restrict__ tasks, const TraceIn *__restrict__ ins) {
  const TraceTask T = tasks[blockIdx.y];
  const int k = T.k;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < k * k; idx += gridDim.x * blockDim.x) {
    const int it = idx / k, itp = idx - it * k;
    double acc = 0.0;
    for (int j = T.in0; j < T.in1; ++j) {
      const TraceIn I = ins[j];
      double s = 0.0;
      for (int il = 0; il < I.d; ++il)
        s += I.rho[int64_t(I.off + it + k * il) * I.ld + (I.off + itp + k * il)];
      acc += s;
    }
    T.out[idx] = acc;
  }
}

// Log-Gaussian broadening of the binned weights (spec.py:27-44).  `le` holds
// ln(e_i); the Gaussian argument is formed in FP64 and only the exponential
// itself runs in FP32 (relative error ~2 ulp = 2.4e-7, inside the 1e-6
// tolerance of the spectral function), accumulated in FP64.
__global__ void k_broaden(const double *__restrict__ le, const double *__restrict__ w, int64_t nbins,
                          const double *__restrict__ omegas, double b, double *__restrict__ out) {
  __shared__ double red[32];
  const double x = omegas[blockIdx.x];
  const double lx = log(x);
  const double ib = 1.0 / b;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < nbins; i += blockDim.x) {
    const double z = fma(lx - le[i], ib, -b * 0.25);
    const double z2 = z * z;
    if (z2 < 80.0) s = fma(w[i], double(expf(-float(z2))), s);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) t += red[i];
    out[blockIdx.x] = (1.0 / x) * t / (b * sqrt(3.14159265358979323846));
  }
}

__device__ __forceinline__ double regulate_exp(double x) {  // fdmThermodynamics.hpp:240-249
  if (x > 100) return exp(100.0);
  if (x < -100) return exp(-100.0);
  return exp(x);
}

// Partition function, entropy and specific heat from the discarded energies
// of every shell (fdmThermodynamics::saveFinalData,
// fdmThermodynamics.hpp:154-226).  disc holds per shell the discarded
// energies already shifted by the shell minimum; gs the corrected shell
// ground energies.
// One CTA per temperature; warp w takes shells w, w + 8, ... and sums, over
// the shell's discarded states with x = E - E_gs(shell) and
// e = regulate_exp(-x / kT), the moments Z_i = sum e, M1_i = sum x e,
// M2_i = sum x^2 e and, per system operator q, Q_qi = sum O_q(x) e in one
// pass (each Boltzmann factor once).  With the reference's shell weights
// w_i = Z_i d^i / sum_j Z_j d^j and per-shell probabilities e / Z_i
// (fdmThermodynamics.hpp:42-236):
//   <E> = sum_i d^i M1_i / L,  <E^2> = sum_i d^i M2_i / L,  L = sum_i d^i Z_i,
//   S = ln L + <E> / kT,  C = (<E^2> - <E>^2) / kT^2,
//   <O_q> = sum_i d^i Q_qi / L   (qsysOPeratorExpValue, :200-218).
// qv: nq arrays in the layout of disc (the diagonal of each operator on the
// discarded states); sums: (3 + nq) * nshell doubles of scratch per
// temperature; opexp: nq x nt.
__global__ void k_thermo(const double *__restrict__ disc, const int64_t *__restrict__ disc_off,
                         const double *__restrict__ gs, int nshell, const double *__restrict__ temps,
                         double bathdim, const double *__restrict__ qv, int nq, int64_t ndisc,
                         double *__restrict__ sums, double *__restrict__ entropy, double *__restrict__ cv,
                         double *__restrict__ opexp, int nt) {
  const double kbt = temps[blockIdx.x], inv = 1.0 / kbt;
  double *z = sums + int64_t(blockIdx.x) * (3 + nq) * nshell, *m1 = z + nshell, *m2 = m1 + nshell;
  double *mq = m2 + nshell;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int i = warp; i < nshell; i += nw) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, sq[kThermoMaxOps];
#pragma unroll
    for (int q = 0; q < kThermoMaxOps; ++q) sq[q] = 0.0;
    const double g = gs[i];
    for (int64_t a = disc_off[i] + lane; a < disc_off[i + 1]; a += 32) {
      const double x = disc[a] - g;
      const double w = regulate_exp(-x * inv);
      s0 += w;
      s1 += x * w;
      s2 += x * x * w;
#pragma unroll
      for (int q = 0; q < kThermoMaxOps; ++q)
        if (q < nq) sq[q] += qv[int64_t(q) * ndisc + a] * w;
    }
    for (int o = 16; o > 0; o >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
#pragma unroll
      for (int q = 0; q < kThermoMaxOps; ++q)
        if (q < nq) sq[q] += __shfl_xor_sync(0xffffffffu, sq[q], o);  // nq is uniform
    }
    if (lane == 0) {
      z[i] = s0;
      m1[i] = s1;
      m2[i] = s2;
      for (int q = 0; q < nq; ++q) mq[int64_t(q) * nshell + i] = sq[q];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double lpart = 0.0, e1 = 0.0, e2 = 0.0;
    for (int i = 0; i < nshell; ++i) {
      const double d = pow(bathdim, double(i));
      lpart += z[i] * d;
      e1 += m1[i] * d;
      e2 += m2[i] * d;
    }
    const double eav = e1 / lpart, esq = e2 / lpart;
    entropy[blockIdx.x] = log(lpart) + eav / kbt;
    cv[blockIdx.x] = (esq - eav * eav) / (kbt * kbt);
    for (int q = 0; q < nq; ++q) {
      double oq = 0.0;
      for (int i = 0; i < nshell; ++i) oq += mq[int64_t(q) * nshell + i] * pow(bathdim, double(i));
      opexp[int64_t(q) * nt + blockIdx.x] = oq / lpart;
    }
  }
}

// Static expectation values of one shell (fdmBackwardIteration::
// rhoDotStaticOperators, dynamics/fdmBackwardIteration.hpp:166-199): for each
// diagonal operator block (i, i), sum over v, v' of O(v, v') rho_i(v', v) with
// the kept x kept part of O left out.  One CTA per task writes its partial
// sum; k_fdm_static_sum then adds the partials of each operator in task order
// (deterministic) to that operator's running total.
__global__ void k_fdm_static(const StaticTask *__restrict__ tasks, double *__restrict__ partial) {
  const StaticTask T = tasks[blockIdx.x];
  __shared__ double red[8];
  double s = 0.0;
  const int64_t nel = int64_t(T.n) * T.n;
  for (int64_t e = threadIdx.x; e < nel; e += blockDim.x) {
    const int r = int(e / T.n), c = int(e - int64_t(r) * T.n);
    if (r < T.kc && c < T.kc) continue;
    s += T.O[int64_t(r) * T.ldo + c] * T.rho[int64_t(c) * T.n + r];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) t += red[i];
    partial[blockIdx.x] = t;
  }
}

__global__ void k_fdm_static_sum(const StaticTask *__restrict__ tasks, int ntasks,
                                 const double *__restrict__ partial, double *__restrict__ acc) {
  if (threadIdx.x != 0) return;
  const int op = blockIdx.x;
  double s = acc[op];
  for (int t = 0; t < ntasks; ++t)
    if (tasks[t].op == op) s += partial[t];
  acc[op] = s;
}

}  // namespace

void launch_fdm_bin(const FdmPair *pairs, int npairs, int64_t nchunks, double delE, int npts, cudaStream_t s) {
  if (npairs == 0 || nchunks == 0) return;
  k_fdm_bin<<<unsigned(nchunks), 256, 0, s>>>(pairs, npairs, delE, npts);
}

void launch_rho_init(const RhoTask *tasks, int ntasks, int64_t nchunks, cudaStream_t s) {
  if (ntasks == 0 || nchunks == 0) return;
  k_rho_init<<<unsigned(nchunks), 256, 0, s>>>(tasks, ntasks);
}

void launch_partial_trace(const TraceTask *tasks, int ntask, const TraceIn *ins, int maxk,
                          cudaStream_t s) {
  if (ntask == 0 || maxk == 0) return;
  int gx = (maxk * maxk + 255) / 256;
  if (gx > 64) gx = 64;
  k_partial_trace<<<dim3(gx, ntask), 256, 0, s>>>(tasks, ins);
}

void launch_broaden(const double *e, const double *w, int64_t nbins, const double *omegas,
                    int64_t nomega, double b, double *out, cudaStream_t s) {
  if (nomega == 0) return;
  k_broaden<<<unsigned(nomega), 256, 0, s>>>(e, w, nbins, omegas, b, out);
}

void launch_thermo(const double *disc, const int64_t *disc_off, const double *gs, int nshell,
                   const double *temps, int nt, double bathdim, const double *qv, int nq, int64_t ndisc,
                   double *sums, double *entropy, double *cv, double *opexp, cudaStream_t s) {
  if (nt == 0) return;
  k_thermo<<<nt, 256, 0, s>>>(disc, disc_off, gs, nshell, temps, bathdim, qv, nq, ndisc, sums, entropy, cv,
                              opexp, nt);
}

void launch_fdm_static(const StaticTask *tasks, int ntasks, int nops, double *partial, double *acc,
                       cudaStream_t s) {
  if (ntasks == 0) return;
  k_fdm_static<<<ntasks, 256, 0, s>>>(tasks, partial);
  k_fdm_static_sum<<<nops, 32, 0, s>>>(tasks, ntasks, partial, acc);
}

}  // namespace nrg
