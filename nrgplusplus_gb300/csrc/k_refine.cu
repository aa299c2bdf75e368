// FP64-accurate refinement of FP32 eigenpairs (mixed-precision path).
//
// The FP32 block solver (k_eig<float>) gives eigenvectors X good to ~1e-6.
// Each refinement step is the Newton-type update of Ogita & Aishima
// ("Iterative refinement for symmetric eigenvalue decomposition", Japan J.
// Indust. Appl. Math. 35 (2018)):
//     S = X^T A X,  G = X^T X  (FP64-accurate GEMMs, all SMs)
//     l_i  = s_ii / g_ii
//     e_ii = (1 - g_ii) / 2
//     e_ij = (s_ij - l_j g_ij) / (l_j - l_i)   if |l_i - l_j| > tau
//          = -g_ij / 2                         otherwise (near-degenerate pair:
//                                               orthonormalise only)
//     X <- X + X E
// which converges quadratically for separated eigenvalues.  The final pass
// takes the Rayleigh quotients l_i and, for every run of sorted l with gaps
// <= tau (a near-degenerate cluster), diagonalises the cluster's block of S
// with a cyclic FP64 Jacobi iteration and rotates the cluster's columns.
// Only these O(n^2) element-wise steps and the tiny cluster problems run on
// the FP64 pipe per block; the O(n^3) work is in the grouped GEMMs.
#include "nrg_internal.h"

namespace nrg {
namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxCluster = 64;
constexpr int kMaxJacobiSweeps = 30;
// Largest remaining Newton correction accepted after the last step.  A
// converged block sits near u |A| / gap <= 1e-16 / tau_rel = 1e-12; a block
// whose FP32 start was too poor for the fixed step count stays far above.
constexpr double kConvTol = 1e-10;

// S and G are symmetric; their lower triangle may not be written (the
// tensor-core path computes only the tiles that meet the upper triangle)
__device__ __forceinline__ double sym(const double *M, int ld, int i, int j) {
  return i <= j ? M[int64_t(i) * ld + j] : M[int64_t(j) * ld + i];
}

__device__ double block_max(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double m = red[0];
  for (int w = 1; w < kWarps; ++w) m = fmax(m, red[w]);
  __syncthreads();
  return m;
}

// The element-wise passes over S and G (the Newton correction, the
// convergence check) run on row strips: one CTA per kStripRows rows of one
// block, one warp per row and lanes along it, so a large block spreads over
// many SMs.  Every CTA recomputes the block's Rayleigh quotients
// lam_i = S_ii / G_ii and tau (n values) in shared memory.
constexpr int kStripRows = 16;
constexpr int kStripThreads = 256;
constexpr int kStripWarps = kStripThreads / 32;

__device__ double strip_max(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double m = red[0];
  for (int w = 1; w < kStripWarps; ++w) m = fmax(m, red[w]);
  __syncthreads();
  return m;
}

// lam into shared memory; returns tau (0 < tau) and sets *bad when a
// Rayleigh quotient is not finite
__device__ double strip_lambdas(const RefineBlock &B, double *lam, double tau_rel, double *red, bool *bad) {
  const int n = B.n;
  double local = 0.0, nf = 0.0;
  for (int i = threadIdx.x; i < n; i += kStripThreads) {
    const double l = B.S[int64_t(i) * B.ld + i] / B.G[int64_t(i) * B.ld + i];
    lam[i] = l;
    if (isfinite(l)) local = fmax(local, fabs(l));
    else nf = 1.0;
  }
  const double m = strip_max(local, red);
  *bad = strip_max(nf, red) > 0.0;
  return tau_rel * fmax(1.0, m);
}

__global__ void __launch_bounds__(kStripThreads)
k_oa_update(const RefineBlock *__restrict__ blocks, const int2 *__restrict__ tiles, double tau_rel) {
  extern __shared__ __align__(16) double lam[];
  __shared__ double red[kStripWarps];
  const int2 t = tiles[blockIdx.x];
  const RefineBlock B = blocks[t.x];
  const int n = B.n;
  bool nf;
  const double tau = strip_lambdas(B, lam, tau_rel, red, &nf);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r1 = min(n, t.y + kStripRows);
  for (int i = t.y + warp; i < r1; i += kStripWarps) {
    const double li = lam[i];
    double *out = B.E2 + int64_t(i) * B.ld;
    for (int j = lane; j < n; j += 32) {
      const double g = sym(B.G, B.ld, i, j);
      double e;
      if (i == j) {
        e = 0.5 * (1.0 - g);
      } else {
        const double d = lam[j] - li;
        e = (fabs(d) > tau) ? (sym(B.S, B.ld, i, j) - lam[j] * g) / d : -0.5 * g;
      }
      out[j] = e;
    }
  }
}

// Convergence: every entry of the correction one more Newton step would
// apply (the k_oa_update formulas; within a cluster only the orthogonality
// part) must be below kConvTol and every Rayleigh quotient finite, otherwise
// flag[b] = 1 and the block is re-solved in FP64.
__global__ void __launch_bounds__(kStripThreads)
k_oa_check(const RefineBlock *__restrict__ blocks, const int2 *__restrict__ tiles, double tau_rel, int *flag) {
  extern __shared__ __align__(16) double lam[];
  __shared__ double red[kStripWarps];
  const int2 t = tiles[blockIdx.x];
  const RefineBlock B = blocks[t.x];
  const int n = B.n;
  bool nf;
  const double tau = strip_lambdas(B, lam, tau_rel, red, &nf);
  double bad = nf ? 1.0 : 0.0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r1 = min(n, t.y + kStripRows);
  for (int i = t.y + warp; i < r1 && bad == 0.0; i += kStripWarps) {
    const double li = lam[i];
    for (int j = lane; j < n; j += 32) {
      const double g = sym(B.G, B.ld, i, j);
      double r;
      if (i == j) {
        r = 1.0 - g;
      } else {
        const double d = lam[j] - li;
        r = (fabs(d) > tau) ? (sym(B.S, B.ld, i, j) - lam[j] * g) / d : g;
      }
      if (!(fabs(r) <= kConvTol)) bad = 1.0;
    }
  }
  if (strip_max(bad, red) > 0.0 && threadIdx.x == 0) flag[t.x] = 1;
}

// Final Rayleigh-Ritz pass: eigenvalues, cluster diagonalisation, sorted
// output (E ascending, U columns in the same order).  status[b] = 2 when
// the refinement has not converged (non-finite Rayleigh quotients or a
// remaining correction above kConvTol): the block is re-solved in FP64.
// Chains longer than kMaxCluster are left as plain columns with status 3
// for k_oa_bigcl, which diagonalises them and clears the status.
__global__ void __launch_bounds__(kThreads)
k_oa_final(const RefineBlock *__restrict__ blocks, double tau_rel, int *status, const int *flag) {
  extern __shared__ __align__(16) double sm[];
  __shared__ double red[kWarps];
  __shared__ int ncl, jac_flag;
  const RefineBlock B = blocks[blockIdx.x];
  const int n = B.n;
  if (flag[blockIdx.x]) {  // k_oa_check: refinement broke down, re-solve in FP64
    if (threadIdx.x == 0) status[blockIdx.x] = 2;
    return;
  }
  double *lam = sm;                                   // n
  double *lams = lam + n;                             // n (sorted)
  double *Sc = lams + n;                              // kMaxCluster^2
  double *Qc = Sc + kMaxCluster * kMaxCluster;        // kMaxCluster^2
  int *perm = reinterpret_cast<int *>(Qc + kMaxCluster * kMaxCluster);  // n
  int *cl = perm + n;                                 // up to n/2 + 1 cluster starts/ends
  int *order = cl + n + 2;                            // kMaxCluster
  double local = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const double l = B.S[int64_t(i) * B.ld + i] / B.G[int64_t(i) * B.ld + i];
    lam[i] = l;
    local = fmax(local, fabs(l));
  }
  const double tau = tau_rel * fmax(1.0, block_max(local, red));
  __syncthreads();  // lam complete
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const double x = lam[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double y = lam[j];
      r += (y < x) || (y == x && j < i);
    }
    perm[r] = i;
    lams[r] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int c = 0, k = 0;
    while (k < n) {
      int e = k + 1;
      while (e < n && lams[e] - lams[e - 1] <= tau) ++e;
      if (e - k > 1) {
        cl[2 * c] = k;
        cl[2 * c + 1] = e;
        ++c;
      }
      k = e;
    }
    ncl = c;
  }
  __syncthreads();
  // plain columns: U[:, k] = X[:, perm[k]], E[k] = lams[k]
  for (int k = threadIdx.x; k < n; k += kThreads) B.Eout[k] = lams[k];
  {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < n; r += kWarps)
      for (int k = lane; k < n; k += 32) B.U[int64_t(r) * B.ldu + k] = B.X[int64_t(r) * B.ld + perm[k]];
  }
  __syncthreads();
  for (int q = 0; q < ncl; ++q) {
    const int a = cl[2 * q], c = cl[2 * q + 1] - a;
    if (c > kMaxCluster) {  // left to k_oa_bigcl (k_eig.cu)
      if (threadIdx.x == 0) status[blockIdx.x] = 3;
      continue;
    }
    for (int idx = threadIdx.x; idx < c * c; idx += kThreads) {
      const int p = idx / c, s = idx - p * c;
      Sc[idx] = sym(B.S, B.ld, perm[a + p], perm[a + s]);
      Qc[idx] = (p == s) ? 1.0 : 0.0;
    }
    __syncthreads();
    // cyclic Jacobi on the c x c cluster block (symmetrised on the fly)
    for (int sweep = 0; sweep < kMaxJacobiSweeps; ++sweep) {
      if (threadIdx.x == 0) jac_flag = 0;
      __syncthreads();
      for (int p = 0; p < c - 1; ++p)
        for (int s = p + 1; s < c; ++s) {
          const double apq = 0.5 * (Sc[p * c + s] + Sc[s * c + p]);
          const double app = Sc[p * c + p], aqq = Sc[s * c + s];
          if (fabs(apq) <= 1e-300 || fabs(apq) <= 1e-17 * (fabs(app) + fabs(aqq))) continue;
          const double th = (aqq - app) / (2.0 * apq);
          const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
          const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
          __syncthreads();
          // rows p, s then columns p, s of Sc; columns p, s of Qc
          for (int k = threadIdx.x; k < c; k += kThreads) {
            const double xp = Sc[p * c + k], xs = Sc[s * c + k];
            Sc[p * c + k] = cs * xp - sn * xs;
            Sc[s * c + k] = sn * xp + cs * xs;
          }
          __syncthreads();
          for (int k = threadIdx.x; k < c; k += kThreads) {
            const double xp = Sc[k * c + p], xs = Sc[k * c + s];
            Sc[k * c + p] = cs * xp - sn * xs;
            Sc[k * c + s] = sn * xp + cs * xs;
            const double qp = Qc[k * c + p], qs = Qc[k * c + s];
            Qc[k * c + p] = cs * qp - sn * qs;
            Qc[k * c + s] = sn * qp + cs * qs;
          }
          if (threadIdx.x == 0) jac_flag = 1;
          __syncthreads();
        }
      __syncthreads();
      const int more = jac_flag;
      __syncthreads();
      if (!more) break;
    }
    // order the cluster's eigenvalues ascending
    if (threadIdx.x == 0) {
      for (int t = 0; t < c; ++t) order[t] = t;
      for (int t = 1; t < c; ++t) {
        int v = order[t], u = t - 1;
        while (u >= 0 && Sc[order[u] * c + order[u]] > Sc[v * c + v]) {
          order[u + 1] = order[u];
          --u;
        }
        order[u + 1] = v;
      }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < c; t += kThreads) B.Eout[a + t] = Sc[order[t] * c + order[t]];
    for (int64_t idx = threadIdx.x; idx < int64_t(n) * c; idx += kThreads) {
      const int r = int(idx / c), t = int(idx - int64_t(r) * c);
      const int col = order[t];
      double v = 0.0;
      for (int p = 0; p < c; ++p) v += B.X[int64_t(r) * B.ld + perm[a + p]] * Qc[p * c + col];
      B.U[int64_t(r) * B.ldu + a + t] = v;
    }
    __syncthreads();
  }
}

size_t final_smem(int n) {
  return sizeof(double) * (2 * size_t(n) + 2 * kMaxCluster * kMaxCluster) +
         sizeof(int) * (2 * size_t(n) + 2 + kMaxCluster) + 64;
}

}  // namespace

int refine_max_n() {
  int n = 64;
  while (final_smem(n + 1) <= 225 * 1024) ++n;
  return n;
}

void launch_oa_update(const RefineBlock *blocks, const int2 *tiles, int ntiles, int max_n, double tau_rel,
                      cudaStream_t s) {
  if (ntiles == 0) return;
  ensure_smem_limit(reinterpret_cast<const void *>(k_oa_update), 225 * 1024);
  k_oa_update<<<ntiles, kStripThreads, sizeof(double) * size_t(max_n) + 16, s>>>(blocks, tiles, tau_rel);
}

void launch_oa_check(const RefineBlock *blocks, const int2 *tiles, int ntiles, int max_n, double tau_rel,
                     int *flag, cudaStream_t s) {
  if (ntiles == 0) return;
  ensure_smem_limit(reinterpret_cast<const void *>(k_oa_check), 225 * 1024);
  k_oa_check<<<ntiles, kStripThreads, sizeof(double) * size_t(max_n) + 16, s>>>(blocks, tiles, tau_rel, flag);
}

int oa_strip_rows() { return kStripRows; }

void launch_oa_final(const RefineBlock *blocks, int nblocks, int max_n, double tau_rel, int *status,
                     const int *flag, cudaStream_t s) {
  if (nblocks == 0) return;
  ensure_smem_limit(reinterpret_cast<const void *>(k_oa_final), 225 * 1024);
  k_oa_final<<<nblocks, kThreads, final_smem(max_n), s>>>(blocks, tau_rel, status, flag);
}

}  // namespace nrg
