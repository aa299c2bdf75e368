// Grouped FP64 GEMM for the operator rotations of the plain FP64 path:
//   f-dagger:  F_new(i,j) = sum_(ii,bb,bb') fb * U_i[rows]^T U_j[rows]
//              (nrgcore::set_current_fdag_operator, nrgcore.hpp:401-477)
//   operators: O_new(i,j) = sum U_i[rows]^T O_prev U_j[rows]
//              (update_system_operator, sysOperator.hpp:36-133)
//   FDM:       rho <- U rho U^T, B rho, rho B (fdmSpectrum.hpp:84-85, 231-232)
// Each CTA owns one 64x64 tile of one output matrix and accumulates every
// contribution of that output in registers, in list order, so the result is
// deterministic and written once.  The sparse f-dagger embedding T of the
// reference is folded into the contribution list as row offsets and a scalar.
#include "nrg_internal.h"

namespace nrg {
namespace {

constexpr int BM = 64, BN = 64, BK = 16;
constexpr int kThreads = 256;  // 16 x 16 threads, 4 x 4 outputs each

__global__ void __launch_bounds__(kThreads)
k_gemm_f64(const GemmTile *__restrict__ tiles, const GemmGroup *__restrict__ groups,
           const GemmContrib *__restrict__ contribs) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const GemmTile t = tiles[blockIdx.x];
  const GemmGroup g = groups[t.group];
  const int m0 = t.tm * BM, n0 = t.tn * BN;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int c = g.c0; c < g.c1; ++c) {
    const GemmContrib q = contribs[c];
    const bool ta = q.trans & 1, tb = (q.trans >> 1) & 1;
    double part[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) part[i][j] = 0.0;
    for (int k0 = 0; k0 < q.K; k0 += BK) {
      // A tile: op(A)[m0 .. m0+63][k0 .. k0+15]
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int idx = threadIdx.x + u * kThreads;  // 0..1023
        int mm, kk;
        if (ta) { mm = idx & 63; kk = idx >> 6; }     // stored K x M: m fastest
        else    { kk = idx & 15; mm = idx >> 4; }     // stored M x K: k fastest
        const int gm = m0 + mm, gk = k0 + kk;
        double v = 0.0;
        if (gm < g.M && gk < q.K)
          v = ta ? q.A[int64_t(gk) * q.lda + gm] : q.A[int64_t(gm) * q.lda + gk];
        As[kk][mm] = v;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int idx = threadIdx.x + u * kThreads;
        int nn, kk;
        if (tb) { kk = idx & 15; nn = idx >> 4; }     // stored N x K: k fastest
        else    { nn = idx & 63; kk = idx >> 6; }     // stored K x N: n fastest
        const int gn = n0 + nn, gk = k0 + kk;
        double v = 0.0;
        if (gn < g.N && gk < q.K)
          v = tb ? q.B[int64_t(gn) * q.ldb + gk] : q.B[int64_t(gk) * q.ldb + gn];
        Bs[kk][nn] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) part[i][j] = fma(a[i], b[j], part[i][j]);
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = fma(q.alpha, part[i][j], acc[i][j]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= g.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx + 16 * j;
      if (gn >= g.N) continue;
      double *cp = g.C + int64_t(gm) * g.ldc + gn;
      *cp = g.accumulate ? (*cp + acc[i][j]) : acc[i][j];
    }
  }
}

}  // namespace

void launch_gemm_f64(const GemmTile *tiles, int ntiles, const GemmGroup *groups,
                     const GemmContrib *contribs, cudaStream_t s) {
  if (ntiles == 0) return;
  k_gemm_f64<<<ntiles, kThreads, 0, s>>>(tiles, groups, contribs);
}

}  // namespace nrg
