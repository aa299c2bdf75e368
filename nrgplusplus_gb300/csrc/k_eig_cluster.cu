// Thread-block-cluster eigensolver for the large sector blocks (the first
// stage of qmatrix::diag -> LAPACKE_dsyevd, qmatrix.hpp:375-404, for blocks
// too large for one SM's shared memory).
//
// One cluster of CS CTAs (CS SMs) owns one block; the matrix lives in the
// cluster's distributed shared memory, row r in CTA r % CS (cyclic rows keep
// the shrinking active part balanced).  The work is the one-CTA solver's
// (k_eig.cu: tred2_reduce, Sturm bisection, inverse iteration, cluster
// re-orthogonalisation), spread over the cluster:
//   Householder step i (n-1 down to 1), reflector u from row i:
//     the owner of row i forms u, h and e_i              | cluster barrier
//     every CTA copies u from the owner (DSMEM loads),
//     p_j = (A u)_j / h for its rows; p_j and the partial
//     u.p to all CTAs                                     | cluster barrier
//     q = p - (u.p / 2h) u locally, rank-2 update A -= u q^T + q u^T of its rows
//   T's diagonal and off-diagonal gathered into every CTA; eigenvalue j is
//   bisected and inverse-iterated by CTA j % CS; eigenvalues gathered again;
//   near-degenerate clusters re-orthogonalised by the CTA owning their first
//   member (one warp each).
// Outputs as k_eig_bi: eigenvalues into E (ascending), the reflectors into W
// (row i: u_i in columns 0..i-1, h_i on the diagonal) and the tridiagonal
// eigenvectors into V, for k_reflect.  T = float is the mixed path's first
// stage (W, V, Bt); T = double the plain FP64 path's reflector solver (W64,
// V64, Bt64).  Every CTA of a cluster passes the same barriers (the control
// flow depends only on n and on values all CTAs read from the same place),
// and no CTA leaves while others may still read its shared memory.
#include <cooperative_groups.h>

#include <algorithm>

#include "eig_tri.cuh"
#include "nrg_internal.h"

namespace nrg {
namespace {

namespace cg = cooperative_groups;

constexpr int kThreadsC = 512;
constexpr int kWarpsC = kThreadsC / 32;
constexpr int kInvIterC = 3;

template <typename T> __device__ __forceinline__ T warp_sum_c(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic CTA-wide sum; red needs kWarpsC + 1 entries.
template <typename T> __device__ T block_sum_c(T v, T *red) {
  v = warp_sum_c(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    T s = (l < kWarpsC) ? red[l] : T(0);
    s = warp_sum_c(s);
    if (l == 0) red[kWarpsC] = s;
  }
  __syncthreads();
  return red[kWarpsC];
}

template <typename T> __device__ T block_max_c(T v, T *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  T m = red[0];
  for (int i = 1; i < kWarpsC; ++i) m = max(m, red[i]);
  __syncthreads();
  return m;
}

struct CtlC {
  double h;    // the current step's h (0: no reflector), set by the row's owner
  int ncl;     // number of near-degenerate clusters
  int pad;
};

__host__ __device__ inline int rows_of(int n, int cs, int rank) { return (n - rank + cs - 1) / cs; }
__host__ __device__ inline int pitch_of(int n) { return (n + 3) & ~3; }

// Dynamic shared memory of one CTA for an n-block on CS CTAs (rank 0 holds
// the most rows; every CTA uses that layout).
template <typename T> __host__ __device__ inline size_t cluster_smem(int n, int cs) {
  const size_t nr = size_t(rows_of(n, cs, 0));
  size_t b = 64 + sizeof(T) * (kWarpsC + 1 + 16 + cs);  // ctl, red, part
  // the CTA's rows; afterwards the staging of the cluster solves (2n per warp)
  b += sizeof(T) * std::max(nr * size_t(pitch_of(n)), size_t(2 * kWarpsC) * size_t(n));
  b += sizeof(T) * (5 * size_t(n) + 16);                 // u, q, d, e, lam
  b += sizeof(T) * (3 * nr + 8);                         // p, h, e of the own rows
  return b + 256;                                        // 16-byte alignment of 12 arrays
}

template <typename T, int CS>
__global__ void __launch_bounds__(kThreadsC, 1)
k_eig_cluster(const EigBlock *__restrict__ blocks) {
  extern __shared__ __align__(16) char smem_c[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = int(cluster.block_rank());
  const EigBlock B = blocks[blockIdx.x / CS];
  const int n = B.n;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nr = rows_of(n, CS, rank), P = pitch_of(n);
  // carve: the layout is the same in every CTA of the cluster (sized for
  // rank 0, which holds the most rows), so a DSMEM address maps 1:1
  const int nr0 = rows_of(n, CS, 0);
  char *sp = smem_c;
  auto take = [&](size_t bytes) {
    char *q = sp;
    sp += (bytes + 15) & ~size_t(15);
    return q;
  };
  CtlC *ctl = reinterpret_cast<CtlC *>(take(sizeof(CtlC)));
  T *red = reinterpret_cast<T *>(take(sizeof(T) * (kWarpsC + 1)));
  T *part = reinterpret_cast<T *>(take(sizeof(T) * CS));
  T *u = reinterpret_cast<T *>(take(sizeof(T) * (n + 4)));
  T *q = reinterpret_cast<T *>(take(sizeof(T) * (n + 4)));
  T *dv = reinterpret_cast<T *>(take(sizeof(T) * n));
  T *ev = reinterpret_cast<T *>(take(sizeof(T) * n));
  T *lam = reinterpret_cast<T *>(take(sizeof(T) * n));
  T *ploc = reinterpret_cast<T *>(take(sizeof(T) * (nr0 + 1)));
  T *hloc = reinterpret_cast<T *>(take(sizeof(T) * (nr0 + 1)));
  T *eloc = reinterpret_cast<T *>(take(sizeof(T) * (nr0 + 1)));
  T *A = reinterpret_cast<T *>(take(sizeof(T) * max(size_t(nr0) * P, size_t(2 * kWarpsC) * size_t(n))));
  T *W = Bufs<T>::W(B), *V = Bufs<T>::V(B), *Bt = Bufs<T>::Bt(B);
  // load the CTA's rows (row g = rank + r * CS)
  for (int64_t idx = tid; idx < int64_t(nr) * n; idx += kThreadsC) {
    const int r = int(idx / n), c = int(idx - int64_t(r) * n);
    A[int64_t(r) * P + c] = T(B.H[int64_t(rank + r * CS) * B.ld + c]);
  }
  for (int r = tid; r <= nr; r += kThreadsC) {
    hloc[r] = T(0);
    eloc[r] = T(0);
  }
  __syncthreads();
  cluster.sync();
  // ---------------- Householder reduction, step i = n-1 .. 1
  for (int i = n - 1; i >= 1; --i) {
    const int l = i - 1;
    const int owner = i % CS, li = i / CS;
    if (rank == owner) {
      T *row = A + int64_t(li) * P;
      T sc = T(0);
      for (int k = tid; k <= l; k += kThreadsC) sc += abs_c(row[k]);
      sc = block_sum_c(sc, red);
      if (l == 0 || sc == T(0)) {
        if (tid == 0) {
          eloc[li] = row[l];
          hloc[li] = T(0);
          ctl->h = 0.0;
        }
      } else {
        T hs = T(0);
        for (int k = tid; k <= l; k += kThreadsC) {
          const T x = row[k] / sc;
          row[k] = x;
          hs += x * x;
        }
        T h = block_sum_c(hs, red);
        if (tid == 0) {
          const T f = row[l];
          const T g = (f >= T(0)) ? -sqrt_c(h) : sqrt_c(h);
          eloc[li] = sc * g;
          h -= f * g;
          row[l] = f - g;
          hloc[li] = h;
          ctl->h = double(h);
        }
      }
    }
    cluster.sync();  // the owner's row i, h and e_i are final
    const CtlC *octl = cluster.map_shared_rank(ctl, owner);
    const T h = T(octl->h);
    if (h == T(0)) continue;  // uniform over the cluster
    const T *orow = cluster.map_shared_rank(A, owner) + int64_t(li) * P;
    for (int k = tid; k <= l; k += kThreadsC) u[k] = orow[k];
    __syncthreads();
    // p_j = (A u)_j / h for the own rows j <= l, one warp per row
    const int nact = (l >= rank) ? (l - rank) / CS + 1 : 0;  // own rows with j <= l
    for (int r = warp; r < nact; r += kWarpsC) {
      const T *rowj = A + int64_t(r) * P;
      T s = T(0);
      for (int k = lane; k <= l; k += 32) s += rowj[k] * u[k];
      s = warp_sum_c(s);
      if (lane == 0) ploc[r] = s / h;
    }
    __syncthreads();
    // p of the own rows and the partial u.p go to every CTA (p gathered into
    // q): one barrier for both, q = p - (u.p / 2h) u is formed locally
    T fs = T(0);
    for (int r = tid; r < nact; r += kThreadsC) fs += ploc[r] * u[rank + r * CS];
    fs = block_sum_c(fs, red);
    if (tid < CS) *cluster.map_shared_rank(part + rank, tid) = fs;
    for (int idx = tid; idx < nact * CS; idx += kThreadsC) {
      const int r = idx / CS, c = idx - r * CS;
      *cluster.map_shared_rank(q + rank + r * CS, c) = ploc[r];
    }
    cluster.sync();
    T f = T(0);
    for (int c = 0; c < CS; ++c) f += part[c];  // same order in every CTA
    const T hh = f / (h + h);
    for (int k = tid; k <= l; k += kThreadsC) q[k] -= hh * u[k];  // q = p - hh u
    __syncthreads();
    // rank-2 update of the own rows, columns 0..l
    for (int r = warp; r < nact; r += kWarpsC) {
      T *rowj = A + int64_t(r) * P;
      const int j = rank + r * CS;
      const T uj = u[j], qj = q[j];
      for (int k = lane; k <= l; k += 32) rowj[k] -= uj * q[k] + qj * u[k];
    }
    __syncthreads();
  }
  // ---------------- T's diagonal / off-diagonal and the reflectors
  // own rows: d_i = A(i, i), e_i from the step that produced it; the
  // reflector row (u in columns 0..i-1, h_i on the diagonal) goes to W
  for (int idx = tid; idx < nr * CS; idx += kThreadsC) {
    const int r = idx / CS, c = idx - r * CS;
    const int g = rank + r * CS;
    *cluster.map_shared_rank(dv + g, c) = A[int64_t(r) * P + g];
    *cluster.map_shared_rank(ev + g, c) = (g == 0) ? T(0) : eloc[r];
  }
  for (int64_t idx = tid; idx < int64_t(nr) * n; idx += kThreadsC) {
    const int r = int(idx / n), c = int(idx - int64_t(r) * n);
    const int g = rank + r * CS;
    if (c < g) W[int64_t(g) * B.ld + c] = A[int64_t(r) * P + c];
    else if (c == g) W[int64_t(g) * B.ld + c] = (g == 0) ? T(0) : hloc[r];
  }
  cluster.sync();
  // ---------------- tridiagonal eigenproblem
  T lo = T(3e38), hi = T(-3e38), tn = T(0);
  for (int i = tid; i < n; i += kThreadsC) {
    const T rr = abs_c(ev[i]) + (i + 1 < n ? abs_c(ev[i + 1]) : T(0));
    lo = min(lo, dv[i] - rr);
    hi = max(hi, dv[i] + rr);
    tn = max(tn, abs_c(dv[i]) + rr);
  }
  lo = -block_max_c(-lo, red);
  hi = block_max_c(hi, red);
  tn = block_max_c(tn, red);
  const T span = max(hi - lo, T(1e-30));
  lo -= T(1e-6) * span;
  hi += T(1e-6) * span;
  const int nown = rows_of(n, CS, rank);  // eigenvalues j = rank + k CS
  for (int k = tid; k < nown; k += kThreadsC) {
    const int j = rank + k * CS;
    T a0 = lo, b0 = hi;
    for (int it = 0; it < 90; ++it) {
      const T mid = T(0.5) * (a0 + b0);
      if (mid <= a0 || mid >= b0) break;
      if (sturm_c(dv, ev, n, mid) > j) b0 = mid; else a0 = mid;
    }
    const T lj = T(0.5) * (a0 + b0);
    for (int c = 0; c < CS; ++c) *cluster.map_shared_rank(lam + j, c) = lj;
  }
  cluster.sync();
  const T pivmin = Tiny<T>::pivmin(tn);
  // inverse iteration of the own eigenvalues
  for (int k = tid; k < nown; k += kThreadsC) {
    const int j = rank + k * CS;
    for (int i = 0; i < n; ++i) V[int64_t(i) * B.ld + j] = T(1) + T(0.25) * T((i * 7919 + j * 104729) % 97) / T(97);
    T s = T(1);
    for (int it = 0; it < kInvIterC; ++it) s = inv_solve_c(dv, ev, n, lam[j], pivmin, s, V, Bt, B.ld, j);
    for (int i = 0; i < n; ++i) V[int64_t(i) * B.ld + j] *= s;
  }
  __threadfence();
  cluster.sync();  // every column written before cluster members are redone
  // near-degenerate clusters [c0, c1): the CTA with c0 % CS == rank redoes
  // them, one warp per cluster, re-orthogonalising against earlier members
  int *cl = reinterpret_cast<int *>(u);  // u, q are free: up to n pairs
  if (tid == 0) {
    int c = 0, k = 0;
    const T gap = Tiny<T>::gap * max(tn, T(1e-30));
    while (k < n) {
      int e2 = k + 1;
      while (e2 < n && lam[e2] - lam[e2 - 1] <= gap) ++e2;
      if (e2 - k > 1 && k % CS == rank) {
        cl[2 * c] = k;
        cl[2 * c + 1] = e2;
        ++c;
      }
      k = e2;
    }
    ctl->ncl = c;
  }
  __syncthreads();
  const int ncl = ctl->ncl;
  // each warp iterates its members in the (now free) matrix area of its own
  // shared memory: the member x and its LU pivots, 2n entries per warp, so
  // the sequential solves run at shared-memory latency
  T *stage = A + size_t(warp) * 2 * n;
  for (int cq = warp; cq < ncl; cq += kWarpsC) {
    const int c0 = cl[2 * cq], c1 = cl[2 * cq + 1];
    for (int j = c0; j < c1; ++j) {
      T *xv = stage, *bv = stage + n;
      for (int i = lane; i < n; i += 32) xv[i] = V[int64_t(i) * B.ld + j];
      __syncwarp();
      for (int rep = 0; rep < 2; ++rep) {
        if (lane == 0) inv_solve_c(dv, ev, n, lam[j], pivmin, T(1), xv, bv, 1, 0);
        __syncwarp();
        for (int k = c0; k < j; ++k) {  // earlier members are final in V
          T dot = T(0);
          for (int i = lane; i < n; i += 32) dot += V[int64_t(i) * B.ld + k] * xv[i];
          dot = warp_sum_c(dot);
          for (int i = lane; i < n; i += 32) xv[i] -= dot * V[int64_t(i) * B.ld + k];
          __syncwarp();
        }
        T nrm = T(0);
        for (int i = lane; i < n; i += 32) nrm += xv[i] * xv[i];
        nrm = warp_sum_c(nrm);
        const T scn = T(1) / sqrt_c(max(nrm, Tiny<T>::small));
        for (int i = lane; i < n; i += 32) xv[i] *= scn;
        __syncwarp();
      }
      for (int i = lane; i < n; i += 32) V[int64_t(i) * B.ld + j] = xv[i];
      __syncwarp();
    }
  }
  for (int k = tid; k < nown; k += kThreadsC) {
    const int j = rank + k * CS;
    B.E[j] = double(lam[j]);
  }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

template <typename T, int CS>
cudaError_t launch_cs(const EigBlock *blocks, int nblocks, int max_n, cudaStream_t s) {
  const size_t bytes = cluster_smem<T>(max_n, CS);
  auto kern = k_eig_cluster<T, CS>;
  ensure_smem_limit(reinterpret_cast<const void *>(kern), int(bytes));
  if (CS > 8) ensure_nonportable_cluster(reinterpret_cast<const void *>(kern));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(nblocks * CS), 1, 1);
  cfg.blockDim = dim3(kThreadsC, 1, 1);
  cfg.dynamicSmemBytes = bytes;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, blocks);
}

constexpr size_t kClusterSmemMax = 225 * 1024;

// Whether clusters of 16 CTAs (above the portable 8) with a full shared
// memory each can run on the current device.
bool sixteen_supported(bool fp64) {
  const void *k = fp64 ? reinterpret_cast<const void *>(k_eig_cluster<double, 16>)
                       : reinterpret_cast<const void *>(k_eig_cluster<float, 16>);
  ensure_smem_limit(k, int(kClusterSmemMax));
  ensure_nonportable_cluster(k);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(16, 1, 1);
  cfg.blockDim = dim3(kThreadsC, 1, 1);
  cfg.dynamicSmemBytes = kClusterSmemMax;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 16;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int ncl = 0;
  const cudaError_t rc = cudaOccupancyMaxActiveClusters(&ncl, k, &cfg);
  if (rc != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return ncl > 0;
}

}  // namespace

int eig_cluster_size_for(int n, bool fp64) {
  for (int cs : {8, 16}) {
    const size_t b = fp64 ? cluster_smem<double>(n, cs) : cluster_smem<float>(n, cs);
    if (b > kClusterSmemMax) continue;
    if (cs == 16) {
      static thread_local int dev_seen = -1, ok16[2] = {0, 0};
      int dev = 0;
      cudaGetDevice(&dev);
      if (dev != dev_seen) {
        ok16[0] = sixteen_supported(false) ? 1 : 0;
        ok16[1] = sixteen_supported(true) ? 1 : 0;
        dev_seen = dev;
      }
      if (!ok16[fp64 ? 1 : 0]) return 0;
    }
    return cs;
  }
  return 0;
}

cudaError_t launch_eig_cluster(const EigBlock *blocks, int nblocks, int max_n, int cs, bool fp64, cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  if (cs != 8 && cs != 16) return cudaErrorInvalidValue;
  if (fp64) return cs == 16 ? launch_cs<double, 16>(blocks, nblocks, max_n, s)
                            : launch_cs<double, 8>(blocks, nblocks, max_n, s);
  return cs == 16 ? launch_cs<float, 16>(blocks, nblocks, max_n, s) : launch_cs<float, 8>(blocks, nblocks, max_n, s);
}

}  // namespace nrg
