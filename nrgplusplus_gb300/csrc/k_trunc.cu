// Global truncation by device select (reference: nrgcore::discard_higher_energies,
// nrgcore.hpp:269-327).
//
// Every block's eigenvalues arrive sorted ascending from the eigensolver, so
// the run-wide sorted list (all_eigenvalue) is a merge: each element finds its
// global rank with one binary search per other block of its run (ties ordered
// by block index, which gives a permutation) and scatters itself.  Then one
// CTA per run applies the reference's rule exactly:
//   total <= Nkeep : keep everything, no shift
//   otherwise      : thr = sorted[Nkeep]; keep E < thr + 1e-8 per block
//                    (a prefix, counted by binary search); shift by E_min when
//                    more than Nkeep states are kept.
// The comparisons are the reference's FP64 comparisons on the same values,
// so the kept counts follow the eigenvalues bit for bit.
#include "nrg_internal.h"

namespace nrg {
namespace {

constexpr double kErrorbarInEnergy = 1e-8;  // nrgcore.hpp:338

__device__ __forceinline__ int lower_bound(const double *a, int n, double x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int upper_bound(const double *a, int n, double x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__global__ void k_rank(const TruncRun *__restrict__ runs, const TruncBlock *__restrict__ blocks,
                       const int *__restrict__ elem_block, const int *__restrict__ block_run,
                       int nelem) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  const int b = elem_block[e];
  const TruncBlock B = blocks[b];
  const TruncRun R = runs[block_run[b]];
  const int p = e - B.e0;
  const double x = B.E[p];
  int64_t rank = p;
  for (int o = R.b0; o < R.b1; ++o) {
    if (o == b) continue;
    const TruncBlock O = blocks[o];
    rank += (o < b) ? upper_bound(O.E, O.n, x) : lower_bound(O.E, O.n, x);
  }
  R.sorted[rank] = x;
}

__global__ void k_select(const TruncRun *__restrict__ runs, const TruncBlock *__restrict__ blocks,
                         int *__restrict__ kept, TruncResult *__restrict__ res) {
  __shared__ long long ssum[32];
  const TruncRun R = runs[blockIdx.x];
  const int64_t total = R.e1 - R.e0;
  const bool trunc = total > R.nkeep;
  const double thr = trunc ? R.sorted[R.nkeep] : R.sorted[total - 1];
  long long local = 0;
  for (int b = R.b0 + threadIdx.x; b < R.b1; b += blockDim.x) {
    const TruncBlock B = blocks[b];
    const int k = trunc ? lower_bound(B.E, B.n, thr + kErrorbarInEnergy) : B.n;
    kept[b] = k;
    local += k;
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) ssum[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long s = 0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) s += ssum[w];
    TruncResult r;
    r.emin = R.sorted[0];
    r.thr = thr;
    r.kept_total = s;
    r.total = total;
    r.truncated = trunc ? 1 : 0;
    r.pad = 0;
    res[blockIdx.x] = r;
  }
}

}  // namespace

void launch_truncate(const TruncRun *runs, int nruns, const TruncBlock *blocks, int nblocks,
                     const int *elem_block, int nelem, int *kept, TruncResult *res,
                     cudaStream_t s) {
  // block_run is stored right after elem_block by the host (nelem + nblocks ints)
  const int *block_run = elem_block + nelem;
  if (nelem > 0) k_rank<<<(nelem + 255) / 256, 256, 0, s>>>(runs, blocks, elem_block, block_run, nelem);
  if (nruns > 0) k_select<<<nruns, 256, 0, s>>>(runs, blocks, kept, res);
}

}  // namespace nrg
