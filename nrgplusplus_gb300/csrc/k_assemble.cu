// Block Hamiltonian assembly (reference: nrgcore::create_next_hamiltonians,
// nrgcore.hpp:146-230).
//
// One flattened grid covers every non-empty block of every run in the batch;
// each CTA owns a 1024-element chunk of one block and each thread computes
// whole output elements in "gather" form: the element's diagonal value (if
// any) plus every hopping term that lands on it, added in the reference's
// loop order (sub-block a, sub-block b, operator).  No atomics, every H
// element is written exactly once with coalesced row-major stores, and the
// kept f-dagger blocks are read along their rows.
#include "nrg_internal.h"

namespace nrg {
namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 4;
constexpr int kChunk = kThreads * kPerThread;

__device__ __forceinline__ int find_sub(const AsmSub *subs, int nsub, int r) {
  int s = 0;
  while (s + 1 < nsub && r >= subs[s + 1].off) ++s;
  return s;
}

__global__ void __launch_bounds__(kThreads)
k_assemble(const AsmBlock *__restrict__ blocks, int nblocks, const AsmSub *__restrict__ subs,
           const int2 *__restrict__ pairs, const AsmTerm *__restrict__ terms) {
  // locate the block owning this chunk (chunk0 is increasing)
  const int64_t chunk = blockIdx.x;
  int lo = 0, hi = nblocks - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (blocks[mid].chunk0 <= chunk) lo = mid; else hi = mid - 1;
  }
  const AsmBlock B = blocks[lo];
  const AsmSub *S = subs + B.sub0;
  const int2 *P = pairs + B.pair0;
  const int64_t n = B.n;
  const int64_t base = (chunk - B.chunk0) * kChunk;

#pragma unroll
  for (int u = 0; u < kPerThread; ++u) {
    const int64_t e = base + u * kThreads + threadIdx.x;
    if (e >= n * n) break;
    const int r = int(e / n), c = int(e - int64_t(r) * n);
    const int sa = find_sub(S, B.nsub, r), sb = find_sub(S, B.nsub, c);
    const AsmSub A = S[sa], C = S[sb];
    const int ra = r - A.off, ca = c - C.off;
    const int ita = ra % A.k, ila = ra / A.k;
    const int itc = ca % C.k, ilc = ca / C.k;
    double h = 0.0;
    if (r == c) {  // diagonal: (E_prev - shift) * rescale + E_bath  (:179-185)
      h = (A.eprev[ita] - B.shift) * B.rescale + A.ebath[ila];
    }
    // direct contribution of pair (sa, sb) and transposed one of (sb, sa),
    // in the reference's (a, b, op) loop order.
    const int first = (sa <= sb) ? 0 : 1;
    for (int pass = 0; pass < 2; ++pass) {
      const bool direct = (pass == first);
      if (!direct && sa == sb) continue;  // same pair: handled below
      const int2 rg = direct ? P[sa * B.nsub + sb] : P[sb * B.nsub + sa];
      for (int t = rg.x; t < rg.y; ++t) {
        const AsmTerm T = terms[t];
        if (direct) {
          // row sub a (it=ita, il=ila), column sub b (it'=itc, il'=ilc)
          double aa = T.F[int64_t(ita) * T.ldf + itc] * T.fb[ilc * A.d + ila] * T.chi;
          h += aa * T.t;
          if (sa == sb) {  // transposed write of the same term lands here too
            double bb = T.F[int64_t(itc) * T.ldf + ita] * T.fb[ila * C.d + ilc] * T.chi;
            h += bb * T.t;
          }
        } else {
          // term (sb, sa): its row index is c, its column index is r
          double aa = T.F[int64_t(itc) * T.ldf + ita] * T.fb[ila * C.d + ilc] * T.chi;
          h += aa * T.t;
        }
      }
    }
    B.H[int64_t(r) * B.ld + c] = h;
  }
}

}  // namespace

void launch_assemble(const AsmBlock *blocks, int nblocks, int64_t nchunks, const AsmSub *subs,
                     const int2 *pairs, const AsmTerm *terms, cudaStream_t s) {
  if (nblocks == 0 || nchunks == 0) return;
  k_assemble<<<unsigned(nchunks), kThreads, 0, s>>>(blocks, nblocks, subs, pairs, terms);
}

}  // namespace nrg
