// FP64-accurate GEMM on the tensor cores (Ozaki-type digit splitting).
//
// Every FP64 operand block is split once (k_split) into 8 bf16 "digit planes":
// with e = ilogb(max|x|) + 1 over the block, X = rint(x * 2^(55-e)) is an
// integer with |X| <= 2^55, written in balanced base 128 as
//     X = sum_p a_p 128^(7-p),   a_p integer in [-64, 64]
// so x = 2^(e-55) sum_p a_p 128^(7-p) to within 2^(e-56).  Each a_p is exact
// in bf16.  A product then is
//     A B = 2^(eA+eB-110) sum_{p,q} 128^(14-p-q) (a_p b_q)
// The digit products are exact in FP32 (|a_p b_q| <= 2^12) and so are their
// sums while |sum| <= 2^24: grouping the pairs by d = p + q (d <= 7; the
// dropped groups weigh below 2^-51 of the result scale) and accumulating each
// group over at most 512 k-terms keeps every partial sum an exact integer.
//
// k_gemm_oz runs the 36 pair products on the 5th-generation tensor cores:
// one CTA owns a 128 x 64 output tile, the eight group sums live in tensor
// memory (TMEM: 8 accumulators x 64 FP32 columns = all 512 columns, lane =
// output row), and one thread issues tcgen05.mma (kind::f16, bf16 inputs,
// FP32 accumulation, M = 128, N = 64, K = 16) on operand tiles that one
// producer thread stages in shared memory with TMA tensor copies
// (cp.async.bulk.tensor, one tensor map per operand view, encoded on the
// host) whose boxes land directly in the canonical no-swizzle core-matrix
// layouts (K-major or MN-major per operand, so transposed operands need no
// transpose).  A four-stage ring overlaps the copies of later k-steps with
// the MMAs of the current one; tcgen05.commit arrives on one mbarrier per
// stage when its MMAs are done.  The group sums are folded into the FP64
// output once per run of contributions that share a scale (at most 512
// deep) by eight warps, two per TMEM lane quadrant: tcgen05.ld to registers,
// integer Horner over the groups, one FP64 fma per element.  Every mbarrier wait is bounded; a wait
// that runs out sets *err, and the kernel drains and releases TMEM.
#include <cuda.h>
#include <cuda_bf16.h>

#include "nrg_internal.h"

namespace nrg {
namespace {

constexpr int kPlanes = 8;
constexpr int kChunkK = 512;
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---------------------------------------------------------------- split
// Two grid-wide passes over the padded elements of every task (chunks of
// kSplitChunk, task located by binary search on the chunk prefix):
//   k_split_max:    per-task max |x| by atomicMax on the IEEE bits (for
//                   non-negative doubles the bit order is the value order);
//   k_split_digits: exponent from the max, then the 8 digits per element.
// Both work on the IEEE-754 fields with integer instructions only: GB300's
// FP64 pipe issues about 2 operations per clock per SM, 64 times fewer than
// its integer pipes, and the split touches every element of every operand.
// Each thread loads its 16 elements before it uses any of them (16
// independent loads in flight per thread).
constexpr int kSplitThreads = 256, kSplitPer = 16, kSplitChunk = kSplitThreads * kSplitPer;
// block exponent of a task whose max is Inf or NaN: 2^(eA+eB-61) overflows,
// so every product with it is NaN and the refinement's convergence check
// sends the block to the FP64 solver
constexpr int kNonFiniteExp = 4096;

__device__ __forceinline__ int find_task(const int64_t *chunk0, int ntasks, int64_t chunk) {
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (chunk0[mid] <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// e with max|x| < 2^e, i.e. ilogb(max) + 1 (0 for an all-zero task)
__device__ __forceinline__ int split_exp(unsigned long long maxbits) {
  if (maxbits == 0) return 0;
  const int ef = int(maxbits >> 52);
  if (ef == 0x7FF) return kNonFiniteExp;
  if (ef == 0) return -1010 - __clzll(static_cast<long long>(maxbits));  // subnormal maximum
  return ef - 1022;
}

// rint(x * 2^s), ties to even, from the fields of x = m 2^ex (m < 2^53):
// shifts of m instead of an FP64 multiply and conversion.  The caller's s
// keeps |x| 2^s < 2^55, so a left shift cannot overflow.
__device__ __forceinline__ long long scale_round(unsigned long long b, int s) {
  const int ef = int((b >> 52) & 0x7FF);
  unsigned long long m = b & ((1ull << 52) - 1);
  int ex = -1074;
  if (ef) {
    m |= 1ull << 52;
    ex = ef - 1075;
  }
  const int sh = ex + s;
  unsigned long long q;
  if (sh >= 0) {
    q = m << sh;
  } else if (sh <= -55) {
    q = 0;  // below half a unit
  } else {
    const int r = -sh;
    q = m >> r;
    const unsigned long long rem = m & ((1ull << r) - 1), half = 1ull << (r - 1);
    q += (rem > half || (rem == half && (q & 1))) ? 1 : 0;
  }
  return (b >> 63) ? -static_cast<long long>(q) : static_cast<long long>(q);
}

// bf16 bits of a small integer (|a| <= 64): 1.5 2^23 + a is exact in FP32,
// subtracting 1.5 2^23 leaves float(a), whose low 16 bits are zero
__device__ __forceinline__ unsigned short small_int_bf16(int a) {
  return static_cast<unsigned short>(__float_as_uint(__int_as_float(0x4B400000 + a) - 12582912.0f) >> 16);
}

// balanced base-128 digits of |X| <= 2^55, least significant first, in
// 32-bit arithmetic: 4 digits from the low 28 bits, their carry into the
// high part, 3 more digits; the most significant digit is the remainder
// itself, which lies in [-64, 64] (the lower digits sum to less than
// 0.504 * 128^7)
__device__ __forceinline__ void store_digits(long long X, unsigned short *pl, int64_t pstride, int64_t i) {
  int L = int(X & 0xFFFFFFF), H = int(X >> 28);
#pragma unroll
  for (int p = kPlanes - 1; p >= 4; --p) {
    const int a = ((L + 64) & 127) - 64;
    L = (L - a) >> 7;
    pl[int64_t(p) * pstride + i] = small_int_bf16(a);
  }
  H += L;
#pragma unroll
  for (int p = 3; p >= 1; --p) {
    const int a = ((H + 64) & 127) - 64;
    H = (H - a) >> 7;
    pl[int64_t(p) * pstride + i] = small_int_bf16(a);
  }
  pl[i] = small_int_bf16(H);
}

__global__ void __launch_bounds__(kSplitThreads)
k_split_max(const SplitTask *__restrict__ tasks, const int64_t *__restrict__ chunk0, int ntasks,
            unsigned long long *__restrict__ maxbits) {
  const int t = find_task(chunk0, ntasks, blockIdx.x);
  const SplitTask T = tasks[t];
  const int base = int(int64_t(blockIdx.x) - chunk0[t]) * kSplitChunk;
  const int nel = T.rows * T.ldp;
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(T.src);
  unsigned long long v[kSplitPer];
#pragma unroll
  for (int u = 0; u < kSplitPer; ++u) {
    const int i = base + u * kSplitThreads + int(threadIdx.x);
    const int r = unsigned(i) / unsigned(T.ldp), c = i - r * T.ldp;
    v[u] = (i < nel && c < T.cols) ? src[int64_t(r) * T.ld + c] : 0ull;
  }
  unsigned long long m = 0;
#pragma unroll
  for (int u = 0; u < kSplitPer; ++u) m = max(m, v[u] & 0x7FFFFFFFFFFFFFFFull);
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(maxbits + t, m);
}

__global__ void __launch_bounds__(kSplitThreads)
k_split_digits(const SplitTask *__restrict__ tasks, const int64_t *__restrict__ chunk0, int ntasks,
               const unsigned long long *__restrict__ maxbits) {
  const int t = find_task(chunk0, ntasks, blockIdx.x);
  const SplitTask T = tasks[t];
  const int e = split_exp(maxbits[t]);
  if (blockIdx.x == chunk0[t] && threadIdx.x == 0) *T.exp = e;
  const int base = int(int64_t(blockIdx.x) - chunk0[t]) * kSplitChunk;
  const int nel = T.rows * T.ldp;
  const unsigned long long *src = reinterpret_cast<const unsigned long long *>(T.src);
  unsigned long long v[kSplitPer];
#pragma unroll
  for (int u = 0; u < kSplitPer; ++u) {
    const int i = base + u * kSplitThreads + int(threadIdx.x);
    const int r = unsigned(i) / unsigned(T.ldp), c = i - r * T.ldp;
    v[u] = (i < nel && c < T.cols) ? src[int64_t(r) * T.ld + c] : 0ull;
  }
  unsigned short *pl = static_cast<unsigned short *>(T.planes);
  const bool finite = e != kNonFiniteExp;
#pragma unroll
  for (int u = 0; u < kSplitPer; ++u) {
    const int i = base + u * kSplitThreads + int(threadIdx.x);
    if (i < nel) store_digits(finite ? scale_round(v[u], 55 - e) : 0ll, pl, T.pstride, i);
  }
}

// ----------------------------------------------------------------- GEMM
constexpr int TM = 128, TN = 64, TK = 16;  // output tile, k-step (one MMA)
constexpr int kStages = 4;
constexpr int kTcThreads = 288;  // 8 consumer warps + 1 producer warp (one issuing thread)
constexpr int kConsumers = 256;
constexpr int kATile = TM * TK * 2, kBTile = TN * TK * 2;  // bytes per plane
constexpr int kAStage = kPlanes * kATile;                  // 32 KB
constexpr int kStageBytes = kPlanes * (kATile + kBTile);   // 48 KB
constexpr int kChunkBox = kPlanes * TK * 32;               // 4 KB: 8 planes x 16 k x 16 elements
constexpr int kWaitLimit = 1 << 24;                        // bounded mbarrier polls

// Stage layouts.  Every operand tile of a stage is written by TMA boxes with
// the 32-byte swizzle straight into the canonical 32-byte-swizzled layouts
// (rows of 32 bytes, the two 16-byte halves of a row exchanged in every
// other group of four rows; atoms of 8 rows = 256 bytes, 256-byte aligned):
//   K-major (rows of m or n, 16 k each):  one box {16 k, R rows, 8 planes}:
//     [plane][row][16 k]; plane p at p * R * 32, 8-row groups 256 bytes apart
//     (SBO; the k extent is one atom wide, LBO unused);
//   MN-major (rows of k, 16 m or n each): R / 16 boxes {16 m, 16 k, 8 planes},
//     one per 16-wide chunk: [chunk][plane][k][16 m]; plane p at p * 512,
//     8-k groups 256 bytes apart (SBO), chunks 4 KB apart (LBO).
// A box row is 32 bytes (16-byte rows halve the TMA unit's throughput).
// The boxes of a stage always total kStageBytes (rows, k and planes beyond
// the operand view are zero-filled by the TMA unit), which the producer
// announces with one expect_tx on the stage's full barrier.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((addr >> 4) & 0x3FFF) | (uint64_t((lbo >> 4) & 0x3FFF) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFF) << 32) | (uint64_t(1) << 46) |  // version 1
         (uint64_t(6) << 61);                                            // 32-byte swizzle
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const OzTensorMap *map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred P1;\n mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n"
        " selp.b32 %0, 1, 0, P1;\n}\n"
        : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// The boxes of the k-step [k0, k0 + 16) of all 8 planes of op(A) (128 x 16)
// and op(B) (64 x 16) into stage `st` (shared address), completing on `bar`.
// x coordinates (k0, m0 + 16 o, n0 + 16 o) are multiples of 16 elements:
// 32-byte aligned (TMA needs 16).
__device__ __forceinline__ void stage_tma(const OzContrib &q, const OzTensorMap *maps, int m0, int n0, int k0,
                                          uint32_t st, uint32_t bar) {
  const bool ta = q.trans & 1, tb = (q.trans >> 1) & 1;
  const OzTensorMap *ma = maps + q.tmA, *mb = maps + q.tmB;
  if (!ta) {
    tma_load_3d(st, ma, k0, m0, 0, bar);
  } else {
    for (int o = 0; o < TM / 16; ++o) tma_load_3d(st + o * kChunkBox, ma, m0 + 16 * o, k0, 0, bar);
  }
  const uint32_t sb = st + kAStage;
  if (tb) {
    tma_load_3d(sb, mb, k0, n0, 0, bar);
  } else {
    for (int o = 0; o < TN / 16; ++o) tma_load_3d(sb + o * kChunkBox, mb, n0 + 16 * o, k0, 0, bar);
  }
}

// Walks the k-steps of a group's contribution list (skipping empty ones).
struct StepIt {
  int c, k0;
  __device__ void skip_empty(const OzGroup &g, const OzContrib *cs) {
    while (c < g.c1 && cs[c].K <= 0) ++c;
  }
  __device__ void next(const OzGroup &g, const OzContrib *cs) {
    k0 += TK;
    if (k0 >= cs[c].K) {
      ++c;
      k0 = 0;
      skip_empty(g, cs);
    }
  }
};

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void consumer_sync() {  // warps 0-7 only
  asm volatile("bar.sync 1, 256;" ::: "memory");
}

// Warp roles: warp 8 lane 0 stages k-steps into a ring of kStages buffers
// with TMA boxes (a stage is released by the tcgen05.commit of its MMAs on
// empty[stage] and completes on full[stage] when its bytes have landed);
// warp 0 lane 0 issues the 36 MMAs of each step; warps 0-7 fold the group
// sums whenever the scale changes, 512 k-terms are used up, or the list ends
// (after a drain commit on `drain`): warp w reads TMEM lanes 32 (w mod 4) ..
// + 31 (the lane quadrant its id gives it access to) and columns
// 32 (w div 4) .. + 31 of each accumulator, so two warps share each
// quadrant's rows.  No CTA-wide barrier sits in the k-loop.
__global__ void __launch_bounds__(kTcThreads, 1)
k_gemm_oz(const GemmTile *__restrict__ tiles, const OzGroup *__restrict__ groups,
          const OzContrib *__restrict__ contribs, const OzTensorMap *__restrict__ maps, int *err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], drain;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  unsigned char *ring = smem_raw;
  const GemmTile t = tiles[blockIdx.x];
  const OzGroup g = groups[t.group];
  const int m0 = t.tm * TM, n0 = t.tn * TN;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int P = (g.planes >= 1 && g.planes <= kPlanes) ? g.planes : kPlanes;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < kStages; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[i])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[i])));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&drain)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    abort_flag = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;

  int nsteps = 0;
  for (int c = g.c0; c < g.c1; ++c)
    if (contribs[c].K > 0) nsteps += (contribs[c].K + TK - 1) / TK;

  if (warp >= 8) {
    // ------------------------------------------------------------- producer
    if (warp == 8 && lane == 0) {
      StepIt it{g.c0, 0};
      it.skip_empty(g, contribs);
      int issued = 0, cur = -1;
      const uint32_t ring0 = smem_u32(ring);
      for (int s = 0; s < nsteps; ++s) {
        const int st = s % kStages, use = s / kStages;
        if (use > 0 && !mbar_wait(smem_u32(&empty[st]), uint32_t((use - 1) & 1))) abort_flag = 1;
        if (abort_flag) break;
        const OzContrib &q = contribs[it.c];
        if (it.c != cur) {  // the tensor maps were written by a copy before the launch
          asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(maps + q.tmA) : "memory");
          asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(maps + q.tmB) : "memory");
          cur = it.c;
        }
        const uint32_t fb = smem_u32(&full[st]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(kStageBytes)
                     : "memory");
        stage_tma(q, maps, m0, n0, it.k0, ring0 + uint32_t(st * kStageBytes), fb);
        ++issued;
        it.next(g, contribs);
      }
      // no TMA write may be in flight when the CTA ends (after an abort the
      // consumer stops waiting for the stages)
      for (int s = (issued > kStages ? issued - kStages : 0); s < issued; ++s)
        mbar_wait(smem_u32(&full[s % kStages]), uint32_t((s / kStages) & 1));
    }
  } else {
    // ------------------------------------------------ MMA issue and folds
    StepIt it{g.c0, 0};
    it.skip_empty(g, contribs);
    int kacc = 0;
    double acc_scale = 0;
    bool first_fold = true;
    uint32_t drain_phase = 0;
    const uint32_t ring0 = smem_u32(ring);
    const int quad = warp & 3, half = warp >> 2;  // TMEM lane quadrant, column half
    const uint32_t tl = tmem + (uint32_t(32 * quad) << 16);
    const int gm = m0 + 32 * quad + lane;

    // Every consumer thread makes the same fold() calls (the fold points
    // depend only on the contribution list), so the named barrier at its end
    // is always reached by all 256; after an abort the waits and TMEM reads
    // are skipped (decided per warp, as tcgen05.ld is warp-collective).
    auto fold = [&]() {
      // drain: every MMA issued so far has completed
      if (__shfl_sync(0xffffffffu, abort_flag, 0) == 0) {
        if (tid == 0) mma_commit(smem_u32(&drain));
        if (!mbar_wait(smem_u32(&drain), drain_phase)) abort_flag = 1;
      }
      drain_phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;");
      // a warp whose 32 rows lie past M, and column chunks past N, have
      // nothing to fold (warp-uniform conditions: tcgen05.ld is collective)
      if (__shfl_sync(0xffffffffu, abort_flag, 0) == 0 && m0 + 32 * quad < g.M) {
        for (int cc = 32 * half; cc < 32 * half + 32 && n0 + cc < g.N; cc += 8) {
          uint32_t v[kPlanes][8];
#pragma unroll
          for (int d = 0; d < kPlanes; ++d) {
            if (d < P) {
              asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                           : "=r"(v[d][0]), "=r"(v[d][1]), "=r"(v[d][2]), "=r"(v[d][3]), "=r"(v[d][4]),
                             "=r"(v[d][5]), "=r"(v[d][6]), "=r"(v[d][7])
                           : "r"(tl + uint32_t(64 * d + cc)));
            } else {  // groups beyond the planes used are not computed
#pragma unroll
              for (int j = 0; j < 8; ++j) v[d][j] = 0u;
            }
          }
          asm volatile("tcgen05.wait::ld.sync.aligned;");
          if (gm < g.M) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const int gn = n0 + cc + j;
              if (gn >= g.N) continue;
              long long hi = __float2int_rz(__uint_as_float(v[0][j]));
#pragma unroll
              for (int d = 1; d < 5; ++d) hi = hi * 128 + __float2int_rz(__uint_as_float(v[d][j]));
              long long lo = __float2int_rz(__uint_as_float(v[5][j]));
#pragma unroll
              for (int d = 6; d < kPlanes; ++d) lo = lo * 128 + __float2int_rz(__uint_as_float(v[d][j]));
              const double h = fma(__ll2double_rn(hi), 2097152.0, __ll2double_rn(lo));  // 128^3
              double *cp = g.C + int64_t(gm) * g.ldc + gn;
              const double base = (first_fold && !g.accumulate) ? 0.0 : *cp;
              *cp = fma(acc_scale, h, base);
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      consumer_sync();  // TMEM read out before the next MMAs overwrite it
      kacc = 0;
      first_fold = false;
    };

    int scale_c = -1;  // contribution whose scale is in `scale`
    double scale = 0.0;
    for (int s = 0; s < nsteps; ++s) {
      const OzContrib &q = contribs[it.c];
      if (it.c != scale_c) {
        scale = fabs(q.alpha) * scalbn(1.0, *q.A.exp + *q.B.exp - 61);
        scale_c = it.c;
      }
      if (kacc > 0 && (scale != acc_scale || kacc + TK > kChunkK)) fold();
      acc_scale = scale;
      if (tid == 0 && !abort_flag) {
        const int st = s % kStages;
        if (!mbar_wait(smem_u32(&full[st]), uint32_t((s / kStages) & 1))) {
          abort_flag = 1;
        } else {
          asm volatile("tcgen05.fence::after_thread_sync;");
          const bool ta = q.trans & 1, tb = (q.trans >> 1) & 1;
          const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(q.alpha < 0.0) << 13) |
                                 (uint32_t(ta) << 15) | (uint32_t(!tb) << 16) | (uint32_t(TN >> 3) << 17) |
                                 (uint32_t(TM >> 4) << 24);
          const uint32_t sa = ring0 + uint32_t(st * kStageBytes), sb = sa + kAStage;
          // plane p of A at a0 + p * astep, plane q of B at b0 + q * bstep
          // (the stage layouts above)
          const uint64_t a0 = ta ? smem_desc(sa, kChunkBox, 256) : smem_desc(sa, 16, 256);
          const uint64_t b0 = tb ? smem_desc(sb, 16, 256) : smem_desc(sb, kChunkBox, 256);
          const uint32_t astep = ta ? TK * 32 : TM * 32, bstep = tb ? TN * 32 : TK * 32;
          const uint32_t first = kacc == 0 ? 0u : 1u;
#pragma unroll
          for (int p = 0; p < kPlanes; ++p) {
#pragma unroll
            for (int qd = 0; qd < kPlanes - p; ++qd) {
              if (p + qd >= P) continue;  // uniform: fewer planes, fewer products
              const uint64_t ad = a0 + uint64_t((p * astep) >> 4);
              const uint64_t bd = b0 + uint64_t((qd * bstep) >> 4);
              const uint32_t acc = p > 0 ? 1u : first;  // the first pair of each group starts it
              asm volatile(
                  "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                  " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
                      tmem + uint32_t(64 * (p + qd))),
                  "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
          }
          mma_commit(smem_u32(&empty[st]));
        }
      }
      kacc += TK;
      it.next(g, contribs);
    }
    if (nsteps > 0) fold();
    if (nsteps == 0 && !g.accumulate) {  // empty contribution list: C = 0
      for (int i = tid; i < TM * TN; i += kConsumers) {
        const int r = i / TN, c = i - r * TN;
        if (m0 + r < g.M && n0 + c < g.N) g.C[int64_t(m0 + r) * g.ldc + n0 + c] = 0.0;
      }
    }
    if (abort_flag && tid == 0) {  // let issued MMAs finish (bounded) before TMEM is released
      mma_commit(smem_u32(&drain));
      mbar_wait(smem_u32(&drain), drain_phase);
      atomicExch(err, 1);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

constexpr size_t kGemmSmem = size_t(kStages) * kStageBytes;

}  // namespace

int split_chunk_elements() { return kSplitChunk; }

void launch_split_grid(const SplitTask *tasks, const int64_t *chunk0, int ntasks, int64_t nchunks,
                       unsigned long long *maxbits, cudaStream_t s) {
  if (ntasks == 0 || nchunks == 0) return;
  cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long) * ntasks, s);
  k_split_max<<<unsigned(nchunks), kSplitThreads, 0, s>>>(tasks, chunk0, ntasks, maxbits);
  k_split_digits<<<unsigned(nchunks), kSplitThreads, 0, s>>>(tasks, chunk0, ntasks, maxbits);
}

void launch_gemm_oz(const GemmTile *tiles, int ntiles, const OzGroup *groups, const OzContrib *contribs,
                    const OzTensorMap *maps, int *err, cudaStream_t s) {
  if (ntiles == 0) return;
  ensure_smem_limit(reinterpret_cast<const void *>(k_gemm_oz), int(kGemmSmem));
  k_gemm_oz<<<ntiles, kTcThreads, kGemmSmem, s>>>(tiles, groups, contribs, maps, err);
}

bool encode_oz_map(OzTensorMap *out, const OzOperand &o, int inner, int outer, int planes, int box_outer) {
  using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  // the driver's encoder, looked up once (the library links the runtime only)
  static const Encode enc = [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<Encode>(f);
  }();
  static_assert(sizeof(CUtensorMap) == sizeof(OzTensorMap), "tensor map size");
  if (!enc || inner <= 0 || outer <= 0 || planes <= 0 || planes > kPlanes) return false;
  const cuuint64_t strides[2] = {cuuint64_t(o.ld) * 2, cuuint64_t(o.pstride) * 2};
  const cuuint32_t box[3] = {16, cuuint32_t(box_outer), cuuint32_t(kPlanes)}, es[3] = {1, 1, 1};
  // planes beyond `planes` are zero-filled (no bytes read) when the driver
  // takes a box deeper than the tensor; otherwise all 8 (always allocated)
  for (const int np : {planes, kPlanes}) {
    const cuuint64_t dims[3] = {cuuint64_t(inner), cuuint64_t(outer), cuuint64_t(np)};
    if (enc(reinterpret_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
            const_cast<__nv_bfloat16 *>(o.p), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
      return true;
  }
  return false;
}

}  // namespace nrg
