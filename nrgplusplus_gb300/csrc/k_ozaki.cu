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
// The 8 group sums are combined once per output element and K-chunk by an
// integer Horner (h = G_0; h = 128 h + G_d) and one FP64 fma, so the FP64
// pipe does a few operations per output element instead of K.  The bf16 products use mma.sync m16n8k16 with
// FP32 accumulation; the result matches an FP64 GEMM to FP64 round-off.
#include <cuda_bf16.h>

#include "nrg_internal.h"

namespace nrg {
namespace {

constexpr int kPlanes = 8;
constexpr int kChunkK = 512;
constexpr int BM = 64, BN = 64, BK = 32;
constexpr int kThreads = 256;
// shared-memory row pitches (bf16 elements): 80-byte and 144-byte rows make
// the 8 row addresses of every ldmatrix fall in distinct 16-byte bank groups
constexpr int kPitchK = BK + 8;   // tiles stored [m or n][k]
constexpr int kPitchMN = BM + 8;  // tiles stored [k][m or n]
constexpr int kTileElems = kPlanes * BM * kPitchK;  // >= kPlanes * BK * kPitchMN

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t &r0, uint32_t &r1, uint32_t &r2, uint32_t &r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------- split
// Two grid-wide passes over every element of every task (chunks of 1024
// elements, task located by binary search on the chunk prefix):
//   k_split_max:    per-task max |x| by atomicMax on the IEEE bits (for
//                   non-negative doubles the bit order is the value order);
//   k_split_digits: exponent from the max, then the 8 digits per element.
__device__ __forceinline__ int find_task(const int64_t *chunk0, int ntasks, int64_t chunk) {
  int lo = 0, hi = ntasks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (chunk0[mid] <= chunk) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(256)
k_split_max(const SplitTask *__restrict__ tasks, const int64_t *__restrict__ chunk0, int ntasks,
            unsigned long long *__restrict__ maxbits) {
  const int t = find_task(chunk0, ntasks, blockIdx.x);
  const SplitTask T = tasks[t];
  const int64_t base = (int64_t(blockIdx.x) - chunk0[t]) * 1024;
  const int64_t nel = int64_t(T.rows) * T.cols;
  double m = 0.0;
  for (int u = 0; u < 4; ++u) {
    const int64_t i = base + u * 256 + threadIdx.x;
    if (i < nel) {
      const int r = int(i / T.cols), c = int(i - int64_t(r) * T.cols);
      m = fmax(m, fabs(T.src[int64_t(r) * T.ld + c]));
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0)
    atomicMax(maxbits + t, static_cast<unsigned long long>(__double_as_longlong(m)));
}

__global__ void __launch_bounds__(256)
k_split_digits(const SplitTask *__restrict__ tasks, const int64_t *__restrict__ chunk0, int ntasks,
               const unsigned long long *__restrict__ maxbits) {
  const int t = find_task(chunk0, ntasks, blockIdx.x);
  const SplitTask T = tasks[t];
  const double mx = __longlong_as_double(static_cast<long long>(maxbits[t]));
  const int e = (mx > 0.0 && isfinite(mx)) ? ilogb(mx) + 1 : 0;
  if (blockIdx.x == chunk0[t] && threadIdx.x == 0) *T.exp = e;
  const int64_t base = (int64_t(blockIdx.x) - chunk0[t]) * 1024;
  const int64_t nel = int64_t(T.rows) * T.ldp;
  __nv_bfloat16 *pl = static_cast<__nv_bfloat16 *>(T.planes);
  for (int u = 0; u < 4; ++u) {
    const int64_t i = base + u * 256 + threadIdx.x;
    if (i >= nel) break;
    const int r = int(i / T.ldp), c = int(i - int64_t(r) * T.ldp);
    long long X = 0;
    if (c < T.cols) X = llrint(scalbn(T.src[int64_t(r) * T.ld + c], 55 - e));
    // balanced base-128 digits, least significant first; the most
    // significant digit is the remainder itself, which lies in [-64, 64]
#pragma unroll
    for (int p = kPlanes - 1; p >= 1; --p) {
      const long long a = ((X + 64) & 127) - 64;
      X = (X - a) >> 7;
      pl[int64_t(p) * T.pstride + i] = __float2bfloat16_rn(float(a));
    }
    pl[i] = __float2bfloat16_rn(float(X));
  }
}

__global__ void __launch_bounds__(256) k_split(const SplitTask *__restrict__ tasks) {
  __shared__ double red[8];
  const SplitTask T = tasks[blockIdx.x];
  const int64_t nel = int64_t(T.rows) * T.cols;
  double m = 0.0;
  for (int64_t i = threadIdx.x; i < nel; i += blockDim.x) {
    const int r = int(i / T.cols), c = int(i - int64_t(r) * T.cols);
    m = fmax(m, fabs(T.src[int64_t(r) * T.ld + c]));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  double mx = red[0];
  for (int w = 1; w < int(blockDim.x >> 5); ++w) mx = fmax(mx, red[w]);
  const int e = (mx > 0.0 && isfinite(mx)) ? ilogb(mx) + 1 : 0;
  if (threadIdx.x == 0) *T.exp = e;
  for (int64_t i = threadIdx.x; i < int64_t(T.rows) * T.ldp; i += blockDim.x) {
    const int r = int(i / T.ldp), c = int(i - int64_t(r) * T.ldp);
    long long X = 0;
    if (c < T.cols) X = llrint(scalbn(T.src[int64_t(r) * T.ld + c], 55 - e));
    // balanced base-128 digits, least significant first; the most
    // significant digit is the remainder itself, which lies in [-64, 64]
    // (|X| <= 2^55 and the lower digits sum to less than 0.504 * 128^7)
    __nv_bfloat16 *pl = static_cast<__nv_bfloat16 *>(T.planes);
#pragma unroll
    for (int p = kPlanes - 1; p >= 1; --p) {
      const long long a = ((X + 64) & 127) - 64;
      X = (X - a) >> 7;
      pl[int64_t(p) * T.pstride + i] = __float2bfloat16_rn(float(a));
    }
    pl[i] = __float2bfloat16_rn(float(X));
  }
}

// ----------------------------------------------------------------- GEMM
struct Frag {
  uint32_t a[kPlanes][4];
};

__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
  const uint32_t d = smem_u32(dst);
  const int sz = valid ? 16 : 0;  // 0: no bytes read, 16 zero bytes written
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(sz));
}
// 8-element vector along k whose tail may run past kend (sub-matrix views
// whose rows continue with real data): copy the first `nvalid` elements,
// zero the rest.  cp.async src-size is in bytes (2 per element).
__device__ __forceinline__ void cp_async16_k(void *dst, const void *src, int nvalid) {
  const uint32_t d = smem_u32(dst);
  const int sz = nvalid <= 0 ? 0 : (nvalid >= 8 ? 16 : 2 * nvalid);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Stage one 32-deep k-slice of every digit plane of op(A) (64 x 32) and
// op(B) (32 x 64) into shared memory with 16-byte cp.async copies.  Plane
// rows are zero-padded to a multiple of 8 elements and row starts are
// 16-byte aligned, so every 8-element vector is either wholly inside the
// operand or zero-filled.
__device__ __forceinline__ void stage_tiles(const OzContrib &q, bool ta, bool tb, int M, int N, int m0,
                                            int n0, int k0, int kend, __nv_bfloat16 *As,
                                            __nv_bfloat16 *Bs) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int p = 0; p < kPlanes; ++p) {
    {  // A: 256 vectors per plane, one per thread
      const __nv_bfloat16 *base = q.A.p + int64_t(p) * q.A.pstride;
      if (!ta) {  // [m][k], 64 rows x 4 vectors
        const int mm = tid >> 2, v = tid & 3;
        const int gm = m0 + mm, gk = k0 + 8 * v;
        const bool ok = gm < M && gk < kend;
        cp_async16_k(As + (p * BM + mm) * kPitchK + 8 * v, ok ? base + int64_t(gm) * q.A.ld + gk : base,
                     ok ? kend - gk : 0);
      } else {    // [k][m], 32 rows x 8 vectors
        const int kk = tid >> 3, v = tid & 7;
        const int gk = k0 + kk, gm = m0 + 8 * v;
        const bool ok = gk < kend && gm < M;
        cp_async16(As + (p * BK + kk) * kPitchMN + 8 * v, ok ? base + int64_t(gk) * q.A.ld + gm : base, ok);
      }
    }
    {  // B
      const __nv_bfloat16 *base = q.B.p + int64_t(p) * q.B.pstride;
      if (tb) {   // [n][k]
        const int nn = tid >> 2, v = tid & 3;
        const int gn = n0 + nn, gk = k0 + 8 * v;
        const bool ok = gn < N && gk < kend;
        cp_async16_k(Bs + (p * BN + nn) * kPitchK + 8 * v, ok ? base + int64_t(gn) * q.B.ld + gk : base,
                     ok ? kend - gk : 0);
      } else {    // [k][n]
        const int kk = tid >> 3, v = tid & 7;
        const int gk = k0 + kk, gn = n0 + 8 * v;
        const bool ok = gk < kend && gn < N;
        cp_async16(Bs + (p * BK + kk) * kPitchMN + 8 * v, ok ? base + int64_t(gk) * q.B.ld + gn : base, ok);
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads, 1)
k_gemm_oz(const GemmTile *__restrict__ tiles, const OzGroup *__restrict__ groups,
          const OzContrib *__restrict__ contribs) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16 *As0 = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
  __nv_bfloat16 *Bs0 = As0 + 2 * kTileElems;
  double *Ct = reinterpret_cast<double *>(Bs0 + 2 * kTileElems);  // BM x BN FP64 totals
  const GemmTile t = tiles[blockIdx.x];
  const OzGroup g = groups[t.group];
  const int m0 = t.tm * BM, n0 = t.tn * BN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 3) * 16, wn = (warp >> 2) * 32;
  for (int i = tid; i < BM * BN; i += kThreads) Ct[i] = 0.0;

  // Group sums of consecutive contributions (and K-chunks) that share the
  // scale |alpha| 2^(eA+eB-61) stay in the same FP32 accumulators while their
  // total depth is <= kChunkK (every partial sum stays an exact integer below
  // 2^24); a negative alpha flips the sign bits of the A fragments.  The
  // accumulators are folded into the FP64 tile only when the scale changes,
  // the depth is used up, or the list ends.
  float acc[kPlanes][4][4];
#pragma unroll
  for (int d = 0; d < kPlanes; ++d)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[d][j][v] = 0.f;
  int kacc = 0;          // depth accumulated since the last fold
  double acc_scale = 0;  // its scale

  auto fold = [&]() {
    // exact group sums -> FP64: 32-bit conversions, Horner over the groups in
    // integers (groups 0-4 into hi <= 2^53, groups 5-7 into lo <= 2^39),
    // then one FP64 fma per element
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        long long hi = __float2int_rz(acc[0][j][v]);
#pragma unroll
        for (int d = 1; d < 5; ++d) hi = hi * 128 + __float2int_rz(acc[d][j][v]);
        long long lo = __float2int_rz(acc[5][j][v]);
#pragma unroll
        for (int d = 6; d < kPlanes; ++d) lo = lo * 128 + __float2int_rz(acc[d][j][v]);
        const double h = fma(__ll2double_rn(hi), 2097152.0, __ll2double_rn(lo));  // 128^3
        const int r = wm + (lane >> 2) + (v >> 1) * 8;
        const int col = wn + j * 8 + (lane & 3) * 2 + (v & 1);
        Ct[r * BN + col] = fma(acc_scale, h, Ct[r * BN + col]);
#pragma unroll
        for (int d = 0; d < kPlanes; ++d) acc[d][j][v] = 0.f;
      }
    kacc = 0;
  };

  for (int c = g.c0; c < g.c1; ++c) {
    const OzContrib q = contribs[c];
    const bool ta = q.trans & 1, tb = (q.trans >> 1) & 1;
    const double scale = fabs(q.alpha) * scalbn(1.0, *q.A.exp + *q.B.exp - 61);
    const uint32_t neg = (q.alpha < 0.0) ? 0x80008000u : 0u;
    for (int kc = 0; kc < q.K; kc += kChunkK) {
      const int kend = min(q.K, kc + kChunkK);
      const int nst = (kend - kc + BK - 1) / BK;
      if (kacc > 0 && (scale != acc_scale || kacc + (kend - kc) > kChunkK)) fold();
      acc_scale = scale;
      kacc += kend - kc;
      __syncthreads();  // previous users of both buffers are done
      stage_tiles(q, ta, tb, g.M, g.N, m0, n0, kc, kend, As0, Bs0);
      cp_async_commit();
      for (int st = 0; st < nst; ++st) {
        const int buf = st & 1;
        if (st + 1 < nst) {
          stage_tiles(q, ta, tb, g.M, g.N, m0, n0, kc + (st + 1) * BK, kend, As0 + (buf ^ 1) * kTileElems,
                      Bs0 + (buf ^ 1) * kTileElems);
          cp_async_commit();
          cp_async_wait<1>();
        } else {
          cp_async_wait<0>();
        }
        __syncthreads();
        const __nv_bfloat16 *As = As0 + buf * kTileElems;
        const __nv_bfloat16 *Bs = Bs0 + buf * kTileElems;
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
          Frag fa;
#pragma unroll
          for (int p = 0; p < kPlanes; ++p) {
            if (!ta) {
              // As[m][k]: rows wm + (lane % 16), k ks + (lane / 16) * 8
              const __nv_bfloat16 *ptr = As + (p * BM + wm + (lane & 15)) * kPitchK + ks + (lane >> 4) * 8;
              ldsm_x4(smem_u32(ptr), fa.a[p][0], fa.a[p][1], fa.a[p][2], fa.a[p][3]);
            } else {
              // As[k][m]: matrix mi = lane / 8 covers k ks + (mi/2)*8, m wm + (mi%2)*8
              const int mi = lane >> 3;
              const __nv_bfloat16 *ptr = As + (p * BK + ks + (mi >> 1) * 8 + (lane & 7)) * kPitchMN + wm + (mi & 1) * 8;
              ldsm_x4_t(smem_u32(ptr), fa.a[p][0], fa.a[p][1], fa.a[p][2], fa.a[p][3]);
            }
#pragma unroll
            for (int x = 0; x < 4; ++x) fa.a[p][x] ^= neg;
          }
#pragma unroll
          for (int qd = 0; qd < kPlanes; ++qd) {
            uint32_t b[4][2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              // matrices (n-tile 2h, k 0-7), (2h, k 8-15), (2h+1, k 0-7), (2h+1, k 8-15)
              const int mi = lane >> 3;
              const int ntile = 2 * h + (mi >> 1), khalf = mi & 1;
              uint32_t r0, r1, r2, r3;
              if (tb) {  // Bs[n][k]
                const __nv_bfloat16 *ptr = Bs + (qd * BN + wn + ntile * 8 + (lane & 7)) * kPitchK + ks + khalf * 8;
                ldsm_x4(smem_u32(ptr), r0, r1, r2, r3);
              } else {   // Bs[k][n]
                const __nv_bfloat16 *ptr = Bs + (qd * BK + ks + khalf * 8 + (lane & 7)) * kPitchMN + wn + ntile * 8;
                ldsm_x4_t(smem_u32(ptr), r0, r1, r2, r3);
              }
              b[2 * h][0] = r0;
              b[2 * h][1] = r1;
              b[2 * h + 1][0] = r2;
              b[2 * h + 1][1] = r3;
            }
#pragma unroll
            for (int p = 0; p < kPlanes; ++p) {
              if (p + qd >= kPlanes) continue;
#pragma unroll
              for (int j = 0; j < 4; ++j) mma_bf16(acc[p + qd][j], fa.a[p], b[j][0], b[j][1]);
            }
          }
        }
        __syncthreads();  // this buffer may be refilled by the next stage
      }
    }
  }
  if (kacc > 0) fold();
  __syncthreads();
  for (int i = tid; i < BM * BN; i += kThreads) {
    const int r = i / BN, col = i - r * BN;
    const int gm = m0 + r, gn = n0 + col;
    if (gm < g.M && gn < g.N) {
      double *cp = g.C + int64_t(gm) * g.ldc + gn;
      *cp = g.accumulate ? (*cp + Ct[i]) : Ct[i];
    }
  }
}

constexpr size_t kGemmSmem = 4 * size_t(kTileElems) * sizeof(__nv_bfloat16) + BM * BN * sizeof(double);

}  // namespace

void launch_split(const SplitTask *tasks, int ntasks, cudaStream_t s) {
  if (ntasks == 0) return;
  k_split<<<ntasks, 256, 0, s>>>(tasks);
}

void launch_split_grid(const SplitTask *tasks, const int64_t *chunk0_max, const int64_t *chunk0_dig,
                       int ntasks, int64_t nchunk_max, int64_t nchunk_dig, unsigned long long *maxbits,
                       cudaStream_t s) {
  if (ntasks == 0) return;
  cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long) * ntasks, s);
  if (nchunk_max > 0) k_split_max<<<unsigned(nchunk_max), 256, 0, s>>>(tasks, chunk0_max, ntasks, maxbits);
  k_split_digits<<<unsigned(nchunk_dig), 256, 0, s>>>(tasks, chunk0_dig, ntasks, maxbits);
}

void launch_gemm_oz(const GemmTile *tiles, int ntiles, const OzGroup *groups, const OzContrib *contribs,
                    cudaStream_t s) {
  if (ntiles == 0) return;
  static bool cfg = false;
  if (!cfg) {
    cudaFuncSetAttribute(k_gemm_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kGemmSmem));
    cfg = true;
  }
  k_gemm_oz<<<ntiles, kThreads, kGemmSmem, s>>>(tiles, groups, contribs);
}

}  // namespace nrg
