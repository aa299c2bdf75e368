// Batched dense symmetric eigensolver for the NRG sector blocks
// (replaces qmatrix::diag -> LAPACKE_dsyevd, qmatrix.hpp:375-404, called per
// block from nrgcore.hpp:85-89).
//
// One CTA solves one block:
//   1. Householder reduction to tridiagonal form, keeping the full symmetric
//      matrix so every access is a row (coalesced in global memory, bank-
//      friendly in shared memory); the reflector u is kept in row i and u/h
//      in column i for step 2.
//   2. Accumulation of the orthogonal transform Q in place.
//   3. Implicit QL with Wilkinson shifts on the tridiagonal (d, e).  One
//      thread runs the Givens chain of a QL sweep and records (c, s); all
//      threads then apply the sweep's rotations to their rows of Q, carrying
//      the running column in a register.
//   4. Eigenvalues ascending with eigenvectors as columns (the LAPACK
//      row-major layout the reference publishes in current_hamiltonQ).
// The matrix lives in shared memory when it fits, otherwise in the block's
// own global buffer (L2 resident).  The QL sweep count per eigenvalue is
// capped; a block that hits the cap sets status[b] = 1 and stops.
// Published algorithms restated here: the Householder tridiagonalisation and
// implicit QL of EISPACK's tred2 / tql2 (Martin, Reinsch and Wilkinson, Numer.
// Math. 11 (1968) 181; Bowdler, Martin, Reinsch and Wilkinson, Numer. Math. 11
// (1968) 293); Sturm-sequence bisection (Barth, Martin and Wilkinson, Numer.
// Math. 9 (1967) 386); inverse iteration with re-orthogonalisation of close
// eigenvalues (Peters and Wilkinson, Linear Algebra (Handbook II/18), 1971).
#include "eig_tri.cuh"
#include "nrg_internal.h"

#include <algorithm>

namespace nrg {
namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxQlIter = 60;
constexpr int kSmemBytes = 225 * 1024;
constexpr int kBiVecs = 6;  // k_eig_bi's shared vectors of n: d, e, two u and two p / q

template <typename T> __device__ __forceinline__ T tabs(T x) { return x < T(0) ? -x : x; }
__device__ __forceinline__ double thypot(double a, double b) { return hypot(a, b); }
__device__ __forceinline__ float thypot(float a, float b) { return hypotf(a, b); }
__device__ __forceinline__ double tsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ float tsqrt(float a) { return sqrtf(a); }

// Givens pair of the QL chain: r = hypot(f, g), s = f / r, c = g / r.
// FP64 keeps IEEE hypot and division; the FP32 first stage of the mixed path
// uses one reciprocal square root (its result is refined in FP64 anyway).
__device__ __forceinline__ double givens(double f, double g, double &s, double &c) {
  const double r = hypot(f, g);
  if (r != 0.0) {
    s = f / r;
    c = g / r;
  }
  return r;
}
__device__ __forceinline__ float givens(float f, float g, float &s, float &c) {
  const float r2 = fmaf(f, f, g * g);
  if (r2 == 0.f) return 0.f;
  const float ri = rsqrtf(r2);
  s = f * ri;
  c = g * ri;
  return r2 * ri;
}

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic CTA-wide sum; red needs kWarps + 1 entries.
template <typename T> __device__ T block_sum(T v, T *red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    T s = (l < kWarps) ? red[l] : T(0);
    s = warp_sum(s);
    if (l == 0) red[kWarps] = s;
  }
  __syncthreads();
  return red[kWarps];
}

struct Ctl {
  int m, istop, done, err;
};

// One reduction step's matrix-vector product p_j = (A u)_j / h (j <= l) and
// rank-2 update A -= u q^T + q u^T for an FP32 matrix in global memory with
// an even leading dimension: every warp streams four rows at a time in 8-byte
// column pairs, so each lane keeps several independent L2 loads in flight
// (one row per warp is latency bound out of L2).  The last pair may cover
// column l + 1, which the caller neutralises with u[l+1] = q[l+1] = 0.
__device__ void matvec_rows_f2(const float *a, int lda, int l, const float *u, float *p, float h) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int npair = (l + 2) >> 1;
  const float2 *u2 = reinterpret_cast<const float2 *>(u);
  for (int j0 = warp; j0 <= l; j0 += 4 * kWarps) {
    const float2 *row[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int j = j0 + r * kWarps;
      row[r] = reinterpret_cast<const float2 *>(a + int64_t(j <= l ? j : j0) * lda);
    }
    float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
    for (int c = lane; c < npair; c += 32) {
      float2 v[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) v[r] = row[r][c];
      const float2 uu = u2[c];
#pragma unroll
      for (int r = 0; r < 4; ++r) s[r] = fmaf(v[r].x, uu.x, fmaf(v[r].y, uu.y, s[r]));
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) s[r] = warp_sum(s[r]);
    if (lane == 0)
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (j0 + r * kWarps <= l) p[j0 + r * kWarps] = s[r] / h;
  }
}

__device__ void update_rows_f2(float *a, int lda, int l, const float *u, const float *q) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int npair = (l + 2) >> 1;
  const float2 *u2 = reinterpret_cast<const float2 *>(u);
  const float2 *q2 = reinterpret_cast<const float2 *>(q);
  for (int j0 = warp; j0 <= l; j0 += 4 * kWarps) {
    float2 *row[4];
    float uj[4], qj[4];
    bool ok[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int j = j0 + r * kWarps;
      ok[r] = j <= l;
      row[r] = reinterpret_cast<float2 *>(a + int64_t(ok[r] ? j : j0) * lda);
      uj[r] = ok[r] ? u[j] : 0.f;
      qj[r] = ok[r] ? q[j] : 0.f;
    }
    for (int c = lane; c < npair; c += 32) {
      float2 v[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) v[r] = row[r][c];
      const float2 uu = u2[c], qq = q2[c];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        v[r].x -= uj[r] * qq.x + qj[r] * uu.x;
        v[r].y -= uj[r] * qq.y + qj[r] * uu.y;
      }
#pragma unroll
      for (int r = 0; r < 4; ++r)
        if (ok[r]) row[r][c] = v[r];
    }
  }
}

// Householder reduction of a (n x n, leading dimension lda, either memory
// space) to tridiagonal form.  Step i (n-1 down to 1) applies the reflector
// P_i = I - u u^T / h with u in row i, entries 0..i-1 (scaled; the scale
// cancels in P_i), h in d[i] (0: no reflector); e[i] = coupling of i-1 and i
// (e[0] = 0).  On return the diagonal of T is a(i, i), so
//     A = Q T Q^T,   Q = P_{n-1} P_{n-2} ... P_1.
// With store_uh, u / h is also written to column i (used by tred2_accumulate).
// wide (FP32, global memory, even lda, no store_uh): the streaming
// matvec_rows_f2 / update_rows_f2 forms.  d, e, u, p: shared arrays of n.
template <typename T>
__device__ void tred2_reduce(T *a, int lda, int n, T *d, T *e, T *u, T *p, T *red, bool store_uh,
                             bool wide = false) {
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
#define A(i, j) a[int64_t(i) * lda + (j)]
  for (int i = n - 1; i >= 1; --i) {
    const int l = i - 1;
    T scale = T(0);
    for (int k = tid; k <= l; k += kThreads) scale += tabs(A(i, k));
    scale = block_sum(scale, red);
    if (l == 0 || scale == T(0)) {
      if (tid == 0) { e[i] = A(i, l); d[i] = T(0); }
      __syncthreads();
      continue;
    }
    T hs = T(0);
    for (int k = tid; k <= l; k += kThreads) {
      T x = A(i, k) / scale;
      A(i, k) = x;
      u[k] = x;
      hs += x * x;
    }
    T h = block_sum(hs, red);
    if (tid == 0) {
      T f = A(i, l);
      T g = (f >= T(0)) ? -tsqrt(h) : tsqrt(h);
      e[i] = scale * g;
      h -= f * g;
      A(i, l) = f - g;
      u[l] = f - g;
      u[i] = T(0);  // column l + 1 = i of the wide forms' last pair
      p[i] = T(0);
      red[kWarps] = h;
    }
    __syncthreads();
    h = red[kWarps];
    __syncthreads();
    if constexpr (sizeof(T) == sizeof(float)) {
      if (wide) {
        matvec_rows_f2(a, lda, l, u, p, h);
        __syncthreads();
        T fs = T(0);
        for (int j = tid; j <= l; j += kThreads) fs += p[j] * u[j];
        const T f = block_sum(fs, red);
        const T hh = f / (h + h);
        for (int j = tid; j <= l; j += kThreads) p[j] = p[j] - hh * u[j];  // q
        __syncthreads();
        update_rows_f2(a, lda, l, u, p);
        if (tid == 0) d[i] = h;
        __syncthreads();
        continue;
      }
    }
    // p_j = (A u)_j / h, and u_j / h stored in column i
    for (int j = warp; j <= l; j += kWarps) {
      T s = T(0);
      for (int k = lane; k <= l; k += 32) s += A(j, k) * u[k];
      s = warp_sum(s);
      if (lane == 0) {
        p[j] = s / h;
        if (store_uh) A(j, i) = u[j] / h;
      }
    }
    __syncthreads();
    T fs = T(0);
    for (int j = tid; j <= l; j += kThreads) fs += p[j] * u[j];
    const T f = block_sum(fs, red);
    const T hh = f / (h + h);
    for (int j = tid; j <= l; j += kThreads) p[j] = p[j] - hh * u[j];  // q
    __syncthreads();
    // rank-2 update of the leading (l+1)^2 block, both triangles
    const int m1 = l + 1;
    for (int j = warp; j <= l; j += kWarps) {
      const T uj = u[j], qj = p[j];
      for (int k = lane; k < m1; k += 32) A(j, k) -= (uj * p[k] + qj * u[k]);
    }
    if (tid == 0) d[i] = h;
    __syncthreads();
  }
  if (tid == 0) { d[0] = T(0); e[0] = T(0); }
  __syncthreads();
#undef A
}

// The reflector solver's reduction (k_eig_bi): the same Householder steps as
// tred2_reduce without store_uh, with each step's rank-2 update deferred
// into the next step's matrix-vector product, so a step makes one pass over
// the active rows (read and write) instead of two reads and a write:
//   step i: row i takes the pending update (u, q of step i + 1), forms
//           u' / h' / e_i; then rows 0..i-1 take the pending update and
//           p'_j = (A u')_j / h' from the updated values in the same pass;
//           q' = p' - (u'.p' / 2h') u' becomes the pending update.
// The values are those of the separate passes.  ua / pa, ub / pb: two pairs
// of shared vectors of n, swapped every step.  wide: global memory, even
// lda, 8- or 16-byte column pairs; otherwise one column per lane.
template <typename T> struct Pair;
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<double> { using type = double2; };

// Rows 0..jn-1: the pending update over ncol columns (UPD) and/or the dot
// products with un (DOT, pn[j] = dot / hn).  Four rows per warp at a time, so
// each lane keeps several independent loads in flight.
template <typename T, bool WIDE, bool UPD, bool DOT>
__device__ void fused_rows(T *a, int lda, int jn, int ncol, const T *u, const T *q, const T *un, T *pn, T hn) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  using P = typename Pair<T>::type;
  const int nc = WIDE ? (ncol + 1) >> 1 : ncol;
  for (int j0 = warp; j0 < jn; j0 += 4 * kWarps) {
    T *row[4];
    T uj[4], qj[4], sd[4];
    bool ok[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int j = j0 + r * kWarps;
      ok[r] = j < jn;
      row[r] = a + int64_t(ok[r] ? j : j0) * lda;
      uj[r] = (UPD && ok[r]) ? u[j] : T(0);
      qj[r] = (UPD && ok[r]) ? q[j] : T(0);
      sd[r] = T(0);
    }
    if constexpr (WIDE) {
      const P *u2 = reinterpret_cast<const P *>(u), *q2 = reinterpret_cast<const P *>(q);
      const P *n2 = reinterpret_cast<const P *>(un);
#pragma unroll 2
      for (int c = lane; c < nc; c += 32) {
        P v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) v[r] = reinterpret_cast<const P *>(row[r])[c];
        if constexpr (UPD) {
          const P uu = u2[c], qq = q2[c];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            v[r].x -= uj[r] * qq.x + qj[r] * uu.x;
            v[r].y -= uj[r] * qq.y + qj[r] * uu.y;
          }
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (ok[r]) reinterpret_cast<P *>(row[r])[c] = v[r];
        }
        if constexpr (DOT) {
          const P w = n2[c];
#pragma unroll
          for (int r = 0; r < 4; ++r) sd[r] = fma(v[r].x, w.x, fma(v[r].y, w.y, sd[r]));
        }
      }
    } else {
      for (int c = lane; c < nc; c += 32) {
        T v[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) v[r] = row[r][c];
        if constexpr (UPD) {
          const T uu = u[c], qq = q[c];
#pragma unroll
          for (int r = 0; r < 4; ++r) v[r] -= uj[r] * qq + qj[r] * uu;
#pragma unroll
          for (int r = 0; r < 4; ++r)
            if (ok[r]) row[r][c] = v[r];
        }
        if constexpr (DOT) {
          const T w = un[c];
#pragma unroll
          for (int r = 0; r < 4; ++r) sd[r] += v[r] * w;
        }
      }
    }
    if constexpr (DOT) {
#pragma unroll
      for (int r = 0; r < 4; ++r) sd[r] = warp_sum(sd[r]);
      if (lane == 0)
#pragma unroll
        for (int r = 0; r < 4; ++r)
          if (ok[r]) pn[j0 + r * kWarps] = sd[r] / hn;
    }
  }
}

template <typename T, bool WIDE>
__device__ void tred2_fused(T *a, int lda, int n, T *d, T *e, T *ua, T *pa, T *ub, T *pb, T *red) {
  const int tid = threadIdx.x;
  T *u = ua, *q = pa, *un = ub, *pn = pb;
  bool pending = false;
  for (int i = n - 1; i >= 1; --i) {
    const int l = i - 1;
    T *ai = a + int64_t(i) * lda;
    // the pending update spans columns 0..i, the new product 0..l; in the
    // wide form the last pair may reach one column further, which u, q and
    // un hold at zero there
    const int ncol = pending ? i + 1 : l + 1;
    // row i (the next reflector): the pending update, staged in un, and its
    // |.| sum over columns 0..l
    T scale = T(0);
    {
      const T ui = pending ? u[i] : T(0), qi = pending ? q[i] : T(0);
      for (int c = tid; c <= i; c += kThreads) {
        T v = ai[c];
        if (pending) {
          v -= ui * q[c] + qi * u[c];
          ai[c] = v;
        }
        if (c <= l) {
          un[c] = v;
          scale += tabs(v);
        }
      }
    }
    scale = block_sum(scale, red);
    if (l == 0 || scale == T(0)) {
      if (tid == 0) { e[i] = un[l]; d[i] = T(0); }
      if (pending) fused_rows<T, WIDE, true, false>(a, lda, i, ncol, u, q, nullptr, nullptr, T(1));
      __syncthreads();
      pending = false;
      continue;
    }
    T hs = T(0);
    for (int k = tid; k <= l; k += kThreads) {
      const T x = un[k] / scale;
      ai[k] = x;
      un[k] = x;
      hs += x * x;
    }
    T h = block_sum(hs, red);
    if (tid == 0) {
      const T f = un[l];
      const T g = (f >= T(0)) ? -tsqrt(h) : tsqrt(h);
      e[i] = scale * g;
      h -= f * g;
      ai[l] = f - g;
      un[l] = f - g;
      un[i] = T(0);
      pn[i] = T(0);
      if (i + 1 < n) {
        un[i + 1] = T(0);
        pn[i + 1] = T(0);
      }
      red[kWarps] = h;
    }
    __syncthreads();
    h = red[kWarps];
    __syncthreads();
    if (pending) fused_rows<T, WIDE, true, true>(a, lda, i, ncol, u, q, un, pn, h);
    else fused_rows<T, WIDE, false, true>(a, lda, i, ncol, u, q, un, pn, h);
    __syncthreads();
    T fs = T(0);
    for (int j = tid; j <= l; j += kThreads) fs += pn[j] * un[j];
    const T f = block_sum(fs, red);
    const T hh = f / (h + h);
    for (int j = tid; j <= l; j += kThreads) pn[j] = pn[j] - hh * un[j];  // q'
    if (tid == 0) d[i] = h;
    __syncthreads();
    T *t = u;
    u = un;
    un = t;
    t = q;
    q = pn;
    pn = t;
    pending = true;
  }
  if (tid == 0) { d[0] = T(0); e[0] = T(0); }
  __syncthreads();
}

// Accumulation of Q from the reflectors left by tred2_reduce(store_uh):
// on return a = Q and d = the diagonal of T.
template <typename T>
__device__ void tred2_accumulate(T *a, int lda, int n, T *d, T *p) {
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
#define A(i, j) a[int64_t(i) * lda + (j)]
  for (int i = 0; i < n; ++i) {
    const int l = i - 1;
    const bool apply = (d[i] != T(0));
    __syncthreads();
    if (apply) {
      // g_j = sum_k u_k Q(k, j); p holds g
      for (int j = tid; j <= l; j += kThreads) {
        T g = T(0);
        for (int k = 0; k <= l; ++k) g += A(i, k) * A(k, j);
        p[j] = g;
      }
      __syncthreads();
      for (int k = warp; k <= l; k += kWarps) {
        const T uk = A(k, i);
        for (int j = lane; j <= l; j += 32) A(k, j) -= p[j] * uk;
      }
      __syncthreads();
    }
    if (tid == 0) {
      d[i] = A(i, i);
      A(i, i) = T(1);
    }
    for (int j = tid; j <= l; j += kThreads) {
      A(j, i) = T(0);
      A(i, j) = T(0);
    }
    __syncthreads();
  }
#undef A
}

// Implicit QL with Wilkinson shifts on (d, e) with the eigenvectors
// accumulated into a (= Q on entry); cs/sn alias u/p.
template <typename T>
__device__ void ql_vectors(T *a, int lda, int n, T *d, T *e, T *u, T *p, Ctl *ctl) {
  const int tid = threadIdx.x;
#define A(i, j) a[int64_t(i) * lda + (j)]
  // ---------------- 3. implicit QL on (d, e)
  // Q is transposed in place first, so that the Givens rotations of the QL
  // sweeps act on contiguous rows (coalesced / bank-conflict free); the
  // eigenvectors end up as rows of the working matrix.
  for (int64_t idx = tid; idx < int64_t(n) * n; idx += kThreads) {
    const int r = int(idx / n), c = int(idx - int64_t(r) * n);
    if (r < c) {
      const T x = A(r, c);
      A(r, c) = A(c, r);
      A(c, r) = x;
    }
  }
  if (tid == 0) {
    for (int i = 1; i < n; ++i) e[i - 1] = e[i];
    e[n - 1] = T(0);
    ctl->err = 0;
  }
  __syncthreads();
  T *cs = u, *sn = p;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    for (;;) {
      if (tid == 0) {
        int m;
        for (m = l; m < n - 1; ++m) {
          T dd = tabs(d[m]) + tabs(d[m + 1]);
          if (tabs(e[m]) + dd == dd) break;
        }
        ctl->m = m;
        ctl->done = (m == l);
        if (m != l) {
          if (iter++ >= kMaxQlIter) {
            ctl->err = 1;
            ctl->done = 1;
          } else {
            T g = (d[l + 1] - d[l]) / (T(2) * e[l]);
            T r = thypot(g, T(1));
            g = d[m] - d[l] + e[l] / (g + (g >= T(0) ? tabs(r) : -tabs(r)));
            T s = T(1), c = T(1), pp = T(0);
            int i;
            for (i = m - 1; i >= l; --i) {
              T f = s * e[i];
              T b = c * e[i];
              T sn_new, cs_new;
              r = givens(f, g, sn_new, cs_new);
              e[i + 1] = r;
              if (r == T(0)) {
                d[i + 1] -= pp;
                e[m] = T(0);
                break;
              }
              s = sn_new;
              c = cs_new;
              g = d[i + 1] - pp;
              r = (d[i] - g) * s + T(2) * c * b;
              d[i + 1] = g + (pp = s * r);
              g = c * r - b;
              cs[i] = c;
              sn[i] = s;
            }
            ctl->istop = i;
            if (!(r == T(0) && i >= l)) {
              d[l] -= pp;
              e[l] = g;
              e[m] = T(0);
            }
          }
        }
      }
      __syncthreads();
      const int done = ctl->done, m = ctl->m, istop = ctl->istop;
      __syncthreads();  // everyone has read ctl before thread 0 rewrites it
      if (done) break;
      // apply rotations i = m-1 .. istop+1 to rows i, i+1 of Q^T; thread k
      // owns column k and carries the running row value in a register
      for (int k = tid; k < n; k += kThreads) {
        T f = A(m, k);
        for (int i = m - 1; i > istop; --i) {
          const T zi = A(i, k);
          A(i + 1, k) = sn[i] * zi + cs[i] * f;
          f = cs[i] * zi - sn[i] * f;
        }
        A(istop + 1, k) = f;
      }
      __syncthreads();
    }
    if (ctl->err) break;
  }
#undef A
}

// Rank eigenvalues (stable ascending) and write E and U (columns permuted).
template <typename T>
__device__ void write_sorted(const T *a, int lda, int n, const T *d, int *rank, double *E, double *U,
                             int ldu) {
  // total order (NaN sorts last, ties by index) so rank is a permutation
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const T x = d[i];
    const T kx = (x == x) ? x : T(INFINITY);
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const T y = d[j];
      const T ky = (y == y) ? y : T(INFINITY);
      r += (ky < kx) || (ky == kx && j < i);
    }
    rank[i] = r;
    E[r] = double(x);
  }
  __syncthreads();
  // eigenvector `vec` is row `vec` of the working matrix
  for (int64_t idx = threadIdx.x; idx < int64_t(n) * n; idx += kThreads) {
    const int vec = int(idx / n), row = int(idx - int64_t(vec) * n);
    U[int64_t(row) * ldu + rank[vec]] = double(a[int64_t(vec) * lda + row]);
  }
}

template <typename T>
__device__ void carve(char *smem, int n, bool matrix_in_smem, T *&amat, T *&d, T *&e, T *&u, T *&p,
                      T *&red, int *&rank, Ctl *&ctl, char **scratch = nullptr, T **ub = nullptr,
                      T **pb = nullptr) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *q = smem + off;
    off += (bytes + 15) & ~size_t(15);
    return q;
  };
  ctl = reinterpret_cast<Ctl *>(take(sizeof(Ctl)));
  red = reinterpret_cast<T *>(take(sizeof(T) * (kWarps + 1)));
  d = reinterpret_cast<T *>(take(sizeof(T) * n));
  e = reinterpret_cast<T *>(take(sizeof(T) * n));
  u = reinterpret_cast<T *>(take(sizeof(T) * n));
  p = reinterpret_cast<T *>(take(sizeof(T) * n));
  rank = reinterpret_cast<int *>(u);  // reused after the solve
  if (ub) {  // the second u / q pair of the fused reduction
    *ub = reinterpret_cast<T *>(take(sizeof(T) * n));
    *pb = reinterpret_cast<T *>(take(sizeof(T) * n));
  }
  if (scratch) *scratch = smem + off;  // the matrix area (free once it is reduced) and beyond
  amat = matrix_in_smem ? reinterpret_cast<T *>(take(sizeof(T) * size_t(n) * (n + 1))) : nullptr;
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 1)
k_eig(const EigBlock *__restrict__ blocks, int max_n_smem, int *status, const int *gate) {
  extern __shared__ __align__(16) char smem[];
  if (gate && gate[blockIdx.x] != 2 && gate[blockIdx.x] != 4) return;  // re-solve only the flagged blocks
  const EigBlock B = blocks[blockIdx.x];
  const int n = B.n;
  if (n == 0) return;
  const bool in_smem = (n <= max_n_smem);
  T *amat, *d, *e, *u, *p, *red;
  int *rank;
  Ctl *ctl;
  carve<T>(smem, n, in_smem, amat, d, e, u, p, red, rank, ctl);
  T *a;
  int lda;
  if (in_smem) {
    a = amat;
    lda = n + 1;
  } else if (sizeof(T) == sizeof(double)) {
    a = reinterpret_cast<T *>(B.H);
    lda = B.ld;
  } else {
    a = reinterpret_cast<T *>(B.W);
    lda = B.ld;
  }
  if (in_smem || sizeof(T) != sizeof(double)) {
    for (int64_t idx = threadIdx.x; idx < int64_t(n) * n; idx += kThreads) {
      const int r = int(idx / n), c = int(idx - int64_t(r) * n);
      a[int64_t(r) * lda + c] = T(B.H[int64_t(r) * B.ld + c]);
    }
  }
  __syncthreads();
  tred2_reduce<T>(a, lda, n, d, e, u, p, red, true);
  tred2_accumulate<T>(a, lda, n, d, p);
  ql_vectors<T>(a, lda, n, d, e, u, p, ctl);
  __syncthreads();
  if (ctl->err) {
    if (threadIdx.x == 0) status[blockIdx.x] = 1;
    return;
  }
  write_sorted<T>(a, lda, n, d, rank, B.E, B.U, B.ldu);
}

// ------------------------------------------------------------------------
// FP32 first stage of the mixed path: the Householder reduction
// (tred2_reduce, reflectors kept instead of forming Q), then the tridiagonal
// problem without the sequential QL chain:
//   * Sturm-sequence bisection, one thread per eigenvalue (all in parallel);
//   * inverse iteration, one thread per eigenvector (tridiagonal LU solve,
//     vectors stored column-wise so every step is a coalesced row access);
//   * near-degenerate clusters (gaps <= 1e-5 |T|) redone one warp per
//     cluster, re-orthogonalising each new iterate against the cluster's
//     earlier vectors (the classic inverse-iteration/Gram-Schmidt scheme).
//     Pairs further apart leave inverse iteration with an overlap of about
//     eps32 |T| / gap <= 1e-2, which the FP64 refinement's orthonormalisation
//     (pairs closer than 1e-4 |H|) or Newton step (the others) removes; a
//     wider cluster gap only made the sequential cluster solves longer;
//   * the back-transform X = Q V applies the reflectors to V in a separate
//     multi-CTA kernel (k_reflect).
// Accuracy is FP32 (~1e-6); the FP64-accurate refinement follows.

constexpr int kInvIter = 3;

template <typename T> __device__ __forceinline__ T block_min(T v, T *red) {
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  T m = red[0];
  for (int w = 1; w < kWarps; ++w) m = min(m, red[w]);
  __syncthreads();
  return m;
}

// number of eigenvalues of the tridiagonal (d, e) below x.  A pivot smaller
// than 1e-30 in magnitude (an exact zero included) is replaced by -1e-30
// before it is counted, so the count and the recurrence see the same sign;
// counting a zero pivot as non-negative while continuing with a negative one
// shifts the count by one and sends the bisection to a neighbouring level.
__device__ __forceinline__ int sturm_count(const float *d, const float *e, int n, float x) {
  float q = d[0] - x;
  if (fabsf(q) < 1e-30f) q = -1e-30f;
  int cnt = q < 0.f;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e[i] * e[i] / q;
    if (fabsf(q) < 1e-30f) q = -1e-30f;
    cnt += q < 0.f;
  }
  return cnt;
}

// One inverse-iteration solve (T - lam I) x = s * v for column j of V (in
// place), with the LU pivots in column j of Bt.  Pivots smaller than pivmin
// are replaced by +-pivmin; growth beyond 1e15 is rescaled on the fly (the
// vector's scale is irrelevant).  Returns 1 / ||x||.
__device__ float inv_solve(const float *d, const float *e, int n, float lam, float pivmin, float s,
                           float *V, float *Bt, int ld, int j) {
  float beta = d[0] - lam;
  if (fabsf(beta) < pivmin) beta = copysignf(pivmin, beta);
  float fb = s;  // scale applied to the remaining right-hand side entries
  float y = V[j] * fb;
  Bt[j] = beta;
  V[j] = y;
  for (int i = 1; i < n; ++i) {
    const float m = e[i] / beta;
    beta = (d[i] - lam) - m * e[i];
    if (fabsf(beta) < pivmin) beta = copysignf(pivmin, beta);
    y = V[int64_t(i) * ld + j] * fb - m * y;
    if (fabsf(y) > 1e15f) {  // rescale the entries computed so far to ~1
      const float sc = 1.f / fabsf(y);
      for (int k = 0; k < i; ++k) V[int64_t(k) * ld + j] *= sc;
      y *= sc;
      fb *= sc;
    }
    Bt[int64_t(i) * ld + j] = beta;
    V[int64_t(i) * ld + j] = y;
  }
  // pivots are >= pivmin >= 1e-20 and entries <= 1e15, so no quotient
  // below overflows before it is rescaled
  float x = y / beta;
  if (!(fabsf(x) <= 1e15f)) x = copysignf(1.f, x);  // first entry: any scale will do
  V[int64_t(n - 1) * ld + j] = x;
  float nrm = x * x;
  for (int i = n - 2; i >= 0; --i) {
    float xi = (V[int64_t(i) * ld + j] - e[i + 1] * x) / Bt[int64_t(i) * ld + j];
    if (fabsf(xi) > 1e15f) {
      const float sc = 1.f / fabsf(xi);
      for (int k = i + 1; k < n; ++k) V[int64_t(k) * ld + j] *= sc;
      xi *= sc;
      nrm *= sc * sc;
    }
    V[int64_t(i) * ld + j] = xi;
    nrm += xi * xi;
    x = xi;
  }
  return rsqrtf(fmaxf(nrm, 1e-37f));
}

// FP32 uses the forms above, FP64 the shared templates (eig_tri.cuh)
__device__ __forceinline__ int sturm_t(const float *d, const float *e, int n, float x) {
  return sturm_count(d, e, n, x);
}
__device__ __forceinline__ int sturm_t(const double *d, const double *e, int n, double x) {
  return sturm_c<double>(d, e, n, x);
}
__device__ __forceinline__ float inv_t(const float *d, const float *e, int n, float lam, float pivmin, float s,
                                       float *V, float *Bt, int ld, int j) {
  return inv_solve(d, e, n, lam, pivmin, s, V, Bt, ld, j);
}
__device__ __forceinline__ double inv_t(const double *d, const double *e, int n, double lam, double pivmin,
                                        double s, double *V, double *Bt, int ld, int j) {
  return inv_solve_c<double>(d, e, n, lam, pivmin, s, V, Bt, ld, j);
}
__device__ __forceinline__ float rnorm_t(float x) { return rsqrtf(fmaxf(x, 1e-37f)); }
__device__ __forceinline__ double rnorm_t(double x) { return 1.0 / sqrt(fmax(x, 1e-300)); }

// One CTA per block.  T = float: the mixed path's first stage (outputs in
// W, V, Bt).  T = double: the plain FP64 path's reflector solver for blocks
// above the shared-memory limit (W64, V64, Bt64), the same work in FP64 with
// no refinement after it.
template <typename T>
__global__ void __launch_bounds__(kThreads, 1)
k_eig_bi(const EigBlock *__restrict__ blocks, int max_n_smem, int smem_total, const int *gate) {
  extern __shared__ __align__(16) char smem[];
  if (gate && gate[blockIdx.x] != 2 && gate[blockIdx.x] != 4) return;  // re-solve only the flagged blocks
  const EigBlock B = blocks[blockIdx.x];
  const int n = B.n;
  if (n == 0) return;
  const bool in_smem = (n <= max_n_smem);
  T *amat, *d, *e, *u, *p, *red;
  int *rank;
  Ctl *ctl;
  char *scratch;
  T *ub, *pb;
  carve<T>(smem, n, in_smem, amat, d, e, u, p, red, rank, ctl, &scratch, &ub, &pb);
  T *const Wg = Bufs<T>::W(B), *const Vg = Bufs<T>::V(B), *const Btg = Bufs<T>::Bt(B);
  T *a = in_smem ? amat : Wg;
  const int lda = in_smem ? n + 1 : B.ld;
  for (int64_t idx = threadIdx.x; idx < int64_t(n) * n; idx += kThreads) {
    const int r = int(idx / n), c = int(idx - int64_t(r) * n);
    a[int64_t(r) * lda + c] = T(B.H[int64_t(r) * B.ld + c]);
  }
  __syncthreads();
  if (!in_smem && lda % 2 == 0) tred2_fused<T, true>(a, lda, n, d, e, u, p, ub, pb, red);
  else tred2_fused<T, false>(a, lda, n, d, e, u, p, ub, pb, red);
  // T's diagonal into d; h_i (0: no reflector) onto the diagonal of the
  // reflector matrix, which k_reflect reads from the block's W buffer
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const T h = (i == 0) ? T(0) : d[i];
    d[i] = a[int64_t(i) * lda + i];
    a[int64_t(i) * lda + i] = h;
  }
  __syncthreads();
  if (in_smem) {  // reflectors (lower triangle and diagonal) out to W
    for (int64_t idx = threadIdx.x; idx < int64_t(n) * n; idx += kThreads) {
      const int r = int(idx / n), c = int(idx - int64_t(r) * n);
      if (c <= r) Wg[int64_t(r) * B.ld + c] = a[int64_t(r) * lda + c];
    }
  }
  // Gershgorin interval and the norm used for pivots and cluster gaps
  T lo = T(3e38f), hi = T(-3e38f), tn = T(0);
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const T r = abs_c(e[i]) + (i + 1 < n ? abs_c(e[i + 1]) : T(0));
    lo = min(lo, d[i] - r);
    hi = max(hi, d[i] + r);
    tn = max(tn, abs_c(d[i]) + r);
  }
  lo = block_min<T>(lo, red);
  hi = -block_min<T>(-hi, red);
  tn = -block_min<T>(-tn, red);
  const T span = max(hi - lo, T(1e-30f));
  lo -= T(1e-6f) * span;
  hi += T(1e-6f) * span;
  T *lam = u;                               // eigenvalues, ascending
  int *cl = reinterpret_cast<int *>(p);     // cluster [start, end) pairs
  for (int j = threadIdx.x; j < n; j += kThreads) {
    T a0 = lo, b0 = hi;
    for (int it = 0; it < 80; ++it) {
      const T mid = T(0.5f) * (a0 + b0);
      if (mid <= a0 || mid >= b0) break;
      if (sturm_t(d, e, n, mid) > j) b0 = mid; else a0 = mid;
    }
    lam[j] = T(0.5f) * (a0 + b0);
  }
  __syncthreads();
  const T pivmin = Tiny<T>::pivmin(tn);
  // inverse iteration for every eigenvalue in parallel
  for (int j = threadIdx.x; j < n; j += kThreads) {
    for (int i = 0; i < n; ++i)
      Vg[int64_t(i) * B.ld + j] = T(1.0f + 0.25f * float((i * 7919 + j * 104729) % 97) / 97.f);
    T sc = T(1);
    for (int it = 0; it < kInvIter; ++it) sc = inv_t(d, e, n, lam[j], pivmin, sc, Vg, Btg, B.ld, j);
    for (int i = 0; i < n; ++i) Vg[int64_t(i) * B.ld + j] *= sc;
  }
  // clusters of near-degenerate eigenvalues
  if (threadIdx.x == 0) {
    int c = 0, k = 0;
    const T gap = Tiny<T>::gap * max(tn, T(1e-30f));
    while (k < n) {
      int q = k + 1;
      while (q < n && lam[q] - lam[q - 1] <= gap) ++q;
      if (q - k > 1) {
        cl[2 * c] = k;
        cl[2 * c + 1] = q;
        ++c;
      }
      k = q;
    }
    ctl->m = c;
  }
  __syncthreads();
  const int ncl = ctl->m;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Each warp iterates its clusters' members in shared memory (the member x
  // and its LU pivots b: 2n values per warp, in the area the matrix used),
  // so the sequential solves run at shared-memory latency.  Without room for
  // one warp's pair the member is iterated in place in V / Bt.
  const size_t avail = size_t(smem_total) - size_t(scratch - smem);
  int nw = int(avail / (sizeof(T) * 2 * size_t(n)));
  const bool staged = nw > 0;
  if (nw > kWarps || !staged) nw = kWarps;
  if (warp < nw) {
    for (int q = warp; q < ncl; q += nw) {
      const int c0 = cl[2 * q], c1 = cl[2 * q + 1];
      for (int j = c0; j < c1; ++j) {
        T *xv, *bv;
        int xs;
        if (staged) {
          xv = reinterpret_cast<T *>(scratch) + size_t(warp) * 2 * n;
          bv = xv + n;
          xs = 1;
          for (int i = lane; i < n; i += 32) xv[i] = Vg[int64_t(i) * B.ld + j];
        } else {
          xv = Vg + j;
          bv = Btg + j;
          xs = B.ld;
        }
        __syncwarp();
        for (int rep = 0; rep < 2; ++rep) {
          if (lane == 0) inv_t(d, e, n, lam[j], pivmin, T(1), xv, bv, xs, 0);
          __syncwarp();
          for (int k = c0; k < j; ++k) {  // earlier members are final in V
            T dot = T(0);
            for (int i = lane; i < n; i += 32) dot += Vg[int64_t(i) * B.ld + k] * xv[int64_t(i) * xs];
            dot = warp_sum(dot);
            for (int i = lane; i < n; i += 32) xv[int64_t(i) * xs] -= dot * Vg[int64_t(i) * B.ld + k];
            __syncwarp();
          }
          T nrm = T(0);
          for (int i = lane; i < n; i += 32) nrm += xv[int64_t(i) * xs] * xv[int64_t(i) * xs];
          nrm = warp_sum(nrm);
          const T scn = rnorm_t(nrm);
          for (int i = lane; i < n; i += 32) xv[int64_t(i) * xs] *= scn;
          __syncwarp();
        }
        if (staged)
          for (int i = lane; i < n; i += 32) Vg[int64_t(i) * B.ld + j] = xv[i];
        __syncwarp();
      }
    }
  }
  for (int j = threadIdx.x; j < n; j += kThreads) B.E[j] = double(lam[j]);
}

// X = Q V for every block, Q = P_{n-1} ... P_1 from the reflectors the
// first stage left in W (row i: u_i in entries 0..i-1, h_i on the diagonal,
// 0 = none): the reflectors are applied to X = V in the order P_1, P_2, ...,
// P_{n-1}.  One CTA owns TW columns of one block in shared memory and each
// warp TW / 8 of them, so a reflector needs no CTA barrier: a warp forms
// u^T x for its columns with lane-strided sums and one shuffle reduction
// each, then updates them.  Reflector rows are staged in panels of `panel`
// rows (one barrier per panel).  The result is written in FP64: the first
// eigenvector estimate of the mixed path (T = float, W / V) or the
// eigenvectors of the FP64 reflector solver (T = double, W64 / V64).
template <typename T> __device__ __forceinline__ const T *refl_W(const EigBlock &b);
template <> __device__ __forceinline__ const float *refl_W<float>(const EigBlock &b) { return b.W; }
template <> __device__ __forceinline__ const double *refl_W<double>(const EigBlock &b) { return b.W64; }
template <typename T> __device__ __forceinline__ const T *refl_V(const EigBlock &b);
template <> __device__ __forceinline__ const float *refl_V<float>(const EigBlock &b) { return b.V; }
template <> __device__ __forceinline__ const double *refl_V<double>(const EigBlock &b) { return b.V64; }

template <typename T, int TW>
__global__ void __launch_bounds__(256)
k_reflect(const EigBlock *__restrict__ blocks, const int2 *__restrict__ tiles, int panel, const int *gate) {
  constexpr int CPW = TW >= 8 ? TW / 8 : 1;  // columns per warp
  constexpr int NWC = TW >= 8 ? 8 : TW;      // warps with columns (TW = 4, the largest blocks: 4)
  constexpr int XP = TW + 1;                 // odd row pitch: lane-strided rows hit distinct banks
  extern __shared__ __align__(16) unsigned char rsm_raw[];
  T *rsm = reinterpret_cast<T *>(rsm_raw);
  const int2 t = tiles[blockIdx.x];
  if (gate && gate[t.x] != 2 && gate[t.x] != 4) return;  // re-solve only the flagged blocks
  const EigBlock B = blocks[t.x];
  const T *Wm = refl_W<T>(B), *Vm = refl_V<T>(B);
  const int n = B.n, c0 = t.y * TW;
  const int nc = min(TW, n - c0);
  T *X = rsm;                      // n x XP
  T *Up = X + size_t(n) * XP;      // panel x n reflector rows
  T *hs = Up + size_t(panel) * n;  // panel h values
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int cw = warp * CPW;
  for (int64_t idx = tid; idx < int64_t(n) * TW; idx += 256) {
    const int r = int(idx / TW), c = int(idx - int64_t(r) * TW);
    X[int64_t(r) * XP + c] = (c < nc) ? Vm[int64_t(r) * B.ld + c0 + c] : T(0);
  }
  for (int p0 = 1; p0 < n; p0 += panel) {
    const int p1 = min(n, p0 + panel);
    __syncthreads();  // previous panel consumed (and X loaded)
    for (int q = p0 + warp; q < p1; q += 8) {
      const T *src = Wm + int64_t(q) * B.ld;
      T *dst = Up + size_t(q - p0) * n;
      for (int k = lane; k < q; k += 32) dst[k] = src[k];
      if (lane == 0) hs[q - p0] = src[q];
    }
    __syncthreads();
    for (int q = p0; q < p1 && warp < NWC; ++q) {
      const T h = hs[q - p0];
      if (h == T(0)) continue;
      const T *uq = Up + size_t(q - p0) * n;
      T w[CPW];
#pragma unroll
      for (int c = 0; c < CPW; ++c) w[c] = T(0);
      for (int k = lane; k < q; k += 32) {
        const T uk = uq[k];
#pragma unroll
        for (int c = 0; c < CPW; ++c) w[c] = fma(uk, X[k * XP + cw + c], w[c]);
      }
#pragma unroll
      for (int c = 0; c < CPW; ++c) w[c] = warp_sum(w[c]) / h;
      for (int k = lane; k < q; k += 32) {
        const T uk = uq[k];
#pragma unroll
        for (int c = 0; c < CPW; ++c) X[k * XP + cw + c] = fma(-uk, w[c], X[k * XP + cw + c]);
      }
    }
  }
  __syncthreads();
  for (int64_t idx = tid; idx < int64_t(n) * nc; idx += 256) {
    const int r = int(idx / nc), c = int(idx - int64_t(r) * nc);
    B.U[int64_t(r) * B.ldu + c0 + c] = double(X[int64_t(r) * XP + c]);
  }
}

constexpr size_t kReflectSmem = 225 * 1024;

size_t reflect_bytes(int n, int tw, int panel, size_t elem = sizeof(float)) {
  return elem * (size_t(n) * (tw + 1) + size_t(panel) * (n + 1)) + 64;
}

template <typename T> size_t smem_bytes(int n, bool in_smem, int nvec = 4) {
  size_t b = 16 + 16 * ((sizeof(T) * (kWarps + 1) + 15) / 16) + nvec * ((sizeof(T) * n + 15) & ~15);
  if (in_smem) b += (sizeof(T) * size_t(n) * (n + 1) + 15) & ~size_t(15);
  return b + 64;
}

template <typename T> int smem_limit(int nvec = 4) {
  int n = 8;
  while (smem_bytes<T>(n + 1, true, nvec) <= size_t(kSmemBytes)) ++n;
  return n;
}

template <typename T>
void launch(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem, int *status,
            cudaStream_t s, const int *gate = nullptr) {
  if (nblocks == 0) return;
  ensure_smem_limit(reinterpret_cast<const void *>(k_eig<T>), kSmemBytes);
  // enough shared memory for the largest block of this launch
  size_t bytes = smem_bytes<T>(max_n, max_n <= max_n_smem);
  if (max_n > max_n_smem) bytes = std::max(bytes, smem_bytes<T>(max_n_smem, true));
  if (bytes > size_t(kSmemBytes)) bytes = kSmemBytes;
  k_eig<T><<<nblocks, kThreads, bytes, s>>>(blocks, max_n_smem, status, gate);
}

// ------------------------------------------------------------------------
// Rayleigh-Ritz on the refinement's long clusters.  The final refinement
// pass (k_refine.cu) diagonalises chains of near-degenerate levels (gaps
// within tau) of up to 64 levels in shared memory; a block with a longer
// chain gets status 3 and comes here: per chain of c levels (c <= 1024) the
// c x c matrix S_CC = X_C^T H X_C (from S, in the sorted order) is
// diagonalised in FP64 by the solver above (tred2 + QL, in the block's free
// E2 buffer), and U_C = X_C Q, E_C = the sorted eigenvalues.  On success the
// status returns to 0; a chain above 1024 levels or a QL failure sets 4 (the
// FP64 re-solve of the whole block follows, as for status 2).
constexpr int kSmallCluster = 64;      // the final pass's own limit (k_refine.cu)
constexpr int kBigCluster = 1024;

__global__ void __launch_bounds__(kThreads, 1)
k_oa_bigcl(const RefineBlock *__restrict__ blocks, double tau_rel, int *status) {
  if (status[blockIdx.x] != 3) return;
  extern __shared__ __align__(16) char smem[];
  __shared__ int ncl;
  const RefineBlock B = blocks[blockIdx.x];
  const int n = B.n, tid = threadIdx.x;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *q = smem + off;
    off += (bytes + 15) & ~size_t(15);
    return q;
  };
  double *lam = reinterpret_cast<double *>(take(sizeof(double) * n));
  int *perm = reinterpret_cast<int *>(take(sizeof(int) * n));
  int *cl = reinterpret_cast<int *>(take(sizeof(int) * (n + 2)));
  double *d = reinterpret_cast<double *>(take(sizeof(double) * kBigCluster));
  double *e = reinterpret_cast<double *>(take(sizeof(double) * kBigCluster));
  double *u = reinterpret_cast<double *>(take(sizeof(double) * kBigCluster));
  double *p = reinterpret_cast<double *>(take(sizeof(double) * kBigCluster));
  double *red = reinterpret_cast<double *>(take(sizeof(double) * (kWarps + 1)));
  int *vof = reinterpret_cast<int *>(take(sizeof(int) * kBigCluster));
  Ctl *ctl = reinterpret_cast<Ctl *>(take(sizeof(Ctl)));
  auto sym = [&](int i, int j) { return i <= j ? B.S[int64_t(i) * B.ld + j] : B.S[int64_t(j) * B.ld + i]; };
  // the final pass's Rayleigh quotients, tau, order and chains
  double local = 0.0;
  for (int i = tid; i < n; i += kThreads) {
    const double l = B.S[int64_t(i) * B.ld + i] / B.G[int64_t(i) * B.ld + i];
    lam[i] = l;
    local = fmax(local, fabs(l));
  }
  const double tau = tau_rel * fmax(1.0, -block_min<double>(-local, red));
  for (int i = tid; i < n; i += kThreads) {
    const double x = lam[i];
    int r = 0;
    for (int j = 0; j < n; ++j) {
      const double y = lam[j];
      r += (y < x) || (y == x && j < i);
    }
    perm[r] = i;
  }
  __syncthreads();
  if (tid == 0) {
    int c = 0, k = 0;
    while (k < n) {
      int q = k + 1;
      while (q < n && lam[perm[q]] - lam[perm[q - 1]] <= tau) ++q;
      if (q - k > kSmallCluster) {
        cl[2 * c] = k;
        cl[2 * c + 1] = q;
        ++c;
      }
      k = q;
    }
    ncl = c;
  }
  __syncthreads();
  for (int q = 0; q < ncl; ++q) {
    const int a0 = cl[2 * q], c = cl[2 * q + 1] - a0;
    if (c > kBigCluster) {
      if (tid == 0) status[blockIdx.x] = 4;
      return;
    }
    double *A = B.E2;  // c x c, leading dimension c
    for (int64_t idx = tid; idx < int64_t(c) * c; idx += kThreads) {
      const int r = int(idx / c), s = int(idx - int64_t(r) * c);
      A[idx] = sym(perm[a0 + r], perm[a0 + s]);
    }
    __syncthreads();
    tred2_reduce<double>(A, c, c, d, e, u, p, red, true);
    tred2_accumulate<double>(A, c, c, d, p);
    ql_vectors<double>(A, c, c, d, e, u, p, ctl);
    __syncthreads();
    if (ctl->err) {
      if (tid == 0) status[blockIdx.x] = 4;
      return;
    }
    // eigenvector v is row v of A; vof[k] = the one of rank k (ascending)
    for (int v = tid; v < c; v += kThreads) {
      const double x = d[v];
      int r = 0;
      for (int j = 0; j < c; ++j) {
        const double y = d[j];
        r += (y < x) || (y == x && j < v);
      }
      vof[r] = v;
    }
    __syncthreads();
    for (int k = tid; k < c; k += kThreads) B.Eout[a0 + k] = d[vof[k]];
    for (int64_t idx = tid; idx < int64_t(n) * c; idx += kThreads) {
      const int r = int(idx / c), k = int(idx - int64_t(r) * c);
      const double *ev = A + int64_t(vof[k]) * c, *xr = B.X + int64_t(r) * B.ld;
      double acc = 0.0;
      for (int m = 0; m < c; ++m) acc = fma(xr[perm[a0 + m]], ev[m], acc);
      B.U[int64_t(r) * B.ldu + a0 + k] = acc;
    }
    __syncthreads();
  }
  if (tid == 0) status[blockIdx.x] = 0;
}

}  // namespace

void launch_oa_bigcl(const RefineBlock *blocks, int nblocks, int max_n, double tau_rel, int *status,
                     cudaStream_t s) {
  if (nblocks == 0) return;
  const size_t bytes = 16 * 16 + sizeof(double) * max_n + sizeof(int) * (2 * size_t(max_n) + 2) +
                       sizeof(double) * (4 * kBigCluster + kWarps + 1) + sizeof(int) * kBigCluster + sizeof(Ctl);
  ensure_smem_limit(reinterpret_cast<const void *>(k_oa_bigcl), int(bytes));
  k_oa_bigcl<<<nblocks, kThreads, bytes, s>>>(blocks, tau_rel, status);
}

int eig_smem_limit_f64() { return smem_limit<double>(); }
int eig_smem_limit_f32() { return smem_limit<float>(kBiVecs); }

// Largest block the solver accepts: its d, e, u, p vectors must fit in shared
// memory even when the matrix itself stays in global memory.
template <typename T> static int max_block() {
  int n = 1024;
  while (smem_bytes<T>(n + 1, false) <= size_t(kSmemBytes)) ++n;
  return n;
}
int eig_max_n_f64() { return max_block<double>(); }
int eig_max_n_f32() { return max_block<float>(); }

void launch_eig_f64(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem, int *status,
                    cudaStream_t s, const int *gate) {
  launch<double>(blocks, nblocks, max_n, max_n_smem, status, s, gate);
}

template <typename T>
static void launch_bisect(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem, cudaStream_t s,
                          const int *gate = nullptr) {
  if (nblocks == 0) return;
  ensure_smem_limit(reinterpret_cast<const void *>(k_eig_bi<T>), kSmemBytes);
  size_t bytes = smem_bytes<T>(max_n, max_n <= max_n_smem, kBiVecs);
  if (max_n > max_n_smem) bytes = std::max(bytes, smem_bytes<T>(max_n_smem, true, kBiVecs));
  if (bytes > size_t(kSmemBytes)) bytes = kSmemBytes;
  k_eig_bi<T><<<nblocks, kThreads, bytes, s>>>(blocks, max_n_smem, int(bytes), gate);
}

void launch_eig_bisect_f32(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem,
                           cudaStream_t s) {
  launch_bisect<float>(blocks, nblocks, max_n, max_n_smem, s);
}

void launch_eig_bisect_f64(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem,
                           cudaStream_t s, const int *gate) {
  launch_bisect<double>(blocks, nblocks, max_n, max_n_smem, s, gate);
}

bool reflect_config(int max_n, int *tw, int *panel, bool fp64) {
  const size_t el = fp64 ? sizeof(double) : sizeof(float);
  for (int w = 64; w >= 4; w /= 2) {
    if (reflect_bytes(max_n, w, 1, el) > kReflectSmem) continue;
    int pn = 32;
    while (pn > 1 && reflect_bytes(max_n, w, pn, el) > kReflectSmem) --pn;
    *tw = w;
    *panel = pn;
    return true;
  }
  return false;
}

bool reflect_fits(int max_n, int tw, int *panel, bool fp64) {
  const size_t el = fp64 ? sizeof(double) : sizeof(float);
  if (reflect_bytes(max_n, tw, 1, el) > kReflectSmem) return false;
  int pn = 32;
  while (pn > 1 && reflect_bytes(max_n, tw, pn, el) > kReflectSmem) --pn;
  *panel = pn;
  return true;
}

int reflect_max_n(bool fp64) {
  const size_t el = fp64 ? sizeof(double) : sizeof(float);
  int n = 8;
  while (reflect_bytes(n + 1, 4, 1, el) <= kReflectSmem) ++n;
  return n;
}

// Largest block the reflector solver's reduction takes (its shared vectors
// of n; the matrix streams from global memory).
int eig_bi_max_n(bool fp64) {
  int n = 64;
  if (fp64) {
    while (smem_bytes<double>(n + 1, false, kBiVecs) <= size_t(kSmemBytes)) ++n;
  } else {
    while (smem_bytes<float>(n + 1, false, kBiVecs) <= size_t(kSmemBytes)) ++n;
  }
  return n;
}

template <typename T, int TW> static void reflect_launch(const EigBlock *blocks, const int2 *tiles, int ntiles,
                                                         int panel, size_t bytes, cudaStream_t s, const int *gate) {
  ensure_smem_limit(reinterpret_cast<const void *>(k_reflect<T, TW>), int(kReflectSmem));
  k_reflect<T, TW><<<ntiles, 256, bytes, s>>>(blocks, tiles, panel, gate);
}

template <typename T>
static void reflect_dispatch(const EigBlock *blocks, const int2 *tiles, int ntiles, int max_n, int tw, int panel,
                             cudaStream_t s, const int *gate) {
  const size_t bytes = reflect_bytes(max_n, tw, panel, sizeof(T));
  switch (tw) {
    case 64: reflect_launch<T, 64>(blocks, tiles, ntiles, panel, bytes, s, gate); break;
    case 32: reflect_launch<T, 32>(blocks, tiles, ntiles, panel, bytes, s, gate); break;
    case 16: reflect_launch<T, 16>(blocks, tiles, ntiles, panel, bytes, s, gate); break;
    case 8: reflect_launch<T, 8>(blocks, tiles, ntiles, panel, bytes, s, gate); break;
    default: reflect_launch<T, 4>(blocks, tiles, ntiles, panel, bytes, s, gate); break;
  }
}

void launch_reflect(const EigBlock *blocks, const int2 *tiles, int ntiles, int max_n, int tw, int panel,
                    cudaStream_t s, bool fp64, const int *gate) {
  if (ntiles == 0) return;
  if (fp64) reflect_dispatch<double>(blocks, tiles, ntiles, max_n, tw, panel, s, gate);
  else reflect_dispatch<float>(blocks, tiles, ntiles, max_n, tw, panel, s, gate);
}
void launch_eig_f32(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem, int *status,
                    cudaStream_t s) {
  launch<float>(blocks, nblocks, max_n, max_n_smem, status, s);
}

}  // namespace nrg
