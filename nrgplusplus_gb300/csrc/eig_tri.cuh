// Tridiagonal stage shared by the one-CTA reflector solver (k_eig.cu:
// k_eig_bi) and the thread-block-cluster solver (k_eig_cluster.cu), in FP32
// (the mixed path's first stage) and FP64 (the plain path's reflector
// solver): Sturm counts for bisection, one inverse-iteration solve, and the
// per-precision block buffers the reflector kernels read and write.
#pragma once

#include "nrg_internal.h"

namespace nrg {

static __device__ __forceinline__ float sqrt_c(float x) { return sqrtf(x); }
static __device__ __forceinline__ double sqrt_c(double x) { return sqrt(x); }
static __device__ __forceinline__ float abs_c(float x) { return fabsf(x); }
static __device__ __forceinline__ double abs_c(double x) { return fabs(x); }

// gap: eigenvalues closer than gap |T| are inverse-iterated as one cluster
// with re-orthogonalisation.  FP32 (the mixed path's first stage): the FP64
// refinement removes the overlap of wider pairs.  FP64 (no refinement): a
// pair further apart keeps an overlap of about eps |T| / gap <= 2e-11; the
// 1e-3 of LAPACK's dstein would chain the dense upper spectrum of an NRG
// block into clusters of hundreds of levels (O(m^2 n) sequential work).
template <typename T> struct Tiny;
template <> struct Tiny<float> {
  static constexpr float piv = 1e-30f, grow = 1e15f, small = 1e-37f, gap = 1e-5f;
  static __device__ float pivmin(float tn) { return fmaxf(tn * 1.2e-7f, 1e-20f); }
};
template <> struct Tiny<double> {
  static constexpr double piv = 1e-290, grow = 1e150, small = 1e-300, gap = 1e-5;
  static __device__ double pivmin(double tn) { return fmax(tn * 2.3e-16, 1e-280); }
};

// Sturm count (eigenvalues of (d, e) below x); a tiny pivot is replaced by
// -piv before it is counted, so count and recurrence see the same sign;
// counting a zero pivot as non-negative while continuing with a negative one
// shifts the count by one and sends the bisection to a neighbouring level.
template <typename T> __device__ int sturm_c(const T *d, const T *e, int n, T x) {
  T q = d[0] - x;
  if (abs_c(q) < Tiny<T>::piv) q = -Tiny<T>::piv;
  int cnt = q < T(0);
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e[i] * e[i] / q;
    if (abs_c(q) < Tiny<T>::piv) q = -Tiny<T>::piv;
    cnt += q < T(0);
  }
  return cnt;
}

// One inverse-iteration solve (T - lam) x = s v on column j of V (stride
// ld), LU pivots in column j of Bt.  Pivots smaller than pivmin are replaced
// by +-pivmin; growth beyond `grow` is rescaled on the fly (the vector's scale
// is irrelevant).  Returns 1 / ||x||.
template <typename T>
__device__ T inv_solve_c(const T *d, const T *e, int n, T lam, T pivmin, T s, T *V, T *Bt, int ld, int j) {
  T beta = d[0] - lam;
  if (abs_c(beta) < pivmin) beta = copysign(pivmin, beta);
  T fb = s;
  T y = V[j] * fb;
  Bt[j] = beta;
  V[j] = y;
  for (int i = 1; i < n; ++i) {
    const T m = e[i] / beta;
    beta = (d[i] - lam) - m * e[i];
    if (abs_c(beta) < pivmin) beta = copysign(pivmin, beta);
    y = V[int64_t(i) * ld + j] * fb - m * y;
    if (abs_c(y) > Tiny<T>::grow) {
      const T sc = T(1) / abs_c(y);
      for (int k = 0; k < i; ++k) V[int64_t(k) * ld + j] *= sc;
      y *= sc;
      fb *= sc;
    }
    Bt[int64_t(i) * ld + j] = beta;
    V[int64_t(i) * ld + j] = y;
  }
  T x = y / beta;
  if (!(abs_c(x) <= Tiny<T>::grow)) x = copysign(T(1), x);
  V[int64_t(n - 1) * ld + j] = x;
  T nrm = x * x;
  for (int i = n - 2; i >= 0; --i) {
    T xi = (V[int64_t(i) * ld + j] - e[i + 1] * x) / Bt[int64_t(i) * ld + j];
    if (abs_c(xi) > Tiny<T>::grow) {
      const T sc = T(1) / abs_c(xi);
      for (int k = i + 1; k < n; ++k) V[int64_t(k) * ld + j] *= sc;
      xi *= sc;
      nrm *= sc * sc;
    }
    V[int64_t(i) * ld + j] = xi;
    nrm += xi * xi;
    x = xi;
  }
  return T(1) / sqrt_c(max(nrm, Tiny<T>::small));
}

template <typename T> struct Bufs;
template <> struct Bufs<float> {
  static __device__ float *W(const EigBlock &b) { return b.W; }
  static __device__ float *V(const EigBlock &b) { return b.V; }
  static __device__ float *Bt(const EigBlock &b) { return b.Bt; }
};
template <> struct Bufs<double> {
  static __device__ double *W(const EigBlock &b) { return b.W64; }
  static __device__ double *V(const EigBlock &b) { return b.V64; }
  static __device__ double *Bt(const EigBlock &b) { return b.Bt64; }
};

}  // namespace nrg
