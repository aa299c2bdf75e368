// Internal descriptors shared by the host engine (engine.cpp) and the CUDA
// kernels.  All device pointers are absolute so one launch can cover the
// blocks of many independent runs.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace nrg {

// Raises `kernel`'s dynamic shared-memory limit to `bytes` on the current
// device.  cudaFuncSetAttribute applies per device, so this runs once per
// (kernel, device) pair, thread-safe; throws the engine's error (NRG_E_CUDA)
// when the runtime refuses.
void ensure_smem_limit(const void *kernel, int bytes);
// Allows `kernel` clusters above the portable 8 CTAs on the current device
// (once per kernel and device); throws like ensure_smem_limit.
void ensure_nonportable_cluster(const void *kernel);

// ---------------------------------------------------------------- assembly
// One device block = one non-empty (Q,Sz) sector of one run.
struct AsmBlock {
  double *H;          // output, row-major n x n with leading dimension ld
  int n, ld;
  int sub0, nsub;     // sub-blocks [sub0, sub0 + nsub) of the AsmSub table
  int pair0;          // nsub*nsub entries of the pair table (int2 term ranges)
  int pad;
  int64_t chunk0;     // first 1024-element chunk of this block (flattened grid)
  double rescale;     // sqrt(Lambda) factor of this run
  double shift;       // ground-state shift of the previous site (0 if none)
};

// Sub-block (ii, bb): previous sector ii (kept prefix k) times bath sector bb
// (d states).  Rows off + it + il*k, it < k, il < d (nrgcore.hpp:179-185).
struct AsmSub {
  int off, k, d, pad;
  const double *eprev;  // previous eigenvalues of sector ii (unshifted)
  const double *ebath;  // bath energies of sector bb
};

// One hopping term between sub-blocks a (rows) and b (columns) for operator
// ip: H[a(it,il), b(it',il')] += F[it,it'] * fb[il',il] * chi * t, plus the
// transpose (nrgcore.hpp:186-224).
struct AsmTerm {
  const double *F;      // previous f-dagger kept block, k_a x k_b, row-major
  const double *fb;     // bath f-dagger block (bb', bb), d_b x d_a, row-major
  int ldf, pad;
  double chi, t;
};

void launch_assemble(const AsmBlock *blocks, int nblocks, int64_t nchunks, const AsmSub *subs,
                     const int2 *pairs, const AsmTerm *terms, cudaStream_t s);

// ------------------------------------------------------------- eigensolve
struct EigBlock {
  double *H;          // input (destroyed when the block is solved in place)
  double *U;          // output eigenvectors as columns, row-major n x ldu
  double *E;          // output eigenvalues, ascending
  float *W;           // FP32 workspace (n x ld): working matrix, then the reflectors
  float *V, *Bt;      // FP32 tridiagonal eigenvectors and LU pivots (n x ld)
  double *W64, *V64, *Bt64;  // the same workspaces of the FP64 reflector solver
  int n, ld, ldu, pad;
};
// FP32 bisection + inverse-iteration solver (mixed path first stage): writes
// E (FP64), the Householder reflectors into W (row i: u_i in columns 0..i-1,
// h_i on the diagonal) and the tridiagonal eigenvectors into V; then
// launch_reflect writes U = Q V (FP64) by applying the reflectors to V.
// reflect_config picks the column-tile width tw (64, 32, 16, 8 or 4) and the
// reflector panel for the largest block of a launch (false: too large);
// tiles: (block, column tile of width tw).
void launch_eig_bisect_f32(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem,
                           cudaStream_t s);
// The same solver in FP64 (W64, V64, Bt64): the plain path's blocks above the
// shared-memory limit, and the mixed path's FP64 re-solve of such blocks
// (with a gate: only blocks with gate[b] == 2 or 4 are solved).
void launch_eig_bisect_f64(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem,
                           cudaStream_t s, const int *gate = nullptr);
// fp64: the FP64 reflector solver's buffers (W64, V64) and tiles.
bool reflect_config(int max_n, int *tw, int *panel, bool fp64 = false);
int reflect_max_n(bool fp64 = false);
// largest block the reflector solver's reduction (k_eig_bi) takes
int eig_bi_max_n(bool fp64);
// whether column tiles of width tw fit for blocks up to max_n (and the
// largest reflector panel that does)
bool reflect_fits(int max_n, int tw, int *panel, bool fp64 = false);
void launch_reflect(const EigBlock *blocks, const int2 *tiles, int ntiles, int max_n, int tw, int panel,
                    cudaStream_t s, bool fp64 = false, const int *gate = nullptr);
// FP64 Householder tridiagonalisation + implicit QL, one CTA per block.
// status[b] != 0 if block b hit the QL iteration cap.
// max_n: largest block of the launch; blocks with n <= max_n_smem are solved
// in shared memory, larger ones in their own global buffer.  With a gate,
// only blocks with gate[b] == 2 or 4 are solved (the others return at once).
void launch_eig_f64(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem, int *status,
                    cudaStream_t s, const int *gate = nullptr);
// Same algorithm in FP32 (mixed path first stage); writes U and E in FP64.
void launch_eig_f32(const EigBlock *blocks, int nblocks, int max_n, int max_n_smem, int *status,
                    cudaStream_t s);
// Thread-block-cluster solver (k_eig_cluster.cu) for blocks above the
// one-CTA shared-memory limit: the cluster size (8 or 16 CTAs) whose
// distributed shared memory holds an n-block, 0 when none does; launches one
// cluster per block (the same outputs as k_eig_bi: E, reflectors in W, V).
int eig_cluster_size_for(int n, bool fp64);
cudaError_t launch_eig_cluster(const EigBlock *blocks, int nblocks, int max_n, int cs, bool fp64,
                               cudaStream_t s);
int eig_smem_limit_f64();
int eig_smem_limit_f32();
int eig_max_n_f64();
int eig_max_n_f32();

// ------------------------------------------- mixed-precision refinement
struct RefineBlock {
  const double *S, *G;  // X^T A X and X^T X (n x n, leading dimension ld)
  double *E2;           // Newton correction E (ld)
  const double *X;      // current eigenvector estimate (ld)
  double *U;            // final eigenvectors, columns ascending (ldu)
  double *Eout;         // final eigenvalues, ascending
  int n, ld, ldu, pad;
};
// The element-wise passes run on row strips: tiles = (block, first row), one
// per oa_strip_rows() rows of each block.
int oa_strip_rows();
void launch_oa_update(const RefineBlock *blocks, const int2 *tiles, int ntiles, int max_n, double tau_rel,
                      cudaStream_t s);
// flag[b] = 1 (zeroed by the caller): the refinement of block b has not
// converged or a Rayleigh quotient is not finite.
void launch_oa_check(const RefineBlock *blocks, const int2 *tiles, int ntiles, int max_n, double tau_rel,
                     int *flag, cudaStream_t s);
// status[b] = 2: flagged by launch_oa_check; the block is re-solved with
// the FP64 solver.  status[b] = 3: a chain of near-degenerate levels too long
// for the in-kernel Jacobi, left to launch_oa_bigcl.
void launch_oa_final(const RefineBlock *blocks, int nblocks, int max_n, double tau_rel, int *status,
                     const int *flag, cudaStream_t s);
// Blocks with status 3 (a chain of near-degenerate levels longer than the
// final pass's 64): Rayleigh-Ritz on each such chain (up to 1024 levels) in
// FP64, status back to 0, or 2 when it cannot (k_eig.cu).
void launch_oa_bigcl(const RefineBlock *blocks, int nblocks, int max_n, double tau_rel, int *status,
                     cudaStream_t s);
int refine_max_n();

// ----------------------------------------------------------- grouped GEMM
// C (M x N) = [C if accumulate] + sum_c alpha_c op(A_c) op(B_c)
struct GemmGroup {
  double *C;
  int ldc, M, N, accumulate;
  int c0, c1;           // contributions [c0, c1)
};
struct GemmContrib {
  const double *A, *B;
  int lda, ldb, K, trans;  // trans bit0: A stored K x M; bit1: B stored N x K
  double alpha;
};
struct GemmTile {
  int group, tm, tn, pad;
};
void launch_gemm_f64(const GemmTile *tiles, int ntiles, const GemmGroup *groups,
                     const GemmContrib *contribs, cudaStream_t s);
constexpr int GEMM_TILE = 64;

// ------------------------------------- FP64-accurate tensor-core GEMM
// Digit planes of one FP64 block (k_ozaki.cu): 8 bf16 planes, plane p at
// planes + p * pstride, row r at + r * ldp; value = 2^(exp-55) *
// sum_p plane_p * 128^(7-p).
struct SplitTask {
  const double *src;
  int rows, cols, ld, ldp;
  void *planes;        // __nv_bfloat16
  int64_t pstride;
  int *exp;            // written: block exponent
};
struct OzOperand {
  const __nv_bfloat16 *p;  // plane 0 (already offset to the first row used)
  int64_t pstride;
  int ld, pad;
  const int *exp;
};
struct OzContrib {
  OzOperand A, B;
  int K, trans;            // trans bit0: A stored K x M; bit1: B stored N x K
  double alpha;
  int tmA, tmB;            // TMA tensor maps of op(A), op(B) in the launch's map array
  int pad0, pad1;
};
// One TMA tensor map (CUtensorMap: 128 bytes, 64-byte aligned).
struct alignas(64) OzTensorMap {
  unsigned char bytes[128];
};
// Tensor map of one operand view for k_gemm_oz's stage boxes: a 3-D tensor
// (inner: the contiguous dimension, `inner` elements; outer: `outer` rows of
// o.ld elements; planes: `planes` of o.pstride elements), box 8 x box_outer x 8.
// K-major operands: inner = K, box_outer = 128 (A) or 64 (B); MN-major ones:
// inner = M or N, outer = K, box_outer = 16.  Returns false if the driver
// rejects the description.
bool encode_oz_map(OzTensorMap *out, const OzOperand &o, int inner, int outer, int planes, int box_outer);
struct OzGroup {
  double *C;
  int ldc, M, N, accumulate;
  int c0, c1;
  int planes, pad;  // digit planes used (1..8): groups d < planes, pairs p + q < planes
};
// Grid-wide split: chunk0 holds per-task prefix counts of chunks of
// split_chunk_elements() padded elements (rows * ldp, below 2^31 per task);
// maxbits: ntasks of scratch.
int split_chunk_elements();
void launch_split_grid(const SplitTask *tasks, const int64_t *chunk0, int ntasks, int64_t nchunks,
                       unsigned long long *maxbits, cudaStream_t s);
// tiles: (group, 128-row tile, 64-column tile); *err is set when a bounded
// wait inside the kernel runs out (the launch then leaves its tile unfinished)
constexpr int OZ_TILE_M = 128, OZ_TILE_N = 64;
void launch_gemm_oz(const GemmTile *tiles, int ntiles, const OzGroup *groups, const OzContrib *contribs,
                    const OzTensorMap *maps, int *err, cudaStream_t s);

// ------------------------------------------------------------- truncation
struct TruncRun {
  int b0, b1;           // device blocks [b0, b1) of this run
  int e0, e1;           // eigenvalues [e0, e1) in the concatenated index space
  int64_t nkeep;
  double *sorted;       // all_eigenvalue output (e1 - e0)
};
struct TruncBlock {
  const double *E;      // ascending eigenvalues of the block
  int n, e0;            // size and first global element index
};
struct TruncResult {    // per run
  double emin, thr;
  int64_t kept_total, total;
  int truncated, pad;
};
void launch_truncate(const TruncRun *runs, int nruns, const TruncBlock *blocks, int nblocks,
                     const int *elem_block, int nelem, int *kept, TruncResult *res,
                     cudaStream_t s);

// ------------------------------------------------------------- FDM / misc
struct FdmPair {          // one (op, i, j) spectral contribution
  const double *rhoA;     // B rho_j   (n_i x n_j, ld nj)
  const double *ARho;     // rho_i B   (n_i x n_j, ld nj)
  const double *B;        // operator block (n_i x n_j, ld nj)
  const double *Ei, *Ej;  // eigenvalues of blocks i and j
  double *pos, *neg;      // this op's histograms (npts each) of the pair's run
  double scale;           // energy scale of the pair's shell
  int ni, nj, kci, kcj;   // sizes and current kept counts
  int64_t chunk0;
};
// chunks of 256 elements; chunk0 of each pair is increasing
void launch_fdm_bin(const FdmPair *pairs, int npairs, int64_t nchunks, double delE, int npts, cudaStream_t s);
struct RhoTask {          // one n x n block of a shell's density matrix
  double *rho;
  const double *diag;     // last shell: Boltzmann weights on the diagonal (or null)
  const double *red;      // earlier shells: reduced density matrix, kc x kc (or null)
  int n, kc;
  int64_t chunk0;         // prefix of 256-element chunks
};
// rho = red in the kept x kept corner, diag on the diagonal elsewhere, 0 otherwise
void launch_rho_init(const RhoTask *tasks, int ntasks, int64_t nchunks, cudaStream_t s);
struct TraceTask {        // one reduced-density-matrix output (k x k)
  double *out;
  int k, in0, in1, pad;
};
struct TraceIn {          // one sub-block (ii, bb) of a rotated rho block
  const double *rho;
  int ld, off, d, pad;
};
void launch_partial_trace(const TraceTask *tasks, int ntask, const TraceIn *ins, int maxk,
                          cudaStream_t s);
void launch_broaden(const double *e, const double *w, int64_t nbins, const double *omegas,
                    int64_t nomega, double b, double *out, cudaStream_t s);
// sums: (3 + nq) * nshell * nt doubles of scratch; qv: nq system-operator
// diagonals in the layout of disc (ndisc entries each), opexp: nq x nt
constexpr int kThermoMaxOps = 8;
void launch_thermo(const double *disc, const int64_t *disc_off, const double *gs, int nshell,
                   const double *temps, int nt, double bathdim, const double *qv, int nq, int64_t ndisc,
                   double *sums, double *entropy, double *cv, double *opexp, cudaStream_t s);
struct StaticTask {       // one diagonal operator block (i, i) of one shell
  const double *O;        // operator block, n x n, leading dimension ldo
  const double *rho;      // the shell's density-matrix block, n x n
  int n, ldo, kc, op;     // kc: kept states of block i (kept x kept part skipped)
};
// acc[op] += sum over the op's tasks, in task order; partial: ntasks doubles
void launch_fdm_static(const StaticTask *tasks, int ntasks, int nops, double *partial, double *acc,
                       cudaStream_t s);

}  // namespace nrg
