/*
 * nrg_gpu.h - C ABI of the GB300 NRG iteration engine.
 *
 * Plain C types only (pointers, sizes, doubles); no CUDA or torch types cross
 * this boundary.  Every call returns 0 on success or a positive NRG_E_* code;
 * nrg_last_error() returns the message of the last failure on this thread.
 * Host buffers passed in are copied before the call returns; host buffers
 * passed out must hold the sizes the matching *_info / count call reported.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the srbhp/nrgplusplus tree).
 */
#ifndef NRG_GPU_H
#define NRG_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* error codes */
#define NRG_OK 0
#define NRG_E_ARG 1        /* invalid argument (reference: std::runtime_error) */
#define NRG_E_STATE 2      /* call out of order */
#define NRG_E_CUDA 3       /* CUDA runtime error */
#define NRG_E_NOMEM 4      /* device memory or HBM budget exhausted */
#define NRG_E_EIG 5        /* block eigensolver did not converge in its sweep cap */
#define NRG_E_NOCUDA 6     /* no usable CUDA device */

/* precision modes */
#define NRG_PREC_FP64 0    /* plain FP64 path */
#define NRG_PREC_MIXED 1   /* FP32 bulk + FP64-accurate refinement */

typedef struct nrg_engine nrg_engine;
typedef struct nrg_run nrg_run;
typedef struct nrg_opset nrg_opset;
typedef struct nrg_fdm nrg_fdm;
typedef struct nrg_thermo nrg_thermo;

typedef struct {
  int device;                 /* CUDA device ordinal */
  int precision;              /* NRG_PREC_* */
  uint64_t hbm_budget_bytes;  /* 0 = no budget */
  int verbose;                /* 0 = silent */
} nrg_engine_opts;

/*
 * One site model (impurity or Wilson site): what nrgcore reads from a model
 * (nrgcore.hpp:44-53, 68-70): get_basis(), get_eigenvaluesQ(), get_chi_Q(),
 * f_dag_operator.  Operator blocks are dense row-major dims[row] x dims[col].
 */
typedef struct {
  int nq;                     /* quantum numbers per sector */
  int nsect;                  /* number of sectors */
  const int *qnum;            /* nsect * nq */
  const int *dims;            /* nsect */
  const double *energies;     /* sum(dims), sector by sector, ascending */
  const double *chi;          /* nsect (bath parity; may be NULL for impurity) */
  int nops;                   /* number of operators (f-dagger list) */
  int nblk;                   /* number of stored operator blocks */
  const int *blk_op;          /* nblk: operator index */
  const int *blk_row;         /* nblk: row sector */
  const int *blk_col;         /* nblk: column sector */
  const double *blk_data;     /* concatenated block data */
} nrg_site_desc;

/* Block-sparse operator list in a run's sector basis (qOperator, qOperator.hpp:18-19). */
typedef struct {
  int nops;
  int nblk;
  const int *blk_op;
  const int *blk_row;
  const int *blk_col;
  const int *blk_rows;        /* rows of each block */
  const int *blk_cols;        /* columns of each block */
  const double *blk_data;
} nrg_op_desc;

typedef struct {
  int64_t iteration;          /* nrg_iterations_cnt (nrgcore.hpp:536) */
  int64_t iteration_min;      /* nrg_iterations_min (nrgcore.hpp:538) */
  int64_t n_pre_sectors;      /* pre_sysmQ.size() */
  int64_t n_cur_sectors;      /* current_sysmQ.size() */
  int64_t n_all;              /* all_eigenvalue.size() */
  int64_t n_kept;             /* no_of_kept_states */
  int64_t n_relgs;            /* relativeGroundStateEnergy.size() */
  int64_t nq;                 /* quantum numbers per sector */
  int64_t n_device_blocks;    /* non-empty sectors held on the device */
  int64_t max_block;          /* largest block dimension this iteration */
  int64_t n_snapshots;
  int64_t device_bytes;       /* device memory held by this run (sites, f-dagger, snapshots) */
} nrg_run_info;

/* ---- engine ------------------------------------------------------------ */
const char *nrg_last_error(void);
int nrg_engine_create(const nrg_engine_opts *opts, nrg_engine **out);
int nrg_engine_destroy(nrg_engine *eng);
/* Wall time of the device phases of the last step, milliseconds:
 * out[0] assemble, out[1] eigensolve, out[2] truncate, out[3] rotate,
 * out[4] operators; n = entries written. */
int nrg_engine_phase_times(nrg_engine *eng, double *out, int cap, int *n);
/* The options the engine was created with. */
int nrg_engine_get_opts(nrg_engine *eng, nrg_engine_opts *out);
/* Number of kernel launches issued by the engine so far. */
int nrg_engine_launch_count(nrg_engine *eng, uint64_t *out);
/* Mixed precision: number of blocks whose refinement did not converge and
 * that were re-solved with the FP64 block solver (0 for NRG_PREC_FP64).
 * No counterpart in the reference (it has one FP64 path). */
int nrg_engine_fallback_count(nrg_engine *eng, uint64_t *out);
/* Device bytes the engine holds now and its high-water mark since creation
 * (or the last reset_peak != 0 call).  No counterpart in the reference. */
int nrg_engine_memory(nrg_engine *eng, uint64_t *used, uint64_t *peak, int reset_peak);
/* Per-kernel CUDA-event timing on the engine stream (off by default). */
int nrg_engine_set_profiling(nrg_engine *eng, int on);
/* Times recorded since the last call, aggregated per kernel: names (each
 * followed by '\n'), total milliseconds, algorithmic flops (bytes for the
 * memory-bound k_split and k_oa_update) and launch counts; nk = kernels
 * written.  Clears the record. */
int nrg_engine_kernel_times(nrg_engine *eng, char *names, uint64_t names_cap, double *ms,
                            double *work, uint64_t *count, int cap, int *nk);
/* Algorithmic work of the steps issued since the last reset (no counterpart
 * in the reference): out[0] F_eig = sum (10/3) n^3 over the blocks solved,
 * out[1] F_rot = sum 2 n_i n_j min(n_i, n_j) over the non-empty f-dagger
 * blocks (operator, i, j) of each new basis, out[2] the FP64-accurate
 * tensor-core GEMM work (2MNK per product), out[3] the bf16 tensor-pipe
 * flops it took (2MNK per digit-plane product); n = entries written. */
int nrg_engine_work_counters(nrg_engine *eng, double *out, int cap, int *n, int reset);
/* Launch-shape autotuner (no counterpart in the reference; on by default):
 * per block-size histogram of a launch (largest block, block count, total
 * size), the reflector back-transform's column-tile width and panel are
 * picked by timing every fitting candidate once, on the first launch that
 * shows the histogram (one stream synchronisation), and reused.  All
 * candidates compute every column in the same order, so results are the
 * same bit for bit whichever is picked.  on = 0: the widest tile that fits. */
int nrg_engine_set_autotune(nrg_engine *eng, int on);
/* Blocks above one SM's shared memory: 0 = the one-CTA eigensolver only,
 * 1 = the thread-block-cluster eigensolver when every cluster of the launch
 * fits one wave of the device (default; env NRG_EIG_CLUSTER), 2 = always. */
int nrg_engine_set_eig_cluster(nrg_engine *eng, int mode);
/* The decisions so far, one line per histogram with the candidates' times;
 * len = bytes of the report (written up to cap, NUL-terminated). */
int nrg_engine_autotune_report(nrg_engine *eng, char *buf, uint64_t cap, uint64_t *len);
int nrg_engine_sync(nrg_engine *eng);

/* ---- one NRG run (nrgcore<Imp,Bath>) ---------------------------------- */
/* nrgcore(im, bath) + set_parameters(nkeep): nrgcore.hpp:44-53, :336-342 */
int nrg_run_create(nrg_engine *eng, const nrg_site_desc *impurity, const nrg_site_desc *bath,
                   uint64_t nkeep, nrg_run **out);
int nrg_run_destroy(nrg_run *run);
/* set_parameters(n): nrgcore.hpp:336-342 (resets the run to iteration 0) */
int nrg_run_set_parameters(nrg_run *run, uint64_t nkeep);
/* bath refresh, nrgcore.hpp:68-70 (dynamic baths); takes effect at the next add_site */
int nrg_run_set_bath(nrg_run *run, const nrg_site_desc *bath);
/* add_bath_site(t, rescale): nrgcore.hpp:65-97 (assembly a2, eigensolve a3,
 * f-dagger rotation a4; the truncation of this site is computed but only
 * published by nrg_run_update_state, as in the reference) */
int nrg_run_add_site(nrg_run *run, const double *t, int nt, double rescale);
/* update_internal_state(): nrgcore.hpp:105-109 (truncation a5) */
int nrg_run_update_state(nrg_run *run);
/* checkHigherEnergyDiscarded(): nrgcore.hpp:384-386 */
int nrg_run_check_discarded(nrg_run *run, int *out);
int nrg_run_get_info(nrg_run *run, nrg_run_info *info);
/* all_eigenvalue (nrgcore.hpp:520), sorted, unshifted */
int nrg_run_get_all_eigenvalues(nrg_run *run, double *out, uint64_t cap);
/* relativeGroundStateEnergy (nrgcore.hpp:522) */
int nrg_run_get_relgs(nrg_run *run, double *out, uint64_t cap);
/* current_sysmQ / pre_sysmQ (nrgcore.hpp:528-530): which = 0 current, 1 pre */
int nrg_run_get_sectors(nrg_run *run, int which, int *qnum, uint64_t cap_sectors);
/* eigenvaluesQ (nrgcore.hpp:532) per current sector: dims[nsect] and the
 * concatenated values (shifted after update_state, as in the reference) */
int nrg_run_get_eigenvalues_q(nrg_run *run, uint64_t *dims, double *values, uint64_t cap_values);
/* eigenvaluesQ_kept_indices sizes per pre sector (nrgcore.hpp:524); the
 * kept indices are always the prefix 0..k-1 of each sector */
int nrg_run_get_kept(nrg_run *run, uint64_t *kept, uint64_t cap);
/* coupled_nQ_index (nrgcore.hpp:534): counts[n_cur] and flattened entries */
int nrg_run_get_coupled(nrg_run *run, uint64_t *counts, uint64_t *entries, uint64_t cap_entries);
/* current_hamiltonQ[sector] (nrgcore.hpp:526): eigenvectors as columns,
 * row-major n x n; n = dims[sector] */
int nrg_run_get_eigenvectors(nrg_run *run, int64_t sector, double *out, uint64_t cap);
/* get_f_dag_operator() / getPreWilsonSiteOperators() (nrgcore.hpp:377, :548):
 * block (ip, i, j) of the rotated f-dagger.  The engine keeps the kept x kept
 * part (all the next site reads, nrgcore.hpp:199-203); rows/cols report it. */
int nrg_run_get_fdag_block(nrg_run *run, int ip, int64_t i, int64_t j, double *out, uint64_t cap,
                           int64_t *rows, int64_t *cols);

/* ---- tracked operators: update_system_operator (sysOperator.hpp:36-133) -- */
/* ops given in the run's current "previous" basis (pre_sysmQ sectors) */
int nrg_opset_create(nrg_run *run, const nrg_op_desc *ops, nrg_opset **out);
int nrg_opset_destroy(nrg_opset *ops);
/* update_system_operator(nrg, ops): call after add_site, before update_state */
int nrg_opset_update(nrg_opset *ops);
/* update_system_operator for n operator sets (of runs on one engine, each
 * after its add_site) in shared launches; same results as n calls.  No
 * counterpart in the reference. */
int nrg_opset_update_batch(nrg_opset *const *ops, int n);
/* block (ip, i, j) of the tracked operator in the current basis */
int nrg_opset_get_block(nrg_opset *ops, int ip, int64_t i, int64_t j, double *out, uint64_t cap,
                        int64_t *rows, int64_t *cols);

/* Enumeration of the blocks behind nrg_opset_get_block / the f-dagger
 * (getPreWilsonSiteOperators) / the loaded snapshot's operator set
 * (NrgData::loadqOperator, nrgData.hpp:213-246): n = number of blocks; the
 * first min(n, cap) (operator, row sector, column sector, rows, cols) are
 * written to the arrays given (any may be NULL).  With these a host layer
 * rebuilds a caller's vector<qOperator> (qOperator::getMap) block by block. */
int nrg_opset_list_blocks(nrg_opset *ops, int *ip, int64_t *i, int64_t *j, int64_t *rows, int64_t *cols,
                          uint64_t cap, uint64_t *n);
int nrg_run_list_fdag_blocks(nrg_run *run, int *ip, int64_t *i, int64_t *j, int64_t *rows, int64_t *cols,
                             uint64_t cap, uint64_t *n);
int nrg_run_list_snapshot_ops(nrg_run *run, int *ip, int64_t *i, int64_t *j, int64_t *rows, int64_t *cols,
                              uint64_t cap, uint64_t *n);
int nrg_run_get_snapshot_op_block(nrg_run *run, int ip, int64_t i, int64_t j, double *out, uint64_t cap);

/* ---- device-resident snapshots (NrgData, nrgData.hpp:134-293) ---------- */
/* saveCurrentData + saveqOperator: keep this site's U, eigenvalues, kept
 * counts, sectors and the tracked operators on the device */
int nrg_run_snapshot(nrg_run *run, nrg_opset *ops);
/* loadCurrentData(iteration): select a stored snapshot for the backward pass */
int nrg_run_load_snapshot(nrg_run *run, int64_t iteration);
/* The run's snapshots written to a file in the layout NrgData writes into its
 * HDF5 file (nrgData.hpp:134-165 saveCurrentData, :175-210 saveqOperator,
 * :106-110 saveFinalState), as a flat container of named float64 arrays
 * (HDF5 itself is not linked): magic "NGRA" (u32 0x4152474e), u32 version 1,
 * then per array u32 name length, name, u64 count, count float64.  Per saved
 * iteration N: /NrgItrN/current_sysmQ, pre_sysmQ (flattened, nq per sector),
 * nq, eigenvaluesQ_kept_indices (kept count per pre sector; the kept states
 * are a prefix), eigenvaluesQ/<sector>, coupled_nQ_index/<sector>, with
 * with_vectors != 0 current_hamiltonQ/<sector> (eigenvectors as columns,
 * row-major), and the saved operator set op/operatorSize,
 * op/at<ip>/{qmat<k>, idVector, rowVector, colVector}; then savedNRGIndex
 * and relativeGroundStateEnergy.  Reader: nrgplusplus_gb300.archive. */
int nrg_run_export_snapshots(nrg_run *run, const char *path, int with_vectors);

/* ---- FDM spectral function, T = 0 (fdmSpectrum.hpp) ------------------- */
int nrg_fdm_create(nrg_run *run, int nops, nrg_fdm **out);     /* ctor + setOperator */
int nrg_fdm_destroy(nrg_fdm *f);
int nrg_fdm_calc(nrg_fdm *f, double energy_scale);               /* calcSpectrum :55-63 */
/* calcSpectrum of n FDM objects of different runs on one engine, each with
 * its snapshot loaded, in shared launches (one per phase); same results as
 * n nrg_fdm_calc calls.  No counterpart in the reference (it runs one). */
int nrg_fdm_calc_batch(nrg_fdm *const *fdms, int n, const double *energy_scales);
/* Finite temperature T (fdmSpectrum is T = 0 only, fdmSpectrum.hpp:27,284):
 * every shell's density matrix takes the Boltzmann weights of its discarded
 * states on the diagonal, the form fdmBackwardIteration::setRhoZero(
 * tBoltzmannFactor) takes (dynamics/fdmBackwardIteration.hpp:207-239), with
 * the weights the thermodynamics average with (w_m exp((E0_m - E)/T) / Z'_m,
 * fdmThermodynamics.hpp:159-218).  `thermo` must already have seen, in the
 * same backward order and energy scales, every shell this object will see
 * (nrg_thermo_calc per shell).  Call before the first nrg_fdm_calc. */
int nrg_fdm_set_temperature(nrg_fdm *f, double T, nrg_thermo *thermo);
/* rhoDotStaticOperators (fdmBackwardIteration.hpp:166-199) summed over the
 * shells computed so far: per operator, Tr(O_ii rho_i) over its diagonal
 * blocks with the kept x kept part of O left out; <O>(T) after the whole
 * backward pass at finite temperature. */
int nrg_fdm_get_static(nrg_fdm *f, double *out, int nops);
/* saveFinalData (:322-337): energy points and the positive/negative weights,
 * each nops x npts; npts = 100000 */
int nrg_fdm_get(nrg_fdm *f, double *energy_points, double *positive, double *negative,
                uint64_t npts);
/* log-Gaussian broadening (examples/fdmSpectrumSiam/spec.py:27-44):
 * out[k] = (1/w_k) sum_i weight_i exp(-(ln(w_k/e_i)/b - b/4)^2) / (b sqrt(pi)) */
int nrg_broaden(nrg_engine *eng, const double *energies, const double *weights, uint64_t nbins,
                const double *omegas, uint64_t nomega, double b, double *out);

/* nrg_broaden on caller-owned DEVICE buffers without any allocation.  No
 * counterpart in the reference (its broadening is host code on host arrays).
 * For callers that hold the histogram on the device and may not let a library
 * allocate device memory (a process whose HBM is reserved up front, e.g. under
 * an nrg_engine_opts budget or another framework's pool).
 * - Its one intermediate (ln e_i per bin) lives in a static device array of
 *   NRG_BROADEN_NOALLOC_MAX_BINS doubles (1 MiB); nbins above that is
 *   rejected with NRG_E_ARG.  No buffer has to start at zero: each call
 *   writes the nbins scratch entries it reads and every out[k].
 * - The current device is used.  Every call looks up the scratch address
 *   with that device current (cudaGetSymbolAddress; no address is cached,
 *   so a cudaDeviceReset between calls is safe); the first call on a device
 *   may load the kernels' module, so make it before any stream capture.
 * - Asynchronous: the kernels are enqueued on `stream` (a cudaStream_t;
 *   NULL = the legacy default stream) and the call returns; read `out` after
 *   that stream has completed.  All pointers must stay valid until then.
 * - The scratch is shared per device: calls whose work may overlap (other
 *   streams, other host threads on the same device) race on it.  Calls on one
 *   stream are ordered and safe. */
#define NRG_BROADEN_NOALLOC_MAX_BINS 131072
int nrg_broaden_noalloc(const double *energies, const double *weights, uint64_t nbins,
                        const double *omegas, uint64_t nomega, double b, double *out,
                        void *stream);

/* ---- thermodynamics (fdmThermodynamics.hpp) ---------------------------- */
/* ctor (:26-38): nrg_iterations from the run, bath dimension from the bath */
int nrg_thermo_create(nrg_run *run, const double *temps, int nt, nrg_thermo **out);
int nrg_thermo_destroy(nrg_thermo *t);
int nrg_thermo_calc(nrg_thermo *t, double energy_scale);        /* calcThermodynamics :42-89 */
int nrg_thermo_final(nrg_thermo *t, double *entropy, double *specific_heat); /* :101-236 */
/* setSystemOperator (:37-39): the operators op_index[0..n) (n <= 8) of the
 * operator set saved with each snapshot (nrg_run_snapshot) are the system
 * operators; calcThermodynamics keeps their (i, i) diagonals on the
 * discarded states (:63-88) and nrg_thermo_final averages them
 * (qsysOPeratorExpValue, :200-218).  Call before the first calc. */
int nrg_thermo_set_operator(nrg_thermo *t, const int *op_index, int n);
/* qsysOPeratorExpValue after nrg_thermo_final: n x nt values, row per operator. */
int nrg_thermo_get_operator(nrg_thermo *t, double *out, int n, int nt);

/* ---- standalone batched symmetric eigensolver --------------------------- */
/* The block solver behind qmatrix::diag (qmatrix.hpp:375-404, LAPACKE_dsyevd
 * 'V','U'): nblk dense symmetric row-major blocks H (concatenated), dims[b]
 * each; eigenvalues ascending into E (concatenated) and eigenvectors as
 * columns into U (row-major, concatenated).  Uses the engine's precision mode. */
int nrg_eigh_batched(nrg_engine *eng, int nblk, const int *dims, const double *H, double *E,
                     double *U);

/* ---- FP64-accurate GEMM on the tensor cores ------------------------------ */
/* C = alpha op(A) op(B) (+ C when beta == 1; beta must be 0 or 1), row-major
 * host buffers; op(X) = X^T when trans is set.  The engine's building block
 * behind the operator rotations of qmatrix::dot (qmatrix.hpp:351-374,
 * cblas_dgemm): digit-split bf16 products with exact FP32 sums, combined in
 * FP64, accurate to FP64 round-off. */
int nrg_dgemm_tc(nrg_engine *eng, int transA, int transB, int M, int N, int K, double alpha,
                 const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc);

/* ---- batched stepping of independent runs (one launch per phase) ------- */
int nrg_batch_add_site(nrg_run *const *runs, int nruns, const double *t, int nt,
                       const double *rescale);
int nrg_batch_update_state(nrg_run *const *runs, int nruns);

/* ---- serving loop: continuous batching of whole runs ------------------- */
/* No counterpart in the reference (its drivers run one nrgcore at a time).
 * A server owns worker threads, each driving one engine (the first worker the
 * engine given to nrg_server_create, every further worker an engine the
 * server creates with the same options and destroys with the server):
 * requests submitted from any thread queue up, are admitted by the workers
 * while a worker has fewer than max_active runs (and no more than its even
 * share of the active and queued runs) and their estimated device footprint
 * fits hbm_budget_bytes next to the reservations of every active run (0 = no
 * budget; an idle server admits one request regardless), and every tick of a
 * worker advances its active runs by one Wilson site in shared launches
 * (nrg_batch_add_site per hopping count), then runs the backward passes
 * (FDM spectrum, thermodynamics) of its runs that finished.  Several workers
 * overlap the host work of one engine's tick with the GPU work of another's.
 * Results are kept until nrg_server_release.  The given engine must not be
 * used by other threads while a server drives it. */
typedef struct nrg_server nrg_server;
typedef struct {
  int max_active;             /* runs stepped together per worker (>= 1) */
  uint64_t hbm_budget_bytes;  /* admission budget over all workers, 0 = none */
  int workers;                /* worker threads / engines, 0 or 1 = one */
} nrg_server_opts;
typedef struct {
  const nrg_site_desc *impurity, *bath;
  uint64_t nkeep;
  int nsites;                 /* add_bath_site calls */
  int nt;                     /* hoppings per site */
  const double *t;            /* nsites * nt */
  const double *rescale;      /* nsites */
  const nrg_op_desc *ops;     /* tracked operators, NULL = none; created after the
                                 first site, in the impurity's sector basis */
  int fdm;                    /* 1: T = 0 FDM spectrum of ops */
  int ntemps;                 /* thermodynamics on temps[ntemps], 0 = none */
  const double *temps;
  const double *shell_scale;  /* nsites: energy scale of the shell kept after each site */
  int first_shell_site;       /* shells are kept after sites >= this one that discard states */
  int keep_eigenvalues;       /* 1: return all_eigenvalue after every site */
} nrg_request;
typedef struct {
  int done;                   /* 1 when finished (ok or failed) */
  int status;                 /* NRG_OK or the failing call's code */
  double latency_s;           /* submit -> finish */
  double queue_s;             /* submit -> admission */
  int nsites, nops, npts, ntemps;
  int64_t n_eig_total;        /* sum of the per-site all_eigenvalue sizes */
  uint64_t peak_device_bytes; /* largest device footprint the run showed */
  char message[256];          /* error text when status != NRG_OK */
} nrg_result_info;
typedef struct {
  uint64_t submitted, completed, failed, queued, max_active_seen, ticks;
  double busy_s;              /* worker time spent in ticks */
  double p50_latency_s, p99_latency_s, mean_latency_s, max_latency_s;
  double footprint_coef;      /* admission estimate: coef * nsites * (bath states * nkeep)^2 bytes */
} nrg_server_stats_t;
int nrg_server_create(nrg_engine *eng, const nrg_server_opts *opts, nrg_server **out);
/* stops the worker after its current tick; unfinished requests fail */
int nrg_server_destroy(nrg_server *srv);
/* copies the request; thread-safe */
int nrg_server_submit(nrg_server *srv, const nrg_request *req, uint64_t *id);
int nrg_server_wait(nrg_server *srv, uint64_t id, double timeout_s, int *done);
int nrg_server_result_info(nrg_server *srv, uint64_t id, nrg_result_info *info);
/* any output may be NULL; sizes from nrg_result_info (eigs: n_eig_total,
 * eig_counts: nsites, energy_points: npts, positive / negative: nops x npts,
 * entropy / cv: ntemps) */
int nrg_server_get_result(nrg_server *srv, uint64_t id, double *eigs, uint64_t *eig_counts,
                          double *energy_points, double *positive, double *negative,
                          double *entropy, double *cv);
int nrg_server_release(nrg_server *srv, uint64_t id);
/* latency percentiles over the requests completed since creation or the
 * last reset != 0 call (nearest rank) */
int nrg_server_stats(nrg_server *srv, nrg_server_stats_t *stats, int reset);

#ifdef __cplusplus
}
#endif
#endif /* NRG_GPU_H */
