// Host-side engine state (C++).  Internal to libnrggpu; the public surface is
// the C ABI in include/nrg_gpu.h.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "nrg_gpu.h"
#include "nrg_internal.h"

namespace nrg {

struct Error {
  int code;
  std::string msg;
};
[[noreturn]] void fail(int code, const std::string &msg);
void check_cuda(cudaError_t e, const char *what);

// Device allocation owned by shared_ptr so snapshots and operator sets can
// keep a site's buffers alive after the run moves on.
struct DevMem {
  void *ptr = nullptr;
  size_t bytes = 0;
  nrg_engine *eng = nullptr;
  ~DevMem();
};
using DevPtr = std::shared_ptr<DevMem>;

struct HostMat {
  int rows = 0, cols = 0;
  std::vector<double> v;
};

struct SiteModel {
  int nq = 0;
  std::vector<std::vector<int>> q;
  std::vector<std::vector<double>> E;
  std::vector<double> chi;
  int nops = 0;
  std::vector<std::map<std::pair<int, int>, HostMat>> op;  // per operator: (row, col) -> block
  // device copies (bath only): energies per sector and f-dagger blocks
  DevPtr dev;
  std::vector<int64_t> e_off;                                      // energies offset per sector
  std::vector<std::map<std::pair<int, int>, int64_t>> op_off;      // block data offsets
};

struct Sub {          // sub-block (ii, bb) of a sector
  int ii, bb, off, k, d;
};

struct Sector {       // one sector of the current basis
  std::vector<Sub> subs;  // only sub-blocks with k*d > 0
  int n = 0;
  int dev = -1;           // device block index, -1 if empty
};

struct DevBlock {     // non-empty sector on the device
  int sector = 0;
  int n = 0, ld = 0;
  double *H = nullptr, *U = nullptr, *E = nullptr;
  OzOperand uop{};    // digit planes of U (mixed path), when present
};

struct FBlock {       // one operator block on the device
  double *p = nullptr;
  int rows = 0, cols = 0, ld = 0;
};
using OpKey = std::tuple<int, int, int>;  // (op, row sector, col sector)

// A site's device data that later passes need: the eigenvectors U, the
// eigenvalues E (unshifted) and the sector layout.
struct SiteData {
  int64_t iteration = 0;
  std::vector<std::vector<int>> cur_q, pre_q;
  std::vector<std::vector<uint64_t>> coupled;
  std::vector<Sector> sectors;
  std::vector<DevBlock> blocks;
  std::vector<int64_t> kept_prev;  // eigenvaluesQ_kept_indices sizes (pre sectors)
  DevPtr mem_U, mem_E;
  std::vector<std::vector<double>> E_host;  // eigenvalues per sector (unshifted)
  DevPtr mem_Uplanes, mem_Uexps;            // digit planes of every U block (mixed path)
  bool has_uplanes = false;
};

// FP64 matrix view and its bf16 digit planes (tensor-core GEMM operands).
constexpr int kDigitPlanes = 8;
struct MatRef {
  const double *p;
  int rows, cols, ld;
};
struct PlaneBuf {
  DevPtr mem, exps;
  std::vector<OzOperand> ops;  // plane-0 operand of each matrix (row 0)
  OzOperand op(size_t i, int row0 = 0) const {
    OzOperand o = ops[i];
    o.p += int64_t(row0) * o.ld;
    return o;
  }
};

PlaneBuf split_matrices(nrg_engine *e, const std::vector<MatRef> &mats, std::vector<DevPtr> &hold);

// One tensor-core (Ozaki) grouped-GEMM launch: C = [C +] sum alpha op(A) op(B).
struct OzList {
  std::vector<OzGroup> groups;
  std::vector<OzContrib> contribs;
  std::vector<GemmTile> tiles;
  double flops = 0;   // bf16 tensor-pipe flops: 2MNK per digit-plane product
  double useful = 0;  // FP64-accurate work: 2MNK per contribution
  int planes = kDigitPlanes;  // digit planes of the products (fewer: a cheaper, less exact product)
  // upper: only the tiles that meet the upper triangle (symmetric outputs whose
  // readers use the upper triangle)
  void out(double *C, int ldc, int M, int N, bool acc, const std::vector<OzContrib> &cs, bool upper = false);
  void launch(nrg_engine *e, std::vector<DevPtr> &hold);
};
OzContrib ozc(const OzOperand &A, const OzOperand &B, int K, int trans, double alpha = 1.0);

struct Snapshot {
  std::shared_ptr<SiteData> site;
  std::map<OpKey, FBlock> ops;
  int nops = 0;
  DevPtr ops_mem;
};

}  // namespace nrg

struct nrg_engine {
  int device = 0;
  int precision = NRG_PREC_FP64;
  uint64_t budget = 0;
  uint64_t used = 0;
  uint64_t peak = 0;  // high-water mark of `used`
  int verbose = 0;
  cudaStream_t stream = nullptr;
  // side stream: work of one phase that may overlap the main stream's
  // (forked and joined with fork_ev / join_ev, both without timing)
  cudaStream_t side = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  cudaEvent_t ev[8] = {};
  double phase_ms[5] = {0, 0, 0, 0, 0};
  uint64_t launches = 0;
  int eig_smem_f64 = 0, eig_smem_f32 = 0;
  // blocks above the one-CTA shared-memory limit go to the cluster solver
  // (NRG_EIG_CLUSTER=0 turns it off)
  // blocks above one SM's shared memory: 0 = one-CTA solver only, 1 = the
  // cluster solver when every cluster of the launch fits one wave of the
  // device (a latency-bound launch), 2 = the cluster solver always
  int eig_cluster = 1;
  int sm_count = 0;
  // launch-shape autotuner (nrg_engine_set_autotune): per block-size
  // histogram, the reflector back-transform's column-tile width and panel,
  // picked by timing every candidate on the first launch that shows the
  // histogram (all candidates give bit-identical results)
  bool autotune = true;
  struct Tuned {
    int tw = 0, panel = 0;
    std::string what;
  };
  std::map<uint64_t, Tuned> tuned;
  int *d_kerr = nullptr;  // set by kernels whose bounded waits ran out (k_gemm_oz)
  // pinned ring for host -> device uploads (descriptor tables): a copy from
  // pageable memory may wait for the stream to drain, one from pinned memory
  // does not, so the host can build the next phase while the GPU runs
  struct PinnedSpan {
    size_t a, b;
    cudaEvent_t ev;
  };
  char *ring = nullptr;
  size_t ring_cap = 0, ring_head = 0;
  std::deque<PinnedSpan> ring_busy;
  std::vector<cudaEvent_t> ring_events;
  uint64_t fallback_blocks = 0;  // mixed path: blocks re-solved in FP64
  // algorithmic work since the last read (nrg_engine_work_counters):
  // [0] F_eig = sum (10/3) n^3 over solved blocks, [1] F_rot = sum
  // 2 n_i n_j min(n_i, n_j) over non-empty f-dagger blocks (i, j) of each
  // operator, [2] FP64-accurate tensor-core GEMM work (2MNK per
  // contribution), [3] the bf16 tensor-pipe flops that work took (2MNK per
  // digit-plane product)
  double work[4] = {0, 0, 0, 0};
  // mixed path: FP64-accurate GEMMs on the tensor cores, bit 0 for the
  // eigenvector refinement, bit 1 for the operator rotations
  int ozaki = 3;
  // optional per-kernel event timing (nrg_engine_set_profiling)
  bool profile = false;
  struct ProfRec {
    std::string name;
    cudaEvent_t a, b;
    double work;  // algorithmic flops (bytes for memory-bound kernels) of the launch
  };
  std::vector<ProfRec> prof;
  std::vector<cudaEvent_t> ev_pool;
};

namespace nrg {
// Fails with NRG_E_CUDA (and clears the word) when a kernel has reported a
// timed-out wait; call after a stream synchronisation.
void check_kernel_error(nrg_engine *e);
// Stream-ordered host -> device copy of `bytes` through the engine's pinned
// ring: returns at once; the host buffer may be reused immediately.
void upload_async(nrg_engine *e, void *dst, const void *src, size_t bytes);
// Releases the pinned ring (engine destruction, after a stream sync).
void release_uploads(nrg_engine *e);
// Records CUDA events around one kernel launch on the engine stream when
// profiling is on; `work` is the launch's algorithmic flop count (byte count
// for the memory-bound kernels k_split and k_oa_update).
struct Prof {
  nrg_engine *e;
  const char *name;
  double work;
  cudaStream_t s;
  cudaEvent_t a = nullptr;
  Prof(nrg_engine *eng, const char *nm, double w = 0.0, cudaStream_t st = nullptr);
  ~Prof();
};
}  // namespace nrg

struct nrg_run {
  nrg_engine *eng = nullptr;
  nrg::SiteModel imp, bath;
  bool bath_pending = false;
  nrg::SiteModel bath_next;
  uint64_t nkeep = 1024;
  // API-visible state, mirroring nrgcore's public members
  int64_t cnt = 0, cnt_min = 0;
  std::vector<std::vector<int>> pre_q;
  std::vector<int64_t> kept;              // per pre sector
  int64_t no_of_kept = 0;
  std::vector<double> relgs;
  std::vector<double> all_eig;
  // previous basis on the device
  std::vector<const double *> prevE;      // per pre sector (null when empty)
  double prev_shift = 0.0;
  std::vector<std::vector<double>> prevE_host;  // eigenvaluesQ of the previous site (shifted view)
  std::shared_ptr<nrg::SiteData> prev_site;     // keeps prevE alive
  std::map<nrg::OpKey, nrg::FBlock> fprev;      // kept x kept f-dagger blocks
  nrg::DevPtr fprev_mem;
  // current site (after add_site)
  bool have_site = false;
  std::shared_ptr<nrg::SiteData> site;
  nrg::DevPtr mem_H;
  std::map<nrg::OpKey, nrg::FBlock> fcur;
  nrg::DevPtr fcur_mem;
  // pending truncation of the current site
  std::vector<int64_t> kept_new;          // per current sector
  std::vector<double> all_eig_pending;    // sorted eigenvalues of the current site
  nrg::TruncResult tres{};
  nrg::DevPtr mem_sorted;
  // snapshots for the backward passes
  std::map<int64_t, std::shared_ptr<nrg::Snapshot>> snaps;
  std::shared_ptr<nrg::Snapshot> loaded;
  int64_t device_bytes = 0;
};

struct nrg_opset {
  nrg_run *run = nullptr;
  int nops = 0;
  std::map<nrg::OpKey, nrg::FBlock> blocks;  // in the basis of the run's pre sectors
  nrg::DevPtr mem;
  bool updated_this_site = false;
};

struct nrg_fdm {
  nrg_run *run = nullptr;
  int nops = 0;
  bool last = true;
  bool have_cur = false;
  std::vector<int64_t> cur_kept, prev_kept;
  std::vector<nrg::DevPtr> reduced_mem;   // per sector of the next (earlier) shell
  std::vector<double *> reduced;          // device pointers, k x k
  std::vector<int64_t> reduced_k;
  bool have_reduced = false;
  nrg::DevPtr hist;                        // 2 * nops * npts
  double local_gs = 0, local_z = 0;
  std::vector<double> partitions;
  // finite temperature (nrg_fdm_set_temperature): per shell in backward
  // order, the Boltzmann weights of its discarded states (thermodynamics
  // layout: sectors in order, states past the kept prefix)
  bool finite_t = false;
  double temperature = 0;
  std::vector<std::vector<double>> shell_weights;
  size_t ncalc = 0;
  nrg::DevPtr static_acc;                  // nops running sums of rhoDotStaticOperators
};

struct nrg_thermo {
  nrg_run *run = nullptr;
  int64_t nmax = 0;
  double bathdim = 0;
  std::vector<double> temps;
  bool have_cur = false;
  std::vector<int64_t> cur_kept, prev_kept;
  std::vector<std::vector<double>> disc, allv;
  // system operators (setSystemOperator): indices into each snapshot's
  // operator set, and per shell their diagonals on the discarded states
  std::vector<int> sysops;
  std::vector<std::vector<double>> qval;  // per shell: nq x (discarded states)
  std::vector<double> opexp;              // nq x nt after nrg_thermo_final
};
