// Host side of the GB300 NRG engine: basis bookkeeping, descriptor tables and
// the launch sequence of one NRG site for a batch of independent runs.
//
// Reference correspondence (srbhp/nrgplusplus):
//   create_next_basis         nrgcore.hpp:238-261   -> build_basis()
//   create_next_hamiltonians  nrgcore.hpp:146-230   -> k_assemble (k_assemble.cu)
//   qmatrix::diag per block   nrgcore.hpp:85-89     -> k_eig (k_eig.cu)
//   discard_higher_energies   nrgcore.hpp:269-327   -> k_rank/k_select (k_trunc.cu)
//   set_current_fdag_operator nrgcore.hpp:401-477   -> grouped GEMM (k_gemm.cu)
//   update_internal_state     nrgcore.hpp:105-109   -> nrg_run_update_state
//
// Empty sectors (no kept states) stay in the API-level sector lists exactly as
// the reference keeps them, but never reach the device.
#include <algorithm>
#include <cstdio>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <unordered_map>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>

#include "engine_core.h"

namespace nrg {

thread_local std::string g_err;

[[noreturn]] void fail(int code, const std::string &msg) { throw Error{code, msg}; }

void check_cuda(cudaError_t e, const char *what) {
  if (e != cudaSuccess)
    fail(e == cudaErrorMemoryAllocation ? NRG_E_NOMEM : NRG_E_CUDA,
         std::string(what) + ": " + cudaGetErrorString(e));
}

DevMem::~DevMem() {
  if (ptr) {
    cudaFreeAsync(ptr, eng->stream);
    eng->used -= bytes;
  }
}

static DevPtr dalloc(nrg_engine *e, size_t bytes) {
  auto m = std::make_shared<DevMem>();
  m->eng = e;
  if (bytes == 0) return m;
  bytes = (bytes + 255) & ~size_t(255);
  if (e->budget && e->used + bytes > e->budget)
    fail(NRG_E_NOMEM, "HBM budget exhausted (" + std::to_string(e->used + bytes) + " > " +
                          std::to_string(e->budget) + " bytes)");
  check_cuda(cudaMallocAsync(&m->ptr, bytes, e->stream), "cudaMallocAsync");
  m->bytes = bytes;
  e->used += bytes;
  if (e->used > e->peak) e->peak = e->used;
  return m;
}

// Host staging of the descriptor tables of one launch phase: one device
// buffer and one copy per phase.
struct Arena {
  std::vector<char> buf;
  template <class T> size_t add(const std::vector<T> &v) {
    size_t off = (buf.size() + 255) & ~size_t(255);
    buf.resize(off + v.size() * sizeof(T) + 16);
    if (!v.empty()) std::memcpy(buf.data() + off, v.data(), v.size() * sizeof(T));
    return off;
  }
  char *push(nrg_engine *e, DevPtr &hold) {
    hold = dalloc(e, buf.size());
    if (!buf.empty())
      upload_async(e, hold->ptr, buf.data(), buf.size());
    return static_cast<char *>(hold->ptr);
  }
};

template <class T> static T *at(char *base, size_t off) { return reinterpret_cast<T *>(base + off); }

static void count_launch(nrg_engine *e, int n = 1) { e->launches += n; }

void upload_async(nrg_engine *e, void *dst, const void *src, size_t bytes) {
  if (bytes == 0) return;
  const size_t need = (bytes + 255) & ~size_t(255);
  if (need > e->ring_cap) {  // (re)allocate: wait for every pending copy first
    check_cuda(cudaStreamSynchronize(e->stream), "upload ring");
    release_uploads(e);
    const size_t cap = std::max<size_t>(size_t(64) << 20, 2 * need);
    check_cuda(cudaHostAlloc(reinterpret_cast<void **>(&e->ring), cap, cudaHostAllocDefault), "cudaHostAlloc");
    e->ring_cap = cap;
    e->ring_head = 0;
  }
  if (e->ring_head + need > e->ring_cap) {
    // wrap: the stream runs in order, so once the newest copy is done every
    // region of the ring is free again
    if (!e->ring_busy.empty()) check_cuda(cudaEventSynchronize(e->ring_busy.back().ev), "upload ring wait");
    for (auto &sp : e->ring_busy) e->ring_events.push_back(sp.ev);
    e->ring_busy.clear();
    e->ring_head = 0;
  }
  const size_t a = e->ring_head, b = a + need;
  // within one lap no region is handed out twice; recycle finished events
  while (!e->ring_busy.empty() && cudaEventQuery(e->ring_busy.front().ev) == cudaSuccess) {
    e->ring_events.push_back(e->ring_busy.front().ev);
    e->ring_busy.pop_front();
  }
  std::memcpy(e->ring + a, src, bytes);
  check_cuda(cudaMemcpyAsync(dst, e->ring + a, bytes, cudaMemcpyHostToDevice, e->stream), "upload");
  cudaEvent_t ev;
  if (e->ring_events.empty()) {
    check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
  } else {
    ev = e->ring_events.back();
    e->ring_events.pop_back();
  }
  check_cuda(cudaEventRecord(ev, e->stream), "event");
  e->ring_busy.push_back({a, b, ev});
  e->ring_head = b;
}

void release_uploads(nrg_engine *e) {
  for (auto &sp : e->ring_busy) e->ring_events.push_back(sp.ev);
  e->ring_busy.clear();
  if (e->ring) cudaFreeHost(e->ring);
  e->ring = nullptr;
  e->ring_cap = e->ring_head = 0;
}

void check_kernel_error(nrg_engine *e) {
  int h = 0;
  check_cuda(cudaMemcpy(&h, e->d_kerr, sizeof(int), cudaMemcpyDeviceToHost), "kernel error word");
  if (h) {
    cudaMemset(e->d_kerr, 0, sizeof(int));
    fail(NRG_E_CUDA, "a tensor-core GEMM wait timed out (results of that launch are incomplete)");
  }
}

static void post_launch(const char *what) { check_cuda(cudaGetLastError(), what); }

void ensure_nonportable_cluster(const void *kernel) {
  static std::mutex mu;
  static std::set<std::pair<const void *, int>> done;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  if (done.count({kernel, dev})) return;
  check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1),
             "cudaFuncSetAttribute(non-portable cluster size)");
  done.insert({kernel, dev});
}

void ensure_smem_limit(const void *kernel, int bytes) {
  // the attribute only ever grows: a launch needing less than the limit set
  // for an earlier launch is fine, one needing more raises it
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, int> limit;  // (kernel, device) -> bytes set
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  int &cur = limit[{kernel, dev}];
  if (bytes <= cur) return;
  check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes),
             "cudaFuncSetAttribute(dynamic shared memory)");
  cur = bytes;
}

// ---------------------------------------------------------------- models
static SiteModel parse_site(const nrg_site_desc *d, bool need_chi) {
  if (!d) fail(NRG_E_ARG, "null site description");
  if (d->nq <= 0 || d->nsect <= 0) fail(NRG_E_ARG, "site needs nq > 0 and nsect > 0");
  if (!d->qnum || !d->dims || !d->energies) fail(NRG_E_ARG, "site arrays missing");
  if (need_chi && !d->chi) fail(NRG_E_ARG, "bath site needs chi (fermion parity per sector)");
  SiteModel m;
  m.nq = d->nq;
  m.q.resize(d->nsect);
  m.E.resize(d->nsect);
  int64_t eo = 0;
  for (int s = 0; s < d->nsect; ++s) {
    m.q[s].assign(d->qnum + int64_t(s) * d->nq, d->qnum + int64_t(s + 1) * d->nq);
    if (d->dims[s] < 0) fail(NRG_E_ARG, "negative sector dimension");
    m.E[s].assign(d->energies + eo, d->energies + eo + d->dims[s]);
    eo += d->dims[s];
  }
  if (d->chi) m.chi.assign(d->chi, d->chi + d->nsect);
  m.nops = d->nops;
  m.op.resize(std::max(0, d->nops));
  int64_t bo = 0;
  for (int b = 0; b < d->nblk; ++b) {
    int ip = d->blk_op[b], r = d->blk_row[b], c = d->blk_col[b];
    if (ip < 0 || ip >= d->nops || r < 0 || r >= d->nsect || c < 0 || c >= d->nsect)
      fail(NRG_E_ARG, "operator block index out of range");
    HostMat hm;
    hm.rows = d->dims[r];
    hm.cols = d->dims[c];
    hm.v.assign(d->blk_data + bo, d->blk_data + bo + int64_t(hm.rows) * hm.cols);
    bo += int64_t(hm.rows) * hm.cols;
    if (m.op[ip].count({r, c})) fail(NRG_E_ARG, "Found operator already");  // qOperator.hpp:58
    m.op[ip][{r, c}] = std::move(hm);
  }
  return m;
}

static void upload_bath(nrg_engine *e, SiteModel &m) {
  std::vector<double> flat;
  m.e_off.clear();
  for (auto &v : m.E) {
    m.e_off.push_back(int64_t(flat.size()));
    flat.insert(flat.end(), v.begin(), v.end());
  }
  m.op_off.assign(m.op.size(), {});
  for (size_t ip = 0; ip < m.op.size(); ++ip)
    for (auto &kv : m.op[ip]) {
      m.op_off[ip][kv.first] = int64_t(flat.size());
      flat.insert(flat.end(), kv.second.v.begin(), kv.second.v.end());
    }
  m.dev = dalloc(e, flat.size() * sizeof(double) + 8);
  check_cuda(cudaMemcpyAsync(m.dev->ptr, flat.data(), flat.size() * sizeof(double),
                             cudaMemcpyHostToDevice, e->stream),
             "bath upload");
  check_cuda(cudaStreamSynchronize(e->stream), "bath upload");
}

static const double *bath_ptr(const SiteModel &m, int64_t off) {
  return static_cast<const double *>(m.dev->ptr) + off;
}

// --------------------------------------------------------------- step
struct RunStep {          // per-run working data of one batched add_site
  nrg_run *run;
  std::shared_ptr<SiteData> site;
  std::vector<double> t;
  double rescale;
  std::map<std::pair<int, int>, std::pair<int, int>> sub_of;  // (ii,bb) -> (sector, off)
  int b0 = 0, e0 = 0, e1 = 0;  // device block / element ranges in the batch
};

static void reference_discard(nrg_run *r, std::vector<std::vector<double>> &E) {
  // host restatement of discard_higher_energies for the impurity step (cnt == 0)
  std::vector<double> all;
  for (auto &v : E) all.insert(all.end(), v.begin(), v.end());
  std::sort(all.begin(), all.end());
  r->all_eig = all;
  r->kept.clear();
  const double emin = all.empty() ? 0.0 : all[0];
  if (all.size() <= r->nkeep) {
    for (auto &v : E) r->kept.push_back(int64_t(v.size()));
  } else {
    const double thr = all[r->nkeep];
    for (auto &v : E) {
      int64_t k = 0;
      for (double x : v)
        if (x < thr + 1e-8) ++k;
      r->kept.push_back(k);
    }
  }
  r->no_of_kept = std::accumulate(r->kept.begin(), r->kept.end(), int64_t(0));
  r->prev_shift = 0.0;
  if (r->no_of_kept <= int64_t(r->nkeep)) {
    r->cnt_min = r->cnt;
  } else {
    r->relgs.push_back(emin);
    r->prev_shift = emin;
  }
}

static void init_from_impurity(nrg_run *r) {
  nrg_engine *e = r->eng;
  r->pre_q = r->imp.q;
  auto E = r->imp.E;
  reference_discard(r, E);
  // previous-site device data: impurity energies and kept f-dagger blocks
  auto sd = std::make_shared<SiteData>();
  std::vector<double> flat;
  std::vector<int64_t> eoff;
  for (auto &v : r->imp.E) {
    eoff.push_back(int64_t(flat.size()));
    flat.insert(flat.end(), v.begin(), v.end());
  }
  std::vector<int64_t> foff;
  std::vector<OpKey> fkeys;
  std::vector<std::pair<int, int>> fdims;
  for (int ip = 0; ip < r->imp.nops; ++ip)
    for (auto &kv : r->imp.op[ip]) {
      int ii = kv.first.first, jj = kv.first.second;
      int k = int(r->kept[ii]), kp = int(r->kept[jj]);
      if (k == 0 || kp == 0) continue;
      fkeys.push_back({ip, ii, jj});
      fdims.push_back({k, kp});
      foff.push_back(int64_t(flat.size()));
      for (int a = 0; a < k; ++a)
        for (int b = 0; b < kp; ++b) flat.push_back(kv.second.v[int64_t(a) * kv.second.cols + b]);
    }
  sd->mem_E = dalloc(e, flat.size() * sizeof(double) + 8);
  check_cuda(cudaMemcpyAsync(sd->mem_E->ptr, flat.data(), flat.size() * sizeof(double),
                             cudaMemcpyHostToDevice, e->stream),
             "impurity upload");
  double *base = static_cast<double *>(sd->mem_E->ptr);
  r->prevE.assign(r->imp.E.size(), nullptr);
  for (size_t s = 0; s < r->imp.E.size(); ++s)
    if (!r->imp.E[s].empty()) r->prevE[s] = base + eoff[s];
  sd->E_host = r->imp.E;
  r->prev_site = sd;
  r->fprev.clear();
  for (size_t i = 0; i < fkeys.size(); ++i)
    r->fprev[fkeys[i]] = FBlock{base + foff[i], fdims[i].first, fdims[i].second, fdims[i].second};
  r->fprev_mem = sd->mem_E;
  r->prevE_host = r->imp.E;
  for (auto &v : r->prevE_host)
    for (auto &x : v) x -= r->prev_shift;
  check_cuda(cudaStreamSynchronize(e->stream), "impurity upload");
}

static void build_basis(RunStep &st) {
  nrg_run *r = st.run;
  const SiteModel &bath = r->bath;
  auto sd = std::make_shared<SiteData>();
  sd->iteration = r->cnt;
  sd->pre_q = r->pre_q;
  sd->kept_prev = r->kept;
  const int nb = int(bath.q.size());
  // new sectors in first-seen order over (previous sector, bath sector), as
  // create_next_basis (nrgcore.hpp:238-261); the basis is never pruned, so
  // this loop runs over every pair: sector keys are packed into 64 bits
  // (up to 4 quantum numbers of 16 bits) for a hash lookup
  const size_t nq = r->pre_q.empty() ? 0 : r->pre_q[0].size();
  for (int j = 0; j < nb; ++j)
    if (bath.q[j].size() != nq) fail(NRG_E_ARG, "quantum number count differs between impurity and bath");
  bool packable = nq <= 4;
  for (auto &q : r->pre_q)
    for (int v : q) packable = packable && v > -16384 && v < 16384;
  for (auto &q : bath.q)
    for (int v : q) packable = packable && v > -16384 && v < 16384;
  std::unordered_map<uint64_t, int> where_packed;
  std::map<std::vector<int>, int> where;
  if (packable) where_packed.reserve(r->pre_q.size() * 2 + 16);
  int tmq[4];
  std::vector<int> tm(nq);
  for (size_t i = 0; i < r->pre_q.size(); ++i) {
    const std::vector<int> &pq = r->pre_q[i];
    if (pq.size() != nq) fail(NRG_E_ARG, "quantum number count differs between sectors");
    for (int j = 0; j < nb; ++j) {
      int idx;
      bool fresh;
      if (packable) {
        uint64_t key = 0;
        for (size_t x = 0; x < nq; ++x) {
          tmq[x] = pq[x] + bath.q[j][x];
          key = (key << 16) | uint64_t(uint16_t(tmq[x] + 32768));
        }
        auto ins = where_packed.emplace(key, int(sd->cur_q.size()));
        idx = ins.first->second;
        fresh = ins.second;
        if (fresh) sd->cur_q.emplace_back(tmq, tmq + nq);
      } else {
        for (size_t x = 0; x < nq; ++x) tm[x] = pq[x] + bath.q[j][x];
        auto ins = where.emplace(tm, int(sd->cur_q.size()));
        idx = ins.first->second;
        fresh = ins.second;
        if (fresh) sd->cur_q.push_back(tm);
      }
      if (fresh) sd->coupled.emplace_back();
      sd->coupled[idx].push_back(uint64_t(i) * nb + j);
    }
  }
  sd->sectors.resize(sd->cur_q.size());
  for (size_t s = 0; s < sd->cur_q.size(); ++s) {
    int off = 0;
    Sector &S = sd->sectors[s];
    for (uint64_t kidx : sd->coupled[s]) {
      int ii = int(kidx / nb), bb = int(kidx % nb);
      int k = int(r->kept[ii]), d = int(bath.E[bb].size());
      if (k * d > 0) {
        S.subs.push_back({ii, bb, off, k, d});
        st.sub_of[{ii, bb}] = {int(s), off};
      }
      off += k * d;
    }
    S.n = off;
  }
  st.site = sd;
}

static int round_up(int x, int m) { return (x + m - 1) / m * m; }

static cudaEvent_t take_event(nrg_engine *e) {
  if (!e->ev_pool.empty()) {
    cudaEvent_t x = e->ev_pool.back();
    e->ev_pool.pop_back();
    return x;
  }
  cudaEvent_t x;
  check_cuda(cudaEventCreate(&x), "event");
  return x;
}

Prof::Prof(nrg_engine *eng, const char *nm, double w, cudaStream_t st)
    : e(eng), name(nm), work(w), s(st ? st : eng->stream) {
  if (e->profile) {
    a = take_event(e);
    cudaEventRecord(a, s);
  }
}
Prof::~Prof() {
  if (a) {
    cudaEvent_t b = take_event(e);
    cudaEventRecord(b, s);
    e->prof.push_back({name, a, b, work});
  }
}

// algorithmic flops of a grouped GEMM: 2 M N K per contribution
double gemm_flops(const std::vector<GemmGroup> &gs, const std::vector<GemmContrib> &cs) {
  double f = 0;
  for (auto &g : gs)
    for (int c = g.c0; c < g.c1; ++c) f += 2.0 * g.M * g.N * double(cs[c].K);
  return f;
}

static double eig_flops(const std::vector<EigBlock> &b) {
  double f = 0;
  for (auto &x : b) f += 10.0 / 3.0 * double(x.n) * x.n * x.n;
  return f;
}

// One grouped-GEMM launch (k_gemm.cu) for a list of outputs.
struct GemmList {
  std::vector<GemmGroup> groups;
  std::vector<GemmContrib> contribs;
  std::vector<GemmTile> tiles;
  void out(double *C, int ldc, int M, int N, bool acc, std::initializer_list<GemmContrib> cs) {
    GemmGroup g{};
    g.C = C;
    g.ldc = ldc;
    g.M = M;
    g.N = N;
    g.accumulate = acc ? 1 : 0;
    g.c0 = int(contribs.size());
    contribs.insert(contribs.end(), cs.begin(), cs.end());
    g.c1 = int(contribs.size());
    const int gi = int(groups.size());
    groups.push_back(g);
    for (int tm = 0; tm < (M + GEMM_TILE - 1) / GEMM_TILE; ++tm)
      for (int tn = 0; tn < (N + GEMM_TILE - 1) / GEMM_TILE; ++tn) tiles.push_back({gi, tm, tn, 0});
  }
  void launch(nrg_engine *e, std::vector<DevPtr> &hold) {
    if (tiles.empty()) return;
    Arena a;
    size_t ot = a.add(tiles), og = a.add(groups), oc = a.add(contribs);
    DevPtr d;
    char *p = a.push(e, d);
    hold.push_back(d);
    Prof pf(e, "k_gemm_f64", gemm_flops(groups, contribs));
    launch_gemm_f64(at<GemmTile>(p, ot), int(tiles.size()), at<GemmGroup>(p, og),
                    at<GemmContrib>(p, oc), e->stream);
    count_launch(e);
    post_launch("grouped gemm");
  }
};

static GemmContrib contrib(const double *A, int lda, const double *B, int ldb, int K, int trans) {
  GemmContrib c{};
  c.A = A;
  c.lda = lda;
  c.B = B;
  c.ldb = ldb;
  c.K = K;
  c.trans = trans;
  c.alpha = 1.0;
  return c;
}

// Split a list of FP64 matrix views (rows x cols, leading dimension ld) into
// bf16 digit planes (k_ozaki.cu) with one grid-wide pass.  All matrices share
// one allocation; plane p of matrix i starts at p * pstride + poff[i].
PlaneBuf split_matrices(nrg_engine *e, const std::vector<MatRef> &mats, std::vector<DevPtr> &hold) {
  PlaneBuf pb;
  const size_t nm = mats.size();
  std::vector<int64_t> poff(nm), chunk0(nm + 1, 0);
  std::vector<int> ldp(nm);
  int64_t tot = 0;
  const int64_t chunk = split_chunk_elements();
  for (size_t i = 0; i < nm; ++i) {
    ldp[i] = round_up(std::max(mats[i].cols, 1), 8);
    poff[i] = tot;
    const int64_t nel = int64_t(mats[i].rows) * ldp[i];
    if (nel >= (int64_t(1) << 31)) fail(NRG_E_ARG, "matrix too large for the digit split");
    tot += nel;
    chunk0[i + 1] = chunk0[i] + (nel + chunk - 1) / chunk;
  }
  pb.mem = dalloc(e, tot * kDigitPlanes * 2 + 16);
  pb.exps = dalloc(e, nm * sizeof(int) + 16);
  hold.push_back(pb.mem);
  hold.push_back(pb.exps);
  std::vector<SplitTask> t(nm);
  pb.ops.resize(nm);
  for (size_t i = 0; i < nm; ++i) {
    t[i] = SplitTask{};
    t[i].src = mats[i].p;
    t[i].rows = mats[i].rows;
    t[i].cols = mats[i].cols;
    t[i].ld = mats[i].ld;
    t[i].ldp = ldp[i];
    t[i].planes = static_cast<__nv_bfloat16 *>(pb.mem->ptr) + poff[i];
    t[i].pstride = tot;
    t[i].exp = static_cast<int *>(pb.exps->ptr) + i;
    OzOperand o{};
    o.p = static_cast<const __nv_bfloat16 *>(pb.mem->ptr) + poff[i];
    o.pstride = tot;
    o.ld = ldp[i];
    o.exp = static_cast<const int *>(pb.exps->ptr) + i;
    pb.ops[i] = o;
  }
  if (nm == 0) return pb;
  const int64_t nchunks = chunk0[nm];
  chunk0.pop_back();
  std::vector<unsigned long long> scratch(nm, 0);
  Arena a;
  size_t ot = a.add(t), oc = a.add(chunk0), os = a.add(scratch);
  DevPtr d;
  char *dp = a.push(e, d);
  hold.push_back(d);
  double bytes = 0;  // algorithmic: 8 + 8 bytes read per element, 8 x 2 bytes written per padded element
  for (size_t i = 0; i < nm; ++i)
    bytes += 16.0 * mats[i].rows * mats[i].cols + 16.0 * mats[i].rows * ldp[i];
  Prof pf(e, "k_split", bytes);
  launch_split_grid(at<SplitTask>(dp, ot), at<int64_t>(dp, oc), int(nm), nchunks, at<unsigned long long>(dp, os),
                    e->stream);
  count_launch(e, 2);
  post_launch("split");
  return pb;
}

// square blocks of one arena (offset off[b], dimension dims[b], ld lds[b])
static PlaneBuf split_blocks(nrg_engine *e, const double *base, const std::vector<int64_t> &off,
                             const std::vector<int> &dims, const std::vector<int> &lds,
                             std::vector<DevPtr> &hold) {
  std::vector<MatRef> m(dims.size());
  for (size_t b = 0; b < dims.size(); ++b) m[b] = MatRef{base + off[b], dims[b], dims[b], lds[b]};
  return split_matrices(e, m, hold);
}

void OzList::out(double *C, int ldc, int M, int N, bool acc, const std::vector<OzContrib> &cs, bool upper) {
  OzGroup g{};
  g.C = C;
  g.ldc = ldc;
  g.M = M;
  g.N = N;
  g.accumulate = acc ? 1 : 0;
  g.planes = planes;
  g.c0 = int(contribs.size());
  const double pairs = 0.5 * planes * (planes + 1);
  for (auto &c : cs) {
    contribs.push_back(c);
    flops += 2.0 * M * N * double(c.K) * pairs;
    useful += 2.0 * M * N * double(c.K);
  }
  g.c1 = int(contribs.size());
  const int gi = int(groups.size());
  groups.push_back(g);
  for (int tm = 0; tm < (M + OZ_TILE_M - 1) / OZ_TILE_M; ++tm)
    for (int tn = 0; tn < (N + OZ_TILE_N - 1) / OZ_TILE_N; ++tn) {
      if (upper && tm * OZ_TILE_M > tn * OZ_TILE_N + OZ_TILE_N - 1) continue;  // wholly below the diagonal
      tiles.push_back({gi, tm, tn, 0});
    }
}

void OzList::launch(nrg_engine *e, std::vector<DevPtr> &hold) {
  if (tiles.empty()) return;
  // one TMA tensor map per distinct operand view (a view is shared by the
  // products of many groups: the same U block, the same X)
  std::vector<OzTensorMap> maps;
  std::map<std::tuple<const void *, int, int, int, int64_t, int>, int> seen;
  auto map_of = [&](const OzOperand &o, int inner, int outer, int box_outer) {
    const auto key = std::make_tuple(static_cast<const void *>(o.p), inner, outer, o.ld, o.pstride, box_outer);
    auto it = seen.find(key);
    if (it != seen.end()) return it->second;
    OzTensorMap m;
    if (!encode_oz_map(&m, o, inner, outer, planes, box_outer))
      fail(NRG_E_CUDA, "TMA tensor map of a digit-plane operand rejected");
    maps.push_back(m);
    seen.emplace(key, int(maps.size()) - 1);
    return int(maps.size()) - 1;
  };
  for (const OzGroup &g : groups)
    for (int c = g.c0; c < g.c1; ++c) {
      OzContrib &q = contribs[c];
      q.tmA = q.tmB = -1;
      if (q.K <= 0) continue;
      const bool ta = q.trans & 1, tb = (q.trans >> 1) & 1;
      q.tmA = ta ? map_of(q.A, g.M, q.K, 16) : map_of(q.A, q.K, g.M, OZ_TILE_M);
      q.tmB = tb ? map_of(q.B, q.K, g.N, OZ_TILE_N) : map_of(q.B, g.N, q.K, 16);
    }
  Arena a;
  size_t ot = a.add(tiles), og = a.add(groups), oc = a.add(contribs), om = a.add(maps);
  DevPtr d;
  char *p = a.push(e, d);
  hold.push_back(d);
  e->work[2] += useful;
  e->work[3] += flops;
  Prof pf(e, "k_gemm_oz", useful);
  launch_gemm_oz(at<GemmTile>(p, ot), int(tiles.size()), at<OzGroup>(p, og), at<OzContrib>(p, oc),
                 at<OzTensorMap>(p, om), e->d_kerr, e->stream);
  count_launch(e);
  post_launch("ozaki gemm");
}

OzContrib ozc(const OzOperand &A, const OzOperand &B, int K, int trans, double alpha) {
  OzContrib c{};
  c.A = A;
  c.B = B;
  c.K = K;
  c.trans = trans;
  c.alpha = alpha;
  return c;
}

// ------------------------------------------------------------ autotuner
// The block-size histogram of one launch, coarsened into a key: the largest
// block in steps of 32 rows, the block count and the total n^2 in powers of
// two, and the precision of the kernel.
// Cluster solver or one-CTA solver for the blocks above one SM's shared
// memory. The cluster solver finishes a block several times sooner but spends
// about six times the SM-time of the one-CTA solver on it, so in the automatic
// mode it takes a launch only when all its clusters run in one wave of the
// device: the launch is then latency-bound and the idle SMs are free.
static bool cluster_wanted(const nrg_engine *e, const std::vector<int> &eligible, bool fp64) {
  if (eligible.empty() || e->eig_cluster == 0) return false;
  if (e->eig_cluster == 2) return true;
  int ctas = 0;
  for (int n : eligible) ctas += eig_cluster_size_for(n, fp64);
  return ctas <= e->sm_count;
}

static uint64_t hist_key(const std::vector<EigBlock> &b, bool fp64) {
  int mx = 0;
  double n2 = 0;
  for (auto &x : b) {
    mx = std::max(mx, x.n);
    n2 += double(x.n) * x.n;
  }
  const uint64_t cnt = uint64_t(std::ilogb(double(b.size()) + 1.0));
  const uint64_t vol = uint64_t(std::ilogb(n2 + 1.0));
  return (uint64_t((mx + 31) / 32) << 24) | (cnt << 16) | (vol << 8) | (fp64 ? 1u : 0u);
}

struct ReflectPlan {
  int tw, panel;
};

// The reflector back-transform's launch shapes for one launch: the tuned one
// when the histogram has been seen, every fitting tile width (largest panel
// each) when it is to be tuned now, else the widest that fits.
static std::vector<ReflectPlan> reflect_plans(nrg_engine *e, uint64_t key, int max_n, bool fp64) {
  std::vector<ReflectPlan> out;
  auto it = e->tuned.find(key);
  if (e->autotune && it != e->tuned.end()) {
    // the key coarsens max_n: the tuned width, with the panel that fits this
    // launch's largest block
    int pn = 1;
    if (reflect_fits(max_n, it->second.tw, &pn, fp64)) return {{it->second.tw, std::min(pn, it->second.panel)}};
  }
  for (int tw : {64, 32, 16, 8, 4}) {
    int pn = 1;
    if (!reflect_fits(max_n, tw, &pn, fp64)) continue;
    out.push_back({tw, pn});
    if (!e->autotune) break;
  }
  if (out.empty())
    fail(NRG_E_ARG, "block dimension " + std::to_string(max_n) + " exceeds the back-transform limit " +
                        std::to_string(reflect_max_n(fp64)));
  return out;
}

// Column tiles (block, tile) of every plan.
static std::vector<std::vector<int2>> reflect_tiles(const std::vector<EigBlock> &b,
                                                    const std::vector<ReflectPlan> &plans) {
  std::vector<std::vector<int2>> t(plans.size());
  for (size_t p = 0; p < plans.size(); ++p)
    for (size_t k = 0; k < b.size(); ++k)
      for (int tn = 0; tn < (b[k].n + plans[p].tw - 1) / plans[p].tw; ++tn) t[p].push_back(make_int2(int(k), tn));
  return t;
}

// Runs the back-transform: one plan as is; several (a histogram seen for the
// first time) each timed with CUDA events after a stream synchronisation,
// the fastest kept for the histogram.  Every plan writes the same U, bit for
// bit (a column's arithmetic does not depend on the tile width or panel).
static void run_reflect(nrg_engine *e, uint64_t key, const std::vector<ReflectPlan> &plans, const char *name,
                        double flops, const std::function<void(size_t)> &launch) {
  if (plans.size() == 1) {
    Prof pf(e, name, flops);
    launch(0);
    count_launch(e);
    post_launch(name);
    return;
  }
  check_cuda(cudaStreamSynchronize(e->stream), "autotune");
  std::vector<float> ms(plans.size(), 0.f);
  for (size_t p = 0; p < plans.size(); ++p) {
    cudaEvent_t a = take_event(e), b = take_event(e);
    check_cuda(cudaEventRecord(a, e->stream), "autotune");
    launch(p);
    count_launch(e);
    post_launch(name);
    check_cuda(cudaEventRecord(b, e->stream), "autotune");
    check_cuda(cudaEventSynchronize(b), "autotune");
    check_cuda(cudaEventElapsedTime(&ms[p], a, b), "autotune");
    e->ev_pool.push_back(a);
    e->ev_pool.push_back(b);
  }
  size_t best = 0;
  for (size_t p = 1; p < plans.size(); ++p)
    if (ms[p] < ms[best]) best = p;
  nrg_engine::Tuned t;
  t.tw = plans[best].tw;
  t.panel = plans[best].panel;
  char buf[64];
  t.what = std::string(name) + " histogram " + std::to_string(key) + ": tw=" + std::to_string(t.tw) +
           " panel=" + std::to_string(t.panel) + " (";
  for (size_t p = 0; p < plans.size(); ++p) {
    std::snprintf(buf, sizeof(buf), "%s%d:%.3f ms", p ? ", " : "", plans[p].tw, double(ms[p]));
    t.what += buf;
  }
  t.what += ")";
  e->tuned[key] = t;
}

constexpr int kRefineSteps = 3;
constexpr double kClusterTau = 1e-4;  // relative gap below which levels form a cluster
// The first Newton step starts from FP32 eigenvectors (errors >= 1e-7), so
// its products need only 5 digit planes (35 bits, relative error ~3e-11,
// 15 instead of 36 digit-plane products); the later steps use all 8.
constexpr int kFirstStepPlanes = 5;

// Mixed-precision eigensolve of every block of the batch: FP32 Householder +
// QL (k_eig<float>), then kRefineSteps Ogita-Aishima Newton steps with
// FP64-accurate grouped GEMMs and a final Rayleigh-Ritz pass with FP64
// Jacobi on near-degenerate clusters (k_refine.cu).  Writes U and E of every
// block; blocks whose refinement did not converge are re-solved with the FP64
// solver in a launch gated on the device by the refinement status, so no host
// round trip is needed.  H is left intact (except in re-solved blocks too
// large for shared memory, which the FP64 solver reduces in place).  Returns
// the device status arrays
// (in `hold`), which the caller reads at its next synchronisation.
struct MixedStatus {
  const int *refine = nullptr;  // per block: 0 ok; re-solved in FP64: 2 not converged, 4 chain too long
  const int *fp64 = nullptr;    // per block: FP64 re-solve status (0 ok)
  int nb = 0;
  std::vector<int> dims;        // block sizes (for the NRG_DEBUG_FALLBACK report)
};

struct F64Solve {
  std::vector<EigBlock> order;  // the blocks in launch order (status index)
  int *d_status = nullptr;      // per block: 1 = tred2 + QL did not converge
};

// Plain FP64 eigensolve of a list of blocks (largest first).  Blocks above
// the one-CTA shared-memory limit (up to the reflector kernel's) go to the
// reflector solver, the mixed path's first stage in FP64 (Householder
// reduction, bisection, inverse iteration, then k_reflect<double>): the
// cluster solver when its clusters fit one wave, else one CTA per block
// streaming the matrix (k_eig_bi<double>).  They are moved to the end of the
// list; the others go to k_eig<double> (tred2 + QL) in shared memory, on the
// side stream.  The caller reads the status at its next synchronisation.
static F64Solve fp64_eigensolve(nrg_engine *e, std::vector<EigBlock> eb, std::vector<DevPtr> &hold,
                                cudaStream_t s) {
  int n_f64 = int(eb.size()), max_r64 = 0, tw64 = 8, panel64 = 1;
  bool cluster64 = false;
  uint64_t key64 = 0;
  std::vector<ReflectPlan> plans64;
  std::vector<std::vector<int2>> tiles64;
  {
    std::vector<EigBlock> one, rs;
    std::vector<int> eligible64;
    int64_t wsz = 0;
    for (auto &b : eb) {
      if (b.n > e->eig_smem_f64 && b.n <= eig_bi_max_n(true) && reflect_config(b.n, &tw64, &panel64, true)) {
        rs.push_back(b);
        wsz += int64_t(b.n) * b.ld;
        max_r64 = std::max(max_r64, b.n);
        if (eig_cluster_size_for(b.n, true) > 0) eligible64.push_back(b.n);
      } else {
        one.push_back(b);
      }
    }
    if (!rs.empty()) {
      cluster64 = eligible64.size() == rs.size() && cluster_wanted(e, eligible64, true);
      key64 = hist_key(rs, true);
      plans64 = reflect_plans(e, key64, max_r64, true);
      tiles64 = reflect_tiles(rs, plans64);
      DevPtr w = dalloc(e, 3 * wsz * sizeof(double) + 16);
      hold.push_back(w);
      double *base = static_cast<double *>(w->ptr);
      int64_t o = 0;
      for (size_t k = 0; k < rs.size(); ++k) {
        EigBlock &b = rs[k];
        b.W64 = base + o;
        b.V64 = base + wsz + o;
        b.Bt64 = base + 2 * wsz + o;
        o += int64_t(b.n) * b.ld;
      }
      n_f64 = int(one.size());
      eb = one;
      eb.insert(eb.end(), rs.begin(), rs.end());
    }
  }

  Arena ar;
  const size_t o_eb = ar.add(eb);
  std::vector<size_t> o_t64(tiles64.size());
  for (size_t p = 0; p < tiles64.size(); ++p) o_t64[p] = ar.add(tiles64[p]);
  std::vector<int> st(eb.size() + 1, 0);
  const size_t o_st = ar.add(st);
  DevPtr desc;
  char *d = ar.push(e, desc);
  hold.push_back(desc);
  {
    const int nrs = int(eb.size()) - n_f64;
    // the tred2 + QL blocks run on the side stream beside the reflector solver
    const bool fork = nrs > 0 && n_f64 > 0;
    if (fork) {
      check_cuda(cudaEventRecord(e->fork_ev, s), "fork");
      check_cuda(cudaStreamWaitEvent(e->side, e->fork_ev, 0), "fork");
    }
    if (nrs > 0) {
      std::vector<EigBlock> rsb(eb.begin() + n_f64, eb.end());
      if (cluster64) {
        Prof pf(e, "k_eig_cluster_f64", eig_flops(rsb) * 0.4);  // tridiagonal reduction: 4/3 n^3
        const int cs = eig_cluster_size_for(max_r64, true);
        const std::string what = "eigensolve f64 (cluster of " + std::to_string(cs) + " CTAs, " +
                                 std::to_string(nrs) + " blocks, largest " + std::to_string(max_r64) + ")";
        check_cuda(launch_eig_cluster(at<EigBlock>(d, o_eb) + n_f64, nrs, max_r64, cs, true, s), what.c_str());
        count_launch(e);
        post_launch("eigensolve f64 (cluster)");
      } else {
        Prof pf(e, "k_eig_bi_f64", eig_flops(rsb) * 0.4);  // tridiagonal reduction: 4/3 n^3
        launch_eig_bisect_f64(at<EigBlock>(d, o_eb) + n_f64, nrs, max_r64, e->eig_smem_f64, s);
        count_launch(e);
        post_launch("eigensolve f64 (reflector solver)");
      }
      double f = 0;  // applying the reflectors: 2 n^3 per block
      for (auto &x : rsb) f += 2.0 * double(x.n) * x.n * x.n;
      run_reflect(e, key64, plans64, "k_reflect_f64", f, [&](size_t p) {
        launch_reflect(at<EigBlock>(d, o_eb) + n_f64, at<int2>(d, o_t64[p]), int(tiles64[p].size()), max_r64,
                       plans64[p].tw, plans64[p].panel, s, true);
      });
    }
    if (n_f64 > 0) {
      cudaStream_t so = fork ? e->side : s;
      int mx = 0;
      for (int b = 0; b < n_f64; ++b) mx = std::max(mx, eb[b].n);
      std::vector<EigBlock> oneb(eb.begin(), eb.begin() + n_f64);
      Prof pf(e, "k_eig_f64", eig_flops(oneb), so);
      launch_eig_f64(at<EigBlock>(d, o_eb), n_f64, mx, e->eig_smem_f64, at<int>(d, o_st), so);
      count_launch(e);
      post_launch("eigensolve");
    }
    if (fork) {
      check_cuda(cudaEventRecord(e->join_ev, e->side), "join");
      check_cuda(cudaStreamWaitEvent(s, e->join_ev, 0), "join");
    }
  }
  F64Solve r;
  r.order = eb;
  r.d_status = at<int>(d, o_st);
  return r;
}

static MixedStatus mixed_eigensolve(nrg_engine *e, std::vector<DevBlock *> &blks, int max_n,
                                    std::vector<DevPtr> &hold) {
  cudaStream_t s = e->stream;
  const size_t nb = blks.size();
  if (nb == 0) return {};
  int64_t sz = 0, esz = 0;
  std::vector<int64_t> off(nb), eoff(nb);
  for (size_t b = 0; b < nb; ++b) {
    off[b] = sz;
    sz += int64_t(blks[b]->n) * blks[b]->ld;
    eoff[b] = esz;
    esz += blks[b]->n;
  }
  DevPtr mx0 = dalloc(e, sz * 8), mx1 = dalloc(e, sz * 8), my = dalloc(e, sz * 8),
         ms = dalloc(e, sz * 8), mg = dalloc(e, sz * 8), me2 = dalloc(e, sz * 8),
         mw = dalloc(e, 3 * sz * 4 + 16), mlam = dalloc(e, esz * 8 + 8);
  hold.insert(hold.end(), {mx0, mx1, my, ms, mg, me2, mw, mlam});
  auto P = [](DevPtr &m, int64_t o) { return static_cast<double *>(m->ptr) + o; };
  double *X[2] = {P(mx0, 0), P(mx1, 0)};
  float *wbase = static_cast<float *>(mw->ptr);
  // FP32 solve: eigenvectors (as FP64) into X0
  std::vector<EigBlock> eb(nb);
  for (size_t b = 0; b < nb; ++b) {
    eb[b] = EigBlock{};
    eb[b].H = blks[b]->H;
    eb[b].U = X[0] + off[b];
    eb[b].E = P(mlam, eoff[b]);
    eb[b].W = wbase + off[b];
    eb[b].V = wbase + sz + off[b];
    eb[b].Bt = wbase + 2 * sz + off[b];
    eb[b].n = blks[b]->n;
    eb[b].ld = blks[b]->ld;
    eb[b].ldu = blks[b]->ld;
  }
  const uint64_t rkey = hist_key(eb, false);
  const std::vector<ReflectPlan> rplans = reflect_plans(e, rkey, max_n, false);
  const std::vector<std::vector<int2>> rtiles = reflect_tiles(eb, rplans);
  std::vector<int> stat(nb + 1, 0);
  std::vector<RefineBlock> rb(nb);
  std::vector<EigBlock> eb64(nb);  // FP64 re-solve of flagged blocks, in place
  for (size_t b = 0; b < nb; ++b) {
    eb64[b] = EigBlock{};
    eb64[b].H = blks[b]->H;
    eb64[b].U = blks[b]->U;
    eb64[b].E = blks[b]->E;
    eb64[b].n = blks[b]->n;
    eb64[b].ld = blks[b]->ld;
    eb64[b].ldu = blks[b]->ld;
  }
  // The FP64 re-solve of the blocks whose refinement failed (gated on the
  // device by their status), as the plain FP64 path solves them: blocks above
  // the reflector kernel's limit by tred2 + QL in global memory, those above
  // shared memory by the FP64 reflector solver, the rest by tred2 + QL in
  // shared memory.  The blocks are sorted by size, largest first, so each set
  // is a range: [0, fb_huge), [fb_huge, fb_refl), [fb_refl, nb).  The
  // reflector solver works in buffers free by then: its reflectors in H (the
  // reduction reads H in place), V and the pivots in the refinement's Y and E
  // buffers of the block.
  int fb_huge = 0, fb_tw = 8, fb_panel = 1;
  const int fb_max = std::min(reflect_max_n(true), eig_bi_max_n(true));
  while (fb_huge < int(nb) && eb64[fb_huge].n > fb_max) ++fb_huge;
  int fb_refl = fb_huge;
  while (fb_refl < int(nb) && eb64[fb_refl].n > e->eig_smem_f64) ++fb_refl;
  std::vector<int2> fb_tiles;
  if (fb_refl > fb_huge) {
    reflect_config(eb64[fb_huge].n, &fb_tw, &fb_panel, true);
    for (int b = fb_huge; b < fb_refl; ++b) {
      eb64[b].W64 = blks[b]->H;
      eb64[b].V64 = P(my, off[b]);
      eb64[b].Bt64 = P(me2, off[b]);
      for (int tn = 0; tn < (eb64[b].n + fb_tw - 1) / fb_tw; ++tn) fb_tiles.push_back(make_int2(b - fb_huge, tn));
    }
  }
  // blocks above the one-CTA shared-memory limit that a cluster's distributed
  // shared memory holds go to k_eig_cluster, the others to k_eig_bi
  std::vector<EigBlock> eb_one, eb_cl;
  int max_one = 0, max_cl = 0;
  std::vector<int> eligible;
  for (size_t b = 0; b < nb; ++b)
    if (eb[b].n > e->eig_smem_f32 && eig_cluster_size_for(eb[b].n, false) > 0) eligible.push_back(eb[b].n);
  const bool cluster_on = cluster_wanted(e, eligible, false);
  for (size_t b = 0; b < nb; ++b) {
    if (cluster_on && eb[b].n > e->eig_smem_f32 && eig_cluster_size_for(eb[b].n, false) > 0) {
      eb_cl.push_back(eb[b]);
      max_cl = std::max(max_cl, eb[b].n);
    } else {
      eb_one.push_back(eb[b]);
      max_one = std::max(max_one, eb[b].n);
    }
  }
  Arena a;
  size_t oeb = a.add(eb), ost = a.add(stat), oeb64 = a.add(eb64), ost64 = a.add(stat), ofbt = a.add(fb_tiles);
  std::vector<size_t> obt(rplans.size());
  for (size_t p = 0; p < rplans.size(); ++p) obt[p] = a.add(rtiles[p]);
  const size_t orb = a.add(rb);  // filled per step below (host copy re-uploaded)
  std::vector<int2> strips;      // (block, first row) of the refinement's row-strip passes
  for (size_t b = 0; b < nb; ++b)
    for (int r0 = 0; r0 < blks[b]->n; r0 += oa_strip_rows()) strips.push_back(make_int2(int(b), r0));
  const size_t ostrip = a.add(strips), oflag = a.add(stat);
  const size_t oone = a.add(eb_one), ocl = a.add(eb_cl);
  DevPtr dd;
  char *dp = a.push(e, dd);
  hold.push_back(dd);
  // the one-CTA solver runs on the side stream, beside the cluster solver
  const bool fork = !eb_cl.empty() && !eb_one.empty();
  if (fork) {
    check_cuda(cudaEventRecord(e->fork_ev, s), "fork");
    check_cuda(cudaStreamWaitEvent(e->side, e->fork_ev, 0), "fork");
  }
  if (!eb_cl.empty()) {
    Prof pf(e, "k_eig_cluster_f32", eig_flops(eb_cl) * 0.4);  // tridiagonal reduction: 4/3 n^3
    const int cs = eig_cluster_size_for(max_cl, false);
    const std::string what = "eigensolve f32 (cluster of " + std::to_string(cs) + " CTAs, " +
                             std::to_string(eb_cl.size()) + " blocks, largest " + std::to_string(max_cl) + ")";
    check_cuda(launch_eig_cluster(at<EigBlock>(dp, ocl), int(eb_cl.size()), max_cl, cs, false, s), what.c_str());
    count_launch(e);
    post_launch("eigensolve f32 (cluster)");
  }
  if (!eb_one.empty()) {
    cudaStream_t so = fork ? e->side : s;
    Prof pf(e, "k_eig_bi_f32", eig_flops(eb_one) * 0.4, so);  // tridiagonal reduction: 4/3 n^3
    launch_eig_bisect_f32(at<EigBlock>(dp, oone), int(eb_one.size()), max_one, e->eig_smem_f32, so);
    count_launch(e);
    post_launch("eigensolve f32");
  }
  if (fork) {
    check_cuda(cudaEventRecord(e->join_ev, e->side), "join");
    check_cuda(cudaStreamWaitEvent(s, e->join_ev, 0), "join");
  }
  {
    double f = 0;  // applying the reflectors: 2 n^3 per block
    for (auto &x : eb) f += 2.0 * double(x.n) * x.n * x.n;
    run_reflect(e, rkey, rplans, "k_reflect", f, [&](size_t p) {
      launch_reflect(at<EigBlock>(dp, oeb), at<int2>(dp, obt[p]), int(rtiles[p].size()), max_n, rplans[p].tw,
                     rplans[p].panel, s);
    });
  }
  int cur = 0;
  // digit planes for the tensor-core GEMMs (H once, X / Y / E per step)
  const bool oz = (e->ozaki & 1) != 0;
  std::vector<int> dims(nb), lds(nb);
  for (size_t b = 0; b < nb; ++b) {
    dims[b] = blks[b]->n;
    lds[b] = blks[b]->ld;
  }
  PlaneBuf pH, pX, pY, pE;
  if (oz) {
    std::vector<MatRef> hm(nb);
    for (size_t b = 0; b < nb; ++b) hm[b] = MatRef{blks[b]->H, dims[b], dims[b], lds[b]};
    pH = split_matrices(e, hm, hold);
  }
  auto splitv = [&](PlaneBuf &pl, double *base) { pl = split_blocks(e, base, off, dims, lds, hold); };
  // Newton steps per block: the FP32 start's error grows with n (about
  // sqrt(n) eps32 |H| / gap) and each step squares it, so blocks above 1536
  // rows take one more step and above 3072 two more; a block whose steps are
  // done sits out the later ones until the final pass
  auto steps_of = [](int n) { return kRefineSteps + (n > 1536 ? 1 : 0) + (n > 3072 ? 1 : 0); };
  int max_steps = 0;
  for (size_t b = 0; b < nb; ++b) max_steps = std::max(max_steps, steps_of(blks[b]->n));
  for (int step = 0; step <= max_steps; ++step) {
    const bool final = (step == max_steps);
    auto active = [&](size_t b) { return final || step < steps_of(blks[b]->n); };
    if (oz) {
      splitv(pX, X[cur]);
      OzList y;
      y.planes = step == 0 ? kFirstStepPlanes : kDigitPlanes;
      for (size_t b = 0; b < nb; ++b) {  // Y = H X
        if (!active(b)) continue;
        const int n = blks[b]->n;
        y.out(P(my, off[b]), lds[b], n, n, false, {ozc(pH.op(b), pX.op(b), n, 0)});
      }
      y.launch(e, hold);
      splitv(pY, P(my, 0));
      OzList sg;
      sg.planes = y.planes;
      for (size_t b = 0; b < nb; ++b) {  // S = X^T Y, G = X^T X
        if (!active(b)) continue;
        const int n = blks[b]->n;
        // symmetric: only the tiles that meet the upper triangle (the refinement
        // kernels read S and G there)
        sg.out(P(ms, off[b]), lds[b], n, n, false, {ozc(pX.op(b), pY.op(b), n, 1)}, true);
        sg.out(P(mg, off[b]), lds[b], n, n, false, {ozc(pX.op(b), pX.op(b), n, 1)}, true);
      }
      sg.launch(e, hold);
    }
    GemmList g1, g2;
    for (size_t b = 0; b < nb; ++b) {
      const int n = blks[b]->n, ld = blks[b]->ld;
      double *x = X[cur] + off[b];
      if (!oz && active(b)) {
        g1.out(P(my, off[b]), ld, n, n, false, {contrib(blks[b]->H, ld, x, ld, n, 0)});     // Y = H X
        g2.out(P(ms, off[b]), ld, n, n, false, {contrib(x, ld, P(my, off[b]), ld, n, 1)});  // S = X^T Y
        g2.out(P(mg, off[b]), ld, n, n, false, {contrib(x, ld, x, ld, n, 1)});              // G = X^T X
      }
      rb[b].S = P(ms, off[b]);
      rb[b].G = P(mg, off[b]);
      rb[b].E2 = P(me2, off[b]);
      rb[b].X = x;
      rb[b].U = blks[b]->U;
      rb[b].Eout = blks[b]->E;
      rb[b].n = n;
      rb[b].ld = ld;
      rb[b].ldu = blks[b]->ld;
    }
    g1.launch(e, hold);
    g2.launch(e, hold);
    upload_async(e, dp + orb, rb.data(), nb * sizeof(RefineBlock));
    if (final) {
      {
        Prof pf(e, "k_oa_check");
        launch_oa_check(at<RefineBlock>(dp, orb), at<int2>(dp, ostrip), int(strips.size()), max_n, kClusterTau,
                        at<int>(dp, oflag), s);
        count_launch(e);
        post_launch("refine check");
      }
      {
        Prof pf(e, "k_oa_final");
        launch_oa_final(at<RefineBlock>(dp, orb), int(nb), max_n, kClusterTau, at<int>(dp, ost),
                        at<int>(dp, oflag), s);
        count_launch(e);
        post_launch("refine final");
      }
      Prof pf(e, "k_oa_bigcl");
      launch_oa_bigcl(at<RefineBlock>(dp, orb), int(nb), max_n, kClusterTau, at<int>(dp, ost), s);
      count_launch(e);
      post_launch("refine long clusters");
      break;
    }
    {
      double bytes = 0;  // S, G read and E written
      for (size_t b = 0; b < nb; ++b) bytes += 24.0 * blks[b]->n * blks[b]->n;
      Prof pf(e, "k_oa_update", bytes);
      launch_oa_update(at<RefineBlock>(dp, orb), at<int2>(dp, ostrip), int(strips.size()), max_n, kClusterTau, s);
      count_launch(e);
      post_launch("refine update");
    }
    // X' = X + X E
    check_cuda(cudaMemcpyAsync(X[1 - cur], X[cur], sz * 8, cudaMemcpyDeviceToDevice, s), "X copy");
    if (oz) {
      splitv(pE, P(me2, 0));
      OzList g3;
      g3.planes = step == 0 ? kFirstStepPlanes : kDigitPlanes;
      for (size_t b = 0; b < nb; ++b) {
        if (!active(b)) continue;
        const int n = blks[b]->n;
        g3.out(X[1 - cur] + off[b], lds[b], n, n, true, {ozc(pX.op(b), pE.op(b), n, 0)});
      }
      g3.launch(e, hold);
    } else {
      GemmList g3;
      for (size_t b = 0; b < nb; ++b) {
        if (!active(b)) continue;
        const int n = blks[b]->n, ld = blks[b]->ld;
        g3.out(X[1 - cur] + off[b], ld, n, n, true, {contrib(X[cur] + off[b], ld, P(me2, off[b]), ld, n, 0)});
      }
      g3.launch(e, hold);
    }
    cur = 1 - cur;
  }
  {
    Prof pf(e, "k_eig_f64_fallback");
    const EigBlock *d64 = at<EigBlock>(dp, oeb64);
    int *st64 = at<int>(dp, ost64), *gate = at<int>(dp, ost);
    if (fb_huge > 0) {
      launch_eig_f64(d64, fb_huge, eb64[0].n, e->eig_smem_f64, st64, s, gate);
      count_launch(e);
    }
    if (fb_refl > fb_huge) {
      launch_eig_bisect_f64(d64 + fb_huge, fb_refl - fb_huge, eb64[fb_huge].n, e->eig_smem_f64, s, gate + fb_huge);
      launch_reflect(d64 + fb_huge, at<int2>(dp, ofbt), int(fb_tiles.size()), eb64[fb_huge].n, fb_tw, fb_panel, s,
                     true, gate + fb_huge);
      count_launch(e, 2);
    }
    if (int(nb) > fb_refl) {
      launch_eig_f64(d64 + fb_refl, int(nb) - fb_refl, eb64[fb_refl].n, e->eig_smem_f64, st64 + fb_refl, s,
                     gate + fb_refl);
      count_launch(e);
    }
    post_launch("eigensolve f64 (refinement fallback)");
  }
  return MixedStatus{at<int>(dp, ost), at<int>(dp, ost64), int(nb), dims};
}

// Host copies of a MixedStatus, filled by enqueue() and checked after the
// caller's synchronisation.
struct MixedCheck {
  std::vector<int> refine, fp64, dims;
  void enqueue(const MixedStatus &m, cudaStream_t s) {
    dims = m.dims;
    refine.assign(m.nb, 0);
    fp64.assign(m.nb, 0);
    if (m.nb == 0) return;
    check_cuda(cudaMemcpyAsync(refine.data(), m.refine, m.nb * sizeof(int), cudaMemcpyDeviceToHost, s),
               "refine status");
    check_cuda(cudaMemcpyAsync(fp64.data(), m.fp64, m.nb * sizeof(int), cudaMemcpyDeviceToHost, s),
               "fallback status");
  }
  void check(nrg_engine *e) const {
    for (size_t b = 0; b < refine.size(); ++b) {
      if (refine[b] == 1) fail(NRG_E_EIG, "FP32 block eigensolver did not converge");
      if (refine[b] == 2 || refine[b] == 4) {
        ++e->fallback_blocks;
        static const bool report = std::getenv("NRG_DEBUG_FALLBACK") != nullptr;
        if (report)
          std::fprintf(stderr, "nrg: FP64 re-solve of a block of %d rows (%s)\n", b < dims.size() ? dims[b] : -1,
                       refine[b] == 2 ? "refinement not converged" : "near-degenerate chain above 1024 levels");
        if (fp64[b]) fail(NRG_E_EIG, "block eigensolver did not converge (FP64 re-solve)");
      }
    }
  }
};

static void batch_add_site(nrg_run *const *runs, int nruns, const double *t, int nt,
                           const double *rescale) {
  if (nruns <= 0) return;
  nrg_engine *e = runs[0]->eng;
  for (int i = 0; i < nruns; ++i) {
    if (!runs[i]) fail(NRG_E_ARG, "null run");
    if (runs[i]->eng != e) fail(NRG_E_ARG, "runs of one batch must share an engine");
    if (runs[i]->have_site) fail(NRG_E_STATE, "add_site called twice without update_state");
  }
  cudaStream_t s = e->stream;
  std::vector<RunStep> steps(nruns);
  for (int i = 0; i < nruns; ++i) {
    nrg_run *r = runs[i];
    if (r->bath_pending) {  // bath refresh, nrgcore.hpp:68-70
      r->bath = std::move(r->bath_next);
      r->bath_pending = false;
      upload_bath(e, r->bath);
    }
    if (nt != r->bath.nops || nt != int(r->imp.nops))
      fail(NRG_E_ARG, "t_hopping " + std::to_string(nt) + " =! pre_fdag_oparator " +
                          std::to_string(r->imp.nops));  // nrgcore.hpp:148-152
    if (r->cnt == 0) init_from_impurity(r);
    steps[i].run = r;
    steps[i].t.assign(t + int64_t(i) * nt, t + int64_t(i + 1) * nt);
    steps[i].rescale = rescale[i];
    build_basis(steps[i]);
  }
  // ---- device blocks and buffers
  std::vector<AsmBlock> ablk;
  std::vector<AsmSub> asub;
  std::vector<int2> apair;
  std::vector<AsmTerm> aterm;
  std::vector<EigBlock> eblk;
  std::vector<TruncRun> trun;
  std::vector<TruncBlock> tblk;
  std::vector<int> elem_block, block_run;
  int64_t chunks = 0;
  int max_n = 0;
  int nblk_total = 0, nelem_total = 0;
  std::vector<DevPtr> hold;
  for (int i = 0; i < nruns; ++i) {
    RunStep &st = steps[i];
    nrg_run *r = st.run;
    SiteData &sd = *st.site;
    int64_t hsz = 0, esz = 0;
    for (size_t sidx = 0; sidx < sd.sectors.size(); ++sidx) {
      Sector &S = sd.sectors[sidx];
      if (S.n == 0) continue;
      DevBlock db;
      db.sector = int(sidx);
      db.n = S.n;
      db.ld = round_up(S.n, 2);
      S.dev = int(sd.blocks.size());
      sd.blocks.push_back(db);
      hsz += int64_t(db.n) * db.ld;
      esz += db.n;
    }
    auto memH = dalloc(e, hsz * sizeof(double));
    sd.mem_U = dalloc(e, hsz * sizeof(double));
    sd.mem_E = dalloc(e, esz * sizeof(double) + 8);
    r->mem_H = memH;
    int64_t ho = 0, eo = 0;
    for (auto &db : sd.blocks) {
      db.H = static_cast<double *>(memH->ptr) + ho;
      db.U = static_cast<double *>(sd.mem_U->ptr) + ho;
      db.E = static_cast<double *>(sd.mem_E->ptr) + eo;
      ho += int64_t(db.n) * db.ld;
      eo += db.n;
    }
    r->mem_sorted = dalloc(e, esz * sizeof(double) + 8);
    st.b0 = nblk_total;
    st.e0 = nelem_total;
    // assembly descriptors
    for (auto &db : sd.blocks) {
      const Sector &S = sd.sectors[db.sector];
      AsmBlock ab{};
      ab.H = db.H;
      ab.n = db.n;
      ab.ld = db.ld;
      ab.sub0 = int(asub.size());
      ab.nsub = int(S.subs.size());
      ab.pair0 = int(apair.size());
      ab.chunk0 = chunks;
      ab.rescale = st.rescale;
      ab.shift = r->prev_shift;
      chunks += (int64_t(db.n) * db.n + 1023) / 1024;
      for (auto &sb : S.subs) {
        AsmSub a{};
        a.off = sb.off;
        a.k = sb.k;
        a.d = sb.d;
        a.eprev = r->prevE[sb.ii];
        a.ebath = bath_ptr(r->bath, r->bath.e_off[sb.bb]);
        asub.push_back(a);
      }
      const int ns = int(S.subs.size());
      for (int sa = 0; sa < ns; ++sa)
        for (int sb = 0; sb < ns; ++sb) {
          int2 rg;
          rg.x = int(aterm.size());
          const Sub &A = S.subs[sa], &B = S.subs[sb];
          for (int ip = 0; ip < r->bath.nops; ++ip) {
            auto f = r->fprev.find(OpKey{ip, A.ii, B.ii});
            if (f == r->fprev.end()) continue;
            auto fb = r->bath.op_off[ip].find({B.bb, A.bb});
            if (fb == r->bath.op_off[ip].end()) continue;
            AsmTerm tm{};
            tm.F = f->second.p;
            tm.ldf = f->second.ld;
            tm.fb = bath_ptr(r->bath, fb->second);
            tm.chi = r->bath.chi[B.bb];
            tm.t = st.t[ip];
            aterm.push_back(tm);
          }
          rg.y = int(aterm.size());
          apair.push_back(rg);
        }
      ablk.push_back(ab);
      EigBlock eb{};
      eb.H = db.H;
      eb.U = db.U;
      eb.E = db.E;
      eb.W = nullptr;
      eb.n = db.n;
      eb.ld = db.ld;
      eb.ldu = db.ld;
      eblk.push_back(eb);
      max_n = std::max(max_n, db.n);
      TruncBlock tb{};
      tb.E = db.E;
      tb.n = db.n;
      tb.e0 = nelem_total;
      for (int x = 0; x < db.n; ++x) elem_block.push_back(nblk_total);
      block_run.push_back(i);
      tblk.push_back(tb);
      nelem_total += db.n;
      ++nblk_total;
    }
    st.e1 = nelem_total;
    TruncRun tr{};
    tr.b0 = st.b0;
    tr.b1 = nblk_total;
    tr.e0 = st.e0;
    tr.e1 = st.e1;
    tr.nkeep = int64_t(r->nkeep);
    tr.sorted = static_cast<double *>(r->mem_sorted->ptr);
    trun.push_back(tr);
    if (st.e1 == st.e0) fail(NRG_E_STATE, "no states left in the basis");
  }
  // eigensolver order: largest blocks first
  std::vector<int> order(eblk.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return eblk[a].n > eblk[b].n; });
  std::vector<EigBlock> eblk_sorted;
  for (int o : order) eblk_sorted.push_back(eblk[o]);
  e->work[0] += eig_flops(eblk);
  elem_block.insert(elem_block.end(), block_run.begin(), block_run.end());
  Arena ar;
  size_t o_ablk = ar.add(ablk), o_asub = ar.add(asub), o_apair = ar.add(apair),
         o_aterm = ar.add(aterm), o_trun = ar.add(trun),
         o_tblk = ar.add(tblk), o_elem = ar.add(elem_block);
  std::vector<int> zeros(nblk_total + 1, 0);
  size_t o_kept = ar.add(zeros);
  std::vector<TruncResult> tres(nruns);
  size_t o_tres = ar.add(tres);
  DevPtr desc;
  char *d = ar.push(e, desc);
  hold.push_back(desc);

  check_cuda(cudaEventRecord(e->ev[0], s), "event");
  {
    Prof pf(e, "k_assemble");
    launch_assemble(at<AsmBlock>(d, o_ablk), int(ablk.size()), chunks, at<AsmSub>(d, o_asub),
                    at<int2>(d, o_apair), at<AsmTerm>(d, o_aterm), s);
    count_launch(e);
    post_launch("assemble");
  }
  check_cuda(cudaEventRecord(e->ev[1], s), "event");
  if (max_n > eig_max_n_f64())
    fail(NRG_E_ARG, "block dimension " + std::to_string(max_n) + " exceeds the solver limit " +
                        std::to_string(eig_max_n_f64()));
  MixedStatus mstat;
  F64Solve f64;
  if (e->precision == NRG_PREC_FP64) {
    f64 = fp64_eigensolve(e, eblk_sorted, hold, s);
  } else {
    if (max_n > refine_max_n())
      fail(NRG_E_ARG, "block dimension " + std::to_string(max_n) + " exceeds the refinement limit");
    std::vector<DevBlock *> blks;
    for (auto &st : steps)
      for (auto &db : st.site->blocks) blks.push_back(&db);
    std::stable_sort(blks.begin(), blks.end(), [](DevBlock *a, DevBlock *b) { return a->n > b->n; });
    mstat = mixed_eigensolve(e, blks, max_n, hold);
    if (e->ozaki & 2) {  // digit planes of every new U: operands of all rotations of this site
      std::vector<MatRef> um;
      for (auto &st : steps)
        for (auto &db : st.site->blocks) um.push_back(MatRef{db.U, db.n, db.n, db.ld});
      std::vector<DevPtr> keep;
      PlaneBuf pu = split_matrices(e, um, keep);
      size_t q = 0;
      for (auto &st : steps) {
        for (auto &db : st.site->blocks) db.uop = pu.ops[q++];
        st.site->mem_Uplanes = pu.mem;
        st.site->mem_Uexps = pu.exps;
        st.site->has_uplanes = true;
      }
    }
  }
  check_cuda(cudaEventRecord(e->ev[2], s), "event");
  {
    Prof pf(e, "k_truncate");
    launch_truncate(at<TruncRun>(d, o_trun), nruns, at<TruncBlock>(d, o_tblk), nblk_total,
                    at<int>(d, o_elem), nelem_total, at<int>(d, o_kept), at<TruncResult>(d, o_tres), s);
    count_launch(e, 2);
    post_launch("truncate");
  }
  check_cuda(cudaEventRecord(e->ev[3], s), "event");
  // results back to the host: kept per block, run results, solver status,
  // sorted eigenvalues and per-block eigenvalues
  std::vector<int> kept_blk(nblk_total);
  check_cuda(cudaMemcpyAsync(kept_blk.data(), d + o_kept, nblk_total * sizeof(int),
                             cudaMemcpyDeviceToHost, s), "kept D2H");
  check_cuda(cudaMemcpyAsync(tres.data(), d + o_tres, nruns * sizeof(TruncResult),
                             cudaMemcpyDeviceToHost, s), "result D2H");
  std::vector<int> stat(f64.order.size() + 1, 0);
  if (!f64.order.empty())
    check_cuda(cudaMemcpyAsync(stat.data(), f64.d_status, f64.order.size() * sizeof(int),
                               cudaMemcpyDeviceToHost, s), "status D2H");
  MixedCheck mcheck;
  mcheck.enqueue(mstat, s);
  std::vector<std::vector<double>> sorted(nruns), evals(nruns);
  for (int i = 0; i < nruns; ++i) {
    RunStep &st = steps[i];
    sorted[i].resize(st.e1 - st.e0);
    evals[i].resize(st.e1 - st.e0);
    check_cuda(cudaMemcpyAsync(sorted[i].data(), st.run->mem_sorted->ptr,
                               sorted[i].size() * sizeof(double), cudaMemcpyDeviceToHost, s),
               "sorted D2H");
    check_cuda(cudaMemcpyAsync(evals[i].data(), st.site->mem_E->ptr, evals[i].size() * sizeof(double),
                               cudaMemcpyDeviceToHost, s),
               "eigenvalues D2H");
  }
  check_cuda(cudaStreamSynchronize(s), "site step");
  check_kernel_error(e);
  mcheck.check(e);
  for (size_t b = 0; b < f64.order.size(); ++b)
    if (stat[b]) fail(NRG_E_EIG, "block eigensolver did not converge (n = " +
                                     std::to_string(f64.order[b].n) + ")");
  // ---- pending truncation per run + rotation descriptors
  std::vector<GemmGroup> groups;
  std::vector<GemmContrib> contribs;
  std::vector<GemmTile> tiles;
  OzList ozrot;
  for (int i = 0; i < nruns; ++i) {
    RunStep &st = steps[i];
    nrg_run *r = st.run;
    SiteData &sd = *st.site;
    r->tres = tres[i];
    r->all_eig_pending = std::move(sorted[i]);
    r->kept_new.assign(sd.sectors.size(), 0);
    sd.E_host.assign(sd.sectors.size(), {});
    int64_t eo = 0;
    for (size_t b = 0; b < sd.blocks.size(); ++b) {
      const DevBlock &db = sd.blocks[b];
      r->kept_new[db.sector] = kept_blk[st.b0 + int(b)];
      sd.E_host[db.sector].assign(evals[i].begin() + eo, evals[i].begin() + eo + db.n);
      eo += db.n;
    }
    // f-dagger rotation into the new basis, kept x kept part only
    // (nrgcore.hpp:409-476; the next site reads only this part, :199-203)
    std::map<OpKey, std::vector<GemmContrib>> outs;
    std::map<OpKey, std::vector<OzContrib>> ozouts;
    const bool use_oz = sd.has_uplanes;
    for (int ip = 0; ip < r->bath.nops; ++ip)
      for (auto &kv : r->bath.op[ip]) {
        const int bb = kv.first.first, bbp = kv.first.second;
        const HostMat &fb = kv.second;
        for (size_t ii = 0; ii < r->kept.size(); ++ii) {
          const int k = int(r->kept[ii]);
          if (k == 0) continue;
          auto ia = st.sub_of.find({int(ii), bb});
          auto ja = st.sub_of.find({int(ii), bbp});
          if (ia == st.sub_of.end() || ja == st.sub_of.end()) continue;
          const int si = ia->second.first, sj = ja->second.first;
          const DevBlock &bi = sd.blocks[sd.sectors[si].dev];
          const DevBlock &bj = sd.blocks[sd.sectors[sj].dev];
          auto &lst = outs[OpKey{ip, si, sj}];
          auto &olst = ozouts[OpKey{ip, si, sj}];
          for (int il = 0; il < fb.rows; ++il)
            for (int ilp = 0; ilp < fb.cols; ++ilp) {
              const double v = fb.v[int64_t(il) * fb.cols + ilp];
              if (v == 0.0) continue;
              if (use_oz) {
                OzOperand a = bi.uop, b = bj.uop;
                a.p += int64_t(ia->second.second + il * k) * a.ld;
                b.p += int64_t(ja->second.second + ilp * k) * b.ld;
                olst.push_back(ozc(a, b, k, 1, v));
                continue;
              }
              GemmContrib c{};
              c.A = bi.U + int64_t(ia->second.second + il * k) * bi.ld;
              c.lda = bi.ld;
              c.B = bj.U + int64_t(ja->second.second + ilp * k) * bj.ld;
              c.ldb = bj.ld;
              c.K = k;
              c.trans = 1;  // A stored K x M
              c.alpha = v;
              lst.push_back(c);
            }
        }
      }
    int64_t fsz = 0;
    for (auto &kv : outs) {
      const int si = std::get<1>(kv.first), sj = std::get<2>(kv.first);
      fsz += r->kept_new[si] * r->kept_new[sj];
      const double ni = sd.sectors[si].n, nj = sd.sectors[sj].n;
      e->work[1] += 2.0 * ni * nj * std::min(ni, nj);
    }
    r->fcur_mem = dalloc(e, fsz * sizeof(double) + 8);
    r->fcur.clear();
    int64_t fo = 0;
    for (auto &kv : outs) {
      const int si = std::get<1>(kv.first), sj = std::get<2>(kv.first);
      const int M = int(r->kept_new[si]), N = int(r->kept_new[sj]);
      if (M == 0 || N == 0) continue;
      FBlock fbk{static_cast<double *>(r->fcur_mem->ptr) + fo, M, N, N};
      fo += int64_t(M) * N;
      r->fcur[kv.first] = fbk;
      if (use_oz) {
        ozrot.out(fbk.p, N, M, N, false, ozouts[kv.first]);
        continue;
      }
      GemmGroup g{};
      g.C = fbk.p;
      g.ldc = N;
      g.M = M;
      g.N = N;
      g.accumulate = 0;
      g.c0 = int(contribs.size());
      contribs.insert(contribs.end(), kv.second.begin(), kv.second.end());
      g.c1 = int(contribs.size());
      const int gi = int(groups.size());
      groups.push_back(g);
      for (int tm = 0; tm < (M + GEMM_TILE - 1) / GEMM_TILE; ++tm)
        for (int tn = 0; tn < (N + GEMM_TILE - 1) / GEMM_TILE; ++tn) tiles.push_back({gi, tm, tn, 0});
    }
  }
  if (!ozrot.tiles.empty()) {
    check_cuda(cudaEventRecord(e->ev[4], s), "event");
    ozrot.launch(e, hold);
    check_cuda(cudaEventRecord(e->ev[5], s), "event");
  } else if (!tiles.empty()) {
    Arena ag;
    size_t o_t = ag.add(tiles), o_g = ag.add(groups), o_c = ag.add(contribs);
    DevPtr gd;
    char *gp = ag.push(e, gd);
    hold.push_back(gd);
    check_cuda(cudaEventRecord(e->ev[4], s), "event");
    Prof pf(e, "k_gemm_f64", gemm_flops(groups, contribs));
    launch_gemm_f64(at<GemmTile>(gp, o_t), int(tiles.size()), at<GemmGroup>(gp, o_g),
                    at<GemmContrib>(gp, o_c), s);
    count_launch(e);
    post_launch("rotate");
    check_cuda(cudaEventRecord(e->ev[5], s), "event");
  } else {
    check_cuda(cudaEventRecord(e->ev[4], s), "event");
    check_cuda(cudaEventRecord(e->ev[5], s), "event");
  }
  for (int i = 0; i < nruns; ++i) {
    nrg_run *r = steps[i].run;
    r->site = steps[i].site;
    r->have_site = true;
  }
  // descriptor buffers are released stream-ordered when `hold` goes out of scope
}

static void update_state(nrg_run *r) {
  if (!r->have_site) fail(NRG_E_STATE, "update_state without add_site");
  SiteData &sd = *r->site;
  r->cnt += 1;
  r->all_eig = std::move(r->all_eig_pending);
  r->kept = r->kept_new;
  r->no_of_kept = r->tres.kept_total;
  double shift = 0.0;
  if (r->no_of_kept <= int64_t(r->nkeep)) {
    r->cnt_min = r->cnt;
  } else {
    r->relgs.push_back(r->tres.emin);
    shift = r->tres.emin;
  }
  r->prev_shift = shift;
  r->prevE.assign(sd.sectors.size(), nullptr);
  for (auto &db : sd.blocks) r->prevE[db.sector] = db.E;
  r->prevE_host = sd.E_host;
  for (auto &v : r->prevE_host)
    for (auto &x : v) x -= shift;
  r->prev_site = r->site;
  r->pre_q = sd.cur_q;
  r->fprev = r->fcur;
  r->fprev_mem = r->fcur_mem;
  r->mem_H.reset();
  r->mem_sorted.reset();
  r->have_site = false;
}

}  // namespace nrg

namespace nrg {
// entry points used by engine_api.cpp
DevPtr engine_alloc(nrg_engine *e, size_t bytes) { return dalloc(e, bytes); }
SiteModel engine_parse_site(const nrg_site_desc *d, bool need_chi) { return parse_site(d, need_chi); }
void engine_upload_bath(nrg_engine *e, SiteModel &m) { upload_bath(e, m); }
void engine_batch_add_site(nrg_run *const *runs, int nruns, const double *t, int nt,
                           const double *rescale) {
  batch_add_site(runs, nruns, t, nt, rescale);
}
void engine_update_state(nrg_run *r) { update_state(r); }
void engine_count_launch(nrg_engine *e, int n) { count_launch(e, n); }
}  // namespace nrg

// ------------------------------------------------ standalone batched eigh
extern "C" int nrg_eigh_batched(nrg_engine *e, int nblk, const int *dims, const double *H, double *E,
                                double *U) {
  using namespace nrg;
  try {
    if (!e || nblk < 0 || (nblk > 0 && (!dims || !H || !E || !U))) fail(NRG_E_ARG, "null argument");
    cudaStream_t s = e->stream;
    int64_t hsz = 0, esz = 0, hin = 0;
    int max_n = 0;
    std::vector<DevBlock> blocks(nblk);
    for (int b = 0; b < nblk; ++b) {
      if (dims[b] <= 0) fail(NRG_E_ARG, "block dimension must be positive");
      blocks[b].n = dims[b];
      blocks[b].ld = round_up(dims[b], 2);
      hsz += int64_t(blocks[b].n) * blocks[b].ld;
      hin += int64_t(dims[b]) * dims[b];
      esz += dims[b];
      max_n = std::max(max_n, dims[b]);
    }
    if (nblk == 0) return NRG_OK;
    if (max_n > eig_max_n_f64()) fail(NRG_E_ARG, "block dimension exceeds the solver limit");
    std::vector<DevPtr> hold;
    DevPtr mh = dalloc(e, hsz * 8), mu = dalloc(e, hsz * 8), me = dalloc(e, esz * 8 + 8);
    int64_t ho = 0, eo = 0, io = 0;
    for (auto &b : blocks) {
      b.H = static_cast<double *>(mh->ptr) + ho;
      b.U = static_cast<double *>(mu->ptr) + ho;
      b.E = static_cast<double *>(me->ptr) + eo;
      check_cuda(cudaMemcpy2DAsync(b.H, b.ld * 8, H + io, b.n * 8, b.n * 8, b.n, cudaMemcpyHostToDevice, s),
                 "H upload");
      ho += int64_t(b.n) * b.ld;
      eo += b.n;
      io += int64_t(b.n) * b.n;
    }
    if (e->precision == NRG_PREC_FP64) {
      std::vector<EigBlock> eb(nblk);
      for (int b = 0; b < nblk; ++b) {
        eb[b] = EigBlock{};
        eb[b].H = blocks[b].H;
        eb[b].U = blocks[b].U;
        eb[b].E = blocks[b].E;
        eb[b].n = blocks[b].n;
        eb[b].ld = blocks[b].ld;
        eb[b].ldu = blocks[b].ld;
      }
      std::stable_sort(eb.begin(), eb.end(), [](const EigBlock &x, const EigBlock &y) { return x.n > y.n; });
      F64Solve f = fp64_eigensolve(e, eb, hold, s);
      std::vector<int> st(nblk + 1, 0);
      check_cuda(cudaMemcpyAsync(st.data(), f.d_status, nblk * sizeof(int), cudaMemcpyDeviceToHost, s), "status");
      check_cuda(cudaStreamSynchronize(s), "eigh");
      check_kernel_error(e);
      for (int b = 0; b < nblk; ++b)
        if (st[b]) fail(NRG_E_EIG, "block eigensolver did not converge");
    } else {
      if (max_n > refine_max_n()) fail(NRG_E_ARG, "block dimension exceeds the refinement limit");
      std::vector<DevBlock *> ptrs;
      for (auto &b : blocks) ptrs.push_back(&b);
      std::stable_sort(ptrs.begin(), ptrs.end(), [](DevBlock *x, DevBlock *y) { return x->n > y->n; });
      MixedCheck mc;
      mc.enqueue(mixed_eigensolve(e, ptrs, max_n, hold), s);
      check_cuda(cudaStreamSynchronize(s), "eigh");
      check_kernel_error(e);
      mc.check(e);
    }
    eo = 0;
    io = 0;
    for (auto &b : blocks) {
      check_cuda(cudaMemcpy2DAsync(U + io, b.n * 8, b.U, b.ld * 8, b.n * 8, b.n, cudaMemcpyDeviceToHost, s),
                 "U download");
      check_cuda(cudaMemcpyAsync(E + eo, b.E, b.n * 8, cudaMemcpyDeviceToHost, s), "E download");
      eo += b.n;
      io += int64_t(b.n) * b.n;
    }
    check_cuda(cudaStreamSynchronize(s), "eigh");
    return NRG_OK;
  } catch (const Error &x) {
    g_err = x.msg;
    return x.code;
  }
}

// ------------------------------------- FP64-accurate tensor-core GEMM ABI
extern "C" int nrg_dgemm_tc(nrg_engine *e, int transA, int transB, int M, int N, int K, double alpha,
                            const double *A, int lda, const double *B, int ldb, double beta, double *C,
                            int ldc) {
  using namespace nrg;
  try {
    if (!e || M < 0 || N < 0 || K < 0 || !A || !B || !C) fail(NRG_E_ARG, "bad argument");
    if (M == 0 || N == 0) return NRG_OK;
    if (beta != 0.0 && beta != 1.0) fail(NRG_E_ARG, "beta must be 0 or 1");
    cudaStream_t s = e->stream;
    std::vector<DevPtr> hold;
    // stored shapes: A is (transA ? K x M : M x K), B is (transB ? N x K : K x N)
    const int ar = transA ? K : M, ac = transA ? M : K, br = transB ? N : K, bc = transB ? K : N;
    if (lda < ac || ldb < bc || ldc < N) fail(NRG_E_ARG, "leading dimension too small");
    DevPtr da = dalloc(e, int64_t(ar) * ac * 8 + 8), db = dalloc(e, int64_t(br) * bc * 8 + 8),
           dc = dalloc(e, int64_t(M) * N * 8 + 8);
    check_cuda(cudaMemcpy2DAsync(da->ptr, ac * 8, A, lda * 8, ac * 8, ar, cudaMemcpyHostToDevice, s), "A");
    check_cuda(cudaMemcpy2DAsync(db->ptr, bc * 8, B, ldb * 8, bc * 8, br, cudaMemcpyHostToDevice, s), "B");
    if (beta != 0.0)
      check_cuda(cudaMemcpy2DAsync(dc->ptr, N * 8, C, ldc * 8, N * 8, M, cudaMemcpyHostToDevice, s), "C");
    const PlaneBuf pl = split_matrices(e, {MatRef{static_cast<const double *>(da->ptr), ar, ac, ac},
                                           MatRef{static_cast<const double *>(db->ptr), br, bc, bc}},
                                       hold);
    const OzOperand oa = pl.op(0), ob = pl.op(1);
    OzList l;
    l.out(static_cast<double *>(dc->ptr), N, M, N, beta != 0.0,
          {ozc(oa, ob, K, (transA ? 1 : 0) | (transB ? 2 : 0), alpha)});
    l.launch(e, hold);
    check_cuda(cudaMemcpy2DAsync(C, ldc * 8, dc->ptr, N * 8, N * 8, M, cudaMemcpyDeviceToHost, s), "C");
    check_cuda(cudaStreamSynchronize(s), "dgemm_tc");
    check_kernel_error(e);
    return NRG_OK;
  } catch (const Error &x) {
    g_err = x.msg;
    return x.code;
  }
}
