// C ABI of the engine (include/nrg_gpu.h): argument checking, the tracked
// operators (update_system_operator), device-resident snapshots (NrgData),
// the FDM spectral pass (fdmSpectrum) and thermodynamics (fdmThermodynamics).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <cstring>
#include <numeric>
#include <set>

#include "engine_core.h"

namespace nrg {
extern thread_local std::string g_err;
DevPtr engine_alloc(nrg_engine *e, size_t bytes);
SiteModel engine_parse_site(const nrg_site_desc *d, bool need_chi);
void engine_upload_bath(nrg_engine *e, SiteModel &m);
void engine_batch_add_site(nrg_run *const *runs, int nruns, const double *t, int nt,
                           const double *rescale);
void engine_update_state(nrg_run *r);
void engine_count_launch(nrg_engine *e, int n);
double gemm_flops(const std::vector<GemmGroup> &gs, const std::vector<GemmContrib> &cs);

constexpr int kFdmPts = 100000;                  // fdmSpectrum.hpp:351
constexpr double kFdmMin = 1e-10, kFdmMax = 10;  // fdmSpectrum.hpp:352-353
constexpr double kFdmEnergyErrorbar = 1e-5;      // fdmSpectrum.hpp:363

static double fdm_delE() { return (kFdmPts - 1.0) / (std::log(kFdmMax / kFdmMin)); }

template <class F> static int guard(F &&f) {
  try {
    f();
    return NRG_OK;
  } catch (const Error &e) {
    g_err = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    g_err = e.what();
    return NRG_E_ARG;
  }
}

struct Staged {  // descriptor tables of one launch phase
  std::vector<char> buf;
  template <class T> size_t add(const std::vector<T> &v) {
    size_t off = (buf.size() + 255) & ~size_t(255);
    buf.resize(off + v.size() * sizeof(T) + 16);
    if (!v.empty()) std::memcpy(buf.data() + off, v.data(), v.size() * sizeof(T));
    return off;
  }
  char *push(nrg_engine *e, DevPtr &hold) {
    hold = engine_alloc(e, buf.size());
    upload_async(e, hold->ptr, buf.data(), buf.size());
    return static_cast<char *>(hold->ptr);
  }
};
template <class T> static T *at(char *b, size_t o) { return reinterpret_cast<T *>(b + o); }

// Grouped GEMM launch helper: one output per group.
struct GemmBatch {
  std::vector<GemmGroup> groups;
  std::vector<GemmContrib> contribs;
  std::vector<GemmTile> tiles;
  void out(double *C, int ldc, int M, int N, bool accumulate,
           const std::vector<GemmContrib> &cs) {
    GemmGroup g{};
    g.C = C;
    g.ldc = ldc;
    g.M = M;
    g.N = N;
    g.accumulate = accumulate ? 1 : 0;
    g.c0 = int(contribs.size());
    contribs.insert(contribs.end(), cs.begin(), cs.end());
    g.c1 = int(contribs.size());
    int gi = int(groups.size());
    groups.push_back(g);
    for (int tm = 0; tm < (M + GEMM_TILE - 1) / GEMM_TILE; ++tm)
      for (int tn = 0; tn < (N + GEMM_TILE - 1) / GEMM_TILE; ++tn) tiles.push_back({gi, tm, tn, 0});
  }
  void run(nrg_engine *e) {
    if (tiles.empty()) return;
    Staged st;
    size_t ot = st.add(tiles), og = st.add(groups), oc = st.add(contribs);
    DevPtr hold;
    char *d = st.push(e, hold);
    Prof pf(e, "k_gemm_f64", gemm_flops(groups, contribs));
    launch_gemm_f64(at<GemmTile>(d, ot), int(tiles.size()), at<GemmGroup>(d, og),
                    at<GemmContrib>(d, oc), e->stream);
    engine_count_launch(e, 1);
    check_cuda(cudaGetLastError(), "grouped gemm");
  }
};
static GemmContrib gc(const double *A, int lda, const double *B, int ldb, int K, int trans,
                      double alpha) {
  GemmContrib c{};
  c.A = A;
  c.lda = lda;
  c.B = B;
  c.ldb = ldb;
  c.K = K;
  c.trans = trans;
  c.alpha = alpha;
  return c;
}

// --------------------------------------------------- update_system_operator
// O_new(i,j) = sum over sub-block pairs with the same bath sector bb of
// U_i[rows (ii,bb,il)]^T O_prev(ii,ii')[:k,:k'] U_j[rows (ii',bb,il)]
// (sysOperator.hpp:36-133), as two grouped-GEMM passes through Y = O U_j.
static void opset_update_batch(const std::vector<nrg_opset *> &os) {
  if (os.empty()) return;
  nrg_engine *e = os[0]->run->eng;
  struct P1 { size_t o; OzOperand u; int kp, k, nj; double *Y; };
  struct Per {
    nrg_opset *o;
    std::map<OpKey, FBlock> nb_blocks;
    DevPtr ymem, omem;
    std::map<OpKey, std::vector<GemmContrib>> p2c;
    std::vector<P1> p1oz;
    std::map<OpKey, std::vector<std::pair<OzOperand, size_t>>> p2oz;  // (U_i rows, Y index)
  };
  std::vector<Per> P(os.size());
  GemmBatch p1, p2;
  std::vector<MatRef> omats, ymats;
  bool oz = false;
  for (size_t w = 0; w < os.size(); ++w) {
    nrg_opset *o = os[w];
    Per &pw = P[w];
    pw.o = o;
    nrg_run *r = o->run;
    if (!r->have_site) fail(NRG_E_STATE, "update_system_operator needs add_site first");
    if (r->eng != e) fail(NRG_E_ARG, "operator sets of one batch must share an engine");
    SiteData &sd = *r->site;
    if (w == 0) oz = sd.has_uplanes;
    else if (oz != sd.has_uplanes) fail(NRG_E_ARG, "operator sets of one batch must share the precision path");
    const SiteModel &bath = r->bath;
    const int nb = int(bath.q.size());
    std::map<std::pair<int, int>, std::pair<int, int>> sub_of;
    for (size_t s = 0; s < sd.sectors.size(); ++s)
      for (auto &sb : sd.sectors[s].subs) sub_of[{sb.ii, sb.bb}] = {int(s), sb.off};
    int64_t ysz = 0;
    std::vector<std::tuple<const FBlock *, int, int, int, int, int>> pend;  // block, ip, ii, iip, bb, il
    std::map<OpKey, int> outs;
    for (auto &kv : o->blocks) {
      const int ip = std::get<0>(kv.first), ii = std::get<1>(kv.first), iip = std::get<2>(kv.first);
      const int k = int(r->kept[ii]), kp = int(r->kept[iip]);
      for (int bb = 0; bb < nb; ++bb) {
        auto a = sub_of.find({ii, bb});
        auto b = sub_of.find({iip, bb});
        // the output block exists whenever both sub-blocks do (hasValue, :244-248)
        const int si = a != sub_of.end() ? a->second.first : -1;
        const int sj = b != sub_of.end() ? b->second.first : -1;
        if (si < 0 || sj < 0) continue;
        outs.emplace(OpKey{ip, si, sj}, 0);
        if (k == 0 || kp == 0) continue;
        for (int il = 0; il < int(bath.E[bb].size()); ++il) {
          pend.emplace_back(&kv.second, ip, ii, iip, bb, il);
          ysz += int64_t(k) * sd.blocks[sd.sectors[sj].dev].n;
        }
      }
    }
    pw.ymem = engine_alloc(e, ysz * sizeof(double) + 8);
    int64_t yo = 0;
    std::map<const double *, size_t> oidx;
    for (auto &t : pend) {
      const FBlock *F = std::get<0>(t);
      const int ip = std::get<1>(t), ii = std::get<2>(t), iip = std::get<3>(t), bb = std::get<4>(t),
                il = std::get<5>(t);
      const int k = int(r->kept[ii]), kp = int(r->kept[iip]);
      auto a = sub_of.at({ii, bb});
      auto b = sub_of.at({iip, bb});
      const DevBlock &bi = sd.blocks[sd.sectors[a.first].dev];
      const DevBlock &bj = sd.blocks[sd.sectors[b.first].dev];
      double *Y = static_cast<double *>(pw.ymem->ptr) + yo;
      yo += int64_t(k) * bj.n;
      if (oz) {
        auto ins = oidx.emplace(F->p, omats.size());
        if (ins.second) omats.push_back(MatRef{F->p, k, kp, F->ld});
        OzOperand uj = bj.uop, ui = bi.uop;
        uj.p += int64_t(b.second + il * kp) * uj.ld;
        ui.p += int64_t(a.second + il * k) * ui.ld;
        pw.p1oz.push_back(P1{ins.first->second, uj, kp, k, bj.n, Y});
        pw.p2oz[OpKey{ip, a.first, b.first}].push_back({ui, ymats.size()});
        ymats.push_back(MatRef{Y, k, bj.n, bj.n});
        continue;
      }
      // pass 1: Y (k x n_j) = O[:k,:k'] U_j[rows (iip,bb,il), :]
      p1.out(Y, bj.n, k, bj.n, false,
             {gc(F->p, F->ld, bj.U + int64_t(b.second + il * kp) * bj.ld, bj.ld, kp, 0, 1.0)});
      // pass 2: O_new(i,j) += U_i[rows (ii,bb,il), :]^T Y
      pw.p2c[OpKey{ip, a.first, b.first}].push_back(
          gc(bi.U + int64_t(a.second + il * k) * bi.ld, bi.ld, Y, bj.n, k, 1, 1.0));
    }
    int64_t osz = 0;
    for (auto &kv : outs) {
      const DevBlock &bi = sd.blocks[sd.sectors[std::get<1>(kv.first)].dev];
      const DevBlock &bj = sd.blocks[sd.sectors[std::get<2>(kv.first)].dev];
      osz += int64_t(bi.n) * bj.n;
    }
    pw.omem = engine_alloc(e, osz * sizeof(double) + 8);
    int64_t oo = 0;
    for (auto &kv : outs) {
      const DevBlock &bi = sd.blocks[sd.sectors[std::get<1>(kv.first)].dev];
      const DevBlock &bj = sd.blocks[sd.sectors[std::get<2>(kv.first)].dev];
      FBlock fb{static_cast<double *>(pw.omem->ptr) + oo, bi.n, bj.n, bj.n};
      oo += int64_t(bi.n) * bj.n;
      pw.nb_blocks[kv.first] = fb;
      if (oz) continue;
      auto it = pw.p2c.find(kv.first);
      p2.out(fb.p, fb.ld, bi.n, bj.n, false, it == pw.p2c.end() ? std::vector<GemmContrib>{} : it->second);
    }
  }
  if (oz) {  // tensor-core variant (mixed path): digit planes of the O views and of Y
    std::vector<DevPtr> hold;
    PlaneBuf po = split_matrices(e, omats, hold);
    OzList l1;
    for (auto &pw : P)
      for (auto &x : pw.p1oz) l1.out(x.Y, x.nj, x.k, x.nj, false, {ozc(po.op(x.o), x.u, x.kp, 0)});
    l1.launch(e, hold);
    PlaneBuf py = split_matrices(e, ymats, hold);
    OzList l2;
    for (auto &pw : P)
      for (auto &kv : pw.nb_blocks) {
        std::vector<OzContrib> cs;
        auto it = pw.p2oz.find(kv.first);
        if (it != pw.p2oz.end())
          for (auto &pr : it->second) cs.push_back(ozc(pr.first, py.op(pr.second), ymats[pr.second].rows, 1));
        l2.out(kv.second.p, kv.second.ld, kv.second.rows, kv.second.cols, false, cs);
      }
    l2.launch(e, hold);
  } else {
    p1.run(e);
    p2.run(e);
  }
  for (auto &pw : P) {
    pw.o->blocks = std::move(pw.nb_blocks);
    pw.o->mem = pw.omem;
    pw.o->updated_this_site = true;
  }
}

static void opset_update(nrg_opset *o) { opset_update_batch({o}); }

// ------------------------------------------------------------- FDM (T = 0)
// One backward-pass shell (fdmSpectrum::calcSpectrum, fdmSpectrum.hpp:55-63)
// for every FDM object of the batch: each must belong to a different run with
// a loaded snapshot.  All of them share one launch per phase: rho set-up,
// digit split, the B rho / rho B GEMMs, binning, rho <- U rho U^T and the
// partial trace.  A single object is the batch of one.
static void fdm_calc_batch(const std::vector<nrg_fdm *> &fs, const std::vector<double> &scales) {
  if (fs.empty()) return;
  nrg_engine *e = fs[0]->run->eng;
  cudaStream_t s = e->stream;
  const size_t nf = fs.size();
  struct Work {
    nrg_fdm *f;
    SiteData *sd;
    Snapshot *S;
    std::vector<double *> rp, rot;
    DevPtr rho, pm, xm, rm;
    bool oz;
  };
  std::vector<Work> W(nf);
  std::vector<DevPtr> hold;
  // ---- setCurrentIndex (:289-298), setRhoZero (:165-199), rho blocks
  std::vector<RhoTask> rtasks;
  std::vector<double> diag_host;     // Boltzmann diagonals of last shells, staged once
  std::vector<std::pair<size_t, size_t>> diag_fix;  // (task, offset into diag_host)
  int64_t rchunks = 0;
  for (size_t w = 0; w < nf; ++w) {
    nrg_fdm *f = fs[w];
    nrg_run *r = f->run;
    if (!r->loaded) fail(NRG_E_STATE, "calcSpectrum needs a loaded snapshot");
    if (r->eng != e) fail(NRG_E_ARG, "FDM objects of one batch must share an engine");
    for (size_t v = 0; v < w; ++v)
      if (fs[v]->run == r) fail(NRG_E_ARG, "FDM objects of one batch must belong to different runs");
    Work &wk = W[w];
    wk.f = f;
    wk.S = r->loaded.get();
    wk.sd = wk.S->site.get();
    SiteData &sd = *wk.sd;
    const int nsec = int(sd.cur_q.size());
    if (!f->have_cur) {
      f->cur_kept.assign(nsec, 0);
      f->have_cur = true;
    } else {
      f->cur_kept = f->prev_kept;
    }
    f->prev_kept = sd.kept_prev;
    if (int(f->cur_kept.size()) != nsec) fail(NRG_E_STATE, "snapshot order does not match the backward pass");
    std::vector<std::vector<double>> boltz;
    if (f->finite_t) {  // setRhoZero(tBoltzmannFactor), fdmBackwardIteration.hpp:207-239
      if (f->ncalc >= f->shell_weights.size())
        fail(NRG_E_STATE, "finite-temperature FDM: more shells than the thermodynamics saw");
      const std::vector<double> &wt = f->shell_weights[f->ncalc];
      size_t o = 0;
      boltz.resize(nsec);
      for (int i = 0; i < nsec; ++i) {
        const size_t n = sd.E_host[i].size(), kc = size_t(f->cur_kept[i]);
        boltz[i].assign(n, 0.0);
        for (size_t x = kc; x < n; ++x) {
          if (o >= wt.size()) fail(NRG_E_STATE, "finite-temperature FDM: shell does not match the thermodynamics");
          boltz[i][x] = wt[o++];
        }
      }
      if (o != wt.size()) fail(NRG_E_STATE, "finite-temperature FDM: shell does not match the thermodynamics");
      f->ncalc++;
    } else if (f->last) {  // setLocalPartitionFunction (:122-155)
      double gs = 0;
      for (auto &v : sd.E_host)
        if (!v.empty()) gs = std::min(gs, *std::min_element(v.begin(), v.end()));
      double z = 0;
      for (auto &v : sd.E_host)
        for (double x : v)
          if (std::fabs(x - gs) < kFdmEnergyErrorbar) z += 1.0;
      boltz.resize(nsec);
      for (int i = 0; i < nsec; ++i) {
        boltz[i].resize(sd.E_host[i].size());
        for (size_t x = 0; x < sd.E_host[i].size(); ++x)
          boltz[i][x] = std::fabs(sd.E_host[i][x] - gs) < kFdmEnergyErrorbar ? 1.0 / z : 0.0;
      }
      f->local_gs = gs;
      f->local_z = z;
    }
    f->partitions.push_back(f->local_z);
    int64_t rsz = 0;
    for (auto &db : sd.blocks) rsz += int64_t(db.n) * db.n;
    wk.rho = engine_alloc(e, rsz * sizeof(double) + 8);
    wk.rp.resize(sd.blocks.size());
    int64_t ro = 0;
    for (size_t b = 0; b < sd.blocks.size(); ++b) {
      const DevBlock &db = sd.blocks[b];
      wk.rp[b] = static_cast<double *>(wk.rho->ptr) + ro;
      ro += int64_t(db.n) * db.n;
      RhoTask t{};
      t.rho = wk.rp[b];
      t.n = db.n;
      if (!boltz.empty()) {
        diag_fix.push_back({rtasks.size(), diag_host.size()});
        diag_host.insert(diag_host.end(), boltz[db.sector].begin(), boltz[db.sector].end());
      }
      if (f->have_reduced) {
        const int kc = int(f->cur_kept[db.sector]);
        if (kc > 0) {
          if (f->reduced_k[db.sector] != kc) fail(NRG_E_STATE, "reduced density matrix size mismatch");
          t.red = f->reduced[db.sector];
          t.kc = kc;
        }
      }
      t.chunk0 = rchunks;
      rchunks += (int64_t(db.n) * db.n + 255) / 256;
      rtasks.push_back(t);
    }
    wk.oz = sd.has_uplanes;
  }
  if (!rtasks.empty()) {
    DevPtr dd;
    if (!diag_host.empty()) {
      Staged sd0;
      size_t od = sd0.add(diag_host);
      char *dp = sd0.push(e, dd);
      for (auto &fx : diag_fix) rtasks[fx.first].diag = at<double>(dp, od) + fx.second;
    }
    Staged st;
    size_t ot = st.add(rtasks);
    DevPtr h;
    char *d = st.push(e, h);
    launch_rho_init(at<RhoTask>(d, ot), int(rtasks.size()), rchunks, s);
    engine_count_launch(e, 1);
    check_cuda(cudaGetLastError(), "rho init");
    hold.push_back(dd);
    hold.push_back(h);
  }
  // ---- rhoDotStaticOperators (fdmBackwardIteration.hpp:166-199): Tr(O_ii rho_i)
  // per operator over its diagonal blocks, the kept x kept part of O left out
  for (size_t w = 0; w < nf; ++w) {
    Work &wk = W[w];
    nrg_fdm *f = wk.f;
    SiteData &sd = *wk.sd;
    std::vector<StaticTask> st;
    for (auto &kv : wk.S->ops) {
      const int ip = std::get<0>(kv.first), i = std::get<1>(kv.first), j = std::get<2>(kv.first);
      if (i != j || ip < 0 || ip >= f->nops || sd.sectors[i].dev < 0) continue;
      const int b = sd.sectors[i].dev;
      StaticTask t{};
      t.O = kv.second.p;
      t.ldo = kv.second.ld;
      t.rho = wk.rp[b];
      t.n = sd.blocks[b].n;
      t.kc = int(f->cur_kept[i]);
      t.op = ip;
      st.push_back(t);
    }
    if (st.empty()) continue;
    if (!f->static_acc) {
      f->static_acc = engine_alloc(e, f->nops * sizeof(double));
      check_cuda(cudaMemsetAsync(f->static_acc->ptr, 0, f->nops * sizeof(double), s), "static sums");
    }
    Staged sg;
    size_t ot = sg.add(st);
    std::vector<double> partial(st.size(), 0.0);
    size_t opart = sg.add(partial);
    DevPtr h;
    char *d = sg.push(e, h);
    hold.push_back(h);
    launch_fdm_static(at<StaticTask>(d, ot), int(st.size()), f->nops, at<double>(d, opart),
                      static_cast<double *>(f->static_acc->ptr), s);
    engine_count_launch(e, 2);
    check_cuda(cudaGetLastError(), "static expectation values");
  }
  // ---- rhoDotOperators (:207-277): B rho_j and rho_i B, then binning
  const bool oz = W[0].oz;
  for (auto &wk : W)
    if (wk.oz != oz) fail(NRG_E_ARG, "FDM objects of one batch must share the precision path");
  std::vector<MatRef> rmats, bmats;
  std::vector<size_t> r0(nf), b0(nf);
  std::vector<std::map<const double *, size_t>> bidx(nf);
  for (size_t w = 0; w < nf; ++w) {
    Work &wk = W[w];
    SiteData &sd = *wk.sd;
    r0[w] = rmats.size();
    b0[w] = bmats.size();
    for (size_t b = 0; b < sd.blocks.size(); ++b)
      rmats.push_back(MatRef{wk.rp[b], sd.blocks[b].n, sd.blocks[b].n, sd.blocks[b].n});
    for (auto &kv : wk.S->ops) {
      const int i = std::get<1>(kv.first), j = std::get<2>(kv.first);
      if (sd.sectors[i].dev < 0 || sd.sectors[j].dev < 0) continue;
      bidx[w][kv.second.p] = bmats.size() - b0[w];
      bmats.push_back(MatRef{kv.second.p, kv.second.rows, kv.second.cols, kv.second.ld});
    }
  }
  PlaneBuf prho, pB;
  if (oz) {
    prho = split_matrices(e, rmats, hold);
    pB = split_matrices(e, bmats, hold);
  }
  GemmBatch g;
  OzList ozg;
  std::vector<FdmPair> pairs;
  int64_t chunk = 0;
  for (size_t w = 0; w < nf; ++w) {
    Work &wk = W[w];
    nrg_fdm *f = wk.f;
    SiteData &sd = *wk.sd;
    int64_t psz = 0;
    for (auto &kv : wk.S->ops) {
      const int i = std::get<1>(kv.first), j = std::get<2>(kv.first);
      if (sd.sectors[i].dev < 0 || sd.sectors[j].dev < 0) continue;
      psz += 2 * int64_t(sd.blocks[sd.sectors[i].dev].n) * sd.blocks[sd.sectors[j].dev].n;
    }
    wk.pm = engine_alloc(e, psz * sizeof(double) + 8);
    int64_t po = 0;
    double *hist = static_cast<double *>(f->hist->ptr);
    for (auto &kv : wk.S->ops) {
      const int ip = std::get<0>(kv.first), i = std::get<1>(kv.first), j = std::get<2>(kv.first);
      if (ip < 0 || ip >= f->nops) fail(NRG_E_ARG, "snapshot operator index exceeds the FDM operator count");
      if (sd.sectors[i].dev < 0 || sd.sectors[j].dev < 0) continue;
      const int bi = sd.sectors[i].dev, bj = sd.sectors[j].dev;
      const DevBlock &Bi = sd.blocks[bi], &Bj = sd.blocks[bj];
      const FBlock &B = kv.second;
      if (B.ld != Bj.n) fail(NRG_E_STATE, "operator block layout");
      double *rhoA = static_cast<double *>(wk.pm->ptr) + po;
      po += int64_t(Bi.n) * Bj.n;
      double *ARho = static_cast<double *>(wk.pm->ptr) + po;
      po += int64_t(Bi.n) * Bj.n;
      if (oz) {
        const size_t q = b0[w] + bidx[w].at(B.p);
        ozg.out(rhoA, Bj.n, Bi.n, Bj.n, false, {ozc(pB.op(q), prho.op(r0[w] + bj), Bj.n, 0)});
        ozg.out(ARho, Bj.n, Bi.n, Bj.n, false, {ozc(prho.op(r0[w] + bi), pB.op(q), Bi.n, 0)});
      } else {
        g.out(rhoA, Bj.n, Bi.n, Bj.n, false, {gc(B.p, B.ld, wk.rp[bj], Bj.n, Bj.n, 0, 1.0)});
        g.out(ARho, Bj.n, Bi.n, Bj.n, false, {gc(wk.rp[bi], Bi.n, B.p, B.ld, Bi.n, 0, 1.0)});
      }
      FdmPair fp{};
      fp.rhoA = rhoA;
      fp.ARho = ARho;
      fp.B = B.p;
      fp.Ei = Bi.E;
      fp.Ej = Bj.E;
      fp.pos = hist + int64_t(ip) * kFdmPts;
      fp.neg = hist + (int64_t(f->nops) + ip) * kFdmPts;
      fp.scale = scales[w];
      fp.ni = Bi.n;
      fp.nj = Bj.n;
      fp.kci = int(f->cur_kept[i]);
      fp.kcj = int(f->cur_kept[j]);
      fp.chunk0 = chunk;
      chunk += (int64_t(Bi.n) * Bj.n + 255) / 256;
      pairs.push_back(fp);
    }
  }
  g.run(e);
  ozg.launch(e, hold);
  if (!pairs.empty()) {
    Staged st;
    size_t op = st.add(pairs);
    DevPtr h;
    char *d = st.push(e, h);
    hold.push_back(h);
    Prof pf(e, "k_fdm_bin");
    launch_fdm_bin(at<FdmPair>(d, op), int(pairs.size()), chunk, fdm_delE(), kFdmPts, s);
    engine_count_launch(e, 1);
    check_cuda(cudaGetLastError(), "fdm binning");
  }
  // ---- setReduceDensityMatrix (:71-114): rho <- U rho U^T, then the partial trace
  GemmBatch g1, g2;
  OzList o1, o2;
  std::vector<MatRef> xmats;
  for (size_t w = 0; w < nf; ++w) {
    Work &wk = W[w];
    SiteData &sd = *wk.sd;
    int64_t rsz = 0;
    for (auto &db : sd.blocks) rsz += int64_t(db.n) * db.n;
    wk.xm = engine_alloc(e, rsz * sizeof(double) + 8);
    wk.rm = engine_alloc(e, rsz * sizeof(double) + 8);
    wk.rot.resize(sd.blocks.size());
    int64_t xo = 0;
    for (size_t b = 0; b < sd.blocks.size(); ++b) {
      const DevBlock &db = sd.blocks[b];
      double *X = static_cast<double *>(wk.xm->ptr) + xo;
      wk.rot[b] = static_cast<double *>(wk.rm->ptr) + xo;
      xo += int64_t(db.n) * db.n;
      if (oz) {
        o1.out(X, db.n, db.n, db.n, false, {ozc(prho.op(r0[w] + b), db.uop, db.n, 2)});  // rho U^T
        xmats.push_back(MatRef{X, db.n, db.n, db.n});
        continue;
      }
      g1.out(X, db.n, db.n, db.n, false, {gc(wk.rp[b], db.n, db.U, db.ld, db.n, 2, 1.0)});  // rho U^T
      g2.out(wk.rot[b], db.n, db.n, db.n, false, {gc(db.U, db.ld, X, db.n, db.n, 0, 1.0)});  // U X
    }
  }
  if (oz) {
    o1.launch(e, hold);
    PlaneBuf px = split_matrices(e, xmats, hold);
    size_t q = 0;
    for (size_t w = 0; w < nf; ++w) {
      SiteData &sd = *W[w].sd;
      for (size_t b = 0; b < sd.blocks.size(); ++b, ++q) {
        const DevBlock &db = sd.blocks[b];
        o2.out(W[w].rot[b], db.n, db.n, db.n, false, {ozc(db.uop, px.op(q), db.n, 0)});  // U X
      }
    }
    o2.launch(e, hold);
  } else {
    g1.run(e);
    g2.run(e);
  }
  std::vector<TraceTask> tasks;
  std::vector<TraceIn> flat;
  int maxk = 0;
  std::vector<std::vector<DevPtr>> red_mem(nf);
  std::vector<std::vector<double *>> red(nf);
  std::vector<std::vector<int64_t>> red_k(nf);
  for (size_t w = 0; w < nf; ++w) {
    Work &wk = W[w];
    SiteData &sd = *wk.sd;
    const int npre = int(sd.pre_q.size());
    const int nsec = int(sd.cur_q.size());
    red_mem[w].resize(npre);
    red[w].assign(npre, nullptr);
    red_k[w].assign(npre, 0);
    std::vector<std::vector<TraceIn>> ins(npre);
    for (int i = 0; i < nsec; ++i) {
      const Sector &Sc = sd.sectors[i];
      if (Sc.dev < 0) continue;
      for (auto &sb : Sc.subs) ins[sb.ii].push_back({wk.rot[Sc.dev], sd.blocks[Sc.dev].n, sb.off, sb.d, 0});
    }
    for (int ii = 0; ii < npre; ++ii) {
      const int k = int(sd.kept_prev[ii]);
      red_k[w][ii] = k;
      if (k == 0) continue;
      red_mem[w][ii] = engine_alloc(e, int64_t(k) * k * sizeof(double));
      red[w][ii] = static_cast<double *>(red_mem[w][ii]->ptr);
      TraceTask t{};
      t.out = red[w][ii];
      t.k = k;
      t.in0 = int(flat.size());
      flat.insert(flat.end(), ins[ii].begin(), ins[ii].end());
      t.in1 = int(flat.size());
      tasks.push_back(t);
      maxk = std::max(maxk, k);
    }
  }
  if (!tasks.empty()) {
    Staged st;
    size_t ot = st.add(tasks), oi = st.add(flat);
    DevPtr h;
    char *d = st.push(e, h);
    hold.push_back(h);
    launch_partial_trace(at<TraceTask>(d, ot), int(tasks.size()), at<TraceIn>(d, oi), maxk, s);
    engine_count_launch(e, 1);
    check_cuda(cudaGetLastError(), "partial trace");
  }
  for (size_t w = 0; w < nf; ++w) {
    nrg_fdm *f = W[w].f;
    f->reduced_mem = std::move(red_mem[w]);
    f->reduced = std::move(red[w]);
    f->reduced_k = std::move(red_k[w]);
    f->have_reduced = true;
    f->last = false;
  }
  // no synchronisation: every buffer above is freed stream-ordered and every
  // host array was staged by its copy call, so the host may queue the next
  // shell while this one runs (errors surface at the next synchronising call)
}

}  // namespace nrg

using namespace nrg;

extern "C" {

const char *nrg_last_error(void) { return g_err.c_str(); }

int nrg_engine_create(const nrg_engine_opts *opts, nrg_engine **out) {
  return guard([&] {
    if (!out) fail(NRG_E_ARG, "null out");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      fail(NRG_E_NOCUDA, "no CUDA device available: the NRG engine has no CPU fallback");
    }
    auto *e = new nrg_engine();
    if (opts) {
      e->device = opts->device;
      e->precision = opts->precision;
      e->budget = opts->hbm_budget_bytes;
      e->verbose = opts->verbose;
    }
    if (e->precision != NRG_PREC_FP64 && e->precision != NRG_PREC_MIXED) {
      delete e;
      fail(NRG_E_ARG, "unknown precision mode");
    }
    check_cuda(cudaSetDevice(e->device), "cudaSetDevice");
    check_cuda(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "stream");
    check_cuda(cudaStreamCreateWithFlags(&e->side, cudaStreamNonBlocking), "side stream");
    check_cuda(cudaEventCreateWithFlags(&e->fork_ev, cudaEventDisableTiming), "event");
    check_cuda(cudaEventCreateWithFlags(&e->join_ev, cudaEventDisableTiming), "event");
    for (auto &ev : e->ev) check_cuda(cudaEventCreate(&ev), "event");
    e->eig_smem_f64 = eig_smem_limit_f64();
    e->eig_smem_f32 = eig_smem_limit_f32();
    check_cuda(cudaMalloc(&e->d_kerr, sizeof(int)), "cudaMalloc (kernel error word)");
    check_cuda(cudaMemset(e->d_kerr, 0, sizeof(int)), "cudaMemset");
    if (const char *oz = std::getenv("NRG_OZAKI")) e->ozaki = std::atoi(oz) & 3;
    if (const char *c = std::getenv("NRG_EIG_CLUSTER")) e->eig_cluster = std::min(2, std::max(0, std::atoi(c)));
    {
      int dev = 0;
      check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
      check_cuda(cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, dev), "SM count");
    }
    if (const char *c = std::getenv("NRG_AUTOTUNE")) e->autotune = std::atoi(c) != 0;
    *out = e;
  });
}

int nrg_engine_destroy(nrg_engine *e) {
  return guard([&] {
    if (!e) return;
    cudaStreamSynchronize(e->stream);
    release_uploads(e);
    for (auto ev : e->ring_events) cudaEventDestroy(ev);
    if (e->d_kerr) cudaFree(e->d_kerr);
    for (auto &ev : e->ev) cudaEventDestroy(ev);
    cudaStreamSynchronize(e->side);
    cudaEventDestroy(e->fork_ev);
    cudaEventDestroy(e->join_ev);
    cudaStreamDestroy(e->side);
    cudaStreamDestroy(e->stream);
    delete e;
  });
}

int nrg_engine_phase_times(nrg_engine *e, double *out, int cap, int *n) {
  return guard([&] {
    if (!e || !out) fail(NRG_E_ARG, "null argument");
    check_cuda(cudaEventSynchronize(e->ev[5]), "event sync");
    float ms[5] = {0, 0, 0, 0, 0};
    cudaEventElapsedTime(&ms[0], e->ev[0], e->ev[1]);
    cudaEventElapsedTime(&ms[1], e->ev[1], e->ev[2]);
    cudaEventElapsedTime(&ms[2], e->ev[2], e->ev[3]);
    cudaEventElapsedTime(&ms[3], e->ev[4], e->ev[5]);
    int m = std::min(cap, 4);
    for (int i = 0; i < m; ++i) out[i] = ms[i];
    if (n) *n = m;
  });
}

int nrg_engine_set_profiling(nrg_engine *e, int on) {
  return guard([&] {
    if (!e) fail(NRG_E_ARG, "null engine");
    e->profile = on != 0;
  });
}

int nrg_engine_kernel_times(nrg_engine *e, char *names, uint64_t names_cap, double *ms, double *work,
                            uint64_t *count, int cap, int *nk) {
  return guard([&] {
    if (!e || !names || !ms || !work || !count || !nk) fail(NRG_E_ARG, "null argument");
    check_cuda(cudaStreamSynchronize(e->stream), "profile sync");
    std::vector<std::string> order;
    std::map<std::string, std::tuple<double, double, uint64_t>> acc;
    for (auto &p : e->prof) {
      float t = 0;
      cudaEventElapsedTime(&t, p.a, p.b);
      if (!acc.count(p.name)) order.push_back(p.name);
      auto &a = acc[p.name];
      std::get<0>(a) += t;
      std::get<1>(a) += p.work;
      std::get<2>(a) += 1;
      e->ev_pool.push_back(p.a);
      e->ev_pool.push_back(p.b);
    }
    e->prof.clear();
    std::string joined;
    int k = 0;
    for (auto &nm : order) {
      if (k >= cap) break;
      auto &a = acc[nm];
      ms[k] = std::get<0>(a);
      work[k] = std::get<1>(a);
      count[k] = std::get<2>(a);
      joined += nm + "\n";
      ++k;
    }
    if (joined.size() + 1 > names_cap) fail(NRG_E_ARG, "names buffer too small");
    std::memcpy(names, joined.c_str(), joined.size() + 1);
    *nk = k;
  });
}

int nrg_engine_get_opts(nrg_engine *e, nrg_engine_opts *out) {
  return guard([&] {
    if (!e || !out) fail(NRG_E_ARG, "null argument");
    *out = nrg_engine_opts{};
    out->device = e->device;
    out->precision = e->precision;
    out->hbm_budget_bytes = e->budget;
    out->verbose = e->verbose;
  });
}

int nrg_engine_launch_count(nrg_engine *e, uint64_t *out) {
  return guard([&] {
    if (!e || !out) fail(NRG_E_ARG, "null argument");
    *out = e->launches;
  });
}

int nrg_engine_memory(nrg_engine *e, uint64_t *used, uint64_t *peak, int reset_peak) {
  return guard([&] {
    if (!e || !used || !peak) fail(NRG_E_ARG, "null argument");
    *used = e->used;
    *peak = e->peak;
    if (reset_peak) e->peak = e->used;
  });
}

int nrg_engine_fallback_count(nrg_engine *e, uint64_t *out) {
  return guard([&] {
    if (!e || !out) fail(NRG_E_ARG, "null argument");
    *out = e->fallback_blocks;
  });
}

int nrg_engine_work_counters(nrg_engine *e, double *out, int cap, int *n, int reset) {
  return guard([&] {
    if (!e || !out || !n || cap < 0) fail(NRG_E_ARG, "null argument");
    const int k = std::min(cap, 4);
    for (int i = 0; i < k; ++i) out[i] = e->work[i];
    *n = k;
    if (reset)
      for (double &w : e->work) w = 0.0;
  });
}

int nrg_engine_set_autotune(nrg_engine *e, int on) {
  return guard([&] {
    if (!e) fail(NRG_E_ARG, "null engine");
    e->autotune = on != 0;
  });
}

int nrg_engine_set_eig_cluster(nrg_engine *e, int mode) {
  return guard([&] {
    if (!e) fail(NRG_E_ARG, "null engine");
    if (mode < 0 || mode > 2) fail(NRG_E_ARG, "cluster mode must be 0, 1 or 2");
    e->eig_cluster = mode;
  });
}

int nrg_engine_autotune_report(nrg_engine *e, char *buf, uint64_t cap, uint64_t *len) {
  return guard([&] {
    if (!e || !len) fail(NRG_E_ARG, "null argument");
    std::string r;
    for (auto &kv : e->tuned) r += kv.second.what + "\n";
    *len = r.size();
    if (buf && cap) {
      const size_t k = std::min<size_t>(r.size(), size_t(cap - 1));
      std::memcpy(buf, r.data(), k);
      buf[k] = 0;
    }
  });
}

int nrg_engine_sync(nrg_engine *e) {
  return guard([&] {
    if (!e) fail(NRG_E_ARG, "null engine");
    check_cuda(cudaStreamSynchronize(e->stream), "sync");
    check_kernel_error(e);
  });
}

int nrg_run_create(nrg_engine *e, const nrg_site_desc *imp, const nrg_site_desc *bath, uint64_t nkeep,
                   nrg_run **out) {
  return guard([&] {
    if (!e || !out) fail(NRG_E_ARG, "null argument");
    auto r = std::make_unique<nrg_run>();
    r->eng = e;
    r->imp = engine_parse_site(imp, false);
    r->bath = engine_parse_site(bath, true);
    if (r->imp.q[0].size() != r->bath.q[0].size())  // nrgcore.hpp:119-122
      fail(NRG_E_ARG, "Number of quantum number is different on model and impurity!");
    if (r->imp.nops != r->bath.nops)  // nrgcore.hpp:124-133
      fail(NRG_E_ARG, "f_dag_operator.size is different on model and impurity!");
    engine_upload_bath(e, r->bath);
    r->nkeep = nkeep;
    r->no_of_kept = int64_t(nkeep);
    *out = r.release();
  });
}

int nrg_run_destroy(nrg_run *r) {
  return guard([&] {
    if (!r) return;
    nrg_engine *e = r->eng;
    delete r;
    cudaStreamSynchronize(e->stream);
  });
}

int nrg_run_set_parameters(nrg_run *r, uint64_t nkeep) {
  return guard([&] {
    if (!r) fail(NRG_E_ARG, "null run");
    r->nkeep = nkeep;
    r->no_of_kept = int64_t(nkeep);
    r->cnt = 0;
    r->cnt_min = 0;
    r->have_site = false;
  });
}

int nrg_run_set_bath(nrg_run *r, const nrg_site_desc *bath) {
  return guard([&] {
    if (!r) fail(NRG_E_ARG, "null run");
    r->bath_next = engine_parse_site(bath, true);
    if (r->bath_next.nops != r->imp.nops) fail(NRG_E_ARG, "bath operator count changed");
    r->bath_pending = true;
  });
}

int nrg_run_add_site(nrg_run *r, const double *t, int nt, double rescale) {
  return guard([&] {
    if (!r || (!t && nt > 0)) fail(NRG_E_ARG, "null argument");
    nrg_run *rs[1] = {r};
    engine_batch_add_site(rs, 1, t, nt, &rescale);
  });
}

int nrg_run_update_state(nrg_run *r) {
  return guard([&] {
    if (!r) fail(NRG_E_ARG, "null run");
    engine_update_state(r);
  });
}

int nrg_batch_add_site(nrg_run *const *runs, int nruns, const double *t, int nt, const double *rescale) {
  return guard([&] {
    if (!runs || nruns < 0 || !rescale || (!t && nt > 0)) fail(NRG_E_ARG, "null argument");
    engine_batch_add_site(runs, nruns, t, nt, rescale);
  });
}

int nrg_batch_update_state(nrg_run *const *runs, int nruns) {
  return guard([&] {
    if (!runs || nruns < 0) fail(NRG_E_ARG, "null argument");
    for (int i = 0; i < nruns; ++i) engine_update_state(runs[i]);
  });
}

int nrg_run_check_discarded(nrg_run *r, int *out) {
  return guard([&] {
    if (!r || !out) fail(NRG_E_ARG, "null argument");
    *out = r->no_of_kept >= int64_t(r->nkeep) ? 1 : 0;  // nrgcore.hpp:384-386
  });
}

int nrg_run_get_info(nrg_run *r, nrg_run_info *info) {
  return guard([&] {
    if (!r || !info) fail(NRG_E_ARG, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->iteration = r->cnt;
    info->iteration_min = r->cnt_min;
    info->n_pre_sectors = int64_t(r->pre_q.size());
    info->n_cur_sectors = r->have_site && r->site ? int64_t(r->site->cur_q.size()) : 0;
    info->n_all = int64_t(r->all_eig.size());
    info->n_kept = r->no_of_kept;
    info->n_relgs = int64_t(r->relgs.size());
    info->nq = r->imp.nq;
    if (r->site) {
      info->n_device_blocks = int64_t(r->site->blocks.size());
      for (auto &b : r->site->blocks) info->max_block = std::max<int64_t>(info->max_block, b.n);
    }
    info->n_snapshots = int64_t(r->snaps.size());
    // device bytes this run holds: its current and previous site, f-dagger
    // blocks and every snapshot (buffers shared between them counted once)
    std::set<const DevMem *> seen;
    int64_t bytes = 0;
    auto add = [&](const DevPtr &m) {
      if (m && m->ptr && seen.insert(m.get()).second) bytes += int64_t(m->bytes);
    };
    auto add_site = [&](const std::shared_ptr<SiteData> &sd) {
      if (!sd) return;
      add(sd->mem_U);
      add(sd->mem_E);
      add(sd->mem_Uplanes);
      add(sd->mem_Uexps);
    };
    add_site(r->site);
    add_site(r->prev_site);
    add(r->mem_H);
    add(r->mem_sorted);
    add(r->fprev_mem);
    add(r->fcur_mem);
    for (auto &kv : r->snaps) {
      add_site(kv.second->site);
      add(kv.second->ops_mem);
    }
    info->device_bytes = bytes;
  });
}

int nrg_run_get_all_eigenvalues(nrg_run *r, double *out, uint64_t cap) {
  return guard([&] {
    if (!r || (!out && cap)) fail(NRG_E_ARG, "null argument");
    if (cap < r->all_eig.size()) fail(NRG_E_ARG, "buffer too small");
    std::copy(r->all_eig.begin(), r->all_eig.end(), out);
  });
}

int nrg_run_get_relgs(nrg_run *r, double *out, uint64_t cap) {
  return guard([&] {
    if (!r || (!out && cap)) fail(NRG_E_ARG, "null argument");
    if (cap < r->relgs.size()) fail(NRG_E_ARG, "buffer too small");
    std::copy(r->relgs.begin(), r->relgs.end(), out);
  });
}

int nrg_run_get_sectors(nrg_run *r, int which, int *qnum, uint64_t cap) {
  return guard([&] {
    if (!r || !qnum) fail(NRG_E_ARG, "null argument");
    const auto *q = which == 0 ? (r->have_site ? &r->site->cur_q : nullptr) : &r->pre_q;
    if (!q) return;
    if (cap < q->size()) fail(NRG_E_ARG, "buffer too small");
    int64_t o = 0;
    for (auto &v : *q)
      for (int x : v) qnum[o++] = x;
  });
}

int nrg_run_get_eigenvalues_q(nrg_run *r, uint64_t *dims, double *values, uint64_t cap) {
  return guard([&] {
    if (!r || !dims) fail(NRG_E_ARG, "null argument");
    // between add_site and update_state: the new, unshifted eigenvalues;
    // afterwards the shifted ones (nrgcore.hpp:317-326)
    const auto &E = r->have_site ? r->site->E_host : r->prevE_host;
    uint64_t o = 0;
    for (size_t s = 0; s < E.size(); ++s) {
      dims[s] = E[s].size();
      if (values) {
        if (o + E[s].size() > cap) fail(NRG_E_ARG, "buffer too small");
        std::copy(E[s].begin(), E[s].end(), values + o);
      }
      o += E[s].size();
    }
  });
}

int nrg_run_get_kept(nrg_run *r, uint64_t *kept, uint64_t cap) {
  return guard([&] {
    if (!r || !kept) fail(NRG_E_ARG, "null argument");
    if (cap < r->kept.size()) fail(NRG_E_ARG, "buffer too small");
    for (size_t i = 0; i < r->kept.size(); ++i) kept[i] = uint64_t(r->kept[i]);
  });
}

int nrg_run_get_coupled(nrg_run *r, uint64_t *counts, uint64_t *entries, uint64_t cap) {
  return guard([&] {
    if (!r || !counts) fail(NRG_E_ARG, "null argument");
    if (!r->site) fail(NRG_E_STATE, "no site yet");
    uint64_t o = 0;
    for (size_t s = 0; s < r->site->coupled.size(); ++s) {
      counts[s] = r->site->coupled[s].size();
      for (uint64_t x : r->site->coupled[s]) {
        if (entries) {
          if (o >= cap) fail(NRG_E_ARG, "buffer too small");
          entries[o] = x;
        }
        ++o;
      }
    }
  });
}

int nrg_run_get_eigenvectors(nrg_run *r, int64_t sector, double *out, uint64_t cap) {
  return guard([&] {
    if (!r || !out) fail(NRG_E_ARG, "null argument");
    if (!r->site || sector < 0 || sector >= int64_t(r->site->sectors.size()))
      fail(NRG_E_ARG, "sector out of range");
    const Sector &S = r->site->sectors[sector];
    if (S.dev < 0) return;
    const DevBlock &b = r->site->blocks[S.dev];
    if (cap < uint64_t(b.n) * b.n) fail(NRG_E_ARG, "buffer too small");
    check_cuda(cudaMemcpy2DAsync(out, b.n * sizeof(double), b.U, b.ld * sizeof(double),
                                 b.n * sizeof(double), b.n, cudaMemcpyDeviceToHost, r->eng->stream),
               "eigenvectors D2H");
    check_cuda(cudaStreamSynchronize(r->eng->stream), "eigenvectors D2H");
  });
}

static void copy_block(nrg_engine *e, const FBlock &b, double *out, uint64_t cap) {
  if (cap < uint64_t(b.rows) * b.cols) fail(NRG_E_ARG, "buffer too small");
  if (b.rows && b.cols)
    check_cuda(cudaMemcpy2DAsync(out, b.cols * sizeof(double), b.p, b.ld * sizeof(double),
                                 b.cols * sizeof(double), b.rows, cudaMemcpyDeviceToHost, e->stream),
               "block D2H");
  check_cuda(cudaStreamSynchronize(e->stream), "block D2H");
}

int nrg_run_get_fdag_block(nrg_run *r, int ip, int64_t i, int64_t j, double *out, uint64_t cap,
                           int64_t *rows, int64_t *cols) {
  return guard([&] {
    if (!r || !rows || !cols) fail(NRG_E_ARG, "null argument");
    const auto &m = r->have_site ? r->fcur : r->fprev;
    auto it = m.find(OpKey{ip, int(i), int(j)});
    *rows = *cols = 0;
    if (it == m.end()) return;
    *rows = it->second.rows;
    *cols = it->second.cols;
    if (out) copy_block(r->eng, it->second, out, cap);
  });
}

int nrg_opset_create(nrg_run *r, const nrg_op_desc *ops, nrg_opset **out) {
  return guard([&] {
    if (!r || !ops || !out) fail(NRG_E_ARG, "null argument");
    auto o = std::make_unique<nrg_opset>();
    o->run = r;
    o->nops = ops->nops;
    int64_t tot = 0;
    for (int b = 0; b < ops->nblk; ++b) tot += int64_t(ops->blk_rows[b]) * ops->blk_cols[b];
    o->mem = engine_alloc(r->eng, tot * sizeof(double) + 8);
    check_cuda(cudaMemcpyAsync(o->mem->ptr, ops->blk_data, tot * sizeof(double), cudaMemcpyHostToDevice,
                               r->eng->stream),
               "opset upload");
    int64_t off = 0;
    for (int b = 0; b < ops->nblk; ++b) {
      FBlock fb{static_cast<double *>(o->mem->ptr) + off, ops->blk_rows[b], ops->blk_cols[b],
                ops->blk_cols[b]};
      off += int64_t(fb.rows) * fb.cols;
      OpKey key{ops->blk_op[b], ops->blk_row[b], ops->blk_col[b]};
      if (o->blocks.count(key)) fail(NRG_E_ARG, "Found operator already");
      o->blocks[key] = fb;
    }
    check_cuda(cudaStreamSynchronize(r->eng->stream), "opset upload");
    *out = o.release();
  });
}

int nrg_opset_destroy(nrg_opset *o) {
  return guard([&] { delete o; });
}

int nrg_opset_update(nrg_opset *o) {
  return guard([&] {
    if (!o) fail(NRG_E_ARG, "null opset");
    opset_update(o);
  });
}

int nrg_opset_update_batch(nrg_opset *const *os, int n) {
  return guard([&] {
    if (n < 0 || (n > 0 && !os)) fail(NRG_E_ARG, "bad argument");
    std::vector<nrg_opset *> v(os, os + n);
    for (size_t a = 0; a < v.size(); ++a) {
      if (!v[a]) fail(NRG_E_ARG, "null operator set");
      for (size_t b = 0; b < a; ++b)
        if (v[b] == v[a]) fail(NRG_E_ARG, "an operator set appears twice in one batch");
    }
    opset_update_batch(v);
  });
}

int nrg_opset_get_block(nrg_opset *o, int ip, int64_t i, int64_t j, double *out, uint64_t cap,
                        int64_t *rows, int64_t *cols) {
  return guard([&] {
    if (!o || !rows || !cols) fail(NRG_E_ARG, "null argument");
    auto it = o->blocks.find(OpKey{ip, int(i), int(j)});
    *rows = *cols = 0;
    if (it == o->blocks.end()) return;
    *rows = it->second.rows;
    *cols = it->second.cols;
    if (out) copy_block(o->run->eng, it->second, out, cap);
  });
}

}  // extern "C"

namespace {
// Enumerates a block map: n = blocks; the first min(n, cap) of each array
// written (any array may be null).
void list_blocks(const std::map<OpKey, FBlock> &m, int *ip, int64_t *i, int64_t *j, int64_t *rows,
                 int64_t *cols, uint64_t cap, uint64_t *n) {
  if (!n) fail(NRG_E_ARG, "null argument");
  uint64_t k = 0;
  for (auto &kv : m) {
    if (k < cap) {
      if (ip) ip[k] = std::get<0>(kv.first);
      if (i) i[k] = std::get<1>(kv.first);
      if (j) j[k] = std::get<2>(kv.first);
      if (rows) rows[k] = kv.second.rows;
      if (cols) cols[k] = kv.second.cols;
    }
    ++k;
  }
  *n = k;
}
}  // namespace

extern "C" {

int nrg_opset_list_blocks(nrg_opset *o, int *ip, int64_t *i, int64_t *j, int64_t *rows, int64_t *cols,
                          uint64_t cap, uint64_t *n) {
  return guard([&] {
    if (!o) fail(NRG_E_ARG, "null opset");
    list_blocks(o->blocks, ip, i, j, rows, cols, cap, n);
  });
}

int nrg_run_list_fdag_blocks(nrg_run *r, int *ip, int64_t *i, int64_t *j, int64_t *rows, int64_t *cols,
                             uint64_t cap, uint64_t *n) {
  return guard([&] {
    if (!r) fail(NRG_E_ARG, "null run");
    list_blocks(r->have_site ? r->fcur : r->fprev, ip, i, j, rows, cols, cap, n);
  });
}

int nrg_run_list_snapshot_ops(nrg_run *r, int *ip, int64_t *i, int64_t *j, int64_t *rows, int64_t *cols,
                              uint64_t cap, uint64_t *n) {
  return guard([&] {
    if (!r) fail(NRG_E_ARG, "null run");
    if (!r->loaded) fail(NRG_E_STATE, "no snapshot loaded");
    list_blocks(r->loaded->ops, ip, i, j, rows, cols, cap, n);
  });
}

int nrg_run_get_snapshot_op_block(nrg_run *r, int ip, int64_t i, int64_t j, double *out, uint64_t cap) {
  return guard([&] {
    if (!r || !out) fail(NRG_E_ARG, "null argument");
    if (!r->loaded) fail(NRG_E_STATE, "no snapshot loaded");
    auto it = r->loaded->ops.find(OpKey{ip, int(i), int(j)});
    if (it == r->loaded->ops.end()) fail(NRG_E_ARG, "no such block in the loaded snapshot");
    copy_block(r->eng, it->second, out, cap);
  });
}

int nrg_run_snapshot(nrg_run *r, nrg_opset *ops) {
  return guard([&] {
    if (!r) fail(NRG_E_ARG, "null run");
    if (!r->have_site) fail(NRG_E_STATE, "snapshot needs add_site first");
    auto s = std::make_shared<Snapshot>();
    s->site = r->site;
    if (ops) {
      s->ops = ops->blocks;
      s->nops = ops->nops;
      s->ops_mem = ops->mem;
    }
    r->snaps[r->cnt] = s;
  });
}

int nrg_run_load_snapshot(nrg_run *r, int64_t iteration) {
  return guard([&] {
    if (!r) fail(NRG_E_ARG, "null run");
    auto it = r->snaps.find(iteration);
    if (it == r->snaps.end()) fail(NRG_E_ARG, "no snapshot for iteration " + std::to_string(iteration));
    r->loaded = it->second;
    r->cnt = iteration;  // loadCurrentData sets nrg_iterations_cnt (nrgData.hpp:273)
  });
}

}  // extern "C"

namespace {
// One named array of the export container: u32 name length, the name, u64
// element count, the elements as little-endian float64.
void put_array(FILE *fp, const std::string &name, const double *v, uint64_t n) {
  const uint32_t len = uint32_t(name.size());
  bool ok = std::fwrite(&len, 4, 1, fp) == 1 && std::fwrite(name.data(), 1, len, fp) == len &&
            std::fwrite(&n, 8, 1, fp) == 1 && (n == 0 || std::fwrite(v, 8, n, fp) == n);
  if (!ok) fail(NRG_E_ARG, "export: write failed");
}
void put_array(FILE *fp, const std::string &name, const std::vector<double> &v) {
  put_array(fp, name, v.data(), v.size());
}
template <class T> std::vector<double> as_doubles(const std::vector<T> &v) {
  return std::vector<double>(v.begin(), v.end());
}
}  // namespace

extern "C" {

int nrg_run_export_snapshots(nrg_run *r, const char *path, int with_vectors) {
  return guard([&] {
    if (!r || !path) fail(NRG_E_ARG, "null argument");
    nrg_engine *e = r->eng;
    FILE *fp = std::fopen(path, "wb");
    if (!fp) fail(NRG_E_ARG, std::string("export: cannot open ") + path);
    std::unique_ptr<FILE, int (*)(FILE *)> guard_fp(fp, std::fclose);
    const uint32_t magic = 0x4152474eu;  // "NGRA"
    const uint32_t version = 1;
    if (std::fwrite(&magic, 4, 1, fp) != 1 || std::fwrite(&version, 4, 1, fp) != 1)
      fail(NRG_E_ARG, "export: write failed");
    std::vector<double> saved;
    for (auto &kv : r->snaps) {
      const int64_t it = kv.first;
      const Snapshot &S = *kv.second;
      const SiteData &sd = *S.site;
      saved.push_back(double(it));
      const std::string g = "/NrgItr" + std::to_string(it) + "/";
      const size_t nq = sd.cur_q.empty() ? 0 : sd.cur_q[0].size();
      std::vector<double> q;
      for (auto &v : sd.cur_q) q.insert(q.end(), v.begin(), v.end());
      put_array(fp, g + "current_sysmQ", q);
      q.clear();
      for (auto &v : sd.pre_q) q.insert(q.end(), v.begin(), v.end());
      put_array(fp, g + "pre_sysmQ", q);
      put_array(fp, g + "nq", std::vector<double>{double(nq)});
      put_array(fp, g + "eigenvaluesQ_kept_indices", as_doubles(sd.kept_prev));
      for (size_t sidx = 0; sidx < sd.cur_q.size(); ++sidx) {
        const std::string k = std::to_string(sidx);
        put_array(fp, g + "eigenvaluesQ/" + k, sidx < sd.E_host.size() ? sd.E_host[sidx] : std::vector<double>{});
        put_array(fp, g + "coupled_nQ_index/" + k, as_doubles(sd.coupled[sidx]));
        if (with_vectors) {  // current_hamiltonQ: eigenvectors as columns, row-major n x n
          const Sector &Sc = sd.sectors[sidx];
          std::vector<double> u;
          if (Sc.dev >= 0) {
            const DevBlock &db = sd.blocks[Sc.dev];
            u.resize(size_t(db.n) * db.n);
            check_cuda(cudaMemcpy2DAsync(u.data(), db.n * sizeof(double), db.U, db.ld * sizeof(double),
                                         db.n * sizeof(double), db.n, cudaMemcpyDeviceToHost, e->stream),
                       "export eigenvectors");
            check_cuda(cudaStreamSynchronize(e->stream), "export eigenvectors");
          }
          put_array(fp, g + "current_hamiltonQ/" + k, u);
        }
      }
      // the operator set saved with the shell (NrgData::saveqOperator layout:
      // per operator the (row, col) block ids, their shapes and the blocks)
      put_array(fp, g + "op/operatorSize", std::vector<double>{double(S.nops)});
      for (int ip = 0; ip < S.nops; ++ip) {
        const std::string og = g + "op/at" + std::to_string(ip) + "/";
        std::vector<double> ids, rows, cols;
        int ic = 0;
        for (auto &b : S.ops) {
          if (std::get<0>(b.first) != ip) continue;
          const FBlock &B = b.second;
          ids.push_back(std::get<1>(b.first));
          ids.push_back(std::get<2>(b.first));
          rows.push_back(B.rows);
          cols.push_back(B.cols);
          std::vector<double> m(size_t(B.rows) * B.cols);
          if (!m.empty()) {
            check_cuda(cudaMemcpy2DAsync(m.data(), B.cols * sizeof(double), B.p, B.ld * sizeof(double),
                                         B.cols * sizeof(double), B.rows, cudaMemcpyDeviceToHost, e->stream),
                       "export operator");
            check_cuda(cudaStreamSynchronize(e->stream), "export operator");
          }
          put_array(fp, og + "qmat" + std::to_string(ic++), m);
        }
        put_array(fp, og + "idVector", ids);
        put_array(fp, og + "rowVector", rows);
        put_array(fp, og + "colVector", cols);
      }
    }
    put_array(fp, "savedNRGIndex", saved);  // NrgData::saveFinalState (nrgData.hpp:106-110)
    put_array(fp, "relativeGroundStateEnergy", r->relgs);
    if (std::fflush(fp) != 0) fail(NRG_E_ARG, "export: write failed");
  });
}

int nrg_fdm_create(nrg_run *r, int nops, nrg_fdm **out) {
  return guard([&] {
    if (!r || !out || nops <= 0) fail(NRG_E_ARG, "bad argument");
    auto f = std::make_unique<nrg_fdm>();
    f->run = r;
    f->nops = nops;
    f->hist = engine_alloc(r->eng, 2 * int64_t(nops) * kFdmPts * sizeof(double));
    check_cuda(cudaMemsetAsync(f->hist->ptr, 0, 2 * int64_t(nops) * kFdmPts * sizeof(double), r->eng->stream),
               "fdm hist");
    *out = f.release();
  });
}

int nrg_fdm_destroy(nrg_fdm *f) {
  return guard([&] { delete f; });
}

int nrg_fdm_calc(nrg_fdm *f, double scale) {
  return guard([&] {
    if (!f) fail(NRG_E_ARG, "null fdm");
    fdm_calc_batch({f}, {scale});
  });
}

int nrg_fdm_calc_batch(nrg_fdm *const *fs, int n, const double *scales) {
  return guard([&] {
    if (n < 0 || (n > 0 && (!fs || !scales))) fail(NRG_E_ARG, "bad argument");
    std::vector<nrg_fdm *> v(fs, fs + n);
    for (auto *f : v)
      if (!f) fail(NRG_E_ARG, "null fdm");
    fdm_calc_batch(v, std::vector<double>(scales, scales + n));
  });
}

int nrg_fdm_get(nrg_fdm *f, double *energy_points, double *positive, double *negative, uint64_t npts) {
  return guard([&] {
    if (!f) fail(NRG_E_ARG, "null fdm");
    if (npts != uint64_t(kFdmPts)) fail(NRG_E_ARG, "npts must be 100000");
    const double de = fdm_delE();
    if (energy_points)
      for (int i = 0; i < kFdmPts; ++i) energy_points[i] = kFdmMin * std::exp(i * 1. / de);
    nrg_engine *e = f->run->eng;
    const double *h = static_cast<const double *>(f->hist->ptr);
    if (positive)
      check_cuda(cudaMemcpyAsync(positive, h, int64_t(f->nops) * kFdmPts * sizeof(double),
                                 cudaMemcpyDeviceToHost, e->stream), "fdm D2H");
    if (negative)
      check_cuda(cudaMemcpyAsync(negative, h + int64_t(f->nops) * kFdmPts,
                                 int64_t(f->nops) * kFdmPts * sizeof(double), cudaMemcpyDeviceToHost,
                                 e->stream), "fdm D2H");
    check_cuda(cudaStreamSynchronize(e->stream), "fdm D2H");
  });
}

int nrg_broaden(nrg_engine *e, const double *energies, const double *weights, uint64_t nbins,
                const double *omegas, uint64_t nomega, double b, double *out) {
  return guard([&] {
    if (!e || !energies || !weights || !omegas || !out) fail(NRG_E_ARG, "null argument");
    std::vector<double> ee, ww;
    for (uint64_t i = 0; i < nbins; ++i)
      if (weights[i] != 0.0) {
        ee.push_back(std::log(energies[i]));  // the kernel takes ln(e_i)
        ww.push_back(weights[i]);
      }
    std::vector<double> om(omegas, omegas + nomega);
    Staged st;
    size_t oe = st.add(ee), ow = st.add(ww), oo = st.add(om);
    std::vector<double> res(nomega, 0.0);
    size_t orr = st.add(res);
    DevPtr hold;
    char *d = st.push(e, hold);
    launch_broaden(at<double>(d, oe), at<double>(d, ow), int64_t(ee.size()), at<double>(d, oo),
                   int64_t(nomega), b, at<double>(d, orr), e->stream);
    engine_count_launch(e, 1);
    check_cuda(cudaGetLastError(), "broaden");
    check_cuda(cudaMemcpyAsync(out, d + orr, nomega * sizeof(double), cudaMemcpyDeviceToHost, e->stream),
               "broaden D2H");
    check_cuda(cudaStreamSynchronize(e->stream), "broaden");
  });
}

int nrg_thermo_create(nrg_run *r, const double *temps, int nt, nrg_thermo **out) {
  return guard([&] {
    if (!r || !out || (!temps && nt > 0)) fail(NRG_E_ARG, "null argument");
    auto t = std::make_unique<nrg_thermo>();
    t->run = r;
    t->nmax = r->cnt;  // nrgMaxIterations (fdmThermodynamics.hpp:30)
    for (auto &v : r->bath.E) t->bathdim += double(v.size());
    t->temps.assign(temps, temps + nt);
    *out = t.release();
  });
}

int nrg_thermo_destroy(nrg_thermo *t) {
  return guard([&] { delete t; });
}

int nrg_thermo_calc(nrg_thermo *t, double scale) {
  return guard([&] {
    if (!t) fail(NRG_E_ARG, "null thermo");
    nrg_run *r = t->run;
    if (!r->loaded) fail(NRG_E_STATE, "calcThermodynamics needs a loaded snapshot");
    SiteData &sd = *r->loaded->site;
    const int nsec = int(sd.cur_q.size());
    if (!t->have_cur) {
      t->cur_kept.assign(nsec, 0);
      t->have_cur = true;
    } else {
      t->cur_kept = t->prev_kept;
    }
    t->prev_kept = sd.kept_prev;
    std::vector<double> disc, all;
    for (int i = 0; i < nsec; ++i)  // discarded states only (:47-52)
      for (size_t j = size_t(t->cur_kept[i]); j < sd.E_host[i].size(); ++j)
        disc.push_back(sd.E_host[i][j] * scale);
    for (int i = 0; i < nsec; ++i)
      for (double x : sd.E_host[i]) all.push_back(x * scale);
    if (!t->sysops.empty()) {  // diagonals of the system operators on the discarded states (:63-88)
      std::vector<double> q(t->sysops.size() * disc.size(), 0.0);
      nrg_engine *e = r->eng;
      for (size_t iq = 0; iq < t->sysops.size(); ++iq) {
        size_t o = 0;
        for (int i = 0; i < nsec; ++i) {
          const size_t n = sd.E_host[i].size(), kc = size_t(t->cur_kept[i]);
          const size_t nd = n > kc ? n - kc : 0;
          auto it = r->loaded->ops.find(OpKey{t->sysops[iq], i, i});
          if (nd && it != r->loaded->ops.end()) {
            const FBlock &B = it->second;
            if (B.rows != int(n) || B.cols != int(n)) fail(NRG_E_STATE, "system operator block size");
            check_cuda(cudaMemcpy2DAsync(q.data() + iq * disc.size() + o, sizeof(double),
                                         B.p + int64_t(kc) * (B.ld + 1), size_t(B.ld + 1) * sizeof(double),
                                         sizeof(double), nd, cudaMemcpyDeviceToHost, e->stream),
                       "system operator diagonal");
          }
          o += nd;
        }
      }
      check_cuda(cudaStreamSynchronize(e->stream), "system operator diagonal");
      t->qval.push_back(std::move(q));
    }
    t->disc.push_back(std::move(disc));
    t->allv.push_back(std::move(all));
  });
}

}  // extern "C"

namespace {
// Discarded energies relative to each shell's minimum (flattened, with
// offsets) and the one-step corrected shell ground energies
// (fdmThermodynamics::saveFinalData, fdmThermodynamics.hpp:114-140).
void thermo_shells(const nrg_thermo *t, std::vector<double> &flat, std::vector<int64_t> &off,
                   std::vector<double> &gs) {
  const int nsh = int(t->allv.size());
  gs.assign(nsh, 0.0);
  off.assign(nsh + 1, 0);
  flat.clear();
  for (int it = 0; it < nsh; ++it) {  // :114-131
    const double m = *std::min_element(t->allv[it].begin(), t->allv[it].end());
    gs[it] = m;
    off[it] = int64_t(flat.size());
    for (double x : t->disc[it]) flat.push_back(x - m);
  }
  off[nsh] = int64_t(flat.size());
  for (int it = 0; it + 1 < nsh; ++it) gs[it] += gs[it + 1];  // one-step correction :133-135
  const double g0 = gs.empty() ? 0.0 : gs[0];
  for (auto &x : gs) x -= g0;
}

double regulate_exp_host(double x) {  // fdmThermodynamics.hpp:240-249
  return std::exp(std::min(100.0, std::max(-100.0, x)));
}
}  // namespace

extern "C" {

int nrg_thermo_final(nrg_thermo *t, double *entropy, double *cv) {
  return guard([&] {
    if (!t || !entropy || !cv) fail(NRG_E_ARG, "null argument");
    nrg_engine *e = t->run->eng;
    const int nsh = int(t->allv.size());
    if (nsh == 0) fail(NRG_E_STATE, "no shells");
    std::vector<double> gs, flat;
    std::vector<int64_t> off;
    thermo_shells(t, flat, off, gs);
    const int nt = int(t->temps.size());
    const int nq = int(t->sysops.size());
    const int64_t ndisc = int64_t(flat.size());
    std::vector<double> qv(size_t(nq) * ndisc, 0.0);  // operator diagonals in the layout of flat
    for (int it = 0; it < nsh && nq; ++it) {
      const int64_t nd = off[it + 1] - off[it];
      for (int iq = 0; iq < nq; ++iq)
        std::copy(t->qval[it].begin() + iq * nd, t->qval[it].begin() + (iq + 1) * nd,
                  qv.begin() + int64_t(iq) * ndisc + off[it]);
    }
    Staged st;
    size_t of = st.add(flat), oo = st.add(off), og = st.add(gs), ot = st.add(t->temps), oq = st.add(qv);
    std::vector<double> scratch(size_t(3 + nq) * nsh * nt + size_t(2 + nq) * nt, 0.0);
    size_t os = st.add(scratch);
    DevPtr hold;
    char *d = st.push(e, hold);
    double *ent = at<double>(d, os) + size_t(3 + nq) * nsh * nt;
    launch_thermo(at<double>(d, of), at<int64_t>(d, oo), at<double>(d, og), nsh, at<double>(d, ot), nt,
                  t->bathdim, at<double>(d, oq), nq, ndisc, at<double>(d, os), ent, ent + nt, ent + 2 * nt,
                  e->stream);
    engine_count_launch(e, 1);
    check_cuda(cudaGetLastError(), "thermo");
    check_cuda(cudaMemcpyAsync(entropy, ent, nt * sizeof(double), cudaMemcpyDeviceToHost, e->stream), "D2H");
    check_cuda(cudaMemcpyAsync(cv, ent + nt, nt * sizeof(double), cudaMemcpyDeviceToHost, e->stream), "D2H");
    t->opexp.assign(size_t(nq) * nt, 0.0);
    if (nq)
      check_cuda(cudaMemcpyAsync(t->opexp.data(), ent + 2 * nt, size_t(nq) * nt * sizeof(double),
                                 cudaMemcpyDeviceToHost, e->stream), "D2H");
    check_cuda(cudaStreamSynchronize(e->stream), "thermo");
  });
}

int nrg_thermo_set_operator(nrg_thermo *t, const int *op_index, int n) {
  return guard([&] {
    if (!t || n < 0 || (n > 0 && !op_index)) fail(NRG_E_ARG, "bad argument");
    if (n > kThermoMaxOps) fail(NRG_E_ARG, "at most " + std::to_string(kThermoMaxOps) + " system operators");
    if (!t->allv.empty()) fail(NRG_E_STATE, "setSystemOperator must come before the first calcThermodynamics");
    for (int i = 0; i < n; ++i)
      if (op_index[i] < 0) fail(NRG_E_ARG, "negative operator index");
    t->sysops.assign(op_index, op_index + n);
  });
}

int nrg_thermo_get_operator(nrg_thermo *t, double *out, int n, int nt) {
  return guard([&] {
    if (!t || (!out && n * nt > 0)) fail(NRG_E_ARG, "bad argument");
    if (n != int(t->sysops.size()) || nt != int(t->temps.size()))
      fail(NRG_E_ARG, "operator / temperature count differs from the thermodynamics object");
    if (t->opexp.size() != size_t(n) * nt) fail(NRG_E_STATE, "nrg_thermo_final has not run");
    std::copy(t->opexp.begin(), t->opexp.end(), out);
  });
}

int nrg_fdm_set_temperature(nrg_fdm *f, double T, nrg_thermo *t) {
  return guard([&] {
    if (!f || !t) fail(NRG_E_ARG, "null argument");
    if (!(T > 0.0)) fail(NRG_E_ARG, "temperature must be > 0");
    if (!f->last || f->ncalc) fail(NRG_E_STATE, "setTemperature must come before the first calcSpectrum");
    if (t->run != f->run) fail(NRG_E_ARG, "the thermodynamics object belongs to another run");
    const int nsh = int(t->allv.size());
    if (nsh == 0) fail(NRG_E_STATE, "the thermodynamics object has seen no shells");
    std::vector<double> gs, flat;
    std::vector<int64_t> off;
    thermo_shells(t, flat, off, gs);
    // w_m (:159-175) and the per-state probabilities exp((E0_m - E)/T) / Z'_m (:183-218)
    std::vector<double> z(nsh, 0.0);
    double lpart = 0.0;
    for (int i = 0; i < nsh; ++i) {
      for (int64_t a = off[i]; a < off[i + 1]; ++a) z[i] += regulate_exp_host((gs[i] - flat[a]) / T);
      lpart += z[i] * std::pow(t->bathdim, double(i));
    }
    f->shell_weights.assign(nsh, {});
    for (int i = 0; i < nsh; ++i) {
      const double wm = z[i] * std::pow(t->bathdim, double(i)) / lpart;
      for (int64_t a = off[i]; a < off[i + 1]; ++a)
        f->shell_weights[i].push_back(z[i] > 0 ? wm * regulate_exp_host((gs[i] - flat[a]) / T) / z[i] : 0.0);
    }
    f->finite_t = true;
    f->temperature = T;
  });
}

int nrg_fdm_get_static(nrg_fdm *f, double *out, int nops) {
  return guard([&] {
    if (!f || (!out && nops > 0)) fail(NRG_E_ARG, "bad argument");
    if (nops != f->nops) fail(NRG_E_ARG, "operator count differs from the FDM object");
    std::fill(out, out + nops, 0.0);
    if (!f->static_acc) return;
    nrg_engine *e = f->run->eng;
    check_cuda(cudaMemcpyAsync(out, f->static_acc->ptr, nops * sizeof(double), cudaMemcpyDeviceToHost, e->stream),
               "static D2H");
    check_cuda(cudaStreamSynchronize(e->stream), "static D2H");
  });
}

}  // extern "C"
