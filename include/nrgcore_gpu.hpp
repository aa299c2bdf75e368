/*
 * nrgcore_gpu.hpp - C++ drop-in for the reference's nrgcore<Imp, Bath> and its
 * companion classes, on top of the C ABI in nrg_gpu.h (header-only, C++17).
 *
 * A driver written against the reference (examples/ * /main.cpp) keeps its
 * model builders, its loops and its calls; it includes this header instead of
 * nrgcore/nrgcore.hpp, nrgcore/sysOperator.hpp, nrgcore/nrgData.hpp,
 * dynamics/fdmSpectrum.hpp and static/fdmThermodynamics.hpp, and adds
 * `using namespace nrg_gpu;` (or names the classes with the prefix):
 *
 *   reference (nrgcore/include/...)                  here
 *   nrgcore<Imp, Bath>            nrgcore.hpp:25-550   nrg_gpu::nrgcore<Imp, Bath>
 *   update_system_operator        sysOperator.hpp:36   nrg_gpu::update_system_operator
 *   NrgData<N>                    nrgData.hpp:31       nrg_gpu::NrgData<N>
 *   fdmSpectrum<N>                fdmSpectrum.hpp:35   nrg_gpu::fdmSpectrum<N>
 *   fdmThermodynamics<N>          fdmThermodynamics.hpp:26  nrg_gpu::fdmThermodynamics<N>
 *
 * Models are read through the reference's model concept (nrgcore.hpp:44-53,
 * 68-70): get_basis() -> vector<vector<int>>, get_eigenvaluesQ() ->
 * vector<vector<double>>, get_chi_Q() -> vector<double>, and a public
 * f_dag_operator: a vector of block operators whose getMap() returns a
 * pointer to a map from {row sector, column sector} (key[0], key[1]) to a
 * row-major matrix with getrow(), getcolumn() and data() (qOperator /
 * qmatrix, qOperator.hpp:18-46).  Operator vectors handed back to the caller
 * (update_system_operator, getPreWilsonSiteOperators, loadqOperator) are
 * rebuilt in the caller's own types; their matrices are constructed as
 * Mat(std::vector<double>, rows, cols) (the qmatrix constructor NrgData uses,
 * nrgData.hpp:242), or Mat(rows, cols, 0.0) and filled through data().
 *
 * Differences a caller can see:
 *  - The nrgcore(Imp&, Bath&) constructor runs on a process-wide engine
 *    (device NRG_GPU_DEVICE, default 0; precision NRG_GPU_PRECISION = "fp64"
 *    or "mixed", default mixed: FP32 block solves refined to FP64 accuracy).
 *    nrgcore(engine&, Imp&, Bath&) picks an engine explicitly.
 *  - current_hamiltonQ[i] is fetched from the device when indexed; the
 *    f-dagger operators (get_f_dag_operator) hold the kept x kept blocks, all
 *    that the next site reads (nrgcore.hpp:199-203).
 *  - update_system_operator(&nrg, ops) rotates on the device and copies the
 *    rotated blocks back into ops (the reference's in-place semantics);
 *    update_system_operator(nrg, system_operators&) skips the copy.
 *  - NrgData keeps its snapshots on the device; saveCurrentData stores the
 *    operator set last passed to update_system_operator with the shell, so
 *    saveqOperator has nothing left to do and loadqOperator copies that set
 *    back.  fdmSpectrum::setOperator and fdmThermodynamics::setSystemOperator
 *    name that same set.
 * Errors become std::runtime_error, as in the reference.
 */
#ifndef NRGCORE_GPU_HPP
#define NRGCORE_GPU_HPP

#include <algorithm>
#include <array>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "nrg_gpu.h"

namespace nrg_gpu {

inline void check(int rc) {
  if (rc != NRG_OK) throw std::runtime_error(std::string("nrg_gpu: ") + nrg_last_error());
}

// One GPU engine: device context, stream, allocator.  precision NRG_PREC_*.
class engine {
 public:
  explicit engine(int precision = NRG_PREC_MIXED, int device = 0, uint64_t hbm_budget_bytes = 0) {
    nrg_engine_opts o{device, precision, hbm_budget_bytes, 0};
    check(nrg_engine_create(&o, &h_));
  }
  ~engine() { nrg_engine_destroy(h_); }
  engine(const engine &) = delete;
  engine &operator=(const engine &) = delete;
  nrg_engine *get() const { return h_; }

 private:
  nrg_engine *h_ = nullptr;
};

// The process-wide engine behind nrgcore(Imp&, Bath&), created on first use
// from NRG_GPU_DEVICE and NRG_GPU_PRECISION ("fp64" or "mixed").
inline engine &default_engine() {
  static engine e([] {
    const char *p = std::getenv("NRG_GPU_PRECISION");
    return (p && std::string(p) == "fp64") ? NRG_PREC_FP64 : NRG_PREC_MIXED;
  }(), [] {
    const char *d = std::getenv("NRG_GPU_DEVICE");
    return d ? std::atoi(d) : 0;
  }());
  return e;
}

// A dense row-major host matrix (qmatrix concept) for current_hamiltonQ.
struct host_matrix {
  size_t r = 0, c = 0;
  std::vector<double> v;
  size_t getrow() const { return r; }
  size_t getcolumn() const { return c; }
  size_t size() const { return v.size(); }
  const double *data() const { return v.data(); }
  double *data() { return v.data(); }
  double &at(size_t i, size_t j) { return v.at(i * c + j); }
  double at(size_t i, size_t j) const { return v.at(i * c + j); }
  double &operator()(size_t i, size_t j) { return v[i * c + j]; }
  double operator()(size_t i, size_t j) const { return v[i * c + j]; }
};

namespace detail {

// Flattened copy of a block-sparse operator list (qOperator concept).
struct op_buffers {
  std::vector<int> op, row, col, rows, cols;
  std::vector<double> data;
  int nops = 0;
  template <class OpVec> void fill(OpVec &ops) {
    nops = int(ops.size());
    for (size_t ip = 0; ip < ops.size(); ++ip) {
      auto *m = ops[ip].getMap();
      for (auto &kv : *m) {
        const auto &mat = kv.second;
        op.push_back(int(ip));
        row.push_back(int(kv.first[0]));
        col.push_back(int(kv.first[1]));
        rows.push_back(int(mat.getrow()));
        cols.push_back(int(mat.getcolumn()));
        const double *p = mat.data();
        data.insert(data.end(), p, p + mat.getrow() * mat.getcolumn());
      }
    }
    if (data.empty()) data.push_back(0.0);
  }
  nrg_op_desc desc() {
    return nrg_op_desc{nops, int(op.size()), op.data(), row.data(), col.data(), rows.data(), cols.data(),
                       data.data()};
  }
};

// nrg_site_desc of a model (its arrays kept alive here).
struct site_buffers {
  std::vector<int> qnum, dims;
  std::vector<double> energies, chi;
  op_buffers ops;
  nrg_site_desc d{};
  template <class Model> void fill(Model &m, bool with_chi) {
    const auto basis = m.get_basis();
    const auto eq = m.get_eigenvaluesQ();
    if (basis.size() != eq.size()) throw std::runtime_error("nrg_gpu: basis and eigenvalue sectors differ");
    const int nq = basis.empty() ? 0 : int(basis[0].size());
    for (auto &q : basis) qnum.insert(qnum.end(), q.begin(), q.end());
    for (auto &v : eq) {
      dims.push_back(int(v.size()));
      energies.insert(energies.end(), v.begin(), v.end());
    }
    if (with_chi) chi = m.get_chi_Q();
    ops.fill(m.f_dag_operator);
    d.nq = nq;
    d.nsect = int(basis.size());
    d.qnum = qnum.data();
    d.dims = dims.data();
    d.energies = energies.data();
    d.chi = with_chi ? chi.data() : nullptr;
    d.nops = ops.nops;
    d.nblk = int(ops.op.size());
    d.blk_op = ops.op.data();
    d.blk_row = ops.row.data();
    d.blk_col = ops.col.data();
    d.blk_data = ops.data.data();
  }
};

// A matrix of the caller's type from row-major data.
template <class Mat> Mat make_matrix(std::vector<double> v, size_t rows, size_t cols) {
  if constexpr (std::is_constructible_v<Mat, std::vector<double>, size_t, size_t>) {
    return Mat(std::move(v), rows, cols);
  } else {
    Mat m(rows, cols, 0.0);
    if (!v.empty()) std::memcpy(m.data(), v.data(), v.size() * sizeof(double));
    return m;
  }
}

// Rebuilds a caller's vector<qOperator> from an enumerated block list:
// list(ip, i, j, rows, cols, cap, &n) and get(ip, i, j, out, cap).
template <class OpVec, class List, class Get> void assign_blocks(OpVec &ops, int nops, List list, Get get) {
  using Op = typename OpVec::value_type;
  using Map = std::remove_pointer_t<decltype(std::declval<Op &>().getMap())>;
  using Mat = typename Map::mapped_type;
  uint64_t n = 0;
  check(list(nullptr, nullptr, nullptr, nullptr, nullptr, 0, &n));
  std::vector<int> ip(n);
  std::vector<int64_t> bi(n), bj(n), rows(n), cols(n);
  if (n) check(list(ip.data(), bi.data(), bj.data(), rows.data(), cols.data(), n, &n));
  if (int(ops.size()) < nops) ops.resize(size_t(nops));
  for (auto &op : ops) op.getMap()->clear();
  for (uint64_t b = 0; b < n; ++b) {
    std::vector<double> v(size_t(rows[b] * cols[b]));
    if (!v.empty()) check(get(ip[b], bi[b], bj[b], v.data(), uint64_t(v.size())));
    typename Map::key_type key{};
    key[0] = size_t(bi[b]);
    key[1] = size_t(bj[b]);
    (*ops[size_t(ip[b])].getMap())[key] = make_matrix<Mat>(std::move(v), size_t(rows[b]), size_t(cols[b]));
  }
}

}  // namespace detail

// Tracked operators in a run's basis (update_system_operator's state on the
// device).
class system_operators {
 public:
  template <class N, class OpVec> system_operators(N &nrg, OpVec &ops) {
    detail::op_buffers b;
    b.fill(ops);
    nrg_op_desc d = b.desc();
    nops_ = b.nops;
    check(nrg_opset_create(nrg.handle(), &d, &h_));
  }
  ~system_operators() { nrg_opset_destroy(h_); }
  system_operators(const system_operators &) = delete;
  system_operators &operator=(const system_operators &) = delete;
  nrg_opset *handle() const { return h_; }
  int size() const { return nops_; }
  // the rotated blocks, rebuilt in the caller's vector<qOperator>
  template <class OpVec> void copy_to(OpVec &ops) const {
    nrg_opset *h = h_;
    detail::assign_blocks(
        ops, nops_,
        [h](int *ip, int64_t *i, int64_t *j, int64_t *r, int64_t *c, uint64_t cap, uint64_t *n) {
          return nrg_opset_list_blocks(h, ip, i, j, r, c, cap, n);
        },
        [h](int ip, int64_t i, int64_t j, double *out, uint64_t cap) {
          int64_t r = 0, c = 0;
          return nrg_opset_get_block(h, ip, i, j, out, cap, &r, &c);
        });
  }

 private:
  nrg_opset *h_ = nullptr;
  int nops_ = 0;
};

// nrgcore<Imp, Bath> (nrgcore.hpp:25-550).  The public data the reference's
// callers read are refreshed by update_internal_state (and the constructor);
// the eigenvectors (current_hamiltonQ[i]) are fetched when indexed.
template <class Imp, class Bath> class nrgcore {
 public:
  using op_type = typename std::decay_t<decltype(std::declval<Imp &>().f_dag_operator)>::value_type;

  nrgcore(Imp &im, Bath &bath) : nrgcore(default_engine(), im, bath) {}  // nrgcore.hpp:44-53
  nrgcore(engine &eng, Imp &im, Bath &bath) : current_hamiltonQ{this}, eng_(eng), imp_(&im), bath_(&bath) {
    test();
    detail::site_buffers si, sb;
    si.fill(im, false);
    sb.fill(bath, true);
    check(nrg_run_create(eng.get(), &si.d, &sb.d, 1024, &h_));  // set_parameters() default
    refresh();
  }
  ~nrgcore() {
    tracked_.clear();
    nrg_run_destroy(h_);
  }
  nrgcore(const nrgcore &) = delete;
  nrgcore &operator=(const nrgcore &) = delete;

  void set_parameters(size_t n = 1024) {  // nrgcore.hpp:336-342
    check(nrg_run_set_parameters(h_, n));
    refresh();
  }
  // add_bath_site (nrgcore.hpp:65-97); the bath is re-read every site as in
  // the reference (:68-70), for baths whose spectrum changes
  void add_bath_site(const std::vector<double> &t, double rescale) {
    detail::site_buffers sb;
    sb.fill(*bath_, true);
    check(nrg_run_set_bath(h_, &sb.d));
    check(nrg_run_add_site(h_, t.data(), int(t.size()), rescale));
    refresh();
  }
  void update_internal_state() {  // nrgcore.hpp:105-109
    check(nrg_run_update_state(h_));
    refresh();
  }
  bool checkHigherEnergyDiscarded() {  // nrgcore.hpp:384-386
    int v = 0;
    check(nrg_run_check_discarded(h_, &v));
    return v != 0;
  }
  // nrgcore.hpp:117-134: the models must agree on the quantum-number count
  // and the number of f-dagger operators
  void test() {
    const auto bi = imp_->get_basis(), bb = bath_->get_basis();
    if (!bi.empty() && !bb.empty() && bi[0].size() != bb[0].size())
      throw std::runtime_error("Number of quantum number is different on model and impurity!");
    if (imp_->f_dag_operator.size() != bath_->f_dag_operator.size())
      throw std::runtime_error("f_dag_operator.size is different on model and impurity!\n"
                               "impurityModel->f_dag_operator.size() = " +
                               std::to_string(imp_->f_dag_operator.size()) +
                               "bath_model->f_dag_operator.size() = " +
                               std::to_string(bath_->f_dag_operator.size()));
  }
  std::vector<std::vector<int>> get_basis_nQ() {  // nrgcore.hpp:350-355
    if (current_sysmQ.empty()) throw std::runtime_error("current_sysmQ.empty!");
    return current_sysmQ;
  }
  std::vector<std::vector<double>> get_eigenvaluesQ() {  // nrgcore.hpp:363-368
    if (eigenvaluesQ.empty()) throw std::runtime_error("eigenvaluesQ.empty!");
    return eigenvaluesQ;
  }
  // nrgcore.hpp:377: the f-dagger operators of the current basis (kept x kept)
  std::vector<op_type> get_f_dag_operator() {
    std::vector<op_type> ops;
    fetch_fdag(ops);
    return ops;
  }
  std::vector<op_type> *getPreWilsonSiteOperators() {  // nrgcore.hpp:548
    fetch_fdag(fdag_);
    return &fdag_;
  }

  nrg_run *handle() const { return h_; }
  engine &eng() const { return eng_; }
  // the device operator set behind a caller's operator vector, created from
  // its blocks on first use (update_system_operator)
  template <class OpVec> system_operators &tracked(OpVec &ops) {
    auto &slot = tracked_[static_cast<const void *>(&ops)];
    if (!slot) slot = std::make_unique<system_operators>(*this, ops);
    return *slot;
  }
  template <class OpVec> system_operators *find_tracked(OpVec *ops) const {
    auto it = tracked_.find(static_cast<const void *>(ops));
    return it == tracked_.end() ? nullptr : it->second.get();
  }
  system_operators *last_updated = nullptr;  // saved with the next NrgData::saveCurrentData

  // current_hamiltonQ[sector] (nrgcore.hpp:526): eigenvectors as columns,
  // row-major, fetched from the device when indexed
  struct hamiltonQ_view {
    const nrgcore *c;
    host_matrix operator[](size_t sector) const {
      const size_t n = c->eigenvaluesQ.at(sector).size();
      host_matrix m;
      m.r = m.c = n;
      m.v.resize(n * n);
      if (n) check(nrg_run_get_eigenvectors(c->h_, int64_t(sector), m.v.data(), m.v.size()));
      return m;
    }
    host_matrix at(size_t sector) const { return (*this)[sector]; }
    size_t size() const { return c->eigenvaluesQ.size(); }
  };

  // public state of the reference (nrgcore.hpp:518-550)
  std::vector<double> all_eigenvalue;
  std::vector<double> relativeGroundStateEnergy;
  std::vector<std::vector<size_t>> eigenvaluesQ_kept_indices;
  hamiltonQ_view current_hamiltonQ;
  std::vector<std::vector<int>> current_sysmQ, pre_sysmQ;
  std::vector<std::vector<double>> eigenvaluesQ;
  std::vector<std::vector<size_t>> coupled_nQ_index;
  int nrg_iterations_cnt = 0, nrg_iterations_min = 0;
  std::vector<std::vector<double>> bath_eigenvaluesQ;
  std::vector<std::vector<int>> nq_bath;

 private:
  void fetch_fdag(std::vector<op_type> &ops) {
    nrg_run *h = h_;
    detail::assign_blocks(
        ops, int(imp_->f_dag_operator.size()),
        [h](int *ip, int64_t *i, int64_t *j, int64_t *r, int64_t *c, uint64_t cap, uint64_t *n) {
          return nrg_run_list_fdag_blocks(h, ip, i, j, r, c, cap, n);
        },
        [h](int ip, int64_t i, int64_t j, double *out, uint64_t cap) {
          int64_t r = 0, c = 0;
          return nrg_run_get_fdag_block(h, ip, i, j, out, cap, &r, &c);
        });
  }
  void refresh() {
    nrg_run_info in{};
    check(nrg_run_get_info(h_, &in));
    nrg_iterations_cnt = int(in.iteration);
    nrg_iterations_min = int(in.iteration_min);
    all_eigenvalue.assign(size_t(in.n_all), 0.0);
    if (in.n_all) check(nrg_run_get_all_eigenvalues(h_, all_eigenvalue.data(), all_eigenvalue.size()));
    relativeGroundStateEnergy.assign(size_t(in.n_relgs), 0.0);
    if (in.n_relgs) check(nrg_run_get_relgs(h_, relativeGroundStateEnergy.data(), relativeGroundStateEnergy.size()));
    auto sectors = [&](int which, int64_t n) {
      std::vector<int> q(static_cast<size_t>(n * in.nq));
      std::vector<std::vector<int>> out(static_cast<size_t>(n));
      if (n) check(nrg_run_get_sectors(h_, which, q.data(), uint64_t(n)));
      for (int64_t s = 0; s < n; ++s) out[size_t(s)].assign(q.begin() + s * in.nq, q.begin() + (s + 1) * in.nq);
      return out;
    };
    current_sysmQ = sectors(0, in.n_cur_sectors);
    pre_sysmQ = sectors(1, in.n_pre_sectors);
    // between add_site and update_state the current sectors, afterwards the
    // truncated site's (which the next site builds on)
    const int64_t nsec = in.n_cur_sectors ? in.n_cur_sectors : in.n_pre_sectors;
    std::vector<uint64_t> dims(static_cast<size_t>(nsec));
    uint64_t tot = 0;
    if (nsec) {
      check(nrg_run_get_eigenvalues_q(h_, dims.data(), nullptr, 0));
      for (auto x : dims) tot += x;
    }
    std::vector<double> vals(tot);
    if (tot) check(nrg_run_get_eigenvalues_q(h_, dims.data(), vals.data(), tot));
    eigenvaluesQ.assign(dims.size(), {});
    size_t o = 0;
    for (size_t s = 0; s < dims.size(); ++s) {
      eigenvaluesQ[s].assign(vals.begin() + o, vals.begin() + o + dims[s]);
      o += dims[s];
    }
    std::vector<uint64_t> kept(static_cast<size_t>(in.n_pre_sectors));
    if (!kept.empty()) check(nrg_run_get_kept(h_, kept.data(), kept.size()));
    eigenvaluesQ_kept_indices.assign(kept.size(), {});
    for (size_t s = 0; s < kept.size(); ++s)
      for (uint64_t k = 0; k < kept[s]; ++k) eigenvaluesQ_kept_indices[s].push_back(size_t(k));
    coupled_nQ_index.assign(size_t(in.n_cur_sectors), {});
    if (in.n_cur_sectors) {
      std::vector<uint64_t> counts(size_t(in.n_cur_sectors));
      check(nrg_run_get_coupled(h_, counts.data(), nullptr, 0));
      uint64_t ne = 0;
      for (auto x : counts) ne += x;
      std::vector<uint64_t> ent(ne);
      if (ne) check(nrg_run_get_coupled(h_, counts.data(), ent.data(), ne));
      size_t e = 0;
      for (size_t s = 0; s < counts.size(); ++s)
        for (uint64_t k = 0; k < counts[s]; ++k) coupled_nQ_index[s].push_back(size_t(ent[e++]));
    }
    bath_eigenvaluesQ = bath_->get_eigenvaluesQ();
    nq_bath = bath_->get_basis();
  }

  engine &eng_;
  Imp *imp_;
  Bath *bath_;
  nrg_run *h_ = nullptr;
  std::vector<op_type> fdag_;
  std::map<const void *, std::unique_ptr<system_operators>> tracked_;
};

// update_system_operator(nrg, ops) (sysOperator.hpp:36-133): rotates the
// caller's operators into the new basis (call after add_bath_site) and writes
// the rotated blocks back into ops, as the reference updates them in place.
template <class N, class OpVec> void update_system_operator(N *nrg, OpVec &ops) {
  system_operators &s = nrg->tracked(ops);
  check(nrg_opset_update(s.handle()));
  s.copy_to(ops);
  nrg->last_updated = &s;
}
// The same rotation without the copy back (the operators stay on the device).
template <class N> void update_system_operator(N &nrg, system_operators &ops) {
  check(nrg_opset_update(ops.handle()));
  nrg.last_updated = &ops;
}

// NrgData<N> (nrgData.hpp:31-293): device-resident snapshots instead of an
// HDF5 file; export() writes them in the file's group layout.
template <class N> class NrgData {
 public:
  explicit NrgData(N *nrg) : nrg_(nrg) {}
  // saveCurrentData (:134-165), with the operator set last rotated by
  // update_system_operator (saveqOperator's data, :175-210)
  void saveCurrentData() {
    check(nrg_run_snapshot(nrg_->handle(), nrg_->last_updated ? nrg_->last_updated->handle() : nullptr));
  }
  void saveCurrentData(system_operators *ops) { check(nrg_run_snapshot(nrg_->handle(), ops ? ops->handle() : nullptr)); }
  // saveqOperator: the operators were stored with the shell by saveCurrentData
  template <class OpVec> void saveqOperator(OpVec *, const std::string &) {}
  // loadCurrentData() (:255-257) reads the caller's (possibly decremented)
  // nrg_iterations_cnt; loadCurrentData(in) (:266-293) sets it
  void loadCurrentData() { loadCurrentData(nrg_->nrg_iterations_cnt); }
  void loadCurrentData(int in) {
    check(nrg_run_load_snapshot(nrg_->handle(), int64_t(in)));
    nrg_->nrg_iterations_cnt = in;
  }
  // loadqOperator (:213-246): the loaded shell's operator set into *ops
  template <class OpVec> void loadqOperator(OpVec *ops, const std::string &) {
    nrg_run *h = nrg_->handle();
    uint64_t n = 0;
    check(nrg_run_list_snapshot_ops(h, nullptr, nullptr, nullptr, nullptr, nullptr, 0, &n));
    std::vector<int> ip(n);
    if (n) check(nrg_run_list_snapshot_ops(h, ip.data(), nullptr, nullptr, nullptr, nullptr, n, &n));
    int nops = int(ops->size());
    for (int x : ip) nops = std::max(nops, x + 1);
    detail::assign_blocks(
        *ops, nops,
        [h](int *p, int64_t *i, int64_t *j, int64_t *r, int64_t *c, uint64_t cap, uint64_t *m) {
          return nrg_run_list_snapshot_ops(h, p, i, j, r, c, cap, m);
        },
        [h](int p, int64_t i, int64_t j, double *out, uint64_t cap) {
          return nrg_run_get_snapshot_op_block(h, p, i, j, out, cap);
        });
  }
  void saveFinalState() {}  // :106-110: savedNRGIndex and relativeGroundStateEnergy live in the run
  void close() {}
  void clear() {}
  // every shell in NrgData's group layout (nrg_run_export_snapshots)
  void exportTo(const std::string &path, bool with_vectors = true) {
    check(nrg_run_export_snapshots(nrg_->handle(), path.c_str(), with_vectors ? 1 : 0));
  }

 private:
  N *nrg_;
};

template <class N> class fdmThermodynamics;

// fdmSpectrum<N> (fdmSpectrum.hpp:35-337).  The spectrum is computed from the
// operator set saved with each snapshot; setOperator names it (the vector the
// caller passed to update_system_operator, or its system_operators).
template <class N> class fdmSpectrum {
 public:
  explicit fdmSpectrum(N *nrg) : nrg_(nrg) {}
  ~fdmSpectrum() {
    if (h_) nrg_fdm_destroy(h_);
  }
  fdmSpectrum(const fdmSpectrum &) = delete;
  fdmSpectrum &operator=(const fdmSpectrum &) = delete;
  // setOperator(bOperator, aOperator = nullptr) (:306-314); A is B^T as in the
  // reference's rhoDotOperators
  template <class OpVec> void setOperator(OpVec *bopr, OpVec * = nullptr) {
    system_operators *s = nrg_->find_tracked(bopr);
    if (!s) throw std::runtime_error("nrg_gpu: setOperator needs the operators passed to update_system_operator");
    create(s->size());
  }
  void setOperator(system_operators &ops) { create(ops.size()); }
  void setTemperature(double) {}  // a no-op in the reference too (fdmSpectrum.hpp:27, 284)
  // finite temperature (no reference counterpart): the shells' Boltzmann
  // weights at T from a thermodynamics object that has seen every shell
  void setTemperature(double T, fdmThermodynamics<N> &thermo) {
    if (!h_) throw std::runtime_error("nrg_gpu: setOperator before setTemperature");
    check(nrg_fdm_set_temperature(h_, T, thermo.handle()));
  }
  void calcSpectrum(double energy_scale) { check(nrg_fdm_calc(h_, energy_scale)); }
  // rhoDotStaticOperators (fdmBackwardIteration.hpp:166-199) summed over the shells
  std::vector<double> staticExpectation() {
    std::vector<double> out(static_cast<size_t>(nops_));
    check(nrg_fdm_get_static(h_, out.data(), nops_));
    return out;
  }
  // filetype: write(const vector<double>&, string), write(const vector<vector<double>>&, string)
  template <class F> void saveFinalData(F *file) {
    const size_t npts = 100000;
    std::vector<double> e(npts), pos(static_cast<size_t>(nops_) * npts), neg(static_cast<size_t>(nops_) * npts);
    check(nrg_fdm_get(h_, e.data(), pos.data(), neg.data(), npts));
    std::vector<std::vector<double>> p(static_cast<size_t>(nops_)), n(static_cast<size_t>(nops_));
    for (int ip = 0; ip < nops_; ++ip) {
      p[size_t(ip)].assign(pos.begin() + ip * npts, pos.begin() + (ip + 1) * npts);
      n[size_t(ip)].assign(neg.begin() + ip * npts, neg.begin() + (ip + 1) * npts);
    }
    file->write(e, "GreenFnEnergyPoints");
    file->write(p, "GreenFnPositiveWeight");
    file->write(n, "GreenFnNegativeWeight");
  }

 private:
  void create(int nops) {
    if (h_) nrg_fdm_destroy(h_);
    h_ = nullptr;
    nops_ = nops;
    check(nrg_fdm_create(nrg_->handle(), nops_, &h_));
  }
  N *nrg_;
  nrg_fdm *h_ = nullptr;
  int nops_ = 0;
};

// fdmThermodynamics<N> (fdmThermodynamics.hpp:26-236)
template <class N> class fdmThermodynamics {
 public:
  fdmThermodynamics(N *nrg, const std::vector<double> &temps) : nrg_(nrg), temps_(temps) {
    check(nrg_thermo_create(nrg->handle(), temps_.data(), int(temps_.size()), &h_));
  }
  ~fdmThermodynamics() { nrg_thermo_destroy(h_); }
  fdmThermodynamics(const fdmThermodynamics &) = delete;
  fdmThermodynamics &operator=(const fdmThermodynamics &) = delete;
  // setSystemOperator (:37-39): every operator of the set passed to
  // update_system_operator (saved with the snapshots)
  template <class OpVec> void setSystemOperator(OpVec *ops) {
    system_operators *s = nrg_->find_tracked(ops);
    if (!s) throw std::runtime_error("nrg_gpu: setSystemOperator needs the operators passed to update_system_operator");
    nops_ = s->size();
    std::vector<int> idx(static_cast<size_t>(nops_));
    for (int i = 0; i < nops_; ++i) idx[size_t(i)] = i;
    check(nrg_thermo_set_operator(h_, idx.data(), nops_));
  }
  void calcThermodynamics(double energy_scale) { check(nrg_thermo_calc(h_, energy_scale)); }
  template <class F> void saveFinalData(F *file) {
    std::vector<double> s(temps_.size()), c(temps_.size());
    check(nrg_thermo_final(h_, s.data(), c.data()));
    file->write(temps_, "temperatureArray");
    file->write(s, "entropy");
    file->write(c, "specificHeat");
    if (nops_) {
      std::vector<double> q(static_cast<size_t>(nops_) * temps_.size());
      check(nrg_thermo_get_operator(h_, q.data(), nops_, int(temps_.size())));
      std::vector<std::vector<double>> qv(static_cast<size_t>(nops_));
      for (int i = 0; i < nops_; ++i)
        qv[size_t(i)].assign(q.begin() + i * temps_.size(), q.begin() + (i + 1) * temps_.size());
      file->write(qv, "qsysOPeratorExpValue");
    }
  }
  nrg_thermo *handle() const { return h_; }

 private:
  N *nrg_;
  std::vector<double> temps_;
  nrg_thermo *h_ = nullptr;
  int nops_ = 0;
};

}  // namespace nrg_gpu

#endif  // NRGCORE_GPU_HPP
