/*
 * nrgcore_gpu.hpp - C++ drop-in for the reference's nrgcore<Imp, Bath> and its
 * companion classes, on top of the C ABI in nrg_gpu.h (header-only, C++17).
 *
 * Drivers written against the reference (examples/ * /main.cpp) keep their model
 * builders and their loops; they include this header, construct one
 * nrg_gpu::engine, and use the classes below under the reference's names:
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
 * pointer to a map from {row sector, column sector} to a row-major matrix with
 * getrow(), getcolumn() and data() (qOperator / qmatrix, qOperator.hpp:18-46).
 * Errors become std::runtime_error, as in the reference.
 */
#ifndef NRGCORE_GPU_HPP
#define NRGCORE_GPU_HPP

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
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

}  // namespace detail

// nrgcore<Imp, Bath> (nrgcore.hpp:25-550).  The public data the reference's
// callers read are refreshed by update_internal_state (and the constructor);
// the eigenvectors (current_hamiltonQ) are fetched on demand.
template <class Imp, class Bath> class nrgcore {
 public:
  nrgcore(engine &eng, Imp &im, Bath &bath) : eng_(eng), bath_(&bath) {
    detail::site_buffers si, sb;
    si.fill(im, false);
    sb.fill(bath, true);
    check(nrg_run_create(eng.get(), &si.d, &sb.d, 1024, &h_));  // set_parameters() default
    refresh();
  }
  ~nrgcore() { nrg_run_destroy(h_); }
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
  // current_hamiltonQ[sector] (nrgcore.hpp:526): eigenvectors as columns, row-major
  std::vector<double> current_hamiltonQ(size_t sector) const {
    const size_t n = eigenvaluesQ.at(sector).size();
    std::vector<double> out(n * n);
    if (n) check(nrg_run_get_eigenvectors(h_, int64_t(sector), out.data(), out.size()));
    return out;
  }
  nrg_run *handle() const { return h_; }
  engine &eng() const { return eng_; }

  // public state of the reference (nrgcore.hpp:518-550)
  std::vector<double> all_eigenvalue;
  std::vector<double> relativeGroundStateEnergy;
  std::vector<std::vector<int>> current_sysmQ, pre_sysmQ;
  std::vector<std::vector<double>> eigenvaluesQ;
  std::vector<size_t> eigenvaluesQ_kept_sizes;  // eigenvaluesQ_kept_indices[i] = 0 .. size - 1
  size_t nrg_iterations_cnt = 0, nrg_iterations_min = 0;

 private:
  void refresh() {
    nrg_run_info in{};
    check(nrg_run_get_info(h_, &in));
    nrg_iterations_cnt = size_t(in.iteration);
    nrg_iterations_min = size_t(in.iteration_min);
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
    eigenvaluesQ_kept_sizes.assign(kept.begin(), kept.end());
  }

  engine &eng_;
  Bath *bath_;
  nrg_run *h_ = nullptr;
};

// Tracked operators (vector<qOperator>) in the run's previous basis; pass to
// update_system_operator after every add_bath_site.
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

 private:
  nrg_opset *h_ = nullptr;
  int nops_ = 0;
};

// update_system_operator(nrg, ops) (sysOperator.hpp:36-133)
template <class N> void update_system_operator(N &, system_operators &ops) { check(nrg_opset_update(ops.handle())); }

// NrgData<N> (nrgData.hpp:31-157): device-resident snapshots instead of HDF5 groups.
template <class N> class NrgData {
 public:
  explicit NrgData(N *nrg) : nrg_(nrg) {}
  void saveCurrentData(system_operators *ops = nullptr) {
    check(nrg_run_snapshot(nrg_->handle(), ops ? ops->handle() : nullptr));
  }
  void loadCurrentData(size_t iteration) { check(nrg_run_load_snapshot(nrg_->handle(), int64_t(iteration))); }

 private:
  N *nrg_;
};

// fdmSpectrum<N> (fdmSpectrum.hpp:35-337), T = 0.  setOperator takes the
// tracked operators whose snapshots the backward pass reads.
template <class N> class fdmSpectrum {
 public:
  explicit fdmSpectrum(N *nrg) : nrg_(nrg) {}
  ~fdmSpectrum() {
    if (h_) nrg_fdm_destroy(h_);
  }
  fdmSpectrum(const fdmSpectrum &) = delete;
  fdmSpectrum &operator=(const fdmSpectrum &) = delete;
  void setOperator(system_operators &ops) {
    if (h_) nrg_fdm_destroy(h_);
    nops_ = ops.size();
    check(nrg_fdm_create(nrg_->handle(), nops_, &h_));
  }
  void setTemperature(double) {}  // a no-op in the reference too (fdmSpectrum.hpp:27, 284)
  void calcSpectrum(double energy_scale) { check(nrg_fdm_calc(h_, energy_scale)); }
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
  N *nrg_;
  nrg_fdm *h_ = nullptr;
  int nops_ = 0;
};

// fdmThermodynamics<N> (fdmThermodynamics.hpp:26-236)
template <class N> class fdmThermodynamics {
 public:
  fdmThermodynamics(N *nrg, const std::vector<double> &temps) : temps_(temps) {
    check(nrg_thermo_create(nrg->handle(), temps_.data(), int(temps_.size()), &h_));
  }
  ~fdmThermodynamics() { nrg_thermo_destroy(h_); }
  fdmThermodynamics(const fdmThermodynamics &) = delete;
  fdmThermodynamics &operator=(const fdmThermodynamics &) = delete;
  void calcThermodynamics(double energy_scale) { check(nrg_thermo_calc(h_, energy_scale)); }
  template <class F> void saveFinalData(F *file) {
    std::vector<double> s(temps_.size()), c(temps_.size());
    check(nrg_thermo_final(h_, s.data(), c.data()));
    file->write(temps_, "temperatureArray");
    file->write(s, "entropy");
    file->write(c, "specificHeat");
  }

 private:
  std::vector<double> temps_;
  nrg_thermo *h_ = nullptr;
};

}  // namespace nrg_gpu

#endif  // NRGCORE_GPU_HPP
