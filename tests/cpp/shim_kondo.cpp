// C++ driver through include/nrgcore_gpu.hpp, written like the reference's
// examples/entropyKondo/main.cpp: Kondo RG flow with the entropy from the
// backward pass.  The models are plain structs with the reference's model
// concept, filled from a binary description written by the Python test.
//
// usage: shim_kondo <models.bin> <out.bin> <precision 0|1> <nsites> <lambda> <nkeep>
#include <cmath>
#include <cstdio>
#include <map>
#include <array>
#include <stdexcept>
#include <string>
#include <vector>

#include "nrgcore_gpu.hpp"

struct Mat {  // qmatrix concept: row-major
  size_t r = 0, c = 0;
  std::vector<double> v;
  size_t getrow() const { return r; }
  size_t getcolumn() const { return c; }
  const double *data() const { return v.data(); }
};
struct Op {  // qOperator concept
  std::map<std::array<size_t, 2>, Mat> storage;
  std::map<std::array<size_t, 2>, Mat> *getMap() { return &storage; }
};
struct Model {  // the model concept nrgcore reads
  std::vector<std::vector<int>> q;
  std::vector<std::vector<double>> e;
  std::vector<double> chi;
  std::vector<Op> f_dag_operator;
  std::vector<std::vector<int>> get_basis() const { return q; }
  std::vector<std::vector<double>> get_eigenvaluesQ() const { return e; }
  std::vector<double> get_chi_Q() const { return chi; }
};

static int rd_i(FILE *f) {
  int v;
  if (std::fread(&v, 4, 1, f) != 1) throw std::runtime_error("short read");
  return v;
}
static double rd_d(FILE *f) {
  double v;
  if (std::fread(&v, 8, 1, f) != 1) throw std::runtime_error("short read");
  return v;
}
static Model read_model(FILE *f) {
  Model m;
  const int nq = rd_i(f), ns = rd_i(f);
  m.q.assign(ns, std::vector<int>(nq));
  for (auto &x : m.q)
    for (auto &y : x) y = rd_i(f);
  m.e.resize(ns);
  for (auto &x : m.e) {
    x.resize(rd_i(f));
    for (auto &y : x) y = rd_d(f);
  }
  m.chi.resize(ns);
  for (auto &x : m.chi) x = rd_d(f);
  const int nops = rd_i(f);
  m.f_dag_operator.resize(nops);
  for (auto &op : m.f_dag_operator) {
    const int nb = rd_i(f);
    for (int b = 0; b < nb; ++b) {
      std::array<size_t, 2> k{size_t(rd_i(f)), size_t(rd_i(f))};
      Mat mat;
      mat.r = rd_i(f);
      mat.c = rd_i(f);
      mat.v.resize(mat.r * mat.c);
      for (auto &y : mat.v) y = rd_d(f);
      op.storage[k] = mat;
    }
  }
  return m;
}

struct Sink {  // the reference's filetype concept
  std::map<std::string, std::vector<double>> d1;
  void write(const std::vector<double> &v, const std::string &name) { d1[name] = v; }
  void write(const std::vector<std::vector<double>> &v, const std::string &name) {
    for (size_t i = 0; i < v.size(); ++i) d1[name + std::to_string(i)] = v[i];
  }
};

static double hopping(int n, double lam) {  // examples/rgflowSIAM/main.cpp:5-10
  return 0.5 * (1.0 + 1.0 / lam) * (1.0 - std::pow(lam, -n - 1)) /
         std::sqrt((1.0 - std::pow(lam, -2.0 * n - 1)) * (1.0 - std::pow(lam, -2.0 * n - 3)));
}

int main(int argc, char **argv) {
  if (argc < 7) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  Model imp = read_model(f), bath = read_model(f);
  const int ntemps = rd_i(f);
  std::vector<double> temps(ntemps);
  for (auto &t : temps) t = rd_d(f);
  std::fclose(f);
  const int precision = std::atoi(argv[3]), nsites = std::atoi(argv[4]);
  const double lam = std::atof(argv[5]);
  const size_t nkeep = size_t(std::atol(argv[6]));
  try {
    nrg_gpu::engine eng(precision);
    nrg_gpu::nrgcore<Model, Model> kondo(eng, imp, bath);
    kondo.set_parameters(nkeep);
    nrg_gpu::NrgData<nrg_gpu::nrgcore<Model, Model>> data(&kondo);
    std::vector<std::vector<double>> eigs;
    int min_it = 0;
    for (int it = 0; it < nsites; ++it) {
      const double t = hopping(it, lam);
      kondo.add_bath_site(std::vector<double>(imp.f_dag_operator.size(), t), std::sqrt(lam));
      if (kondo.checkHigherEnergyDiscarded()) data.saveCurrentData();
      else ++min_it;
      kondo.update_internal_state();
      eigs.push_back(kondo.all_eigenvalue);
    }
    nrg_gpu::fdmThermodynamics<nrg_gpu::nrgcore<Model, Model>> thermo(&kondo, temps);
    size_t cnt = kondo.nrg_iterations_cnt;
    for (int it = nsites; it > min_it + 1; --it) {  // the Kondo drivers skip the first kept shell
      --cnt;
      data.loadCurrentData(cnt);
      thermo.calcThermodynamics(std::pow(lam, -(it - 1.0) / 2.0));
    }
    Sink sink;
    thermo.saveFinalData(&sink);
    FILE *o = std::fopen(argv[2], "wb");
    const int n = int(eigs.size());
    std::fwrite(&n, 4, 1, o);
    for (auto &v : eigs) {
      const int m = int(v.size());
      std::fwrite(&m, 4, 1, o);
      std::fwrite(v.data(), 8, v.size(), o);
    }
    const auto &s = sink.d1["entropy"];
    const int ns = int(s.size());
    std::fwrite(&ns, 4, 1, o);
    std::fwrite(s.data(), 8, s.size(), o);
    std::fclose(o);
  } catch (const std::exception &x) {
    std::fprintf(stderr, "%s\n", x.what());
    return 1;
  }
  return 0;
}
