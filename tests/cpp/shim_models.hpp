// Models for the C++ drivers of the drop-in header: plain structs with the
// reference's model concept (get_basis, get_eigenvaluesQ, get_chi_Q, public
// f_dag_operator of block operators with getMap), filled from the binary
// description tests/test_cpp_shim.py writes.
#pragma once
#include <array>
#include <cmath>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

struct Mat {  // qmatrix concept: row-major
  size_t r = 0, c = 0;
  std::vector<double> v;
  Mat() = default;
  Mat(std::vector<double> data, size_t rows, size_t cols) : r(rows), c(cols), v(std::move(data)) {}
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

static std::vector<Op> read_ops(FILE *f) {
  std::vector<Op> ops(rd_i(f));
  for (auto &op : ops) {
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
  return ops;
}

static double hopping(int n, double lam) {  // examples/rgflowSIAM/main.cpp:5-10
  return 0.5 * (1.0 + 1.0 / lam) * (1.0 - std::pow(lam, -n - 1)) /
         std::sqrt((1.0 - std::pow(lam, -2.0 * n - 1)) * (1.0 - std::pow(lam, -2.0 * n - 3)));
}

static void write_vec(FILE *o, const std::vector<double> &v) {
  const int m = int(v.size());
  std::fwrite(&m, 4, 1, o);
  std::fwrite(v.data(), 8, v.size(), o);
}
