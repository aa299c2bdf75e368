// Oracle driver: runs the reference's own NRG engine (headers compiled
// unchanged from the reference tree by oracle/build_ref.sh) on one workload
// and writes every result array to a flat binary file of named float64
// arrays.  Test infrastructure only: it checks the engine and is never part of it.
//
// The loop mirrors the reference's example drivers:
//   examples/rgflowSIAM/main.cpp:27-42       (SIAM forward RG flow)
//   examples/rgflowKondo/main.cpp:20-39      (Kondo: no V site, rescale sqrt(L))
//   examples/twoChannelSiam/main.cpp:22-56   (impurity f-dag duplicated to 4 ops)
//   examples/fdmSpectrumSiam/main.cpp:61-135 (d-dag chi tracked, FDM backward)
//   examples/entropySIAM/main.cpp:67-93      (thermodynamics backward pass)
// with HDF5 snapshots (nrgData.hpp) replaced by in-memory copies of the same
// public members that nrgData.hpp:150-157 saves.
//
// usage: ref_nrg <siam|kondo|twochannel|zero|sc> <out.bin> key=value ...
//   keys: eps U V J lambda nkeep nsites fdm thermo dumpops opsites sysop
//   sysop=1 (with thermo): the impurity occupancy n_d is tracked through
//   update_system_operator and handed to fdmThermodynamics::setSystemOperator
//   (static/fdmThermodynamics.hpp:37-39, :63-88, :200-218), whose
//   qsysOPeratorExpValue (<n_d>(T)) is written out.
#include "dynamics/fdmSpectrum.hpp"
#include "models/fermionBasis.hpp"
#include "models/spinhalf.hpp"
#include "models/spinhalfKondo.hpp"
#include "models/spinhalfSC.hpp"
#include "models/twoChannel.hpp"
#include "nrgcore/nrgcore.hpp"
#include "nrgcore/sysOperator.hpp"
#include "static/fdmThermodynamics.hpp"
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <map>
#include <string>
#include <vector>

struct Out {
  std::vector<std::pair<std::string, std::vector<double>>> d;
  void write(const std::vector<double> &v, const std::string &s) { d.push_back({s, v}); }
  void write(const std::vector<std::vector<double>> &v, const std::string &s) {
    for (size_t i = 0; i < v.size(); i++) write(v[i], s + std::to_string(i));
  }
  void save(const char *fn) {
    FILE *f = fopen(fn, "wb");
    for (auto &kv : d) {
      fputs(kv.first.c_str(), f);
      fputc(0, f);
      unsigned long long n = kv.second.size();
      fwrite(&n, 8, 1, f);
      fwrite(kv.second.data(), 8, n, f);
    }
    fclose(f);
  }
};

static double hopping(int site, double l) {
  return 0.5 * (1.0 + 1.0 / l) * (1. - std::pow(l, -site - 1)) /
         std::sqrt((1.0 - std::pow(l, -2. * site - 1)) * (1.0 - std::pow(l, -2. * site - 3)));
}

struct Snap {
  std::vector<qmatrix<double>> H;
  std::vector<std::vector<int>> cur, pre;
  std::vector<std::vector<double>> ev;
  std::vector<std::vector<size_t>> cpl, kept;
  std::vector<qOperator> op, sysop;
};

template <class N> static void dump_ops(Out &o, std::vector<qOperator> &ops, const std::string &tag) {
  for (size_t ip = 0; ip < ops.size(); ip++) {
    for (auto &kv : *ops[ip].getMap()) {
      std::string nm = tag + "_op" + std::to_string(ip) + "_" + std::to_string(kv.first[0]) + "_" +
                       std::to_string(kv.first[1]);
      std::vector<double> v = {double(kv.second.getrow()), double(kv.second.getcolumn())};
      v.insert(v.end(), kv.second.begin(), kv.second.end());
      o.write(v, nm);
    }
  }
}

template <class IMP, class BATH>
static void run(IMP &imp, BATH &bath, std::map<std::string, double> &P, bool firstV, bool kondoRescale,
                int nops, Out &o, std::function<void(int)> pre_site = nullptr) {
  double L = P["lambda"], V = P["V"];
  size_t nk = size_t(P["nkeep"]);
  int nMax = int(P["nsites"]);
  bool fdm = P["fdm"] != 0, thermo = P["thermo"] != 0;
  int dumpops = int(P["dumpops"]);
  nrgcore<IMP, BATH> n(imp, bath);
  n.set_parameters(nk);
  std::vector<qOperator> d, nd;
  const bool sysop = thermo && P["sysop"] != 0;
  if (sysop) {
    fermionBasis b(2, fermionBasis::chargeAndSpin);
    auto f = b.get_raw_f_dag_operator();
    auto nt = f[0].dot(f[0].cTranspose());
    for (size_t i = 1; i < f.size(); i++) nt = nt + f[i].dot(f[i].cTranspose());
    nd = b.get_block_operators(std::vector<qmatrix<>>{nt});
  }
  if (fdm) {
    fermionBasis b(2, fermionBasis::chargeAndSpin);
    auto f = b.get_raw_f_dag_operator();
    auto nt = f[0].dot(f[0].cTranspose());
    for (size_t i = 1; i < f.size(); i++) nt = nt + f[i].dot(f[i].cTranspose());
    auto chi = nt;
    for (size_t i = 0; i < chi.getrow(); i++) chi(i, i) = std::pow(-1, nt(i, i));
    for (auto &a : f) a = a.dot(chi);
    d = b.get_block_operators(f);
  }
  std::map<int, Snap> st;
  size_t minIt = 0;
  auto record = [&](const std::string &tag) {
    o.write(n.all_eigenvalue, "Eigenvalues" + tag);
    std::vector<double> kept, dims;
    for (size_t i = 0; i < n.eigenvaluesQ_kept_indices.size(); i++) kept.push_back(n.eigenvaluesQ_kept_indices[i].size());
    for (auto &e : n.eigenvaluesQ) dims.push_back(e.size());
    o.write(kept, "kept" + tag);
    o.write(dims, "dims" + tag);
    std::vector<double> q;
    for (auto &s : n.pre_sysmQ) for (int x : s) q.push_back(x);
    o.write(q, "sysQ" + tag);
  };
  if (firstV) {
    std::vector<double> t(nops, V);
    if (pre_site) pre_site(-1);
    n.add_bath_site(t, 1.0);
    if (fdm) update_system_operator(&n, d);
    if (sysop) update_system_operator(&n, nd);
    n.update_internal_state();
    record("V");
  }
  for (int in = 0; in < nMax; in++) {
    double r = kondoRescale ? std::sqrt(L) : (in > 0 ? std::sqrt(L) : 1.0);
    std::vector<double> t(nops, hopping(in, L));
    if (pre_site) pre_site(in);
    n.add_bath_site(t, r);
    if (fdm) update_system_operator(&n, d);
    if (sysop) update_system_operator(&n, nd);
    if (fdm || thermo) {
      if (n.checkHigherEnergyDiscarded())
        st[n.nrg_iterations_cnt] = {n.current_hamiltonQ, n.current_sysmQ, n.pre_sysmQ, n.eigenvaluesQ,
                                    n.coupled_nQ_index, n.eigenvaluesQ_kept_indices, d, nd};
      else
        minIt++;
    }
    if (dumpops > 0 && in < dumpops) {
      auto *fo = n.getPreWilsonSiteOperators();
      dump_ops<decltype(n)>(o, *fo, "F" + std::to_string(in));
      std::vector<double> evs;
      for (size_t i = 0; i < n.eigenvaluesQ.size(); i++) {
        evs.push_back(double(n.eigenvaluesQ[i].size()));
        evs.insert(evs.end(), n.eigenvaluesQ[i].begin(), n.eigenvaluesQ[i].end());
      }
      o.write(evs, "EQ" + std::to_string(in));
      if (fdm) dump_ops<decltype(n)>(o, d, "D" + std::to_string(in));
    }
    n.update_internal_state();
    record(std::to_string(in));
  }
  o.write(n.relativeGroundStateEnergy, "relativeGroundStateEnergy");
  o.write(std::vector<double>{double(minIt)}, "minIterations");
  if (fdm) {
    fdmSpectrum<decltype(n)> f(&n);
    f.setOperator(&d);
    for (size_t in = nMax; in > minIt; in--) {
      n.nrg_iterations_cnt--;
      auto &s = st.at(n.nrg_iterations_cnt);
      n.current_hamiltonQ = s.H; n.current_sysmQ = s.cur; n.pre_sysmQ = s.pre;
      n.eigenvaluesQ = s.ev; n.coupled_nQ_index = s.cpl; n.eigenvaluesQ_kept_indices = s.kept; d = s.op;
      f.calcSpectrum(std::pow(L, -(in - 1.0) / 2.0));
    }
    f.saveFinalData(&o);
  }
  if (thermo && !fdm) {
    double vMax = 2, vMin = 1e-10;
    int tP = 200;
    double dT = (tP - 1.0) / std::log(vMax / vMin);
    std::vector<double> T(tP);
    for (int i = 0; i < tP; i++) T[i] = vMin * std::exp(std::fabs(i) * 1. / dT);
    fdmThermodynamics<decltype(n)> th(&n, T);
    std::vector<qOperator> ndShell;
    if (sysop) th.setSystemOperator(&ndShell);
    size_t lo = minIt + (kondoRescale ? 1 : 0);
    for (size_t in = nMax; in > lo; in--) {
      double sc = std::pow(L, -(1.0 * in - 1.0) / 2.0);
      n.nrg_iterations_cnt--;
      auto &s = st.at(n.nrg_iterations_cnt);
      n.current_hamiltonQ = s.H; n.current_sysmQ = s.cur; n.pre_sysmQ = s.pre;
      n.eigenvaluesQ = s.ev; n.coupled_nQ_index = s.cpl; n.eigenvaluesQ_kept_indices = s.kept;
      ndShell = s.sysop;
      th.calcThermodynamics(sc);
    }
    th.saveFinalData(&o);
  }
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: ref_nrg <siam|kondo|twochannel|zero> <out.bin> key=value...\n");
    return 2;
  }
  std::string model = argv[1];
  std::map<std::string, double> P = {{"eps", -0.25}, {"U", 0.5},  {"V", 0.1},   {"J", 0.25},
                                     {"lambda", 2.0}, {"nkeep", 512}, {"nsites", 40}, {"fdm", 0},
                                     {"thermo", 0},  {"dumpops", 0},  {"sysop", 0}, {"delta", 0}};
  for (int i = 3; i < argc; i++) {
    std::string a = argv[i];
    auto p = a.find('=');
    P[a.substr(0, p)] = atof(a.substr(p + 1).c_str());
  }
  Out o;
  if (model == "siam") {
    spinhalf imp(P["eps"], P["U"]), bath(0, 0);
    run(imp, bath, P, true, false, 2, o);
  } else if (model == "zero") {  // free chain: spinhalf(0,0) impurity, Kondo-style loop
    spinhalf imp(0, 0), bath(0, 0);
    run(imp, bath, P, false, true, 2, o);
  } else if (model == "kondo") {
    spinhalfKondo imp(P["J"], 0.5);
    spinhalf bath(0, 0);
    run(imp, bath, P, false, true, 2, o);
  } else if (model == "twochannel") {
    spinhalf imp(P["eps"], P["U"]);
    imp.f_dag_operator.push_back(imp.f_dag_operator[0]);
    imp.f_dag_operator.push_back(imp.f_dag_operator[1]);
    twoChannel bath;
    run(imp, bath, P, true, false, 4, o);
  } else if (model == "sc") {
    // superconducting bath: spinhalfSC sites (S_z sectors only) whose pairing
    // is refreshed before every site, delta Lambda^(n/2) at Wilson site n
    // (delta at the V site); models/spinhalfSC.hpp:26-125, nrgcore.hpp:68-70
    spinhalfSC imp(P["eps"], P["U"], 0.0), bath(0, 0, 0);
    const double delta = P["delta"], L = P["lambda"];
    run(imp, bath, P, true, false, 2, o,
        [&](int site) { bath.addSCDelta(site < 0 ? delta : delta * std::pow(L, 0.5 * site)); });
  } else {
    fprintf(stderr, "unknown model %s\n", model.c_str());
    return 2;
  }
  o.save(argv[2]);
  return 0;
}
