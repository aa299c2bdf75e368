// A driver in the form of the reference's examples/entropySIAM/main.cpp
// (forward RG flow, NrgData snapshots, fdmThermodynamics backward pass with
// the caller decrementing nrg_iterations_cnt before loadCurrentData()), with
// the impurity occupancy n_d tracked by update_system_operator(&siam, nd)
// and averaged through setSystemOperator(&nd).  Only the includes and the
// `using namespace` differ from a reference driver: the constructor, the
// calls and the class template argument deduction are the reference's.
//
// usage: shim_entropy_siam <models.bin> <out.bin> <nsites> <lambda> <nkeep> <V>
// models.bin: impurity, bath, the n_d operator, the temperature grid.
#include <cstdlib>
#include <iostream>

#include "nrgcore_gpu.hpp"
#include "shim_models.hpp"
using namespace nrg_gpu;

int main(int argc, char **argv) {
  if (argc < 7) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  Model impurity = read_model(f), bathModel = read_model(f);
  std::vector<Op> nd = read_ops(f);
  std::vector<double> temperatureArray(rd_i(f));
  for (auto &t : temperatureArray) t = rd_d(f);
  std::fclose(f);
  const int nMax = std::atoi(argv[3]);
  const double LAMBDA = std::atof(argv[4]), V = std::atof(argv[6]);
  const size_t nkeep = size_t(std::atol(argv[5]));
  try {
    nrgcore<Model, Model> siam(impurity, bathModel);
    siam.set_parameters(nkeep);
    siam.add_bath_site({V, V}, 1.0);
    update_system_operator(&siam, nd);
    siam.update_internal_state();
    NrgData rawData(&siam);
    size_t minIterations = 0;
    std::vector<std::vector<double>> eigs;
    for (int in = 0; in < nMax; in++) {
      double rescale = 1.0;
      if (in > 0) rescale = std::sqrt(LAMBDA);
      siam.add_bath_site({hopping(in, LAMBDA), hopping(in, LAMBDA)}, rescale);
      update_system_operator(&siam, nd);
      if (siam.checkHigherEnergyDiscarded()) {
        rawData.saveCurrentData();
      } else {
        minIterations++;
      }
      siam.update_internal_state();
      eigs.push_back(siam.all_eigenvalue);
    }
    // public members a driver reads
    size_t kept = 0;
    for (auto &k : siam.eigenvaluesQ_kept_indices) kept += k.size();
    if (kept < nkeep) throw std::runtime_error("eigenvaluesQ_kept_indices: fewer kept states than Nkeep");
    // as in the reference, update_internal_state moved current_sysmQ into
    // pre_sysmQ (nrgcore.hpp:105-109), so get_basis_nQ() throws here
    bool threw = false;
    try {
      siam.get_basis_nQ();
    } catch (const std::runtime_error &) {
      threw = true;
    }
    if (!threw || siam.pre_sysmQ.empty() || siam.get_eigenvaluesQ().size() != siam.pre_sysmQ.size())
      throw std::runtime_error("sector members");
    if (siam.nq_bath.size() != bathModel.get_basis().size()) throw std::runtime_error("nq_bath");
    auto *fdag = siam.getPreWilsonSiteOperators();
    if (fdag->size() != impurity.f_dag_operator.size() || (*fdag)[0].getMap()->empty())
      throw std::runtime_error("getPreWilsonSiteOperators");
    double nd_norm2 = 0;  // basis-invariant content of the rotated n_d
    for (auto &kv : *nd[0].getMap())
      for (double x : kv.second.v) nd_norm2 += x * x;
    // backward iteration (entropySIAM/main.cpp:79-93)
    fdmThermodynamics fdmTc(&siam, temperatureArray);
    fdmTc.setSystemOperator(&nd);
    for (size_t in = size_t(nMax); in > minIterations; in--) {
      double enScale = std::pow(LAMBDA, -(1.0 * static_cast<double>(in) - 1.0) / 2.0);
      siam.nrg_iterations_cnt--;
      rawData.loadCurrentData();
      fdmTc.calcThermodynamics(enScale);
    }
    Sink rfile;
    fdmTc.saveFinalData(&rfile);
    // the last loaded shell's operator set back in the caller's type
    std::vector<Op> ndShell;
    rawData.loadqOperator(&ndShell, "ndOperator");
    FILE *o = std::fopen(argv[2], "wb");
    const int n = int(eigs.size());
    std::fwrite(&n, 4, 1, o);
    for (auto &v : eigs) write_vec(o, v);
    write_vec(o, rfile.d1["entropy"]);
    write_vec(o, rfile.d1["qsysOPeratorExpValue0"]);
    write_vec(o, {nd_norm2, double(ndShell.size()), double(ndShell.empty() ? 0 : ndShell[0].getMap()->size())});
    std::fclose(o);
  } catch (const std::exception &x) {
    std::cerr << x.what() << std::endl;
    return 1;
  }
  return 0;
}
