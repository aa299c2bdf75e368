// C++ driver through include/nrgcore_gpu.hpp, written like the reference's
// examples/entropyKondo/main.cpp: Kondo RG flow with the entropy from the
// backward pass.  The models are plain structs with the reference's model
// concept, filled from a binary description written by the Python test.
//
// usage: shim_kondo <models.bin> <out.bin> <precision 0|1> <nsites> <lambda> <nkeep>
#include "nrgcore_gpu.hpp"
#include "shim_models.hpp"

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
