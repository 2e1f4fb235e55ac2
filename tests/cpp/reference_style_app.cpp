// A reference-style application (the call sequence of a classicalDFT app) built
// against include/classicaldft_gb300.hpp: config 1 (hard spheres, WhiteBearI,
// 32^3 at dx = 0.2, rho = 0.7 (1 + noise)), one evaluation, then FIRE2 steps.
// Prints "Omega F_hs mu steps F_final sum(Hv) sum|Hv| max|snapshot - density| Omega_AO log_det
// lambda_max max|dF| sum(dF) F_resumed steps_resumed" for the test to compare.
#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "classicaldft_gb300.hpp"

using namespace classicaldft_gb300;

static double splitmix_uniform(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

int main(int argc, char** argv) {
  int fire_steps = argc > 1 ? std::atoi(argv[1]) : 20;
  double L[3] = {6.4, 6.4, 6.4};
  Density density(0.2, L);
  uint64_t seed = 20240601;
  for (long p = 0; p < density.Ntot(); ++p) density.set(p, 0.7 * (1.0 + 0.05 * (2.0 * splitmix_uniform(seed) - 1.0)));
  FMT_Species species(density, 1.0, 0.0);
  WhiteBearI fmt;
  DFT dft(&species);
  dft.addHardCoreContribution(&fmt);
  species.setChemPotential(dft.mu_times_beta(0.7));
  double F = dft.calculateFreeEnergyAndDerivatives(false);
  double Fhs = dft.get_f_hs();
  // the derivative as the reference hands it out: a DFT_Vec with its BLAS-1 calls
  const double dF_inf = dft.getDF(0).inf_norm(), dF_accu = dft.getDF(0).accu();
  // Hessian . v at this density (DFT::matrix_dot_v1), v_i = 0.3 (2u - 1) from splitmix64(77)
  DFT_Vec v(density.Ntot()), Hv;
  uint64_t vs = 77;
  for (unsigned i = 0; i < v.size(); ++i) v.set(i, 0.3 * (2.0 * splitmix_uniform(vs) - 1.0));
  dft.matrix_dot_v1(v, Hv, nullptr);
  double hsum = Hv.accu(), habs = 0;
  for (unsigned i = 0; i < Hv.size(); ++i) habs += std::fabs(Hv.get(i));
  // the spectral drivers at this density: Log_Det (order 6, one probe, seed 1234, spectrum
  // bracket [0.005, 0.2]) and Eigenvalues with change_sign (the largest eigenvalue)
  Log_Det ld(dft, 6, 0.2, 0.005);
  double ld_var = 0;
  const double logdet = ld.calculate_log_det(1234, 1, false, ld_var);
  Eigenvalues eig(dft);
  eig.set_change_sign(true);
  eig.set_tolerence(1e-10);
  eig.calculate_eigenvector();
  const double lam_max = eig.get_eigenvalue();
  // FIRE2 writes snapshot_s0.dat at its 1st, 11th, ... step, as the reference does; its
  // state is saved after the run and a second minimizer resumes it for 10 more steps
  fireMinimizer2 fire(&dft);
  fire.setForceTerminationCriterion(0.0);
  fire.run(fire_steps);
  fire.save_state("fire.state");
  const double F_run = fire.getF();
  const long steps_run = fire.report().total_steps;
  fireMinimizer2 resumed(&dft);
  resumed.setSnapshots(false);
  resumed.load_state("fire.state");
  resumed.run(10);
  const double F_resumed = resumed.getF();
  // the density files (src/Density.cpp:197-244): snapshot round trip, and the VTK file
  density.writeDensity("snapshot.dat");
  Density back(0.2, L);
  back.readDensity("snapshot.dat");
  double snap_diff = 0;
  for (long p = 0; p < density.Ntot(); ++p) snap_diff = std::max(snap_diff, std::fabs(back.get(p) - density.get(p)));
  density.write_VTK_File("snapshot");
  // optional: an FMT_AO_Species system (WhiteBearI, d = 1, Rp = 0.35, reservoir 0.4) on the
  // 16^3, dx = 0.2 density read from the snapshot argv[2]
  double FA = 0;
  if (argc > 2) {
    double LA[3] = {3.2, 3.2, 3.2};
    Density dA(0.2, LA);
    dA.readDensity(argv[2]);
    FMT_AO_Species sa(dA, 1.0, 0.35, 0.4, 0.0, 0);
    WhiteBearI fmtA;
    DFT dftA(&sa);
    dftA.addHardCoreContribution(&fmtA);
    sa.setChemPotential(dftA.mu_times_beta(0.4));
    FA = dftA.calculateFreeEnergyAndDerivatives(false);
  }
  std::printf("%.17g %.17g %.17g %ld %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %ld\n", F, Fhs,
              species.getChemPotential(), steps_run, F_run, hsum, habs, snap_diff, FA, logdet, lam_max, dF_inf, dF_accu, F_resumed,
              resumed.report().total_steps);
  return 0;
}
