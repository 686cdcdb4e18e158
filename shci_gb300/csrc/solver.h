// Host-side solver flow on top of the device stages.
#pragma once

#include <cstddef>
#include <vector>

struct shci_ctx;

namespace shci {

struct VarIter {
  size_t n_dets;
  size_t nnz_sym;     // the reference's symmetric element count
  double energy;      // reported energy (FP64-corrected in mixed mode)
  double eval;        // Davidson eigenvalue
  bool converged;
  int n_matvec;
  std::vector<double> energies;  // every state's reported energy (n_states > 1)
};

std::vector<double> run_all_variations(shci_ctx* c, const std::vector<double>& eps_vars,
                                       const std::vector<double>& schedule, double target_error,
                                       int precision, bool var_sd, std::vector<VarIter>* trace);

}  // namespace shci
