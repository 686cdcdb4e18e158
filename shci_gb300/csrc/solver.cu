// Variational stage on the device: Solver<S>::run_all_variations / run_variation
// (src/solver/solver.h:338-397, 413-539), driving selection (select.cu), the Hamiltonian build
// (hbuild.cu) and Davidson (davidson.cu; several states when c->n_states > 1).
#include <cmath>

#include "ctx.h"
#include "kernels.h"
#include "solver.h"

namespace shci {

// src/solver/solver.h:413-539
static double run_variation(shci_ctx* c, double eps_var, bool until_converged, double target_error,
                            int precision, bool var_sd, std::vector<VarIter>* trace) {
  size_t n_dets = c->up.size();
  size_t n_dets_new = n_dets;
  double energy_prev = 0.0;
  bool converged = false, dets_converged = false;
  while (!converged) {
    if (!dets_converged) {
      n_dets_new = n_dets + select_dets(c, eps_var, var_sd);
      build_hamiltonian(c, precision);
    }
    const double tol = until_converged ? target_error / 500000 : target_error / 50;
    DavidsonOut r;
    if (c->n_states == 1) {
      r = davidson(c, tol);
      c->state_energy.assign(1, r.eval);
      if (precision == SHCI_PREC_MIXED) c->state_energy[0] = rayleigh_fp64(c);  // FP64 correction
    } else {
      DavidsonStatesOut rs = davidson_states(c, tol);
      r.eval = rs.evals[0];
      r.converged = rs.converged;
      r.n_matvec = rs.n_matvec;
      c->state_energy = rs.evals;
      if (precision == SHCI_PREC_MIXED)
        for (unsigned k = 0; k < c->n_states && k < c->H.n; k++)
          c->state_energy[k] = rayleigh_fp64_of(c, state_coef(c, k));
    }
    const double e = c->state_energy[0];
    if (trace)
      trace->push_back(VarIter{n_dets_new, 2 * (c->H.nnz + c->H.n) - c->H.n, e, r.eval,
                               r.converged, r.n_matvec, c->state_energy});
    if (n_dets_new < n_dets * 1.001) dets_converged = true;
    if (dets_converged && r.converged) converged = true;
    n_dets = n_dets_new;
    energy_prev = e;
    if (!until_converged) break;
  }
  return energy_prev;
}

std::vector<double> run_all_variations(shci_ctx* c, const std::vector<double>& eps_vars,
                                       const std::vector<double>& schedule, double target_error,
                                       int precision, bool var_sd, std::vector<VarIter>* trace) {
  if (!c->Q.built) upload_queues(c);
  std::vector<double> energies;
  double eps_var_prev = 1.0e100;
  size_t it = 0;
  for (double eps_var : eps_vars) {
    while (it < schedule.size() && schedule[it] >= eps_var_prev) it++;
    while (it < schedule.size() && schedule[it] > eps_var) {
      run_variation(c, schedule[it], false, target_error, precision, var_sd, trace);
      it++;
    }
    energies.push_back(run_variation(c, eps_var, true, target_error, precision, var_sd, trace));
    eps_var_prev = eps_var;
  }
  return energies;
}

}  // namespace shci
