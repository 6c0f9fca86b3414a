/* Prints sizeof/offsetof of the C-ABI structs, compared by tests/test_host.py
 * with the ctypes declarations of the Python host binding. */
#include <stddef.h>
#include <stdio.h>
#include "qgybj.h"
#define OFF(s, f) printf("%s.%s %zu\n", #s, #f, offsetof(s, f))
int main(void) {
  printf("sizeof.qg_config %zu\n", sizeof(qg_config));
  OFF(qg_config, n1); OFF(qg_config, n3); OFF(qg_config, precision); OFF(qg_config, device);
  OFF(qg_config, ybj_plus); OFF(qg_config, inviscid); OFF(qg_config, dz); OFF(qg_config, Bu);
  OFF(qg_config, delt); OFF(qg_config, gamma); OFF(qg_config, nuh1); OFF(qg_config, nuh2w);
  OFF(qg_config, ilap1); OFF(qg_config, ilap2w); OFF(qg_config, nuz); OFF(qg_config, a_ell_ut);
  OFF(qg_config, rho_ut); OFF(qg_config, rho_st); OFF(qg_config, r_2ut); OFF(qg_config, levels_per_batch);
  OFF(qg_config, use_graphs); OFF(qg_config, solve_columns);
  printf("sizeof.qg_tuning %zu\n", sizeof(qg_tuning));
  OFF(qg_tuning, levels_per_batch); OFF(qg_tuning, ms_per_step); OFF(qg_tuning, ncandidates);
  OFF(qg_tuning, candidates); OFF(qg_tuning, candidate_ms); OFF(qg_tuning, solve_columns);
  OFF(qg_tuning, nsolve); OFF(qg_tuning, solve_candidates); OFF(qg_tuning, solve_candidate_ms);
  printf("sizeof.qg_energy %zu\n", sizeof(qg_energy));
  OFF(qg_energy, wke); OFF(qg_energy, wpe); OFF(qg_energy, wce); OFF(qg_energy, ke); OFF(qg_energy, pe);
  OFF(qg_energy, zeta2); OFF(qg_energy, omegah2);
  return 0;
}
