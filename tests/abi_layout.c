/* Prints sizeof/offsetof of the C-ABI structs, compared by tests/test_host.py
 * with the ctypes declarations of the Python host binding. */
#include <stddef.h>
#include <stdio.h>
#include "qgybj.h"
#define OFF(f) printf("%s %zu\n", #f, offsetof(qg_config, f))
int main(void) {
  printf("sizeof %zu\n", sizeof(qg_config));
  OFF(n1); OFF(n3); OFF(precision); OFF(device); OFF(ybj_plus); OFF(inviscid); OFF(dz); OFF(Bu); OFF(delt);
  OFF(gamma); OFF(nuh1); OFF(nuh2w); OFF(ilap1); OFF(ilap2w); OFF(nuz); OFF(a_ell_ut); OFF(rho_ut); OFF(rho_st);
  OFF(r_2ut); OFF(levels_per_batch); OFF(use_graphs); OFF(solve_columns);
  printf("tuning %zu\n", sizeof(qg_tuning));
  printf("energy %zu\n", sizeof(qg_energy));
  return 0;
}
