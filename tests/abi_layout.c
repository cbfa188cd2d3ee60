/* Prints the size and field offsets of the C ABI structs of include/scft.h, one
   per line, so that tests/test_abi.py can check the ctypes mirror against the
   compiler's layout. */
#include <stddef.h>
#include <stdio.h>

#include "scft.h"

#define F(T, m) printf(#T "." #m " %zu\n", offsetof(T, m))
int main(void) {
  printf("scft_config %zu\n", sizeof(scft_config));
  F(scft_config, n_nodes); F(scft_config, x); F(scft_config, L); F(scft_config, f0);
  F(scft_config, nsteps); F(scft_config, ds); F(scft_config, rule); F(scft_config, sign);
  F(scft_config, precision); F(scft_config, scheme); F(scft_config, wmode); F(scft_config, w_wall);
  printf("scft_instance %zu\n", sizeof(scft_instance));
  F(scft_instance, n_nodes); F(scft_instance, x); F(scft_instance, L); F(scft_instance, f0);
  F(scft_instance, w0); F(scft_instance, nsteps); F(scft_instance, ds); F(scft_instance, rule);
  printf("scft_solve_opts %zu\n", sizeof(scft_solve_opts));
  F(scft_solve_opts, precision); F(scft_solve_opts, tol); F(scft_solve_opts, tol32_factor);
  F(scft_solve_opts, verify64); F(scft_solve_opts, maxit); F(scft_solve_opts, depth);
  F(scft_solve_opts, beta); F(scft_solve_opts, clip); F(scft_solve_opts, grow); F(scft_solve_opts, reg);
  F(scft_solve_opts, residual_mode); F(scft_solve_opts, precond); F(scft_solve_opts, iters_per_graph);
  F(scft_solve_opts, beta_schedule); F(scft_solve_opts, weighted); F(scft_solve_opts, step_cap);
  F(scft_solve_opts, field_floor); F(scft_solve_opts, fused);
  F(scft_solve_opts, finish_stall); F(scft_solve_opts, finish_tol); F(scft_solve_opts, budget_ms);
  F(scft_solve_opts, forks); F(scft_solve_opts, fork_at); F(scft_solve_opts, fork_grace);
  F(scft_solve_opts, fork_first); F(scft_solve_opts, fork_err); F(scft_solve_opts, transfer_stride);
  F(scft_solve_opts, fork_scale); F(scft_solve_opts, graded_ratio); F(scft_solve_opts, precond_hfloor);
  printf("scft_result %zu\n", sizeof(scft_result));
  F(scft_result, status); F(scft_result, iterations); F(scft_result, err); F(scft_result, Q);
  return 0;
}
