/* Prints sizeof/offsetof of every struct in include/gpe.h as JSON, so the
 * ctypes declarations of the Python host mirror can be checked against the
 * C compiler's layout (tests/test_abi.py). */
#include <stddef.h>
#include <stdio.h>

#include "gpe.h"

#define F(T, m) printf("\"%s.%s\": %zu, ", #T, #m, offsetof(T, m))
#define S(T) printf("\"%s\": %zu, ", #T, sizeof(T))

int main(void) {
    printf("{");
    S(gpe_grid_desc); F(gpe_grid_desc, n); F(gpe_grid_desc, dx); F(gpe_grid_desc, span);
    F(gpe_grid_desc, precision); F(gpe_grid_desc, device);
    S(gpe_params); F(gpe_params, n_recalc); F(gpe_params, itp_adjust_stepsize); F(gpe_params, omega);
    S(gpe_itp_params); F(gpe_itp_params, fp64_polish); F(gpe_itp_params, switch_delta);
    S(gpe_itp_result); F(gpe_itp_result, final_dt); F(gpe_itp_result, last_delta); F(gpe_itp_result, ms_fp64);
    S(gpe_split_params); F(gpe_split_params, vtd); F(gpe_split_params, on_step); F(gpe_split_params, step_user);
    S(gpe_adjoint_params); F(gpe_adjoint_params, checkpoint_every); F(gpe_adjoint_params, mem_budget);
    F(gpe_adjoint_params, precision);
    S(gpe_sgpe_params); F(gpe_sgpe_params, ecut); F(gpe_sgpe_params, seed);
    S(gpe_current); F(gpe_current, current_time);
    S(gpe_obs); F(gpe_obs, energy); F(gpe_obs, ecpl);
    S(gpe_spinor_params); F(gpe_spinor_params, coupling_re); F(gpe_spinor_params, nlincpl);
    S(gpe_kernel_stat); F(gpe_kernel_stat, launches); F(gpe_kernel_stat, bytes_per_launch);
    printf("\"end\": 0}\n");
    return 0;
}
