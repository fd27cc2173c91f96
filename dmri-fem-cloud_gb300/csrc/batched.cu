// Batched mixed-precision stepper (placeholder until the SpMM path lands).
#include "bt_common.cuh"

namespace bt {

struct SolverMixed {};

void solve_mixed(bt_ctx*, int32_t, const double*, const double*, const int32_t*, const double*, double, int32_t,
                 double*, double*, bt_stats*) {
    throw Error(BT_ERR_INVALID, "mixed precision is not available in this build");
}
void get_solution_mixed(bt_ctx*, int32_t, double*) {
    throw Error(BT_ERR_INVALID, "mixed precision is not available in this build");
}
void free_solver_mixed(bt_ctx* ctx) {
    delete ctx->smx;
    ctx->smx = nullptr;
}

}  // namespace bt
