// Tensor-core (tcgen05) E-step and M-step of the fused iteration.
#include "plan.cuh"

namespace emc {
int tc_bind(emc_plan* p) { return fail(p->ctx, EMC_ERR_UNSUPPORTED, "mixed precision path not built yet"); }
int tc_estep(emc_plan* p, float) { return fail(p->ctx, EMC_ERR_UNSUPPORTED, "mixed precision path not built yet"); }
int tc_mstep(emc_plan* p, float*, float*) { return fail(p->ctx, EMC_ERR_UNSUPPORTED, "mixed precision path not built yet"); }
}  // namespace emc
