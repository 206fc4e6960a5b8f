// euler_split.cu -- split-precision DG Euler stage (placeholder until the
// tensor-core kernel lands: reports "not built").
#include "../../include/dgcu.h"
#include "dg_ctx.hpp"

namespace dgk {

cudaError_t launch_euler_split(int, const EulerArgs&, const SplitPlan&, cudaStream_t) { return cudaErrorNotSupported; }

}  // namespace dgk

int split_setup(dg_ctx* c) {
    c->split.ready = false;
    return DG_ERR_UNSUPPORTED;
}

void split_teardown(dg_ctx*) {}
