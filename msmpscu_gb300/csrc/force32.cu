// force32.cu -- mixed-precision force passes (placeholder until the FP32 kernels land).
#include "msmgb_internal.cuh"

namespace msmgb {

int launch_density32(msmgb_ctx *c)
{
    return set_err(c, MSMGB_ERR_ARG, "mixed-precision passes are not built in this library");
}

int launch_force32(msmgb_ctx *c)
{
    return set_err(c, MSMGB_ERR_ARG, "mixed-precision passes are not built in this library");
}

}  // namespace msmgb
