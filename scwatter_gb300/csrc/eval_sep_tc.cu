// Tensor-core (tcgen05) output GEMM of the separable evaluator -- placeholder until the
// UMMA path lands; every call reports SCW_ERR_UNSUPPORTED.
#include "scw_sep.h"

namespace scw {
scw_status sep_synth_tc(scw_ctx, const float2*, const float2*, int, int, int, float*, int) {
    return SCW_ERR_UNSUPPORTED;
}
}  // namespace scw
