// Mixed-precision regular-box RHS (placeholder until the FP32 kernels land).
#include "ocfd_internal.h"
#include "rhs_regular.h"

namespace ocfd {

ocfd_status rhs_regular_box_f32(ocfd_context*, const ocfd_array4*, const ocfd_array4*,
                                const ocfd_array4*, const ocfd_box&, const double*, unsigned,
                                void*) {
    return fail(OCFD_UNSUPPORTED, "OCFD_FLUX_FP32 not available in this build");
}

ocfd_status launch_rhs_regular_f32(int, bool, const RegBoxArgs*, const int*, int, const RegBoxArgs&,
                                   int, const DevParm&, cudaStream_t) {
    return fail(OCFD_UNSUPPORTED, "OCFD_FLUX_FP32 not available in this build");
}

ocfd_status configure_rhs_regular_f32() { return OCFD_OK; }

}  // namespace ocfd
