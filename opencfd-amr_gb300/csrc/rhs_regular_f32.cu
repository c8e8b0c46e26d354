// Mixed-precision regular-box RHS (placeholder until the FP32 kernels land).
#include "ocfd_internal.h"
#include "rhs_regular.h"

namespace ocfd {

ocfd_status rhs_regular_box_f32(ocfd_context*, const ocfd_array4*, const ocfd_array4*,
                                const ocfd_array4*, const ocfd_box&, const double*, unsigned,
                                void*) {
    return fail(OCFD_UNSUPPORTED, "OCFD_FLUX_FP32 not available in this build");
}

}  // namespace ocfd
