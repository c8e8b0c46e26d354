// Li-Dryer chemistry on the GPU: mechanism tables in constant memory and the
// kernels that read them (real-gas primitives, transport, multispecies RHS,
// implicit chemistry substep).
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "mechanism.h"
#include "ocfd_internal.h"

namespace ocfd {

void mech_builtin(MechTables* t);

__constant__ MechTables c_mech;

ocfd_status mech_upload(const ocfd_parm& p) {
    MechTables t;
    mech_builtin(&t);
    auto fetch = [](double* dst, const double* src, size_t n) -> bool {
        if (!src) return true;
        return cudaMemcpy(dst, src, n * sizeof(double), cudaMemcpyDefault) == cudaSuccess;
    };
    const double* lo[NSP] = {p.H2_lo, p.O2_lo, p.H2O_lo, p.H_lo, p.O_lo, p.OH_lo, p.HO2_lo, p.H2O2_lo, p.N2_lo};
    const double* hi[NSP] = {p.H2_hi, p.O2_hi, p.H2O_hi, p.H_hi, p.O_hi, p.OH_hi, p.HO2_hi, p.H2O2_hi, p.N2_hi};
    bool ok = fetch(t.mw, p.mw, NSP);
    for (int n = 0; n < NSP; ++n) ok = ok && fetch(t.lo[n], lo[n], 7) && fetch(t.hi[n], hi[n], 7);
    ok = ok && fetch(t.HP, p.HP, NSP) && fetch(t.A0, p.A0, NSP) && fetch(t.visc, p.visccoeff, NSP * 5) &&
         fetch(t.cond, p.conductcoeff, NSP * 5) && fetch(t.diff, p.diffcoeff, 45 * 5);
    if (!ok) {
        cudaGetLastError();
        return fail(OCFD_BAD_ARG, "mechanism tables: cannot read the Parm table pointers");
    }
    if (cudaMemcpyToSymbol(c_mech, &t, sizeof(t)) != cudaSuccess) {
        cudaError_t e = cudaGetLastError();
        return fail(OCFD_LAUNCH_FAIL, std::string("mechanism upload: ") + cudaGetErrorString(e));
    }
    return OCFD_OK;
}

}  // namespace ocfd
