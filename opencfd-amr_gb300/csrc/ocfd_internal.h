// Internal host/device declarations of the ocfd library (not installed).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "ocfd/ocfd.h"

namespace ocfd {

// Scalars of Parm the kernels read, plus constants derived once on the host
// (in double, exactly as the reference derives them per point).
struct DevParm {
    double gamma, Rg, smallr, smallp;
    double C_s, T_s, kOverMu, twoThirds;
    double Ru, Patm;
    double sw_tmp1, sw_tmp2, sw_tmp3;  // 1/(2g), 2(g-1), (3-g)/(2(g-1)): FluxSplit.H:31-34
    double sw_gm1;                     // (g - 1) as written `(gamma - 1)` in FluxSplit.H:41
    double invRg;                      // 1 / Rg
    double vl_rg, vl_rg21, vl_ggm1;    // 1/g, 1/(2(g^2-1)), g/(g-1): the Van Leer flux (EBkernels.H:73-171)
    double grav;                       // 0, or g = -9.8 when a call asks for OCFD_GRAVITY
    uint32_t* err;                     // the context's device error word (bit 1: a bounded wait ran out)
    // the same constants rounded to FP32 once on the host, for the mixed form
    float f_gamma, f_smallr, f_smallp, f_invRg, f_C_s, f_T_s, f_kOverMu, f_twoThirds;
    float f_sw_tmp1, f_sw_tmp2, f_sw_tmp3, f_sw_gm1;
    float f_vl_rg, f_vl_rg21, f_vl_ggm1;
};

// Device view of an Array4 (same addressing as amrex::Array4).
template <class T>
struct View {
    T* p;
    long long js, ks, ns;
    int b0, b1, b2;
    __host__ __device__ __forceinline__ T& operator()(int i, int j, int k, int n = 0) const {
        return p[(long long)(i - b0) + (long long)(j - b1) * js + (long long)(k - b2) * ks +
                 (long long)n * ns];
    }
};

template <class T>
inline View<T> view_of(const ocfd_array4* a) {
    return View<T>{reinterpret_cast<T*>(a->p), a->jstride, a->kstride, a->nstride,
                   a->begin[0], a->begin[1], a->begin[2]};
}
inline View<const uint32_t> view_of_flag(const ocfd_flag4* a) {
    return View<const uint32_t>{a->p, a->jstride, a->kstride, a->nstride,
                                a->begin[0], a->begin[1], a->begin[2]};
}

}  // namespace ocfd

struct ocfd_context {
    int device = 0;
    ocfd::DevParm parm{};
    ocfd_parm host_parm{};
    uint32_t* d_error = nullptr;   // device error word
    void* scratch = nullptr;       // scratch pool owned by the context
    size_t scratch_bytes = 0;
    int num_sms = 0;
    double* eb_static_scratch = nullptr;  // device address of the allocation-free variant's array
};

namespace ocfd {

void set_error(const std::string& msg);
ocfd_status fail(ocfd_status s, const std::string& msg);
ocfd_status check_launch(const char* what);

// Checks that `a` covers the cell box [lo-grow, hi+grow] (nodal in `nodal_dir`
// when >= 0) with at least `ncomp` components.
bool covers(const ocfd_array4* a, const ocfd_box& bx, int grow, int ncomp, int nodal_dir = -1);
bool covers_flag(const ocfd_flag4* a, const ocfd_box& bx, int grow);

// Ensures the context scratch pool holds at least `bytes`; returns its pointer.
void* scratch(ocfd_context* ctx, size_t bytes);

// Looks up the device address of the allocation-free cut-cell entry point's
// static array for ctx's device (which must be current); loads eb.cu's device
// code, so that the array is resident from context creation on.
ocfd_status eb_static_scratch_resolve(ocfd_context* ctx);

}  // namespace ocfd
