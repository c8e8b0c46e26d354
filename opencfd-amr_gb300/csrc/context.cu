// Context, parameters, status reporting and argument checks of the C ABI.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>

#include "ocfd_internal.h"
#include "mechanism.h"
#include "rhs_regular.h"
#include "eb_level.h"

namespace ocfd {

ocfd_status configure_chem();

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

ocfd_status fail(ocfd_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

ocfd_status check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(OCFD_LAUNCH_FAIL, std::string(what) + ": " + cudaGetErrorString(e));
    return OCFD_OK;
}

bool covers(const ocfd_array4* a, const ocfd_box& bx, int grow, int ncomp, int nodal_dir) {
    if (!a || !a->p || a->ncomp < ncomp) return false;
    for (int d = 0; d < 3; ++d) {
        int lo = bx.lo[d] - grow;
        int hi = bx.hi[d] + grow + (d == nodal_dir ? 1 : 0);
        if (a->begin[d] > lo || a->end[d] <= hi) return false;
    }
    return a->jstride > 0 && a->kstride > 0 && (ncomp <= 1 || a->nstride > 0);
}

bool covers_flag(const ocfd_flag4* a, const ocfd_box& bx, int grow) {
    if (!a || !a->p) return false;
    for (int d = 0; d < 3; ++d)
        if (a->begin[d] > bx.lo[d] - grow || a->end[d] <= bx.hi[d] + grow) return false;
    return true;
}

void* scratch(ocfd_context* ctx, size_t bytes) {
    if (bytes <= ctx->scratch_bytes) return ctx->scratch;
    if (ctx->scratch) cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    size_t want = bytes + bytes / 4;
    if (cudaMalloc(&ctx->scratch, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    ctx->scratch_bytes = want;
    return ctx->scratch;
}

DevParm make_dev_parm(const ocfd_parm& p) {
    DevParm d{};
    d.gamma = p.eos_gamma;
    d.Rg = p.Rg;
    d.smallr = p.smallr;
    d.smallp = p.smallp;
    d.C_s = p.C_s;
    d.T_s = p.T_s;
    d.kOverMu = p.kOverMu;
    d.twoThirds = p.twoThirds;
    d.Ru = p.Ru;
    d.Patm = p.Patm;
    double g = p.eos_gamma;
    d.sw_tmp1 = 1.0 / (2.0 * g);
    d.sw_tmp2 = 2.0 * (g - 1.0);
    d.sw_tmp3 = (3.0 - g) / (2.0 * (g - 1.0));
    d.sw_gm1 = g - 1;
    d.invRg = 1.0 / d.Rg;
    d.vl_rg = 1.0 / d.gamma;
    d.vl_rg21 = 1.0 / (2.0 * (d.gamma * d.gamma - 1.0));
    d.vl_ggm1 = d.gamma * (1.0 / (d.gamma - 1.0));
    d.f_gamma = (float)d.gamma;
    d.f_smallr = (float)d.smallr;
    d.f_smallp = (float)d.smallp;
    d.f_invRg = (float)(1.0 / d.Rg);
    d.f_C_s = (float)d.C_s;
    d.f_T_s = (float)d.T_s;
    d.f_kOverMu = (float)d.kOverMu;
    d.f_twoThirds = (float)d.twoThirds;
    d.f_sw_tmp1 = (float)d.sw_tmp1;
    d.f_sw_tmp2 = (float)d.sw_tmp2;
    d.f_sw_tmp3 = (float)d.sw_tmp3;
    d.f_sw_gm1 = (float)d.sw_gm1;
    // as the FP32 faces formed them from the rounded gamma
    const float fg = d.f_gamma;
    d.f_vl_rg = 1.0f / fg;
    d.f_vl_rg21 = 1.0f / (2.0f * (fg * fg - 1.0f));
    d.f_vl_ggm1 = fg * (1.0f / (fg - 1.0f));
    return d;
}

}  // namespace ocfd

using namespace ocfd;

extern "C" {

ocfd_status ocfd_parm_default(ocfd_parm* p) {
    if (!p) return fail(OCFD_BAD_ARG, "ocfd_parm_default: null parm");
    std::memset(p, 0, sizeof(*p));
    p->eos_gamma = 1.4;
    p->eos_m = 28.97e-3;
    p->Patm = 101325.0;
    p->Ru = 8.31446261815324;
    p->Pr = 0.72;
    p->C_s = 1.458e-6;
    p->T_s = 110.4;
    p->smallr = 1.e-19;
    p->smallp = 1.e-10;
    p->eps = 1.e-40;
    p->twoThirds = 2.0 / 3.0;
    p->oneSix = 1.0 / 6.0;
    p->Rg = p->Ru / p->eos_m;
    p->cv = p->Rg / (p->eos_gamma - 1.0);
    p->cp = p->eos_gamma * p->cv;
    p->kOverMu = p->cp / p->Pr;
    mech_host_tables(p);
    return OCFD_OK;
}

ocfd_status ocfd_context_create(const ocfd_parm* parm, int device, ocfd_context** out) {
    if (!parm || !out) return fail(OCFD_BAD_ARG, "ocfd_context_create: null argument");
    // the kernels apply the density and pressure floors by integer compares,
    // which order doubles correctly against a non-negative floor
    if (!(parm->smallr >= 0.0) || !(parm->smallp >= 0.0))
        return fail(OCFD_BAD_ARG, "ocfd_context_create: smallr and smallp must be >= 0");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(OCFD_NO_DEVICE, "ocfd_context_create: no CUDA device");
    }
    if (device < 0 || device >= ndev) return fail(OCFD_BAD_ARG, "ocfd_context_create: bad device index");
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return fail(OCFD_NO_DEVICE, "ocfd_context_create: cannot query device");
    if (prop.major != 10 || prop.minor != 3)
        return fail(OCFD_NO_DEVICE, "ocfd_context_create: library built for sm_103a, device is sm_" +
                                        std::to_string(prop.major) + std::to_string(prop.minor));
    if (cudaSetDevice(device) != cudaSuccess) return fail(OCFD_NO_DEVICE, "cudaSetDevice failed");
    ocfd_context* ctx = new ocfd_context();
    ctx->device = device;
    ctx->host_parm = *parm;
    ctx->parm = make_dev_parm(*parm);
    ctx->num_sms = prop.multiProcessorCount;
    if (cudaMalloc(&ctx->d_error, sizeof(uint32_t)) != cudaSuccess ||
        cudaMemset(ctx->d_error, 0, sizeof(uint32_t)) != cudaSuccess) {
        delete ctx;
        return fail(OCFD_OUT_OF_MEMORY, "ocfd_context_create: error word allocation");
    }
    ctx->parm.err = ctx->d_error;
    ocfd_status s = mech_upload(*parm);
    if (s == OCFD_OK) s = configure_rhs_regular();
    if (s == OCFD_OK) s = configure_rhs_regular_f32();
    if (s == OCFD_OK) s = configure_chem();
    if (s == OCFD_OK) s = configure_eb_tile();
    if (s == OCFD_OK) s = eb_static_scratch_resolve(ctx);
    if (s != OCFD_OK) {
        cudaFree(ctx->d_error);
        delete ctx;
        return s;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaFree(ctx->d_error);
        delete ctx;
        return fail(OCFD_LAUNCH_FAIL, "ocfd_context_create: device synchronize failed");
    }
    *out = ctx;
    return OCFD_OK;
}

ocfd_status ocfd_context_destroy(ocfd_context* ctx) {
    if (!ctx) return OCFD_OK;
    cudaSetDevice(ctx->device);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->d_error) cudaFree(ctx->d_error);
    delete ctx;
    return OCFD_OK;
}

ocfd_status ocfd_context_check(ocfd_context* ctx, void* stream, uint32_t* device_error) {
    if (!ctx) return fail(OCFD_BAD_ARG, "ocfd_context_check: null context");
    uint32_t w = 0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(&w, ctx->d_error, sizeof(w), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaError_t e = cudaGetLastError();
        return fail(OCFD_LAUNCH_FAIL, std::string("ocfd_context_check: ") + cudaGetErrorString(e));
    }
    if (device_error) *device_error = w;
    if (w & 1u) return fail(OCFD_NONFINITE, "device reported non-finite values");
    if (w & 2u) return fail(OCFD_TIMEOUT, "device reported a bounded wait that ran out");
    return OCFD_OK;
}

const char* ocfd_status_string(ocfd_status s) {
    switch (s) {
        case OCFD_OK: return "ok";
        case OCFD_BAD_ARG: return "bad argument";
        case OCFD_LAUNCH_FAIL: return "launch failure";
        case OCFD_TIMEOUT: return "device wait timed out";
        case OCFD_NONFINITE: return "non-finite values";
        case OCFD_GUARD_FALLBACK: return "surrogate guard fallback";
        case OCFD_NO_DEVICE: return "no suitable device";
        case OCFD_OUT_OF_MEMORY: return "out of memory";
        case OCFD_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

const char* ocfd_last_error(void) { return ocfd::g_last_error.c_str(); }

int ocfd_version(void) { return 1; }

int ocfd_built_arch(void) { return 1030; }

}  // extern "C"
