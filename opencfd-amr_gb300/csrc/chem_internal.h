// Multispecies internals shared by chem.cu (kernels) and react.cu (the
// reacting level driver).
#pragma once

#include <cuda_runtime.h>

#include "mechanism.h"
#include "ocfd_internal.h"

namespace ocfd {

constexpr int kChemThreads = 128;

// Per-thread 9x10 matrix in shared memory, element-major so that the threads
// of a warp touch consecutive words.
struct SmemMat {
    double* base;
    int stride;
    __device__ __forceinline__ double& operator()(int r, int c) const { return base[(r * 10 + c) * stride]; }
};

struct CellBox {
    int lo[3], n[3];
    __host__ __device__ __forceinline__ long long count() const { return (long long)n[0] * n[1] * n[2]; }
    __device__ __forceinline__ void cell(long long c, int& i, int& j, int& k) const {
        i = lo[0] + (int)(c % n[0]);
        j = lo[1] + (int)((c / n[0]) % n[1]);
        k = lo[2] + (int)(c / ((long long)n[0] * n[1]));
    }
};

struct ChemBoxArgs {
    View<const double> S, sp;
    View<double> dsdt, dsdts;
    View<double> flux[3], fluxs[3];
    View<double> q;    // 8 primitives over grow(bx, qg)
    int qg;            // primitive halo: 3 (WENO, regular boxes) or 2 (MUSCL, cut boxes)
    View<double> tr;   // mu, lambda, D[9] over grow(bx, 1)
    int lo[3], hi[3];
    double dxinv[3];
    int visc;
    // mixed precision: split and WENO-Z of the faces in FP32 (the viscous,
    // diffusive and enthalpy fluxes, the primitives and the transport stay FP64)
    int f32;
    // cut-cell variant
    int eb;
    View<const uint32_t> flag;
    View<const double> vfrac;
    View<const double> ap[3];
};

// Scratch (doubles) of one regular box's multispecies RHS without external
// face arrays, and the argument block carving it.
size_t chem_rhs_scratch_doubles(const ocfd_box& bx);
void chem_rhs_args(ChemBoxArgs& B, View<const double> S, View<const double> sp, View<double> dsdt,
                   View<double> dsdts, const ocfd_box& bx, const double dxinv[3], bool visc, double* scr);
ocfd_status launch_chem_rhs(const ChemBoxArgs& B, const DevParm& P, int sms, cudaStream_t st);
// the cut-cell chain of a box (B.eb set) and the switch of regular arguments
// (chem_rhs_args) to it: primitive halo 2, the box's cut-cell geometry; FP64
ocfd_status launch_chem_eb_rhs(const ChemBoxArgs& B, const DevParm& P, int sms, cudaStream_t st);
void chem_args_as_cut(ChemBoxArgs& B, View<const uint32_t> flag, View<const double> vfrac,
                      const View<const double> ap[3]);
// one implicit chemistry substep per cell; with `renorm` the species clip and
// rescale of Source/EBR.cpp:333-357 follows in the same thread (a step's last
// substep)
ocfd_status launch_chem_advance(View<double> S, View<double> sp, const CellBox& B, double dt, const DevParm& P,
                                cudaStream_t st, bool renorm = false);
ocfd_status launch_chem_advance_list(const long long* off, const long long* stride, long long ncell, double* U,
                                     double dt, const DevParm& P, cudaStream_t st, const unsigned* count = nullptr,
                                     const double* dtc = nullptr, bool renorm = false);
ocfd_status launch_chem_surrogate(const ocfd_mlp* mlp, const long long* off, const long long* stride, long long ncell,
                                  double* U, double dt, const DevParm& P, const ocfd_surrogate_guard& g,
                                  long long* fb_off, long long* fb_stride, unsigned* fb_count,
                                  unsigned long long* fb_total, unsigned* err, int sms, cudaStream_t st);
ocfd_status launch_spec_renorm(View<const double> S, View<double> sp, const CellBox& B, int sms, cudaStream_t st);

}  // namespace ocfd
