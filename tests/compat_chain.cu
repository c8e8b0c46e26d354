// Test driver of include/ocfd/compat.H, compiled for the host by
// tests/test_compat.py: the reference's regular-box chain of
// Source/Advance.cpp:245-329 - c2prim and the Steger-Warming split over
// grow(bx, 4), WENO-Z and the viscous flux over each direction's faces, divop over
// the box - written with the source-compatible per-point functions, in the
// reference's loop order.
#include <vector>

#include "ocfd/compat.H"
#include "ocfd/ocfd.h"

namespace {

// an amrex::Array4-like view: (i, j, k, n) with a lower corner
struct Arr {
    double* p;
    int b[3], e[3];  // begin, end (exclusive)
    long long js, ks, ns;
    Arr(double* ptr, const int lo[3], const int hi[3]) : p(ptr) {
        for (int d = 0; d < 3; ++d) {
            b[d] = lo[d];
            e[d] = hi[d] + 1;
        }
        js = e[0] - b[0];
        ks = js * (e[1] - b[1]);
        ns = ks * (e[2] - b[2]);
    }
    double& operator()(int i, int j, int k, int n = 0) const {
        return p[(i - b[0]) + (j - b[1]) * js + (k - b[2]) * ks + n * ns];
    }
};

struct Dx {
    double v[3];
    double operator[](int d) const { return v[d]; }
};

}  // namespace

// S: (5, nz+8, ny+8, nx+8) state of box 0..n-1 grown by 4; dsdt: (5, nz, ny, nx)
extern "C" int compat_rhs_regular(const double* S, int nx, int ny, int nz, const double* dxinv, int do_visc,
                                  const ocfd_parm* parm, double* dsdt) {
    const int lo[3] = {0, 0, 0}, hi[3] = {nx - 1, ny - 1, nz - 1};
    const int glo[3] = {-4, -4, -4}, ghi[3] = {nx + 3, ny + 3, nz + 3};
    const long long ng = (long long)(nx + 8) * (ny + 8) * (nz + 8);
    std::vector<double> q(7 * ng), fp(5 * ng), fm(5 * ng);
    Arr s(const_cast<double*>(S), glo, ghi), qa(q.data(), glo, ghi), fpa(fp.data(), glo, ghi),
        fma(fm.data(), glo, ghi), out(dsdt, lo, hi);
    const Dx dx{{dxinv[0], dxinv[1], dxinv[2]}};
    std::vector<double> fl[3];
    std::vector<Arr> fa;
    for (int d = 0; d < 3; ++d) {
        int h[3] = {hi[0], hi[1], hi[2]};
        h[d] += 1;
        fl[d].assign(5LL * (h[0] + 1) * (h[1] + 1) * (h[2] + 1), 0.0);
        fa.emplace_back(fl[d].data(), lo, h);
    }
    for (int k = glo[2]; k <= ghi[2]; ++k)
        for (int j = glo[1]; j <= ghi[1]; ++j)
            for (int i = glo[0]; i <= ghi[0]; ++i) ocfd_compat::c2prim(i, j, k, s, qa, *parm);
    for (int d = 0; d < 3; ++d) {
        for (int k = glo[2]; k <= ghi[2]; ++k)
            for (int j = glo[1]; j <= ghi[1]; ++j)
                for (int i = glo[0]; i <= ghi[0]; ++i) {
                    if (d == 0) ocfd_compat::flux_split_x(i, j, k, fpa, fma, qa, s, *parm);
                    if (d == 1) ocfd_compat::flux_split_y(i, j, k, fpa, fma, qa, s, *parm);
                    if (d == 2) ocfd_compat::flux_split_z(i, j, k, fpa, fma, qa, s, *parm);
                }
        const Arr& f = fa[d];
        for (int n = 0; n < 5; ++n)
            for (int k = f.b[2]; k < f.e[2]; ++k)
                for (int j = f.b[1]; j < f.e[1]; ++j)
                    for (int i = f.b[0]; i < f.e[0]; ++i) {
                        if (d == 0) ocfd_compat::reconstruction_x(i, j, k, n, fpa, fma, f, *parm);
                        if (d == 1) ocfd_compat::reconstruction_y(i, j, k, n, fpa, fma, f, *parm);
                        if (d == 2) ocfd_compat::reconstruction_z(i, j, k, n, fpa, fma, f, *parm);
                    }
        if (do_visc)
            for (int k = f.b[2]; k < f.e[2]; ++k)
                for (int j = f.b[1]; j < f.e[1]; ++j)
                    for (int i = f.b[0]; i < f.e[0]; ++i) {
                        if (d == 0) ocfd_compat::compute_visc_x(i, j, k, qa, f, dx, *parm);
                        if (d == 1) ocfd_compat::compute_visc_y(i, j, k, qa, f, dx, *parm);
                        if (d == 2) ocfd_compat::compute_visc_z(i, j, k, qa, f, dx, *parm);
                    }
    }
    for (int n = 0; n < 5; ++n)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) ocfd_compat::divop(i, j, k, n, out, fa[0], fa[1], fa[2], dx);
    return 0;
}
