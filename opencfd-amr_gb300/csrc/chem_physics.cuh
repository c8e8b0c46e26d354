// Li-Dryer H2/O2 thermochemistry and transport on the GPU (device functions).
// Included by exactly one translation unit (chem.cu), which owns c_mech.
//
// Each routine keeps the operation order of the reference routine it replaces
// (Source/CHEM/LiDryer.H, Source/CHEM/ChemViscous.H); exp/log/pow are CUDA's,
// so results agree with the CPU build to a few ulps, not bit for bit.
#pragma once

#include "device_physics.cuh"
#include "mechanism.h"

namespace ocfd {

__constant__ MechTables c_mech;

// Quantities derived from the tables once on the host, so that the per-cell
// routines divide less (GB300's FP64 pipe runs a division as ~10 instructions):
//   q3, q5   a2 / 3, a4 / 5 of the internal energy and enthalpy polynomials, and
//   g6, g12, g20   a2 / 6, a3 / 12, a4 / 20 of the Gibbs polynomial - the same
//            quotients the expressions form first, so these are bit-identical;
//   inv_mw   1 / W_n and wratio[a][b] = W_a / W_b, which replace divisions by W
//            (a rounding of the last bit differs from dividing).
struct MechDerived {
    double q3[2][NSP], q5[2][NSP];
    double g6[2][NSP], g12[2][NSP], g20[2][NSP];
    double inv_mw[NSP];
    double wratio[NSP][NSP];
    // e_n(T)/(R T W_n) at the bounds 250 K and 3500 K of the temperature
    // inversion (the mixture energies there are then 9 products)
    double umin_w[NSP], umax_w[NSP];
};
__constant__ MechDerived c_mder;

// NASA-7 coefficient row of species n for temperature T
__device__ __forceinline__ const double* nasa(double T, int n) {
    return T < 1000 ? c_mech.lo[n] : c_mech.hi[n];
}

// speciesInternalEnergy, LiDryer.H:531-614: e/(RT), tc = {., T, T^2, T^3, T^4}
__device__ __forceinline__ void species_internal_energy(double* e, const double* tc) {
    const double T = tc[1];
    const double invT = 1.0 / T;
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        if (T < 1000) {
            const double* a = c_mech.lo[n];
            e[n] = a[0] - 1.0 + a[1] / 2.0 * tc[1] + c_mder.q3[0][n] * tc[2] + a[3] / 4.0 * tc[3] +
                   c_mder.q5[0][n] * tc[4];
        } else {
            const double* a = c_mech.hi[n];
            e[n] = a[0] - 1.0 + a[1] / 2.0 * tc[1] + c_mder.q3[1][n] * tc[2] + a[3] / 4.0 * tc[3] +
                   c_mder.q5[1][n] * tc[4] + (a[5] - c_mech.lo[n][5]) * invT;
        }
    }
}

// speciesEnthalpy, LiDryer.H:616-695: h/R [K]
__device__ __forceinline__ void species_enthalpy(double T, double* h) {
    const double tc[5] = {T, T * T, T * T * T, T * T * T * T, T * T * T * T * T};
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        if (T < 1000) {
            const double* a = c_mech.lo[n];
            h[n] = a[0] * tc[0] + a[1] / 2.0 * tc[1] + c_mder.q3[0][n] * tc[2] + a[3] / 4.0 * tc[3] +
                   c_mder.q5[0][n] * tc[4];
        } else {
            const double* a = c_mech.hi[n];
            h[n] = a[0] * tc[0] + a[1] / 2.0 * tc[1] + c_mder.q3[1][n] * tc[2] + a[3] / 4.0 * tc[3] +
                   c_mder.q5[1][n] * tc[4] + (a[5] - c_mech.lo[n][5]);
        }
    }
}

// CKUBMS, LiDryer.H:697-714: mixture internal energy per volume [J/m^3]
__device__ __forceinline__ double ckubms(double T, const double* rhoi, double Ru) {
    double result = 0;
    const double tc[5] = {0, T, T * T, T * T * T, T * T * T * T};
    double ums[NSP];
    const double RT = Ru * T;
    species_internal_energy(ums, tc);
#pragma unroll
    for (int n = 0; n < NSP; ++n) result += rhoi[n] * ums[n] * c_mder.inv_mw[n];
    return result * RT;
}

// CKCVBS, LiDryer.H:801-815
__device__ __forceinline__ double ckcvbs(double T, const double* rhoi, double Ru) {
    double result = 0;
    const double tc[5] = {0, T, T * T, T * T * T, T * T * T * T};
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        const double* a = nasa(T, n);
        const double cpor = a[0] + a[1] * tc[1] + a[2] * tc[2] + a[3] * tc[3] + a[4] * tc[4];
        result += (cpor - 1.0) * rhoi[n] * c_mder.inv_mw[n];
    }
    return result * Ru;
}

// CKPY, LiDryer.H:10-18
__device__ __forceinline__ double ckpy(const double* rhoi, double T, double Ru) {
    double YOW = 0;
#pragma unroll
    for (int i = 0; i < NSP; ++i) YOW += rhoi[i] * c_mder.inv_mw[i];
    return Ru * T * YOW;
}

// CKYTX, LiDryer.H:36-54
__device__ __forceinline__ void ckytx(const double* y, double* x) {
    double YOW = 0, tmp[NSP];
#pragma unroll
    for (int i = 0; i < NSP; ++i) tmp[i] = y[i] / c_mech.mw[i];
#pragma unroll
    for (int i = 0; i < NSP; ++i) YOW += tmp[i];
    const double YOWINV = 1.0 / YOW;
#pragma unroll
    for (int i = 0; i < NSP; ++i) x[i] = y[i] / c_mech.mw[i] * YOWINV;
}

// GET_T_GIVEN_EY, LiDryer.H:833-888: bounded Newton for T from e on NASA-7
__device__ __forceinline__ double get_t_given_ey(double e, const double* rhoi, double Ru) {
    const int maxiter = 200;
    const double tol = 1e-7;
    const double ein = e, tmin = 250, tmax = 3500;
    double smin = 0, smax = 0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        smin += rhoi[n] * c_mder.umin_w[n];
        smax += rhoi[n] * c_mder.umax_w[n];
    }
    const double emin = smin * (Ru * tmin), emax = smax * (Ru * tmax);
    if (ein < emin) return tmin - (emin - ein) / ckcvbs(tmin, rhoi, Ru);
    if (ein > emax) return tmax - (emax - ein) / ckcvbs(tmax, rhoi, Ru);
    double As = 0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) As += c_mech.A0[n] * Ru * c_mder.inv_mw[n] * rhoi[n];
    double t1 = e / As;
    if (t1 < tmin || t1 > tmax) t1 = tmin + (tmax - tmin) / (emax - emin) * (ein - emin);
    for (int i = 0; i < maxiter; ++i) {
        const double e1 = ckubms(t1, rhoi, Ru);
        const double cv = ckcvbs(t1, rhoi, Ru);
        double dt = (ein - e1) / cv;
        if (dt > 100.0) dt = 100.0;
        else if (dt < -100.0) dt = -100.0;
        else if (fabs(dt) < tol) break;
        else if (t1 + dt == t1) break;
        t1 += dt;
    }
    return t1;
}

// ------------------------------------------------------------ production rates
// vproductionRate, LiDryer.H:156-529.  Reaction m contributes to wdot and to
// the analytic Jacobian Arate only through the species it involves; the
// reference's loops over all species add exact zeros elsewhere, so adding the
// non-zero terms in the same reaction order gives the same sums.
//   A(l, n): accessor of Arate[l][n]
struct Stoich {
    int s[4];   // distinct species of the reaction (-1 = unused)
    int vf[4];  // forward stoichiometric coefficients of s[]
    int vr[4];  // reverse
};

template <class Mat>
__device__ __forceinline__ void rxn_accum(const Stoich& X, double wf, double wr, const double* sc,
                                          double* wdot, Mat& A) {
    const double eps = 1e-20;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (X.s[a] < 0) continue;
        wdot[X.s[a]] += (wf - wr) * (X.vr[a] - X.vf[a]);
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        if (X.s[b] < 0) continue;
        const int n = X.s[b];
        const double Awf = X.vf[b] * wf / (sc[n] + eps);
        const double Awr = X.vr[b] * wr / (sc[n] + eps);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (X.s[a] < 0) continue;
            A(X.s[a], n) += (Awf - Awr) * (X.vr[a] - X.vf[a]);
        }
    }
}

template <class Mat>
__device__ __forceinline__ void production_rate(double* wdot, Mat& A, const double* sc, double T,
                                                double Ru, double Patm) {
    double tc[5], gi[NSP];
    tc[0] = log(T);
    tc[1] = T;
    tc[2] = T * (T);
    tc[3] = tc[2] * tc[1];
    tc[4] = tc[2] * tc[2];
    const double invT = 1.0 / T;
    // gibbs, LiDryer.H:70-154: g/(RT)
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        const double* a = nasa(T, n);
        const int h = T < 1000 ? 0 : 1;
        gi[n] = a[0] * (1.0 - tc[0]) - a[1] / 2.0 * tc[1] - c_mder.g6[h][n] * tc[2] - c_mder.g12[h][n] * tc[3] -
                c_mder.g20[h][n] * tc[4] + a[5] * invT - a[6];
    }
    const double RsT = Ru / Patm * 1e6 * T;
    const double iRsT = 1.0 / RsT;
    double mixture = 0.0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) {
        mixture += sc[n];
        wdot[n] = 0.0;
    }
    const double alpha_a = mixture + 1.5 * sc[0] + 11 * sc[2];
    // forward rate k = A exp(b lnT - Ta/T), LiDryer.H:171-191
#define KF(A_, b_, Ta_) ((A_) * exp((b_) * tc[0] - (Ta_) * invT))
#define ST(s0, s1, s2, s3, f0, f1, f2, f3, r0, r1, r2, r3) \
    Stoich { {s0, s1, s2, s3}, {f0, f1, f2, f3}, {r0, r1, r2, r3} }
    double wf, wr, kf, iKc;  // the inverse equilibrium constant: kf * iKc is the reverse rate constant
    // 0: H + O2 <=> O + OH
    kf = KF(3.55e+15, -0.41, 8353.444256079512);
    iKc = exp((gi[4] + gi[5]) - (gi[3] + gi[1]));
    wf = sc[3] * sc[1] * kf;
    wr = sc[4] * sc[5] * (kf * iKc);
    rxn_accum(ST(3, 1, 4, 5, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 1: O + H2 <=> H + OH
    kf = KF(50800.0, 2.67, 3165.2508657072367);
    iKc = exp((gi[3] + gi[5]) - (gi[4] + gi[0]));
    wf = sc[4] * sc[0] * kf;
    wr = sc[3] * sc[5] * (kf * iKc);
    rxn_accum(ST(4, 0, 3, 5, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 2: H2 + OH <=> H2O + H
    kf = KF(2.16e+08, 1.51, 1726.0429999007667);
    iKc = exp((gi[2] + gi[3]) - (gi[0] + gi[5]));
    wf = sc[0] * sc[5] * kf;
    wr = sc[2] * sc[3] * (kf * iKc);
    rxn_accum(ST(0, 5, 2, 3, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 3: O + H2O <=> OH + OH
    kf = KF(2.97e+06, 2.02, 6743.141748883461);
    iKc = exp((gi[5] + gi[5]) - (gi[4] + gi[2]));
    wf = sc[4] * sc[2] * kf;
    wr = sc[5] * sc[5] * (kf * iKc);
    rxn_accum(ST(4, 2, 5, -1, 1, 1, 0, 0, 0, 0, 2, 0), wf, wr, sc, wdot, A);
    // 4: H2 + M <=> H + H + M
    kf = alpha_a * KF(4.58e+19, -1.4, 52526.05490660117);
    iKc = RsT * exp((gi[3] + gi[3]) - (gi[0]));
    wf = sc[0] * kf;
    wr = sc[3] * sc[3] * (kf * iKc);
    rxn_accum(ST(0, 3, -1, -1, 1, 0, 0, 0, 0, 2, 0, 0), wf, wr, sc, wdot, A);
    // 5: O + O + M <=> O2 + M
    kf = alpha_a * KF(6.16e+15, -0.5, 0.0);
    iKc = iRsT * exp((gi[1]) - (gi[4] + gi[4]));
    wf = sc[4] * sc[4] * kf;
    wr = sc[1] * (kf * iKc);
    rxn_accum(ST(4, 1, -1, -1, 2, 0, 0, 0, 0, 1, 0, 0), wf, wr, sc, wdot, A);
    // 6: O + H + M <=> OH + M
    kf = alpha_a * KF(4.71e+18, -1.0, 0.0);
    iKc = iRsT * exp((gi[5]) - (gi[4] + gi[3]));
    wf = sc[4] * sc[3] * kf;
    wr = sc[5] * (kf * iKc);
    rxn_accum(ST(4, 3, 5, -1, 1, 1, 0, 0, 0, 0, 1, 0), wf, wr, sc, wdot, A);
    // 7: H + OH + M <=> H2O + M
    kf = alpha_a * KF(3.8e+22, -2.0, 0.0);
    iKc = iRsT * exp((gi[2]) - (gi[3] + gi[5]));
    wf = sc[3] * sc[5] * kf;
    wr = sc[2] * (kf * iKc);
    rxn_accum(ST(3, 5, 2, -1, 1, 1, 0, 0, 0, 0, 1, 0), wf, wr, sc, wdot, A);
    // 8: H + O2 (+M) <=> HO2 (+M), Troe falloff, Fcent = 0.8
    {
        const double alpha = mixture + sc[0] + 10 * sc[2] + -0.22 * sc[1];
        kf = KF(1.48e+12, 0.6, 0.0);
        const double redP = alpha / kf * 6.37e+20 * exp(-1.72 * tc[0] - 261.6741574193582 * invT);
        const double logPred = log10(redP);
        const double logFcent = log10(0.8);
        const double troe_c = -0.4 - 0.67 * logFcent;
        const double troe_n = 0.75 - 1.27 * logFcent;
        const double troe = (troe_c + logPred) / (troe_n - 0.14 * (troe_c + logPred));
        const double F_troe = pow(10.0, logFcent / (1.0 + troe * troe));
        kf *= (redP / (1.0 + redP)) * F_troe;
    }
    iKc = iRsT * exp((gi[6]) - (gi[3] + gi[1]));
    wf = sc[3] * sc[1] * kf;
    wr = sc[6] * (kf * iKc);
    rxn_accum(ST(3, 1, 6, -1, 1, 1, 0, 0, 0, 0, 1, 0), wf, wr, sc, wdot, A);
    // 9: HO2 + H <=> H2 + O2
    kf = KF(1.66e+13, 0.0, 412.64001746898793);
    iKc = exp((gi[0] + gi[1]) - (gi[6] + gi[3]));
    wf = sc[6] * sc[3] * kf;
    wr = sc[0] * sc[1] * (kf * iKc);
    rxn_accum(ST(6, 3, 0, 1, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 10: HO2 + H <=> OH + OH
    kf = KF(7.08e+13, 0.0, 150.96586004962973);
    iKc = exp((gi[5] + gi[5]) - (gi[6] + gi[3]));
    wf = sc[6] * sc[3] * kf;
    wr = sc[5] * sc[5] * (kf * iKc);
    rxn_accum(ST(6, 3, 5, -1, 1, 1, 0, 0, 0, 0, 2, 0), wf, wr, sc, wdot, A);
    // 11: HO2 + O <=> O2 + OH
    kf = KF(3.25e+13, 0.0, 0.0);
    iKc = exp((gi[1] + gi[5]) - (gi[6] + gi[4]));
    wf = sc[6] * sc[4] * kf;
    wr = sc[1] * sc[5] * (kf * iKc);
    rxn_accum(ST(6, 4, 1, 5, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 12: HO2 + OH <=> H2O + O2
    kf = KF(2.89e+13, 0.0, -251.60976674938289);
    iKc = exp((gi[2] + gi[1]) - (gi[6] + gi[5]));
    wf = sc[6] * sc[5] * kf;
    wr = sc[2] * sc[1] * (kf * iKc);
    rxn_accum(ST(6, 5, 2, 1, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 13: HO2 + HO2 <=> H2O2 + O2 (two rate expressions, DUPLICATE)
    {
        const double kf1 = KF(4.2e+14, 0.0, 6028.570011315214);
        const double kf2 = KF(1.3e+11, 0.0, -820.2478396029883);
        iKc = exp((gi[7] + gi[1]) - (gi[6] + gi[6]));
        const double phi_f = sc[6] * sc[6], phi_r = sc[7] * sc[1];
        wf = phi_f * kf1;
        wr = phi_r * (kf1 * iKc);
        wf += phi_f * kf2;
        wr += phi_r * (kf2 * iKc);
        rxn_accum(ST(6, 7, 1, -1, 2, 0, 0, 0, 0, 1, 1, 0), wf, wr, sc, wdot, A);
    }
    // 14: H2O2 (+M) <=> OH + OH (+M), Troe falloff, Fcent = 0.5
    {
        kf = KF(2.95e+14, 0.0, 24355.825421340265);
        const double redP = alpha_a / kf * 1.20e+17 * exp(-22846.166820843966 * invT);
        const double logPred = log10(redP);
        const double logFcent = log10(0.5);
        const double troe_c = -0.4 - 0.67 * logFcent;
        const double troe_n = 0.75 - 1.27 * logFcent;
        const double troe = (troe_c + logPred) / (troe_n - 0.14 * (troe_c + logPred));
        const double F_troe = pow(10.0, logFcent / (1.0 + troe * troe));
        kf *= (redP / (1.0 + redP)) * F_troe;
    }
    iKc = RsT * exp((gi[5] + gi[5]) - (gi[7]));
    wf = sc[7] * kf;
    wr = sc[5] * sc[5] * (kf * iKc);
    rxn_accum(ST(7, 5, -1, -1, 1, 0, 0, 0, 0, 2, 0, 0), wf, wr, sc, wdot, A);
    // 15: H2O2 + H <=> H2O + OH
    kf = KF(2.41e+13, 0.0, 1997.7815479901);
    iKc = exp((gi[2] + gi[5]) - (gi[7] + gi[3]));
    wf = sc[7] * sc[3] * kf;
    wr = sc[2] * sc[5] * (kf * iKc);
    rxn_accum(ST(7, 3, 2, 5, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 16: H2O2 + H <=> HO2 + H2
    kf = KF(4.82e+13, 0.0, 4000.595291315188);
    iKc = exp((gi[6] + gi[0]) - (gi[7] + gi[3]));
    wf = sc[7] * sc[3] * kf;
    wr = sc[6] * sc[0] * (kf * iKc);
    rxn_accum(ST(7, 3, 6, 0, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 17: H2O2 + O <=> OH + HO2
    kf = KF(9.55e+06, 2.0, 1997.7815479901);
    iKc = exp((gi[5] + gi[6]) - (gi[7] + gi[4]));
    wf = sc[7] * sc[4] * kf;
    wr = sc[5] * sc[6] * (kf * iKc);
    rxn_accum(ST(7, 4, 5, 6, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    // 18: H2O2 + OH <=> HO2 + H2O (two rate expressions, DUPLICATE)
    {
        const double kf1 = KF(1.0e+12, 0.0, 0.0);
        const double kf2 = KF(5.8e+14, 0.0, 4810.778740248201);
        iKc = exp((gi[6] + gi[2]) - (gi[7] + gi[5]));
        const double phi_f = sc[7] * sc[5], phi_r = sc[6] * sc[2];
        wf = phi_f * kf1;
        wr = phi_r * (kf1 * iKc);
        wf += phi_f * kf2;
        wr += phi_r * (kf2 * iKc);
        rxn_accum(ST(7, 5, 6, 2, 1, 1, 0, 0, 0, 0, 1, 1), wf, wr, sc, wdot, A);
    }
#undef KF
#undef ST
}

// gauss, LiDryer.H:890-942: partial-pivot elimination of the augmented 9x10
// system held by accessor U (column 9 = right-hand side); solution in x.
template <class Mat>
__device__ __forceinline__ void gauss_solve(Mat& U, double* x) {
    for (int k = 0; k < NSP; k++) {
        int pv = k;
        double maxPivot = 0.0;
        for (int i = k; i < NSP; i++) {
            const double a = fabs(U(i, k));
            if (a > maxPivot) {
                maxPivot = a;
                pv = i;
            }
        }
        if (pv != k)
            for (int i = k; i < NSP + 1; i++) {
                const double t = U(pv, i);
                U(pv, i) = U(k, i);
                U(k, i) = t;
            }
        // one reciprocal of the pivot instead of a division per row
        const double ipiv = 1.0 / U(k, k);
        for (int i = k + 1; i < NSP; i++) {
            const double m = U(i, k) * ipiv;
            for (int j = k; j < NSP + 1; j++) U(i, j) -= m * U(k, j);
        }
    }
#pragma unroll
    for (int k = NSP - 1; k >= 0; k--) {
        double sum = U(k, NSP);
#pragma unroll
        for (int j = k + 1; j < NSP; j++) sum -= U(k, j) * x[j];
        x[k] = sum / U(k, k);
    }
}

// ------------------------------------------------------------------ transport
__device__ __forceinline__ double dot5(const double* x, const double* y) {
    return x[0] * y[0] + x[1] * y[1] + x[2] * y[2] + x[3] * y[3] + x[4] * y[4];
}

// mixtureProperties, ChemViscous.H:16-64 (Wilke mixing rule)
__device__ __forceinline__ void mixture_properties(double T, const double* X, double& mu,
                                                   double& lambda) {
    double mui[NSP], sqmui[NSP], lambdai[NSP];
    const double sqT = sqrt(T), logT = log(T);
    const double sqsqT = sqrt(sqT);
    const double poly[5] = {1.0, logT, logT * logT, logT * logT * logT, logT * logT * logT * logT};
#pragma unroll
    for (int k = 0; k < NSP; k++) {
        sqmui[k] = sqsqT * dot5(poly, &c_mech.visc[k * 5]);
        lambdai[k] = sqT * dot5(poly, &c_mech.cond[k * 5]);
        mui[k] = (sqmui[k] * sqmui[k]);
    }
    double sum1 = 0.0, sum2 = 0.0;
#pragma unroll
    for (int k = 0; k < NSP; k++) {
        sum1 += X[k] * lambdai[k];
        sum2 += X[k] / lambdai[k];
    }
    lambda = 0.5 * (sum1 + 1.0 / sum2);
    // phi[k][j] for j < k and its mirror, accumulated row by row
    double rowsum[NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) rowsum[k] = 0.0;
    // the reference sums tmp_k = sum_j X[j] phi[k][j] in j order; build phi fully
    double phi[NSP][NSP];
#pragma unroll
    for (int k = 0; k < NSP; k++) {
#pragma unroll
        for (int j = 0; j < k; j++) {
            const double wratiojk = c_mech.mw[j] / c_mech.mw[k];
            const double vratiokj = mui[k] / mui[j];
            const double factor1 = 1.0 + (sqmui[k] / sqmui[j]) * sqrt(sqrt(wratiojk));
            const double tmp = factor1 * factor1 / sqrt(8.0 + 8.0 * c_mech.mw[k] / c_mech.mw[j]);
            phi[k][j] = tmp;
            phi[j][k] = tmp / (vratiokj * wratiojk);
        }
        phi[k][k] = 1.0;
    }
    double m = 0;
#pragma unroll
    for (int k = 0; k < NSP; k++) {
        double tmp = 0;
#pragma unroll
        for (int j = 0; j < NSP; j++) tmp += X[j] * phi[k][j];
        m += X[k] * mui[k] / tmp;
    }
    (void)rowsum;
    mu = m;
}

// ---- FP32 transport of the mixed form: the same fits and mixing rules with the
// species-pair constants of the Wilke rule precomputed in FP64 and rounded once
struct TransF {
    float visc[NSP * 5], cond[NSP * 5], diff[45 * 5];
    float mw[NSP];
    float wr14[NSP][NSP];   // (W_j / W_k)^(1/4)
    float den[NSP][NSP];    // 1 / sqrt(8 + 8 W_k / W_j)
    float wratio[NSP][NSP]; // W_j / W_k
};
__constant__ TransF c_trf;

__device__ __forceinline__ float dot5f(const float* x, const float* y) {
    return x[0] * y[0] + x[1] * y[1] + x[2] * y[2] + x[3] * y[3] + x[4] * y[4];
}

// mixtureProperties (ChemViscous.H:16-64) and getMixDiffCoeffsMass
// (ChemViscous.H:66-106) in FP32: mole fractions from the mass fractions,
// Wilke viscosity, averaged conductivity, mixture-averaged diffusivities
__device__ __forceinline__ void transport_f32(float T, float p, const float* Y, float& mu, float& lambda, float* D) {
    float X[NSP], tmp[NSP], yow = 0.0f;
#pragma unroll
    for (int i = 0; i < NSP; ++i) {
        tmp[i] = __fdividef(Y[i], c_trf.mw[i]);
        yow += tmp[i];
    }
    const float yowinv = __frcp_rn(yow);
#pragma unroll
    for (int i = 0; i < NSP; ++i) X[i] = tmp[i] * yowinv;
    const float sqT = sqrtf(T), logT = __logf(T), sqsqT = sqrtf(sqT);
    const float poly[5] = {1.0f, logT, logT * logT, logT * logT * logT, logT * logT * logT * logT};
    float mui[NSP], sqmui[NSP], lami[NSP];
    float s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int k = 0; k < NSP; ++k) {
        sqmui[k] = sqsqT * dot5f(poly, &c_trf.visc[k * 5]);
        lami[k] = sqT * dot5f(poly, &c_trf.cond[k * 5]);
        mui[k] = sqmui[k] * sqmui[k];
        s1 += X[k] * lami[k];
        s2 += __fdividef(X[k], lami[k]);
    }
    lambda = 0.5f * (s1 + __frcp_rn(s2));
    float phi[NSP][NSP];
#pragma unroll
    for (int k = 0; k < NSP; ++k) {
#pragma unroll
        for (int j = 0; j < k; ++j) {
            const float f1 = 1.0f + __fdividef(sqmui[k], sqmui[j]) * c_trf.wr14[k][j];
            const float t = f1 * f1 * c_trf.den[k][j];
            phi[k][j] = t;
            phi[j][k] = __fdividef(t, __fdividef(mui[k], mui[j]) * c_trf.wratio[k][j]);
        }
        phi[k][k] = 1.0f;
    }
    float m = 0.0f;
#pragma unroll
    for (int k = 0; k < NSP; ++k) {
        float t = 0.0f;
#pragma unroll
        for (int j = 0; j < NSP; ++j) t += X[j] * phi[k][j];
        m += __fdividef(X[k] * mui[k], t);
    }
    mu = m;
    const float t32 = T * sqT;
    float mmw = 0.0f;
#pragma unroll
    for (int n = 0; n < NSP; ++n) mmw += X[n] * c_trf.mw[n];
#pragma unroll
    for (int n = 0; n < NSP; n++) {
        float a1 = 0.0f, a2 = 0.0f;
#pragma unroll
        for (int nn = 0; nn < NSP; nn++) {
            if (nn == n) continue;
            const int a = n < nn ? n : nn, b = n < nn ? nn : n;
            const int ic = a * NSP - (a * (a - 1)) / 2 + (b - a);
            const float bdinv = __frcp_rn(t32 * dot5f(poly, &c_trf.diff[ic * 5]));
            a1 += X[nn] * bdinv;
            a2 += X[nn] * c_trf.mw[nn] * bdinv;
        }
        a1 *= p;
        a2 *= __fdividef(p * X[n], mmw - c_trf.mw[n] * X[n]);
        D[n] = __frcp_rn(a1 + a2);
    }
}

// getMixDiffCoeffsMass, ChemViscous.H:66-106
__device__ __forceinline__ void mix_diff_coeffs(double T, double p, const double* X, double* D) {
    const double logT = log(T);
    const double poly[5] = {1.0, logT, logT * logT, logT * logT * logT, logT * logT * logT * logT};
    const double t32 = T * sqrt(T);
    double mmw = 0;
#pragma unroll
    for (int n = 0; n < NSP; ++n) mmw += X[n] * c_mech.mw[n];
#pragma unroll
    for (int n = 0; n < NSP; n++) {
        double sum1 = 0.0, sum2 = 0.0;
#pragma unroll
        for (int nn = 0; nn < NSP; nn++) {
            if (nn == n) continue;
            const int a = n < nn ? n : nn, b = n < nn ? nn : n;
            const int ic = a * NSP - (a * (a - 1)) / 2 + (b - a);  // upper-triangle index
            const double bd = t32 * dot5(poly, &c_mech.diff[ic * 5]);
            sum1 += X[nn] / bd;
            sum2 += X[nn] * c_mech.mw[nn] / bd;
        }
        sum1 *= p;
        sum2 *= p * X[n] / (mmw - c_mech.mw[n] * X[n]);
        D[n] = 1.0 / (sum1 + sum2);
    }
}

}  // namespace ocfd
