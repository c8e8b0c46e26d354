// AMReX plotfile output (HyperCLaw-V1.1 layout) and an fcompare-equivalent
// comparison of two plotfiles, in host C++.
//
// Layout written (the format AmrLevel::writePlotFile produces, Source/IO.cpp:32-35):
//   <dir>/Header                  text: version, variable names, dimension, time,
//                                 finest level, problem extents, ratios, level
//                                 domains, steps, cell sizes, grids per level
//   <dir>/Level_<l>/Cell_H        VisMF header: boxes, file offsets, per-box min/max
//   <dir>/Level_<l>/Cell_D_00000  one FAB per box: a text line
//                                 "FAB ((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8)))(box) ncomp"
//                                 then the components (little-endian IEEE doubles),
//                                 each over the box with i fastest
// The comparison follows Util/Plotfile/fcompare.cpp:150-290: per level and variable
// the difference of the two files over level-l valid data; norm 0 = max |b - a|
// (relative to max |a|), norm 1 / 2 = the discrete L1 / L2 norm times dV^(1/p)
// (relative to the same norm of a), NaNs reported per variable.
#include <sys/stat.h>
#include <sys/types.h>

#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>

#include "ocfd_internal.h"

namespace ocfd {

static const char* kRealDesc = "(8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8))";

static bool make_dir(const std::string& d) {
    if (mkdir(d.c_str(), 0755) == 0) return true;
    struct stat sb;
    return stat(d.c_str(), &sb) == 0 && S_ISDIR(sb.st_mode);
}

static std::string box_text(const ocfd_box& b) {
    std::ostringstream os;
    os << "((" << b.lo[0] << "," << b.lo[1] << "," << b.lo[2] << ") (" << b.hi[0] << "," << b.hi[1] << ","
       << b.hi[2] << ") (0,0,0))";
    return os.str();
}

static long long box_cells(const ocfd_box& b) {
    return (long long)(b.hi[0] - b.lo[0] + 1) * (b.hi[1] - b.lo[1] + 1) * (b.hi[2] - b.lo[2] + 1);
}

ocfd_status plotfile_write(const std::string& dir, int nlev, const ocfd_plot_level* levels, int ncomp,
                           const char* const* names, const ocfd_box& dom0, const double* prob_lo,
                           const double* prob_hi, int ratio, double time) {
    if (nlev < 1 || ncomp < 1 || !levels || !names) return fail(OCFD_BAD_ARG, "plotfile: bad arguments");
    if (!make_dir(dir)) return fail(OCFD_BAD_ARG, "plotfile: cannot create " + dir);
    std::ofstream h(dir + "/Header");
    if (!h) return fail(OCFD_BAD_ARG, "plotfile: cannot write the header");
    h.precision(17);
    h << "HyperCLaw-V1.1\n" << ncomp << "\n";
    for (int n = 0; n < ncomp; ++n) h << names[n] << "\n";
    h << 3 << "\n" << time << "\n" << nlev - 1 << "\n";
    h << prob_lo[0] << " " << prob_lo[1] << " " << prob_lo[2] << "\n";
    h << prob_hi[0] << " " << prob_hi[1] << " " << prob_hi[2] << "\n";
    for (int l = 0; l < nlev - 1; ++l) h << ratio << (l + 1 < nlev - 1 ? " " : "");
    h << "\n";
    for (int l = 0; l < nlev; ++l) {
        ocfd_box d = dom0;
        for (int e = 0; e < 3; ++e) {
            d.lo[e] = dom0.lo[e] * (1 << l);
            d.hi[e] = (dom0.hi[e] + 1) * (1 << l) - 1;
        }
        h << box_text(d) << (l + 1 < nlev ? " " : "");
    }
    h << "\n";
    for (int l = 0; l < nlev; ++l) h << levels[l].step << (l + 1 < nlev ? " " : "");
    h << "\n";
    for (int l = 0; l < nlev; ++l) h << levels[l].dx[0] << " " << levels[l].dx[1] << " " << levels[l].dx[2] << "\n";
    h << 0 << "\n" << 0 << "\n";  // Cartesian coordinates, no boundary data
    for (int l = 0; l < nlev; ++l) {
        const ocfd_plot_level& L = levels[l];
        h << l << " " << L.nbox << " " << time << "\n" << L.step << "\n";
        for (int b = 0; b < L.nbox; ++b)
            for (int e = 0; e < 3; ++e)
                h << prob_lo[e] + L.dx[e] * L.boxes[b].lo[e] << " " << prob_lo[e] + L.dx[e] * (L.boxes[b].hi[e] + 1)
                  << "\n";
        h << "Level_" << l << "/Cell\n";
        // FAB data and the VisMF header of the level
        const std::string ld = dir + "/Level_" + std::to_string(l);
        if (!make_dir(ld)) return fail(OCFD_BAD_ARG, "plotfile: cannot create " + ld);
        std::ofstream d(ld + "/Cell_D_00000", std::ios::binary);
        if (!d) return fail(OCFD_BAD_ARG, "plotfile: cannot write level data");
        std::vector<long long> off(L.nbox);
        std::vector<double> mn((size_t)L.nbox * ncomp), mx((size_t)L.nbox * ncomp);
        for (int b = 0; b < L.nbox; ++b) {
            off[b] = (long long)d.tellp();
            d << "FAB (" << kRealDesc << ")" << box_text(L.boxes[b]) << " " << ncomp << "\n";
            const long long nc = box_cells(L.boxes[b]);
            const double* p = L.fabs[b];
            d.write(reinterpret_cast<const char*>(p), sizeof(double) * nc * ncomp);
            for (int n = 0; n < ncomp; ++n) {
                double a = std::numeric_limits<double>::infinity(), z = -a;
                for (long long c = 0; c < nc; ++c) {
                    a = std::fmin(a, p[n * nc + c]);
                    z = std::fmax(z, p[n * nc + c]);
                }
                mn[(size_t)b * ncomp + n] = a;
                mx[(size_t)b * ncomp + n] = z;
            }
        }
        if (!d) return fail(OCFD_BAD_ARG, "plotfile: write failed");
        std::ofstream c(ld + "/Cell_H");
        c.precision(17);
        c << 1 << "\n" << 0 << "\n" << ncomp << "\n" << 0 << "\n";
        c << "(" << L.nbox << " 0\n";
        for (int b = 0; b < L.nbox; ++b) c << box_text(L.boxes[b]) << "\n";
        c << ")\n" << L.nbox << "\n";
        for (int b = 0; b < L.nbox; ++b) c << "FabOnDisk: Cell_D_00000 " << off[b] << "\n";
        c << "\n" << L.nbox << "," << ncomp << "\n";
        for (int b = 0; b < L.nbox; ++b) {
            for (int n = 0; n < ncomp; ++n) c << mn[(size_t)b * ncomp + n] << ",";
            c << "\n";
        }
        c << "\n" << L.nbox << "," << ncomp << "\n";
        for (int b = 0; b < L.nbox; ++b) {
            for (int n = 0; n < ncomp; ++n) c << mx[(size_t)b * ncomp + n] << ",";
            c << "\n";
        }
        if (!c) return fail(OCFD_BAD_ARG, "plotfile: cell header write failed");
    }
    if (!h) return fail(OCFD_BAD_ARG, "plotfile: header write failed");
    return OCFD_OK;
}

// ---------------------------------------------------------------- reading
struct PlotData {
    int ncomp = 0, nlev = 0;
    std::vector<std::string> names;
    std::vector<std::array<double, 3>> dx;
    std::vector<std::vector<ocfd_box>> boxes;
    std::vector<std::vector<std::vector<double>>> fab;  // [lev][box] ncomp x cells
};

static bool parse_box(const std::string& s, size_t& pos, ocfd_box& b) {
    int v[9];
    const char* p = s.c_str() + pos;
    int used = 0;
    if (std::sscanf(p, " ((%d,%d,%d) (%d,%d,%d) (%d,%d,%d))%n", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6],
                    &v[7], &v[8], &used) != 9)
        return false;
    for (int e = 0; e < 3; ++e) {
        b.lo[e] = v[e];
        b.hi[e] = v[3 + e];
    }
    pos += used;
    return true;
}

static ocfd_status plotfile_read(const std::string& dir, PlotData& P) {
    std::ifstream h(dir + "/Header");
    if (!h) return fail(OCFD_BAD_ARG, "plotfile: no header in " + dir);
    std::string line;
    std::getline(h, line);
    if (line.rfind("HyperCLaw-V1.1", 0) != 0) return fail(OCFD_BAD_ARG, "plotfile: unknown version " + line);
    h >> P.ncomp;
    std::getline(h, line);
    for (int n = 0; n < P.ncomp; ++n) {
        std::getline(h, line);
        P.names.push_back(line);
    }
    int dim, finest;
    double time;
    h >> dim >> time >> finest;
    if (dim != 3) return fail(OCFD_BAD_ARG, "plotfile: only 3D files");
    P.nlev = finest + 1;
    double plo[3], phi[3];
    h >> plo[0] >> plo[1] >> plo[2] >> phi[0] >> phi[1] >> phi[2];
    std::getline(h, line);
    std::getline(h, line);  // ratios
    std::getline(h, line);  // level domains
    std::getline(h, line);  // level steps
    P.dx.resize(P.nlev);
    for (int l = 0; l < P.nlev; ++l) h >> P.dx[l][0] >> P.dx[l][1] >> P.dx[l][2];
    int coord, bw;
    h >> coord >> bw;
    P.boxes.resize(P.nlev);
    P.fab.resize(P.nlev);
    for (int l = 0; l < P.nlev; ++l) {
        int lev, ngrid, step;
        double t;
        h >> lev >> ngrid >> t >> step;
        double x0, x1;
        for (int b = 0; b < ngrid * 3; ++b) h >> x0 >> x1;
        std::string rel;
        h >> rel;
        // VisMF header of the level
        const std::string ld = dir + "/" + rel.substr(0, rel.find('/'));
        std::ifstream c(ld + "/Cell_H");
        if (!c) return fail(OCFD_BAD_ARG, "plotfile: no Cell_H in " + ld);
        int version, how, nc, ng;
        c >> version >> how >> nc >> ng;
        if (nc != P.ncomp) return fail(OCFD_BAD_ARG, "plotfile: component count mismatch");
        std::string rest;
        std::getline(c, rest);
        std::getline(c, rest);  // "(n 0"
        for (int b = 0; b < ngrid; ++b) {
            std::getline(c, rest);
            ocfd_box bx{};
            size_t pos = 0;
            if (!parse_box(rest, pos, bx)) return fail(OCFD_BAD_ARG, "plotfile: bad box line");
            P.boxes[l].push_back(bx);
        }
        std::getline(c, rest);  // ")"
        int nfab;
        c >> nfab;
        for (int b = 0; b < nfab; ++b) {
            std::string tag, fname;
            long long off;
            c >> tag >> fname >> off;
            std::ifstream d(ld + "/" + fname, std::ios::binary);
            if (!d) return fail(OCFD_BAD_ARG, "plotfile: missing " + fname);
            d.seekg(off);
            std::string fl;
            std::getline(d, fl);
            const size_t q = fl.find(")((");
            if (fl.rfind("FAB ", 0) != 0 || q == std::string::npos) return fail(OCFD_BAD_ARG, "plotfile: bad FAB header");
            if (fl.find(kRealDesc) == std::string::npos)
                return fail(OCFD_UNSUPPORTED, "plotfile: only little-endian IEEE double data");
            ocfd_box fb{};
            size_t pos = q + 1;
            if (!parse_box(fl, pos, fb)) return fail(OCFD_BAD_ARG, "plotfile: bad FAB box");
            const long long ncell = box_cells(fb);
            std::vector<double> v((size_t)ncell * P.ncomp);
            d.read(reinterpret_cast<char*>(v.data()), sizeof(double) * v.size());
            if (!d) return fail(OCFD_BAD_ARG, "plotfile: short FAB data");
            P.fab[l].push_back(std::move(v));
        }
    }
    return OCFD_OK;
}

static double value_at(const PlotData& P, int l, int n, const int* c, bool* found) {
    for (size_t b = 0; b < P.boxes[l].size(); ++b) {
        const ocfd_box& B = P.boxes[l][b];
        if (c[0] < B.lo[0] || c[0] > B.hi[0] || c[1] < B.lo[1] || c[1] > B.hi[1] || c[2] < B.lo[2] || c[2] > B.hi[2])
            continue;
        const long long nx = B.hi[0] - B.lo[0] + 1, ny = B.hi[1] - B.lo[1] + 1;
        const long long idx = (c[0] - B.lo[0]) + nx * ((c[1] - B.lo[1]) + ny * (long long)(c[2] - B.lo[2]));
        *found = true;
        return P.fab[l][b][(size_t)n * box_cells(B) + idx];
    }
    *found = false;
    return 0.0;
}

}  // namespace ocfd

using namespace ocfd;

extern "C" {

ocfd_status ocfd_plotfile_write(const char* dir, int32_t nlev, const ocfd_plot_level* levels, int32_t ncomp,
                                const char* const* names, const ocfd_box* domain0, const double prob_lo[3],
                                const double prob_hi[3], int32_t ref_ratio, double time) {
    if (!dir || !domain0 || !prob_lo || !prob_hi || ref_ratio != 2)
        return fail(OCFD_BAD_ARG, "ocfd_plotfile_write: bad arguments (ratio 2 only)");
    return plotfile_write(dir, nlev, levels, ncomp, names, *domain0, prob_lo, prob_hi, ref_ratio, time);
}

ocfd_status ocfd_plotfile_info(const char* file, int32_t* nlev, int32_t* ncomp) {
    if (!file) return fail(OCFD_BAD_ARG, "ocfd_plotfile_info");
    PlotData P;
    ocfd_status s = plotfile_read(file, P);
    if (s != OCFD_OK) return s;
    if (nlev) *nlev = P.nlev;
    if (ncomp) *ncomp = P.ncomp;
    return OCFD_OK;
}

ocfd_status ocfd_plotfile_compare(const char* file_a, const char* file_b, int32_t norm, int32_t allow_diff_grids,
                                  int32_t cap, double* abs_err, double* rel_err, int32_t* nan_flags,
                                  int32_t* nlev_out, int32_t* ncomp_out) {
    if (!file_a || !file_b || norm < 0 || norm > 2) return fail(OCFD_BAD_ARG, "ocfd_plotfile_compare: arguments");
    PlotData A, B;
    ocfd_status s = plotfile_read(file_a, A);
    if (s == OCFD_OK) s = plotfile_read(file_b, B);
    if (s != OCFD_OK) return s;
    if (A.nlev != B.nlev) return fail(OCFD_BAD_ARG, "fcompare: number of levels do not match");
    if (A.ncomp != B.ncomp) return fail(OCFD_BAD_ARG, "fcompare: number of variables do not match");
    for (int n = 0; n < A.ncomp; ++n)
        if (A.names[n] != B.names[n]) return fail(OCFD_BAD_ARG, "fcompare: variable " + A.names[n] + " not in both files");
    if (nlev_out) *nlev_out = A.nlev;
    if (ncomp_out) *ncomp_out = A.ncomp;
    for (int l = 0; l < A.nlev; ++l) {
        for (int e = 0; e < 3; ++e)
            if (A.dx[l][e] != B.dx[l][e]) return fail(OCFD_BAD_ARG, "fcompare: grid dx does not match");
        bool same = A.boxes[l].size() == B.boxes[l].size();
        for (size_t b = 0; same && b < A.boxes[l].size(); ++b)
            same = std::memcmp(&A.boxes[l][b], &B.boxes[l][b], sizeof(ocfd_box)) == 0;
        if (!same && !allow_diff_grids) return fail(OCFD_BAD_ARG, "fcompare: grids do not match");
        const double dv = A.dx[l][0] * A.dx[l][1] * A.dx[l][2];
        for (int n = 0; n < A.ncomp; ++n) {
            double num = 0.0, den = 0.0;
            bool nan_a = false, nan_b = false;
            for (size_t b = 0; b < A.boxes[l].size(); ++b) {
                const ocfd_box& X = A.boxes[l][b];
                const long long nc = box_cells(X);
                const double* pa = A.fab[l][b].data() + (size_t)n * nc;
                const double* pb = same ? B.fab[l][b].data() + (size_t)n * nc : nullptr;
                long long c = 0;
                for (int k = X.lo[2]; k <= X.hi[2]; ++k)
                    for (int j = X.lo[1]; j <= X.hi[1]; ++j)
                        for (int i = X.lo[0]; i <= X.hi[0]; ++i, ++c) {
                            const double a = pa[c];
                            double bv;
                            if (pb) {
                                bv = pb[c];
                            } else {
                                const int cc[3] = {i, j, k};
                                bool found;
                                bv = value_at(B, l, n, cc, &found);
                                if (!found) return fail(OCFD_BAD_ARG, "fcompare: grids do not cover the same domain");
                            }
                            nan_a = nan_a || std::isnan(a);
                            nan_b = nan_b || std::isnan(bv);
                            const double d = std::fabs(bv - a);
                            if (norm == 0) {
                                num = std::fmax(num, d);
                                den = std::fmax(den, std::fabs(a));
                            } else if (norm == 1) {
                                num += d;
                                den += std::fabs(a);
                            } else {
                                num += d * d;
                                den += a * a;
                            }
                        }
            }
            double ab = num, rel;
            if (norm == 2) {
                ab = std::sqrt(num);
                den = std::sqrt(den);
            }
            rel = den > 0 ? ab / den : (ab > 0 ? std::numeric_limits<double>::infinity() : 0.0);
            if (norm >= 1) ab *= std::pow(dv, 1.0 / norm);
            const int q = l * A.ncomp + n;
            if (q < cap) {
                if (abs_err) abs_err[q] = ab;
                if (rel_err) rel_err[q] = rel;
                if (nan_flags) nan_flags[q] = (nan_a ? 1 : 0) | (nan_b ? 2 : 0);
            }
        }
    }
    return OCFD_OK;
}

}  // extern "C"
