/* CPU oracle: restatement of OpenCFD-AMR's hot-path arithmetic (test
 * infrastructure; see ocfd_oracle.h).  Every routine cites the reference
 * source it restates and keeps that source's operation order, because the
 * bit-for-bit comparison against the compiled reference depends on it. */
#include "ocfd_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NG OCFDO_NG
#define NS OCFDO_NSPEC
#define OCFDO_PI 3.14159265358979323846
/* conserved / primitive component indices (Source/IndexDefines.H:4-23) */
enum { URHO = 0, UMX = 1, UMY = 2, UMZ = 3, UEDEN = 4, NCONS = 5 };
enum { QRHO = 0, QU = 1, QV = 2, QW = 3, QPRES = 4, QT = 5, QC = 6, QGAMA = 7 };

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }

/* ------------------------------------------------------------------ layout */
typedef struct {
    int nx, ny, nz;
    long long gx, gy, gz;
} box_t;

static box_t mkbox(int nx, int ny, int nz) {
    box_t b = {nx, ny, nz, nx + 2 * NG, ny + 2 * NG, nz + 2 * NG};
    return b;
}
static inline long long gN(const box_t* b) { return b->gx * b->gy * b->gz; }
static inline long long gI(const box_t* b, int i, int j, int k) {
    return (long long)(i + NG) + (long long)(j + NG) * b->gx + (long long)(k + NG) * b->gx * b->gy;
}
static inline long long bN(const box_t* b) { return (long long)b->nx * b->ny * b->nz; }
static inline long long bI(const box_t* b, int i, int j, int k) {
    return (long long)i + (long long)j * b->nx + (long long)k * b->nx * b->ny;
}
/* face box of direction d */
static inline long long fN(const box_t* b, int d) {
    return (long long)(b->nx + (d == 0)) * (b->ny + (d == 1)) * (b->nz + (d == 2));
}
static inline long long fI(const box_t* b, int d, int i, int j, int k) {
    long long sx = b->nx + (d == 0), sy = b->ny + (d == 1);
    return (long long)i + (long long)j * sx + (long long)k * sx * sy;
}
/* all-nodal box */
static inline long long nN(const box_t* b) {
    return (long long)(b->nx + 1) * (b->ny + 1) * (b->nz + 1);
}
static inline long long nI(const box_t* b, int i, int j, int k) {
    return (long long)i + (long long)j * (b->nx + 1) + (long long)k * (b->nx + 1) * (b->ny + 1);
}
static const int E[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

static void* xcalloc(long long n, size_t sz) {
    void* p = calloc((size_t)(n > 0 ? n : 1), sz);
    if (!p) abort();
    return p;
}

/* -------------------------------------------------------------------- Parm */
/* Source/Constants.H:9-30 defaults and Source/Constants.cpp:7-180.  The
 * Li-Dryer data tables have to be the reference's values exactly; they are
 * checked against the compiled reference in tests/test_oracle_vs_ref.py. */
static const double MW[NS] = {2.016e-3, 31.998e-3, 18.015e-3, 1.008e-3, 15.999e-3,
                              17.007e-3, 33.006e-3, 34.014e-3, 28.014e-3};
static const double NASA_LO[NS][7] = {
    {3.29812, 8.24944e-4, -81.43015e-8, -9.47543e-11, 413.48718e-15, -0.01013e+5, -3.29409},
    {3.21294, 11.27486e-4, -57.56150e-8, 131.38770e-11, -876.8554e-15, -0.01005e+5, 6.03474},
    {3.38684, 34.74982e-4, -635.4696e-8, 696.8581e-11, -2506.588e-15, -0.30208e+5, 2.59023},
    {2.5, 0.0, 0.0, 0.0, 0.0, 0.25472e+5, -0.46012},
    {2.94643, -16.3817e-4, 242.10320e-8, -160.284e-11, 389.06961e-15, 0.29148e+5, 2.96399},
    {3.63727, 1.85091e-4, -167.6165e-8, 238.72031e-11, -843.1442e-15, 0.03607e+5, 1.35886},
    {2.97996, 49.96697e-4, -379.0997e-8, 235.41919e-11, -808.9024e-15, 0.00176e+5, 9.22272},
    {3.38875, 65.69226e-4, -14.85013e-8, -462.58060e-11, 2471.515e-15, -0.17663e+5, 6.78536},
    {3.29868, 14.08240e-4, -396.3222e-8, 564.15149e-11, -2444.855e-15, -0.01021e+5, 3.95037}};
static const double NASA_HI[NS][7] = {
    {2.99142, 7.00064e-4, -5.63383e-8, -0.92316e-11, 1.58275e-15, -0.00835e+5, -1.35511},
    {3.69758, 6.13520e-4, -12.58842e-8, 1.77528e-11, -1.13644e-15, -0.01234e+5, 3.18917},
    {2.67215, 30.56293e-4, -87.30260e-8, 12.00996e-11, -6.39162e-15, -0.29899e+5, 6.86282},
    {2.5, 0.0, 0.0, 0.0, 0.0, 0.25472e+5, -0.46012},
    {2.54206, -0.27551e-4, -0.31028e-8, 0.45511e-11, -0.43681e-15, 0.29231e+5, 4.92031},
    {2.88273, 10.13974e-4, -22.76877e-8, 2.17468e-11, -0.51263e-15, 0.03887e+5, 5.59571},
    {4.07219, 21.31296e-4, -53.08145e-8, 6.11227e-11, -2.84116e-15, -0.00158e+5, 3.47603},
    {4.57317, 43.36136e-4, -147.4689e-8, 23.48904e-11, -14.31654e-15, -0.18007e+5, 0.50114},
    {2.92664, 14.87977e-4, -56.84761e-8, 10.09704e-11, -6.75335e-15, -0.00923e+5, 5.98053}};
static const double VISC[NS * 5] = {
    -1.85174759e-04, 3.89197447e-04, -6.98160471e-05, 6.36454790e-06, -2.11216442e-07,
    -5.80149070e-03, 3.39295201e-03, -6.36767978e-04, 5.43779133e-05, -1.73237416e-06,
    1.49332282e-02, -8.19367041e-03, 1.68282727e-03, -1.45738528e-04, 4.60116686e-06,
    -5.03440195e-03, 2.77694310e-03, -5.05779281e-04, 4.17970313e-05, -1.28989348e-06,
    -4.25439228e-03, 2.69409815e-03, -5.12461257e-04, 4.46919118e-05, -1.45052986e-06,
    -4.31987570e-03, 2.73556559e-03, -5.20349037e-04, 4.53798077e-05, -1.47285635e-06,
    -5.84665026e-03, 3.41936319e-03, -6.41724663e-04, 5.48011981e-05, -1.74585918e-06,
    -5.89078698e-03, 3.44517618e-03, -6.46569083e-04, 5.52148957e-05, -1.75903878e-06,
    -4.86883676e-03, 2.91081563e-03, -5.49840279e-04, 4.73395563e-05, -1.51957597e-06};
static const double COND[NS * 5] = {
    -5.28463600e-01, 3.15473947e-01, -6.87861093e-02, 6.58583530e-03, -2.30878456e-04,
    3.45755008e-02, -2.10056875e-02, 4.78193956e-03, -4.69828968e-04, 1.73609698e-05,
    -2.42370932e-01, 1.55066730e-01, -3.67910197e-02, 3.82882196e-03, -1.45626051e-04,
    -2.05169993e-01, 1.03579992e-01, -1.83028199e-02, 1.47068561e-03, -4.35660111e-05,
    5.22190001e-02, -3.07414624e-02, 7.02757543e-03, -7.03400778e-04, 2.64083229e-05,
    -1.41026759e-01, 8.85651492e-02, -2.02651378e-02, 2.03706447e-03, -7.50266004e-05,
    -7.12040025e-02, 4.31981643e-02, -9.82859052e-03, 1.00407694e-03, -3.78442817e-05,
    -1.18157269e-02, 9.27318610e-03, -2.71924641e-03, 3.59761794e-04, -1.62746865e-05,
    4.77081884e-02, -2.51859514e-02, 4.94733498e-03, -4.15782937e-04, 1.29219096e-05};
static const double DIFF[45 * 5] = {
    -0.006098424587788583, 0.004074726320140367, -0.0007655079217743792, 7.01945414920243e-05, -2.283978048241683e-06,
    -0.007361772345996411, 0.0042187108652972285, -0.0007832424157195558, 6.805076239783791e-05, -2.1468141590124147e-06,
    -0.012714368881604958, 0.005800464307529211, -0.0008628173792959883, 5.797865818973548e-05, -1.3148664989894858e-06,
    -0.02331895278393948, 0.012988306044054893, -0.0023909974764966175, 0.00020481645048811995, -6.393432695483336e-06,
    -0.008203316666546017, 0.004854681011212246, -0.0009069544030339767, 7.98972126021157e-05, -2.5440602562722086e-06,
    -0.008176066416389936, 0.004838554451993892, -0.0009039416296196897, 7.963180543591231e-05, -2.535609250271386e-06,
    -0.007355106588534061, 0.004214891010226138, -0.000782533224544873, 6.798914545886926e-05, -2.144870314265137e-06,
    -0.00734883038938788, 0.0042112943940458315, -0.0007818654797209853, 6.793112951970908e-05, -2.143040071146875e-06,
    -0.006631024777860074, 0.0038397370846872426, -0.0007137696048348218, 6.226499117199988e-05, -1.968810850179303e-06,
    -0.003165622529780972, 0.0016565295961648823, -0.0002955102867456441, 2.4323268960998937e-05, -7.332687938295335e-07,
    0.0017962300955720687, -0.0016252040565658543, 0.00047039226523034656, -5.1041731991760684e-05, 1.9707403545544835e-06,
    -0.02065558573348347, 0.01049932817565325, -0.0018228205967741945, 0.00014586133392843038, -4.265266434634806e-06,
    -0.004477615809775433, 0.002401743913536847, -0.00043555046112257176, 3.6523201605646507e-05, -1.1207561496132533e-06,
    -0.004388261916818509, 0.002353815467310766, -0.00042685875309455987, 3.579435608041233e-05, -1.0983906923530078e-06,
    -0.003141360101617588, 0.0016438333792438298, -0.0002932453934942289, 2.4136846998057358e-05, -7.276487676670712e-07,
    -0.0031183633828342915, 0.001631799491779716, -0.00029109865398359785, 2.3960150196485035e-05, -7.223219240282344e-07,
    -0.0030766151054801255, 0.001623930137648841, -0.0002916902121621802, 2.4185952795909278e-05, -7.345781692660118e-07,
    0.015418678757875483, -0.008276025270343653, 0.0016022988850484384, -0.0001292488075144311, 3.7780416116707573e-06,
    0.015491646067634311, -0.012297762819716031, 0.0033220236270480115, -0.00034981378874120536, 1.3233960398093872e-05,
    -0.0031409034359764906, 0.000964215499007546, -1.5256977763517157e-05, -1.0009613901179592e-05, 6.865263141553794e-07,
    -0.00309121182555696, 0.0009489608368058763, -1.501560014564807e-05, -9.851253784321545e-06, 6.756649174673959e-07,
    -9.806367280891379e-05, -0.0005259982739909082, 0.00023777270488750687, -2.9610758656448636e-05, 1.2409556192468912e-06,
    -9.754926582674518e-05, -0.0005232390750052945, 0.00023652543424357053, -2.945543119768198e-05, 1.2344460095131642e-06,
    0.0009009636432407803, -0.0010975268417085945, 0.0003568805024623778, -4.047906132942509e-05, 1.6078992712041145e-06,
    -0.049547371639744826, 0.02420786673131437, -0.0040039853524907396, 0.0003046592732139884, -8.373772281551857e-06,
    -0.027018754679375097, 0.014131423473429378, -0.0025198932193017465, 0.00020732039220446453, -6.247265305088386e-06,
    -0.026971255852400414, 0.01410658050614936, -0.002515463260429814, 0.00020695592405809058, -6.236282645924077e-06,
    -0.020645950902716106, 0.01049443074735431, -0.0018219703392133265, 0.00014579329667774188, -4.2632768943398505e-06,
    -0.02063688301930936, 0.010489821500976207, -0.0018211701137997654, 0.00014572926297830028, -4.261404425595428e-06,
    -0.019430526862365516, 0.00997359743800644, -0.0017481642351558765, 0.00014128443680858248, -4.177030598880565e-06,
    -0.0059382904901673595, 0.0032649962117391896, -0.0005991311922260038, 5.1014036740744293e-05, -1.5859623241784843e-06,
    -0.00584963856139101, 0.0032162535286223044, -0.0005901868443753459, 5.02524551442533e-05, -1.5622857089560921e-06,
    -0.0044547665185479274, 0.0023894878048250404, -0.00043332784539284135, 3.633682356306633e-05, -1.1150369265388267e-06,
    -0.004433163993709295, 0.0023779004479025216, -0.00043122650618556915, 3.616061519603177e-05, -1.109629771571358e-06,
    -0.00419972224671333, 0.0022703026942310655, -0.0004131673665395828, 3.48089622951453e-05, -1.0723125190961097e-06,
    -0.005759622266467147, 0.003166760688484433, -0.0005811048417034481, 4.947915269564291e-05, -1.538244707164061e-06,
    -0.004364944907483492, 0.002341308479746039, -0.0004245906410903713, 3.5604162935439344e-05, -1.0925543985047233e-06,
    -0.004342895613050795, 0.0023294814805234227, -0.0004224458433307047, 3.542431033976762e-05, -1.0870354162206174e-06,
    -0.004119743857368838, 0.0022270676557828092, -0.0004052991175070151, 3.414606970952483e-05, -1.05189168573903e-06,
    -0.003116908817255142, 0.0016310383363007772, -0.00029096287055129454, 2.3948973946122656e-05, -7.219849958113728e-07,
    -0.0030937303493271603, 0.0016189093418438713, -0.00028879916479071873, 2.37708806629901e-05, -7.166160527175076e-07,
    -0.0030546059172749706, 0.0016123130250736487, -0.00028960354725398777, 2.40129336925455e-05, -7.293232158117316e-07,
    -0.003070376910660832, 0.001606688787447522, -0.00028661912554336986, 2.35914429806519e-05, -7.112065802854437e-07,
    -0.0030337554543677816, 0.0016013075226178426, -0.00028762673971045356, 2.3849023585380798e-05, -7.243449216977582e-07,
    -0.0029800170761932095, 0.0015859694924580709, -0.000286608674495536, 2.3921390316404743e-05, -7.312450753144484e-07};

void ocfdo_parm_default(ocfdo_parm* p) {
    memset(p, 0, sizeof(*p));
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
    /* Parm::Initialize, Source/Constants.cpp:9-12 */
    p->Rg = p->Ru / p->eos_m;
    p->cv = p->Rg / (p->eos_gamma - 1.0);
    p->cp = p->eos_gamma * p->cv;
    p->kOverMu = p->cp / p->Pr;
    for (int n = 0; n < NS; ++n) {
        p->mw[n] = MW[n];
        for (int c = 0; c < 7; ++c) {
            p->nasa_lo[n][c] = NASA_LO[n][c];
            p->nasa_hi[n][c] = NASA_HI[n][c];
        }
        p->HP[n] = NASA_LO[n][5];
        p->A0[n] = NASA_LO[n][0] - 1.0;
    }
    memcpy(p->visccoeff, VISC, sizeof VISC);
    memcpy(p->conductcoeff, COND, sizeof COND);
    memcpy(p->diffcoeff, DIFF, sizeof DIFF);
}

/* ------------------------------------------------------------ ideal gas */
/* c2prim, Source/kernel/Kernels.H:13-40 */
static void c2prim_ideal(const ocfdo_parm* p, const double* u, double* q) {
    double rho = dmax(u[URHO], p->smallr);
    double rhoinv = 1.0 / rho;
    double ux = u[UMX] * rhoinv, uy = u[UMY] * rhoinv, uz = u[UMZ] * rhoinv;
    double kineng = 0.5 * (ux * ux + uy * uy + uz * uz);
    double ei = u[UEDEN] - rho * kineng;
    double pr = dmax((p->eos_gamma - 1.0) * ei, p->smallp);
    double T = pr / (rho * p->Rg);
    q[QRHO] = rho; q[QU] = ux; q[QV] = uy; q[QW] = uz;
    q[QPRES] = pr; q[QT] = T;
    q[QC] = sqrt(p->eos_gamma * p->Rg * T);
}

/* Steger-Warming split along d, Source/kernel/FluxSplit.H:11-193 (the three
 * direction copies differ only in which velocity is normal). */
static void sw_split(double gamma, const double* q, int d, double* fp, double* fm) {
    double dd = q[QRHO], c = q[QC];
    double vel[3] = {q[QU], q[QV], q[QW]};
    double un = vel[d];
    double tmp1 = 1.0 / (2.0 * gamma);
    double tmp2 = 2.0 * (gamma - 1.0);
    double tmp3 = (3.0 - gamma) / (2.0 * (gamma - 1.0));
    double a[3] = {vel[0], vel[1], vel[2]}, b[3] = {vel[0], vel[1], vel[2]};
    double uc1 = un - c, uc2 = un + c;
    a[d] = uc1; b[d] = uc2;
    double vvc1 = 0.5 * (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    double vvc2 = 0.5 * (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    double v2 = (gamma - 1) * (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
    double w2 = tmp3 * c * c;
    double E1 = un, E2 = un - c, E3 = un + c;
    double E1P = (E1 + fabs(E1)) * 0.5, E2P = (E2 + fabs(E2)) * 0.5, E3P = (E3 + fabs(E3)) * 0.5;
    double E1M = E1 - E1P, E2M = E2 - E2P, E3M = E3 - E3P;
    double tmp0 = dd * tmp1;
    fp[URHO] = tmp0 * (tmp2 * E1P + E2P + E3P);
    fm[URHO] = tmp0 * (tmp2 * E1M + E2M + E3M);
    for (int m = 0; m < 3; ++m) {
        if (m == d) {
            fp[UMX + m] = tmp0 * (tmp2 * E1P * un + E2P * uc1 + E3P * uc2);
            fm[UMX + m] = tmp0 * (tmp2 * E1M * un + E2M * uc1 + E3M * uc2);
        } else {
            fp[UMX + m] = tmp0 * vel[m] * (tmp2 * E1P + E2P + E3P);
            fm[UMX + m] = tmp0 * vel[m] * (tmp2 * E1M + E2M + E3M);
        }
    }
    fp[UEDEN] = tmp0 * (E1P * v2 + E2P * vvc1 + E3P * vvc2 + w2 * (E2P + E3P));
    fm[UEDEN] = tmp0 * (E1M * v2 + E2M * vvc1 + E3M * vvc2 + w2 * (E2M + E3M));
}

/* WENO-Z, Source/kernel/Reconstruction.H:83-138.  Upwind-biased value from
 * f+ at cells i-3..i+1 (V1..V5) ... */
static double wenoz_plus(double V1, double V2, double V3, double V4, double V5) {
    const double eps = 1e-6;
    double s11 = (13.0 / 12.0) * (V1 - 2.0 * V2 + V3) * (V1 - 2.0 * V2 + V3) +
                 0.25 * (V1 - 4.0 * V2 + 3.0 * V3) * (V1 - 4.0 * V2 + 3.0 * V3);
    double s22 = (13.0 / 12.0) * (V2 - 2.0 * V3 + V4) * (V2 - 2.0 * V3 + V4) +
                 0.25 * (V2 - V4) * (V2 - V4);
    double s33 = (13.0 / 12.0) * (V3 - 2.0 * V4 + V5) * (V3 - 2.0 * V4 + V5) +
                 0.25 * (3.0 * V3 - 4.0 * V4 + V5) * (3.0 * V3 - 4.0 * V4 + V5);
    double s55 = fabs(s11 - s33);
    s11 = 1.0 + (s55 / (eps + s11)) * (s55 / (eps + s11));
    s22 = 1.0 + (s55 / (eps + s22)) * (s55 / (eps + s22));
    s33 = 1.0 + (s55 / (eps + s33)) * (s55 / (eps + s33));
    double a1 = s11, a2 = 6.0 * s22, a3 = 3.0 * s33;
    double invsum = 1.0 / (a1 + a2 + a3);
    double v1 = 2.0 * V1 - 7.0 * V2 + 11.0 * V3;
    double v2 = -V2 + 5.0 * V3 + 2.0 * V4;
    double v3 = 2.0 * V3 + 5.0 * V4 - V5;
    return (1.0 / 6.0) * invsum * (a1 * v1 + a2 * v2 + a3 * v3);
}
/* ... and from f- at cells i-2..i+2 (V1..V5), the mirrored stencil. */
static double wenoz_minus(double V1, double V2, double V3, double V4, double V5) {
    const double eps = 1e-6;
    double s11 = (13.0 / 12.0) * (V5 - 2.0 * V4 + V3) * (V5 - 2.0 * V4 + V3) +
                 0.25 * (V5 - 4.0 * V4 + 3.0 * V3) * (V5 - 4.0 * V4 + 3.0 * V3);
    double s22 = (13.0 / 12.0) * (V2 - 2.0 * V3 + V4) * (V2 - 2.0 * V3 + V4) +
                 0.25 * (V4 - V2) * (V4 - V2);
    double s33 = (13.0 / 12.0) * (V3 - 2.0 * V2 + V1) * (V3 - 2.0 * V2 + V1) +
                 0.25 * (3.0 * V3 - 4.0 * V2 + V1) * (3.0 * V3 - 4.0 * V2 + V1);
    double s55 = fabs(s11 - s33);
    s11 = 1.0 + (s55 / (eps + s11)) * (s55 / (eps + s11));
    s22 = 1.0 + (s55 / (eps + s22)) * (s55 / (eps + s22));
    s33 = 1.0 + (s55 / (eps + s33)) * (s55 / (eps + s33));
    double a1 = s11, a2 = 6.0 * s22, a3 = 3.0 * s33;
    double invsum = 1.0 / (a1 + a2 + a3);
    double v1 = 11.0 * V3 - 7.0 * V4 + 2.0 * V5;
    double v2 = -V4 + 5.0 * V3 + 2.0 * V2;
    double v3 = 2.0 * V3 + 5.0 * V2 - V1;
    return (1.0 / 6.0) * invsum * (a1 * v1 + a2 * v2 + a3 * v3);
}

/* face value of component array f+ (fp) / f- (fm) at the d-face of cell (i,j,k) */
static double weno_face(const box_t* b, const double* fp, const double* fm, int d, int i, int j,
                        int k) {
    int di = E[d][0], dj = E[d][1], dk = E[d][2];
#define AT(a, o) a[gI(b, i + (o) * di, j + (o) * dj, k + (o) * dk)]
    double fpx = wenoz_plus(AT(fp, -3), AT(fp, -2), AT(fp, -1), AT(fp, 0), AT(fp, 1));
    double fmx = wenoz_minus(AT(fm, -2), AT(fm, -1), AT(fm, 0), AT(fm, 1), AT(fm, 2));
#undef AT
    return fpx + fmx;
}

static inline double sutherland(const ocfdo_parm* p, double T) {
    return p->C_s * T * sqrt(T) / (T + p->T_s);
}

/* transverse central derivative of primitive m along t at the d-face of cell c,
 * averaging the two cells c and c-e_d (Source/kernel/Diffusion.H:31-34 etc.) */
static double tderiv(const box_t* b, const double* q, int m, int d, int t, int i, int j, int k,
                     double dxinv_t) {
    const double* qm = q + (long long)m * gN(b);
    int ti = E[t][0], tj = E[t][1], tk = E[t][2];
    int li = i - E[d][0], lj = j - E[d][1], lk = k - E[d][2];
    return (qm[gI(b, i + ti, j + tj, k + tk)] + qm[gI(b, li + ti, lj + tj, lk + tk)] -
            qm[gI(b, i - ti, j - tj, k - tk)] - qm[gI(b, li - ti, lj - tj, lk - tk)]) *
           (0.25 * dxinv_t);
}

/* Viscous stress and heat flux added to the d-face flux,
 * Source/kernel/Diffusion.H:7-131.  multi != 0 selects the multispecies form of
 * Source/CHEM/ChemViscous.H:201-355 (face-averaged mu, lambda and the species
 * enthalpy flux `hflux`). */
static void visc_face(const ocfdo_parm* p, const box_t* b, const double* q, int d, int i, int j,
                      int k, const double* dxinv, double* f /* 5 comps, stride fs */, long long fs,
                      int multi, double mu_f, double lam_f, double hflux) {
    long long c = gI(b, i, j, k), l = gI(b, i - E[d][0], j - E[d][1], k - E[d][2]);
    long long N = gN(b);
    double Tr = q[QT * N + c], Tl = q[QT * N + l];
    double muf = 0, ksum = 0;
    if (!multi) {
        double mutl = sutherland(p, Tl), mutr = sutherland(p, Tr);
        double ktl = mutl * p->kOverMu, ktr = mutr * p->kOverMu;
        muf = 0.5 * (mutl + mutr);
        ksum = ktl + ktr;
    } else {
        muf = mu_f;
    }
    double dT = (Tr - Tl) * dxinv[d];
    /* g[m][t]: d(vel m)/d(x_t) at the face */
    double g[3][3];
    for (int m = 0; m < 3; ++m) g[m][d] = (q[(QU + m) * N + c] - q[(QU + m) * N + l]) * dxinv[d];
    for (int t = 0; t < 3; ++t) {
        if (t == d) continue;
        g[d][t] = tderiv(b, q, QU + d, d, t, i, j, k, dxinv[t]);
        g[t][t] = tderiv(b, q, QU + t, d, t, i, j, k, dxinv[t]);
    }
    double divu = g[0][0] + g[1][1] + g[2][2];
    double tau[3];
    for (int m = 0; m < 3; ++m) {
        if (m == d)
            tau[m] = muf * (2.0 * g[d][d] - p->twoThirds * divu);
        else
            tau[m] = muf * (g[m][d] + g[d][m]);
    }
    for (int m = 0; m < 3; ++m) f[(UMX + m) * fs] += -tau[m];
    double ubar0 = q[QU * N + c] + q[QU * N + l];
    double ubar1 = q[QV * N + c] + q[QV * N + l];
    double ubar2 = q[QW * N + c] + q[QW * N + l];
    if (!multi) {
        f[UEDEN * fs] += -0.5 * (ubar0 * tau[0] + ubar1 * tau[1] + ubar2 * tau[2] + ksum * dT);
    } else {
        f[UEDEN * fs] += -0.5 * (ubar0 * tau[0] + ubar1 * tau[1] + ubar2 * tau[2]) - lam_f * dT - hflux;
    }
}

void ocfdo_c2prim(const ocfdo_parm* p, int chem, const double* S, const double* spec, int nx,
                  int ny, int nz, double* q);

void ocfdo_rhs_regular(const ocfdo_parm* p, const double* S, int nx, int ny, int nz,
                       const double* dxinv, int do_visc, double* dSdt, double* fx, double* fy,
                       double* fz) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b);
    double* q = (double*)xcalloc(N * 7, sizeof(double));
    double* fp = (double*)xcalloc(N * NCONS, sizeof(double));
    double* fm = (double*)xcalloc(N * NCONS, sizeof(double));
    double* fl[3] = {fx, fy, fz};
    ocfdo_c2prim(p, 0, S, NULL, nx, ny, nz, q);
    for (int d = 0; d < 3; ++d) {
        long long FN = fN(&b, d);
        memset(fl[d], 0, sizeof(double) * FN * NCONS);
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (long long c = 0; c < N; ++c) {
            double qc[7], a[5], m[5];
            for (int n = 0; n < 7; ++n) qc[n] = q[n * N + c];
            sw_split(p->eos_gamma, qc, d, a, m);
            for (int n = 0; n < 5; ++n) { fp[n * N + c] = a[n]; fm[n * N + c] = m[n]; }
        }
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int k = 0; k < nz + (d == 2); ++k)
            for (int j = 0; j < ny + (d == 1); ++j)
                for (int i = 0; i < nx + (d == 0); ++i) {
                    long long fi = fI(&b, d, i, j, k);
                    for (int n = 0; n < NCONS; ++n)
                        fl[d][n * FN + fi] = weno_face(&b, fp + n * N, fm + n * N, d, i, j, k);
                    if (do_visc & 1) visc_face(p, &b, q, d, i, j, k, dxinv, fl[d] + fi, FN, 0, 0, 0, 0);
                }
    }
    long long BN = bN(&b);
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                for (int n = 0; n < NCONS; ++n) {
                    /* divop, Source/kernel/Kernels.H:84-97 */
                    dSdt[n * BN + bI(&b, i, j, k)] =
                        dxinv[0] * (fx[n * fN(&b, 0) + fI(&b, 0, i, j, k)] - fx[n * fN(&b, 0) + fI(&b, 0, i + 1, j, k)]) +
                        dxinv[1] * (fy[n * fN(&b, 1) + fI(&b, 1, i, j, k)] - fy[n * fN(&b, 1) + fI(&b, 1, i, j + 1, k)]) +
                        dxinv[2] * (fz[n * fN(&b, 2) + fI(&b, 2, i, j, k)] - fz[n * fN(&b, 2) + fI(&b, 2, i, j, k + 1)]);
                }
    if (do_visc & 2) {
        /* do_gravity, Source/Advance.cpp:331-342: g = -9.8 on the z momentum and the energy */
        const double g = -9.8;
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    long long c = bI(&b, i, j, k), gc = gI(&b, i, j, k);
                    dSdt[3 * BN + c] += g * S[0 * N + gc];
                    dSdt[4 * BN + c] += g * S[3 * N + gc];
                }
    }
    free(q); free(fp); free(fm);
}

/* ------------------------------------------------------------------ EB */
static inline int conn(uint32_t f, int i, int j, int k) {
    int p = 4 + (i + 1) + 3 * (j + 1) + 9 * (k + 1);
    return p >= 0 && p < 32 && ((f >> p) & 1u);
}
static inline int is_covered(uint32_t f) { return (f & 3u) == 3u; }
static inline int is_regular(uint32_t f) { return (f & 3u) == 0u; }

static double minmod(double a, double b) {
    /* Source/kernel/Reconstruction.H:8-19 */
    if (a * b > 0) return fabs(a) > fabs(b) ? b : a;
    return 0.0;
}

/* eb_recon_x/y/z, Source/EB/EBkernels.H:9-71: MUSCL-minmod left/right states at
 * the d-face of cell (i,j,k) for one component array v (grown layout). */
static void eb_recon(const box_t* b, const uint32_t* flag, const double* v, int d, int i, int j,
                     int k, double* l, double* r) {
    int di = E[d][0], dj = E[d][1], dk = E[d][2];
    double v0 = v[gI(b, i, j, k)], vm1 = v[gI(b, i - di, j - dj, k - dk)];
    double vm2 = v[gI(b, i - 2 * di, j - 2 * dj, k - 2 * dk)], vp1 = v[gI(b, i + di, j + dj, k + dk)];
    uint32_t f = flag[gI(b, i, j, k)];
    *l = vm1;
    *r = v0;
    if (conn(f, -di, -dj, -dk)) {
        if (conn(f, -2 * di, -2 * dj, -2 * dk)) *l = vm1 + 0.5 * minmod(v0 - vm1, vm1 - vm2);
        if (conn(f, di, dj, dk)) *r = v0 - 0.5 * minmod(vp1 - v0, v0 - vm1);
    }
}

/* Van Leer flux, Source/EB/EBkernels.H:73-171 */
static void vanleer(const ocfdo_parm* p, int chem, const double* ql, const double* qr, int d,
                    double* flx) {
    double fp[5] = {0, 0, 0, 0, 0}, fm[5] = {0, 0, 0, 0, 0};
    double dl = ql[QRHO], ul = ql[QU], vl = ql[QV], wl = ql[QW], pl = dmax(ql[QPRES], p->smallp);
    double dr = qr[QRHO], ur = qr[QU], vr = qr[QV], wr = qr[QW], pr = dmax(qr[QPRES], p->smallp);
    double gamma = chem ? 0.5 * (ql[QGAMA] + qr[QGAMA]) : p->eos_gamma;
    double cL = ql[QC], cR = qr[QC];
    int nn[3] = {d == 0, d == 1, d == 2};
    double UL = d == 0 ? ul : (d == 1 ? vl : wl);
    double UR = d == 0 ? ur : (d == 1 ? vr : wr);
    double ML = UL / cL, MR = UR / cR;
    double lv[3] = {ul, vl, wl}, rv[3] = {ur, vr, wr};
    if (ML >= 1.0) {
        fp[0] = dl * UL;
        for (int m = 0; m < 3; ++m) fp[1 + m] = dl * UL * lv[m] + nn[m] * pl;
        fp[4] = UL * (gamma * pl / (gamma - 1.0) + 0.5 * dl * (ul * ul + vl * vl + wl * wl));
    } else if (fabs(ML) < 1.0) {
        double Mp = 0.250 * (1.0 + ML) * (1.0 + ML);
        double tmp0 = dl * cL * Mp;
        fp[0] = tmp0;
        for (int m = 0; m < 3; ++m) fp[1 + m] = tmp0 * (nn[m] * (-UL + 2.0 * cL) / gamma + lv[m]);
        fp[4] = tmp0 * (((gamma - 1) * UL + 2 * cL) * ((gamma - 1) * UL + 2 * cL) / (2 * (gamma * gamma - 1)) +
                        (ul * ul + vl * vl + wl * wl - UL * UL) / 2);
    }
    if (fabs(MR) < 1.0) {
        double Mm = -0.250 * (MR - 1.0) * (MR - 1.0);
        double tmp0 = dr * cR * Mm;
        fm[0] = tmp0;
        for (int m = 0; m < 3; ++m) fm[1 + m] = tmp0 * (nn[m] * (-UR - 2.0 * cR) / gamma + rv[m]);
        fm[4] = tmp0 * (((gamma - 1) * UR - 2 * cR) * ((gamma - 1) * UR - 2 * cR) / (2 * (gamma * gamma - 1)) +
                        (ur * ur + vr * vr + wr * wr - UR * UR) / 2);
    } else if (MR <= -1.0) {
        fm[0] = dr * UR;
        for (int m = 0; m < 3; ++m) fm[1 + m] = dr * UR * rv[m] + nn[m] * pr;
        fm[4] = UR * (gamma * pr / (gamma - 1.0) + 0.5 * dr * (ur * ur + vr * vr + wr * wr));
    }
    for (int n = 0; n < NCONS; ++n) flx[n] = fp[n] + fm[n];
}

/* connectivity-aware transverse derivative, Source/EB/EBdiffusion.H:36-58 */
static double eb_tderiv(const box_t* b, const uint32_t* flag, const double* q, int m, int d, int t,
                        int i, int j, int k, double dxinv_t) {
    static const double weights[3] = {0., 1., 0.5};
    const double* qm = q + (long long)m * gN(b);
    int ti = E[t][0], tj = E[t][1], tk = E[t][2];
    int li = i - E[d][0], lj = j - E[d][1], lk = k - E[d][2];
    uint32_t fh = flag[gI(b, i, j, k)], fl = flag[gI(b, li, lj, lk)];
    int hip = conn(fh, ti, tj, tk), him = conn(fh, -ti, -tj, -tk);
    int lop = conn(fl, ti, tj, tk), lom = conn(fl, -ti, -tj, -tk);
    double whi = weights[hip + him], wlo = weights[lop + lom];
    return (0.5 * dxinv_t) *
           ((qm[gI(b, i + hip * ti, j + hip * tj, k + hip * tk)] - qm[gI(b, i - him * ti, j - him * tj, k - him * tk)]) * whi +
            (qm[gI(b, li + lop * ti, lj + lop * tj, lk + lop * tk)] - qm[gI(b, li - lom * ti, lj - lom * tj, lk - lom * tk)]) * wlo);
}

/* eb_compute_visc_x/y/z (Source/EB/EBdiffusion.H:8-203) and the multispecies
 * compute_visc_*_multi_eb (Source/CHEM/ChemViscous.H:357-575) */
static void eb_visc_face(const ocfdo_parm* p, const box_t* b, const uint32_t* flag,
                         const double* q, int d, int i, int j, int k, const double* dxinv,
                         double* f, long long fs, int multi, double mu_f, double lam_f,
                         double hflux) {
    long long N = gN(b);
    long long c = gI(b, i, j, k), l = gI(b, i - E[d][0], j - E[d][1], k - E[d][2]);
    double Tc = q[QT * N + c], Tm = q[QT * N + l];
    double muf, ksum = 0;
    if (!multi) {
        double mutl = sutherland(p, Tc), mutr = sutherland(p, Tm);
        muf = 0.5 * (mutl + mutr);
        ksum = mutl * p->kOverMu + mutr * p->kOverMu;
    } else {
        muf = mu_f;
    }
    double dT = (Tc - Tm) * dxinv[d];
    double g[3][3];
    for (int m = 0; m < 3; ++m) g[m][d] = (q[(QU + m) * N + c] - q[(QU + m) * N + l]) * dxinv[d];
    for (int t = 0; t < 3; ++t) {
        if (t == d) continue;
        g[d][t] = eb_tderiv(b, flag, q, QU + d, d, t, i, j, k, dxinv[t]);
        g[t][t] = eb_tderiv(b, flag, q, QU + t, d, t, i, j, k, dxinv[t]);
    }
    double divu = g[0][0] + g[1][1] + g[2][2];
    double tau[3];
    for (int m = 0; m < 3; ++m) {
        if (m == d)
            tau[m] = muf * (2.0 * g[d][d] - p->twoThirds * divu);
        else
            tau[m] = muf * (g[m][d] + g[d][m]);
    }
    for (int m = 0; m < 3; ++m) f[(UMX + m) * fs] += -tau[m];
    double ub0 = q[QU * N + c] + q[QU * N + l];
    double ub1 = q[QV * N + c] + q[QV * N + l];
    double ub2 = q[QW * N + c] + q[QW * N + l];
    if (!multi)
        f[UEDEN * fs] += -0.5 * (ub0 * tau[0] + ub1 * tau[1] + ub2 * tau[2] + ksum * dT);
    else
        f[UEDEN * fs] += -0.5 * (ub0 * tau[0] + ub1 * tau[1] + ub2 * tau[2]) - lam_f * dT - hflux;
}

/* Cut-cell divergence of one cell, Source/EB/EBkernels.H:216-338.  Writes the
 * negated divergence to out[n*os]. */
static void eb_div_cell(const ocfdo_parm* p, int chem, const box_t* b, const uint32_t* flag,
                        const double* vfrac, const double* ap[3], const double* q,
                        const double* fl[3], int ncomp, int i, int j, int k, const double* dxinv,
                        int visc_wall, double* out, long long os) {
    long long N = gN(b);
    long long c = gI(b, i, j, k);
    uint32_t f = flag[c];
    double tmp = dxinv[0] / vfrac[c];
    long long F0 = fN(b, 0), F1 = fN(b, 1), F2 = fN(b, 2);
    long long x0 = fI(b, 0, i, j, k), x1 = fI(b, 0, i + 1, j, k);
    long long y0 = fI(b, 1, i, j, k), y1 = fI(b, 1, i, j + 1, k);
    long long z0 = fI(b, 2, i, j, k), z1 = fI(b, 2, i, j, k + 1);
    if (is_covered(f)) {
        for (int n = 0; n < ncomp; ++n) out[n * os] = 0.0;
    } else if (is_regular(f)) {
        for (int n = 0; n < ncomp; ++n)
            out[n * os] = dxinv[0] * (fl[0][n * F0 + x1] - fl[0][n * F0 + x0]) +
                          dxinv[1] * (fl[1][n * F1 + y1] - fl[1][n * F1 + y0]) +
                          dxinv[2] * (fl[2][n * F2 + z1] - fl[2][n * F2 + z0]);
    } else {
        double axm = ap[0][x0], axp = ap[0][x1], aym = ap[1][y0], ayp = ap[1][y1];
        double azm = ap[2][z0], azp = ap[2][z1];
        for (int n = 0; n < ncomp; ++n)
            out[n * os] = tmp * (axp * fl[0][n * F0 + x1] - axm * fl[0][n * F0 + x0] +
                                 ayp * fl[1][n * F1 + y1] - aym * fl[1][n * F1 + y0] +
                                 azp * fl[2][n * F2 + z1] - azm * fl[2][n * F2 + z0]);
        if (ncomp == NCONS) {
            double fw[5];
            if (!visc_wall) {
                /* slip-wall pressure flux, EBkernels.H:305-311 */
                double pr = q[QPRES * N + c];
                fw[0] = 0.0;
                fw[1] = (axm - axp) * pr;
                fw[2] = (aym - ayp) * pr;
                fw[3] = (azm - azp) * pr;
                fw[4] = 0.0;
            } else {
                /* eb_wallflux, EBkernels.H:173-214 */
                double d = q[QRHO * N + c], u = q[QU * N + c], v = q[QV * N + c],
                       w = q[QW * N + c], pr = q[QPRES * N + c], cs = q[QC * N + c];
                double apnorm = sqrt((axm - axp) * (axm - axp) + (aym - ayp) * (aym - ayp) +
                                     (azm - azp) * (azm - azp));
                double un = u * (axm - axp) + v * (aym - ayp) + w * (azm - azp);
                double lambda0 = fabs(un) + cs * apnorm;
                double gamma = chem ? q[QGAMA * N + c] : p->eos_gamma;
                double E0 = pr / (gamma - 1) + 0.50 * d * (u * u + v * v + w * w);
                double fpw[5], fmw[5];
                fpw[0] = 0.5 * (d * un + lambda0 * d);
                fpw[1] = 0.5 * (d * u * un + (axm - axp) * pr + lambda0 * d * u);
                fpw[2] = 0.5 * (d * v * un + (aym - ayp) * pr + lambda0 * d * v);
                fpw[3] = 0.5 * (d * w * un + (azm - azp) * pr + lambda0 * d * w);
                fpw[4] = 0.5 * ((E0 + pr) * un + lambda0 * E0);
                fmw[0] = 0.5 * (d * (-un) - lambda0 * d);
                fmw[1] = fpw[1];
                fmw[2] = fpw[2];
                fmw[3] = fpw[3];
                fmw[4] = 0.5 * (-(E0 + pr) * un - lambda0 * E0);
                for (int n = 0; n < 5; ++n) fw[n] = fpw[n] + fmw[n];
            }
            for (int n = 0; n < NCONS; ++n) out[n * os] += fw[n] * tmp;
        }
    }
}

/* Zeroes the flux arrays of the three directions */
static void zero_faces(const box_t* b, double* fl[3], int ncomp) {
    for (int d = 0; d < 3; ++d) memset(fl[d], 0, sizeof(double) * fN(b, d) * ncomp);
}

void ocfdo_rhs_eb(const ocfdo_parm* p, const double* S, const uint32_t* flag,
                  const double* vfrac, const double* apx, const double* apy, const double* apz,
                  int nx, int ny, int nz, const double* dxinv, int do_visc, int do_redistribute,
                  double* dSdt, double* fx, double* fy, double* fz) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b), BN = bN(&b);
    double* q = (double*)xcalloc(N * 7, sizeof(double));
    double* divc = (double*)xcalloc(BN * NCONS, sizeof(double));
    double* fl[3] = {fx, fy, fz};
    const double* cfl[3] = {fx, fy, fz};
    const double* ap[3] = {apx, apy, apz};
    zero_faces(&b, fl, NCONS);
    ocfdo_c2prim(p, 0, S, NULL, nx, ny, nz, q);
    for (int d = 0; d < 3; ++d) {
        long long FN = fN(&b, d);
        for (int k = 0; k < nz + (d == 2); ++k)
            for (int j = 0; j < ny + (d == 1); ++j)
                for (int i = 0; i < nx + (d == 0); ++i) {
                    double ql[7], qr[7], flx[5];
                    for (int n = 0; n < 7; ++n) eb_recon(&b, flag, q + n * N, d, i, j, k, &ql[n], &qr[n]);
                    vanleer(p, 0, ql, qr, d, flx);
                    long long fi = fI(&b, d, i, j, k);
                    for (int n = 0; n < NCONS; ++n) fl[d][n * FN + fi] = flx[n];
                    if (do_visc) eb_visc_face(p, &b, flag, q, d, i, j, k, dxinv, fl[d] + fi, FN, 0, 0, 0, 0);
                }
    }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = bI(&b, i, j, k);
                eb_div_cell(p, 0, &b, flag, vfrac, ap, q, cfl, NCONS, i, j, k, dxinv, do_visc,
                            divc + c, BN);
                for (int n = 0; n < NCONS; ++n) divc[n * BN + c] *= -1.0;
            }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = bI(&b, i, j, k);
                double vf = vfrac[gI(&b, i, j, k)];
                if (do_redistribute && vf < 0.5 && vf > 0.0) {
                    /* flux_redist, Source/EB/EBkernels.H:341-377 (only the local rescale is live) */
                    for (int n = 0; n < NCONS; ++n) dSdt[n * BN + c] = vf * divc[n * BN + c];
                } else {
                    for (int n = 0; n < NCONS; ++n) dSdt[n * BN + c] = divc[n * BN + c];
                }
            }
    free(q); free(divc);
}

/* ------------------------------------------------------------- CFL bound */
double ocfdo_estdt(const ocfdo_parm* p, const double* S, int nx, int ny, int nz,
                   const double* dx) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b);
    double dt = DBL_MAX;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = gI(&b, i, j, k);
                double rho = S[URHO * N + c], mx = S[UMX * N + c], my = S[UMY * N + c],
                       mz = S[UMZ * N + c], En = S[UEDEN * N + c];
                double rhoinv = 1.0 / dmax(rho, p->smallr);
                double vx = mx * rhoinv, vy = my * rhoinv, vz = mz * rhoinv;
                double pr = dmax((p->eos_gamma - 1.0) * (En - 0.5 * rho * (vx * vx + vy * vy + vz * vz)),
                                 p->smallp);
                double cs = sqrt(p->eos_gamma * pr * rhoinv);
                double dtx = dx[0] / (fabs(vx) + cs);
                double dty = dx[1] / (fabs(vy) + cs);
                double dtz = dx[2] / (fabs(vz) + cs);
                dt = dmin(dt, dmin(dtx, dmin(dty, dtz)));
            }
    return dt;
}

/* =========================================================== chemistry */
static void nasa_coef(const ocfdo_parm* p, double T, int n, const double** a) {
    *a = T < 1000 ? p->nasa_lo[n] : p->nasa_hi[n];
}

/* gibbs, Source/CHEM/LiDryer.H:70-154: g/(RT) */
static void gibbs(const ocfdo_parm* p, double* g, const double* tc) {
    double T = tc[1];
    double invT = 1 / T;
    for (int n = 0; n < NS; ++n) {
        const double* a;
        nasa_coef(p, T, n, &a);
        g[n] = a[0] * (1.0 - tc[0]) - a[1] / 2.0 * tc[1] - a[2] / 6.0 * tc[2] - a[3] / 12.0 * tc[3] -
               a[4] / 20.0 * tc[4] + a[5] * invT - a[6];
    }
}

/* speciesInternalEnergy, LiDryer.H:531-614: e/(RT) */
static void species_internal_energy(const ocfdo_parm* p, double* e, const double* tc) {
    double T = tc[1];
    double invT = 1.0 / T;
    for (int n = 0; n < NS; ++n) {
        if (T < 1000) {
            const double* a = p->nasa_lo[n];
            e[n] = a[0] - 1.0 + a[1] / 2.0 * tc[1] + a[2] / 3.0 * tc[2] + a[3] / 4.0 * tc[3] + a[4] / 5.0 * tc[4];
        } else {
            const double* a = p->nasa_hi[n];
            e[n] = a[0] - 1.0 + a[1] / 2.0 * tc[1] + a[2] / 3.0 * tc[2] + a[3] / 4.0 * tc[3] + a[4] / 5.0 * tc[4] +
                   (a[5] - p->nasa_lo[n][5]) * invT;
        }
    }
}

/* speciesEnthalpy, LiDryer.H:616-695: h/R in K */
void ocfdo_species_enthalpy(const ocfdo_parm* p, double T, double* h) {
    double tc[5] = {T, T * T, T * T * T, T * T * T * T, T * T * T * T * T};
    for (int n = 0; n < NS; ++n) {
        if (T < 1000) {
            const double* a = p->nasa_lo[n];
            h[n] = a[0] * tc[0] + a[1] / 2.0 * tc[1] + a[2] / 3.0 * tc[2] + a[3] / 4.0 * tc[3] + a[4] / 5.0 * tc[4];
        } else {
            const double* a = p->nasa_hi[n];
            h[n] = a[0] * tc[0] + a[1] / 2.0 * tc[1] + a[2] / 3.0 * tc[2] + a[3] / 4.0 * tc[3] + a[4] / 5.0 * tc[4] +
                   (a[5] - p->nasa_lo[n][5]);
        }
    }
}

/* cp_R, LiDryer.H:716-783 */
static void cp_R(const ocfdo_parm* p, double* cp, const double* tc) {
    double T = tc[1];
    for (int n = 0; n < NS; ++n) {
        const double* a;
        nasa_coef(p, T, n, &a);
        cp[n] = a[0] + a[1] * tc[1] + a[2] * tc[2] + a[3] * tc[3] + a[4] * tc[4];
    }
}

double ocfdo_ckubms(const ocfdo_parm* p, double T, const double* rhoi) {
    /* CKUBMS, LiDryer.H:697-714 */
    double result = 0;
    double tc[5] = {0, T, T * T, T * T * T, T * T * T * T};
    double ums[NS];
    double RT = p->Ru * T;
    species_internal_energy(p, ums, tc);
    for (int n = 0; n < NS; ++n) result += rhoi[n] * ums[n] / p->mw[n];
    return result * RT;
}

double ocfdo_ckcvbs(const ocfdo_parm* p, double T, const double* rhoi) {
    /* CKCVBS, LiDryer.H:801-815 */
    double result = 0;
    double tc[5] = {0, T, T * T, T * T * T, T * T * T * T};
    double cpor[NS];
    cp_R(p, cpor, tc);
    for (int n = 0; n < NS; ++n) result += (cpor[n] - 1.0) * rhoi[n] / p->mw[n];
    return result * p->Ru;
}

double ocfdo_ckpy(const ocfdo_parm* p, const double* rhoi, double T) {
    /* CKPY, LiDryer.H:10-18 */
    double YOW = 0;
    for (int i = 0; i < NS; ++i) YOW += rhoi[i] / p->mw[i];
    return p->Ru * T * YOW;
}

double ocfdo_ckrhoy(const ocfdo_parm* p, double P, double T, const double* y) {
    /* CKRHOY, LiDryer.H:20-34 */
    double YOW = 0, tmp[NS];
    for (int i = 0; i < NS; ++i) tmp[i] = y[i] / p->mw[i];
    for (int i = 0; i < NS; ++i) YOW += tmp[i];
    return P / (p->Ru * T * YOW);
}

void ocfdo_ckytx(const ocfdo_parm* p, const double* y, double* x) {
    /* CKYTX, LiDryer.H:36-54 */
    double YOW = 0, tmp[NS];
    for (int i = 0; i < NS; i++) tmp[i] = y[i] / p->mw[i];
    for (int i = 0; i < NS; ++i) YOW += tmp[i];
    double YOWINV = 1.0 / YOW;
    for (int i = 0; i < NS; i++) x[i] = y[i] / p->mw[i] * YOWINV;
}

void ocfdo_ckxty(const ocfdo_parm* p, const double* x, double* y) {
    /* CKXTY, LiDryer.H:56-68 */
    double XW = 0.0;
    for (int i = 0; i < NS; ++i) XW += x[i] * p->mw[i];
    for (int i = 0; i < NS; ++i) y[i] = x[i] * p->mw[i] / XW;
}

double ocfdo_get_t_given_ey(const ocfdo_parm* p, double e, const double* rhoi) {
    /* GET_T_GIVEN_EY, LiDryer.H:833-888: bounded Newton on e(T) */
    const int maxiter = 200;
    const double tol = 1e-7;
    double ein = e, tmin = 250, tmax = 3500;
    double emin = ocfdo_ckubms(p, tmin, rhoi), emax = ocfdo_ckubms(p, tmax, rhoi);
    if (ein < emin) return tmin - (emin - ein) / ocfdo_ckcvbs(p, tmin, rhoi);
    if (ein > emax) return tmax - (emax - ein) / ocfdo_ckcvbs(p, tmax, rhoi);
    double As = 0;
    for (int n = 0; n < NS; ++n) As += p->A0[n] * p->Ru / p->mw[n] * rhoi[n];
    double t1 = e / As;
    if (t1 < tmin || t1 > tmax) t1 = tmin + (tmax - tmin) / (emax - emin) * (ein - emin);
    for (int i = 0; i < maxiter; ++i) {
        double e1 = ocfdo_ckubms(p, t1, rhoi);
        double cv = ocfdo_ckcvbs(p, t1, rhoi);
        double dt = (ein - e1) / cv;
        if (dt > 100.0) dt = 100.0;
        else if (dt < -100.0) dt = -100.0;
        else if (fabs(dt) < tol) break;
        else if (t1 + dt == t1) break;
        t1 += dt;
    }
    return t1;
}

/* Li-Dryer 9-species / 19-reaction mechanism as data for vproductionRate
 * (Source/CHEM/LiDryer.H:156-529): forward rates k = A exp(b lnT - Ta/T)
 * (LiDryer.H:171-191), reaction stoichiometry, third-body kind and Troe data. */
typedef struct { double A, b, Ta; } arrh_t;
static const arrh_t KF[21] = {
    {3.55e+15, -0.41, 8353.444256079512}, {50800.0, 2.67, 3165.2508657072367},
    {2.16e+08, 1.51, 1726.0429999007667}, {2.97e+06, 2.02, 6743.141748883461},
    {4.58e+19, -1.4, 52526.05490660117},  {6.16e+15, -0.5, 0.0},
    {4.71e+18, -1, 0.0},                  {3.8e+22, -2, 0.0},
    {1.48e+12, 0.6, 0.0},                 {1.66e+13, 0.0, 412.64001746898793},
    {7.08e+13, 0.0, 150.96586004962973},  {3.25e+13, 0.0, 0.0},
    {2.89e+13, 0.0, -251.60976674938289}, {4.2e+14, 0.0, 6028.570011315214},
    {1.3e+11, 0.0, -820.2478396029883},   {2.95e+14, 0.0, 24355.825421340265},
    {2.41e+13, 0.0, 1997.7815479901},     {4.82e+13, 0.0, 4000.595291315188},
    {9.55e+06, 2, 1997.7815479901},       {1.0e+12, 0.0, 0.0},
    {5.8e+14, 0.0, 4810.778740248201}};
/* reaction r: up to two reactant / product species (-1 = none); kf[2] indexes
 * into KF (second entry for the duplicate reactions 13 and 18); tb 0 none,
 * 1 M = mixture+1.5 H2+11 H2O, 2 Troe with M = mixture+H2+10 H2O-0.22 O2,
 * 3 Troe with kind-1 efficiencies; kc_pre: 0 none, +1 RsT, -1 1/RsT. */
typedef struct {
    int re[2], pr[2];
    int kf[2];
    int tb;
    int kc_pre;
    double troe_A, troe_b, troe_Ta, fcent;
} rxn_t;
static const rxn_t RX[19] = {
    {{3, 1}, {4, 5}, {0, -1}, 0, 0, 0, 0, 0, 0},
    {{4, 0}, {3, 5}, {1, -1}, 0, 0, 0, 0, 0, 0},
    {{0, 5}, {2, 3}, {2, -1}, 0, 0, 0, 0, 0, 0},
    {{4, 2}, {5, 5}, {3, -1}, 0, 0, 0, 0, 0, 0},
    {{0, -1}, {3, 3}, {4, -1}, 1, -1, 0, 0, 0, 0},
    {{4, 4}, {1, -1}, {5, -1}, 1, 1, 0, 0, 0, 0},
    {{4, 3}, {5, -1}, {6, -1}, 1, 1, 0, 0, 0, 0},
    {{3, 5}, {2, -1}, {7, -1}, 1, 1, 0, 0, 0, 0},
    {{3, 1}, {6, -1}, {8, -1}, 2, 1, 6.37e+20, -1.72, 261.6741574193582, 0.8},
    {{6, 3}, {0, 1}, {9, -1}, 0, 0, 0, 0, 0, 0},
    {{6, 3}, {5, 5}, {10, -1}, 0, 0, 0, 0, 0, 0},
    {{6, 4}, {1, 5}, {11, -1}, 0, 0, 0, 0, 0, 0},
    {{6, 5}, {2, 1}, {12, -1}, 0, 0, 0, 0, 0, 0},
    {{6, 6}, {7, 1}, {13, 14}, 0, 0, 0, 0, 0, 0},
    {{7, -1}, {5, 5}, {15, -1}, 3, -1, 1.20e+17, 0.0, 22846.166820843966, 0.5},
    {{7, 3}, {2, 5}, {16, -1}, 0, 0, 0, 0, 0, 0},
    {{7, 3}, {6, 0}, {17, -1}, 0, 0, 0, 0, 0, 0},
    {{7, 4}, {5, 6}, {18, -1}, 0, 0, 0, 0, 0, 0},
    {{7, 5}, {6, 2}, {19, 20}, 0, 0, 0, 0, 0, 0}};

static double sum2g(const double* g, const int* sp) {
    return sp[1] < 0 ? g[sp[0]] : g[sp[0]] + g[sp[1]];
}
static double prod2c(const double* c, const int* sp) {
    return sp[1] < 0 ? c[sp[0]] : c[sp[0]] * c[sp[1]];
}

void ocfdo_production_rate(const ocfdo_parm* p, const double* sc, double T, double* wdot,
                           double* arate) {
    double tc[5], invT, k_f_s[21], gi_T[NS], mixture;
    const double eps = 1e-20;
    tc[0] = log(T);
    tc[1] = T;
    tc[2] = T * (T);
    tc[3] = tc[2] * tc[1];
    tc[4] = tc[2] * tc[2];
    invT = 1.0 / T;
    for (int r = 0; r < 21; ++r) k_f_s[r] = KF[r].A * exp(KF[r].b * tc[0] - KF[r].Ta * invT);
    gibbs(p, gi_T, tc);
    double RsT = p->Ru / p->Patm * 1e6 * T;
    mixture = 0.0;
    for (int n = 0; n < NS; n++) {
        mixture += sc[n];
        wdot[n] = 0.0;
        for (int l = 0; l < NS; l++) arate[n * NS + l] = 0.0;
    }
    double q_f[19], q_r[19];
    int vf[19][NS], vr[19][NS];
    memset(vf, 0, sizeof vf);
    memset(vr, 0, sizeof vr);
    for (int r = 0; r < 19; ++r) {
        const rxn_t* x = &RX[r];
        for (int s = 0; s < 2; ++s) {
            if (x->re[s] >= 0) vf[r][x->re[s]] += 1;
            if (x->pr[s] >= 0) vr[r][x->pr[s]] += 1;
        }
        double dG = sum2g(gi_T, x->re) - sum2g(gi_T, x->pr);
        double phi_f = prod2c(sc, x->re), phi_r = prod2c(sc, x->pr);
        double k_f = k_f_s[x->kf[0]];
        if (x->tb == 1) {
            double alpha = mixture + 1.5 * sc[0] + 11 * sc[2];
            k_f = alpha * k_f;
        } else if (x->tb == 2 || x->tb == 3) {
            double alpha = x->tb == 2 ? mixture + sc[0] + 10 * sc[2] + -0.22 * sc[1]
                                      : mixture + 1.5 * sc[0] + 11 * sc[2];
            double redP = alpha / k_f * x->troe_A * exp(x->troe_b * tc[0] - x->troe_Ta * invT);
            double logPred = log10(redP);
            double logFcent = log10(x->fcent);
            double troe_c = -0.4 - 0.67 * logFcent;
            double troe_n = 0.75 - 1.27 * logFcent;
            double troe = (troe_c + logPred) / (troe_n - 0.14 * (troe_c + logPred));
            double F_troe = pow(10.0, logFcent / (1.0 + troe * troe));
            k_f *= (redP / (1.0 + redP)) * F_troe;
        }
        double Kc = exp(dG);
        if (x->kc_pre > 0) Kc = RsT * exp(dG);
        if (x->kc_pre < 0) Kc = 1.0 / RsT * exp(dG);
        q_f[r] = phi_f * k_f;
        q_r[r] = phi_r * (k_f / Kc);
        if (x->kf[1] >= 0) {
            /* duplicate reaction: second rate expression added */
            double k2 = k_f_s[x->kf[1]];
            double Kc2 = exp(dG);
            q_f[r] += phi_f * k2;
            q_r[r] += phi_r * (k2 / Kc2);
        }
    }
    for (int m = 0; m < 19; ++m) {
        double wf1 = q_f[m], wr1 = q_r[m];
        for (int n = 0; n < NS; ++n) wdot[n] += (wf1 - wr1) * (vr[m][n] - vf[m][n]);
        for (int n = 0; n < NS; ++n) {
            double Awf = vf[m][n] * wf1 / (sc[n] + eps);
            double Awr = vr[m][n] * wr1 / (sc[n] + eps);
            for (int l = 0; l < NS; ++l) arate[l * NS + n] += (Awf - Awr) * (vr[m][l] - vf[m][l]);
        }
    }
}

void ocfdo_gauss(const double* A, const double* b, double* x) {
    /* gauss, LiDryer.H:890-942: partial-pivot elimination on the augmented matrix */
    double U[NS][NS + 1];
    for (int i = 0; i < NS; i++) {
        U[i][NS] = b[i];
        for (int j = 0; j < NS; j++) U[i][j] = A[i * NS + j];
    }
    for (int k = 0; k < NS; k++) {
        int pv = k;
        double maxPivot = 0.0;
        for (int i = k; i < NS; i++)
            if (fabs(U[i][k]) > maxPivot) { maxPivot = fabs(U[i][k]); pv = i; }
        if (pv != k)
            for (int i = k; i < NS + 1; i++) { double t = U[pv][i]; U[pv][i] = U[k][i]; U[k][i] = t; }
        for (int i = k + 1; i < NS; i++) {
            double m = U[i][k] / U[k][k];
            for (int j = k; j < NS + 1; j++) U[i][j] -= m * U[k][j];
        }
    }
    for (int k = NS - 1; k >= 0; k--) {
        double sum = U[k][NS];
        for (int j = k + 1; j < NS; j++) sum -= U[k][j] * x[j];
        x[k] = sum / U[k][k];
    }
}

static double dot5(const double* x, const double* y) {
    return x[0] * y[0] + x[1] * y[1] + x[2] * y[2] + x[3] * y[3] + x[4] * y[4];
}

void ocfdo_mixture_properties(const ocfdo_parm* p, double T, const double* X, double* mu,
                              double* lambda) {
    /* mixtureProperties, Source/CHEM/ChemViscous.H:16-64 (Wilke mixing) */
    double mui[NS], sqmui[NS], lambdai[NS], phi[NS][NS];
    memset(phi, 0, sizeof phi);
    double sqT = sqrt(T), logT = log(T);
    double sqsqT = sqrt(sqT);
    double poly[5] = {1.0, logT, logT * logT, logT * logT * logT, logT * logT * logT * logT};
    for (int k = 0; k < NS; k++) {
        sqmui[k] = sqsqT * dot5(poly, &p->visccoeff[k * 5]);
        lambdai[k] = sqT * dot5(poly, &p->conductcoeff[k * 5]);
        mui[k] = (sqmui[k] * sqmui[k]);
    }
    double sum1 = 0.0, sum2 = 0.0;
    for (int k = 0; k < NS; k++) {
        sum1 += X[k] * lambdai[k];
        sum2 += X[k] / lambdai[k];
    }
    *lambda = 0.5 * (sum1 + 1.0 / sum2);
    for (int k = 0; k < NS; k++) {
        for (int j = 0; j < k; j++) {
            double wratiojk = p->mw[j] / p->mw[k];
            double vratiokj = mui[k] / mui[j];
            double factor1 = 1.0 + (sqmui[k] / sqmui[j]) * sqrt(sqrt(wratiojk));
            double tmp = factor1 * factor1 / sqrt(8.0 + 8.0 * p->mw[k] / p->mw[j]);
            phi[k][j] = tmp;
            phi[j][k] = tmp / (vratiokj * wratiojk);
        }
        phi[k][k] = 1.0;
    }
    double m = 0;
    for (int k = 0; k < NS; k++) {
        double tmp = 0;
        for (int j = 0; j < NS; j++) tmp += X[j] * phi[k][j];
        m += X[k] * mui[k] / tmp;
    }
    *mu = m;
}

void ocfdo_mix_diff_coeffs(const ocfdo_parm* p, double T, double P, const double* X, double* D) {
    /* getMixDiffCoeffsMass, Source/CHEM/ChemViscous.H:66-106 */
    double logT = log(T);
    double poly[5] = {1.0, logT, logT * logT, logT * logT * logT, logT * logT * logT * logT};
    double bdiff[NS][NS];
    int ic = 0;
    for (int n = 0; n < NS; n++)
        for (int nn = n; nn < NS; nn++) {
            bdiff[n][nn] = T * sqrt(T) * dot5(poly, &p->diffcoeff[ic * 5]);
            bdiff[nn][n] = bdiff[n][nn];
            ic++;
        }
    double mmw = 0;
    for (int n = 0; n < NS; ++n) mmw += X[n] * p->mw[n];
    for (int n = 0; n < NS; n++) {
        double sum1 = 0.0, sum2 = 0.0;
        for (int nn = 0; nn < NS; nn++) {
            if (nn == n) continue;
            sum1 += X[nn] / bdiff[n][nn];
            sum2 += X[nn] * p->mw[nn] / bdiff[n][nn];
        }
        sum1 *= P;
        sum2 *= P * X[n] / (mmw - p->mw[n] * X[n]);
        D[n] = 1.0 / (sum1 + sum2);
    }
}

/* c2prim_rgas, Source/kernel/Kernels.H:42-81 */
static void c2prim_real(const ocfdo_parm* p, const double* u, const double* rhoi_in, double* q) {
    double rho = dmax(u[URHO], p->smallr);
    double rhoinv = 1.0 / rho;
    double ux = u[UMX] * rhoinv, uy = u[UMY] * rhoinv, uz = u[UMZ] * rhoinv;
    double kineng = 0.5 * (ux * ux + uy * uy + uz * uz);
    double ei = u[UEDEN] - rho * kineng;
    double rhoi[NS];
    q[QRHO] = rho; q[QU] = ux; q[QV] = uy; q[QW] = uz;
    for (int n = 0; n < NS; ++n) rhoi[n] = rhoi_in[n];
    double T = ocfdo_get_t_given_ey(p, ei, rhoi);
    double pr = ocfdo_ckpy(p, rhoi, T);
    q[QT] = T;
    q[QPRES] = pr;
    double gama = pr / ei + 1.0;
    q[QGAMA] = gama;
    q[QC] = sqrt(gama * pr / rho);
}

void ocfdo_c2prim(const ocfdo_parm* p, int chem, const double* S, const double* spec, int nx,
                  int ny, int nz, double* q) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b);
    int nq = chem ? 8 : 7;
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long long c = 0; c < N; ++c) {
        double u[5], qc[8], r[NS];
        for (int n = 0; n < 5; ++n) u[n] = S[n * N + c];
        if (chem) {
            for (int n = 0; n < NS; ++n) r[n] = spec[n * N + c];
            c2prim_real(p, u, r, qc);
        } else {
            c2prim_ideal(p, u, qc);
        }
        for (int n = 0; n < nq; ++n) q[n * N + c] = qc[n];
    }
}

/* transport properties over the grown box, Source/CHEM/FlowAdvance.cpp:188-202 */
static void transport_q(const ocfdo_parm* p, const box_t* b, const double* q, const double* spec,
                        double* mu, double* lam, double* D) {
    long long N = gN(b);
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long long c = 0; c < N; ++c) {
        double Yt[NS], Xt[NS], Dc[NS];
        double T = q[QT * N + c], pr = q[QPRES * N + c];
        for (int n = 0; n < NS; ++n) Yt[n] = spec[n * N + c] / q[QRHO * N + c];
        ocfdo_ckytx(p, Yt, Xt);
        ocfdo_mixture_properties(p, T, Xt, &mu[c], &lam[c]);
        ocfdo_mix_diff_coeffs(p, T, pr, Xt, Dc);
        for (int n = 0; n < NS; ++n) D[n * N + c] = Dc[n];
    }
}

void ocfdo_transport(const ocfdo_parm* p, const double* S, const double* spec, int nx, int ny,
                     int nz, double* mu, double* lambda, double* D) {
    box_t b = mkbox(nx, ny, nz);
    double* q = (double*)xcalloc(gN(&b) * 8, sizeof(double));
    ocfdo_c2prim(p, 1, S, spec, nx, ny, nz, q);
    transport_q(p, &b, q, spec, mu, lambda, D);
    free(q);
}

/* Species split factor, Source/CHEM/FlowAdvance.cpp:214-242 */
static void spec_split_cell(const double* qc, int d, double* tp, double* tm, double* tmp1) {
    double un = qc[QU + d], c = qc[QC], gamma = qc[QGAMA];
    double E1 = un, E2 = un - c, E3 = un + c;
    double E1P = (E1 + fabs(E1)) * 0.5, E2P = (E2 + fabs(E2)) * 0.5, E3P = (E3 + fabs(E3)) * 0.5;
    double E1M = E1 - E1P, E2M = E2 - E2P, E3M = E3 - E3P;
    *tmp1 = 1.0 / (2.0 * gamma);
    double tmp2 = 2.0 * (gamma - 1.0);
    *tp = tmp2 * E1P + E2P + E3P;
    *tm = tmp2 * E1M + E2M + E3M;
}

/* species diffusion flux at the d-face, Source/CHEM/ChemViscous.H:108-199 */
static void diffusion_face(const box_t* b, const double* q, const double* spec, const double* D,
                           int d, int i, int j, int k, const double* dxinv, double* fs,
                           double* fd, long long FN) {
    long long N = gN(b);
    long long c = gI(b, i, j, k), l = gI(b, i - E[d][0], j - E[d][1], k - E[d][2]);
    double rhor = q[QRHO * N + c], rhol = q[QRHO * N + l];
    double rho = 0.5 * (rhol + rhor);
    double di[NS], Ytr[NS], Ytl[NS];
    for (int n = 0; n < NS; ++n) {
        Ytr[n] = spec[n * N + c] / rhor;
        Ytl[n] = spec[n * N + l] / rhol;
        di[n] = 0.5 * (D[n * N + c] + D[n * N + l]);
    }
    for (int n = 0; n < NS; ++n) {
        double tmp = rho * di[n] * (Ytl[n] - Ytr[n]) * dxinv[d];
        fd[n * FN] = tmp;
        fs[n * FN] += tmp;
    }
}

/* face-averaged mu, lambda and species-enthalpy flux for the multispecies viscous term */
static void multi_face_props(const ocfdo_parm* p, const box_t* b, const double* q,
                             const double* mu, const double* lam, const double* fd, long long FN,
                             int d, int i, int j, int k, double* muf, double* lamf,
                             double* hflux) {
    long long N = gN(b);
    long long c = gI(b, i, j, k), l = gI(b, i - E[d][0], j - E[d][1], k - E[d][2]);
    double Tr = q[QT * N + c], Tl = q[QT * N + l];
    double T = 0.5 * (Tl + Tr);
    *muf = 0.5 * (mu[c] + mu[l]);
    *lamf = 0.5 * (lam[c] + lam[l]);
    double hi[NS];
    ocfdo_species_enthalpy(p, T, hi);
    double tmp = 0;
    for (int n = 0; n < NS; ++n) tmp += fd[n * FN] * hi[n];
    *hflux = tmp;
}

void ocfdo_rhs_chem(const ocfdo_parm* p, const double* S, const double* spec, int nx, int ny,
                    int nz, const double* dxinv, int do_visc, double* dSdt, double* dSdt_spec,
                    double* fx, double* fy, double* fz, double* fxs, double* fys, double* fzs,
                    double* fxd, double* fyd, double* fzd) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b), BN = bN(&b);
    double* q = (double*)xcalloc(N * 8, sizeof(double));
    double* fp = (double*)xcalloc(N * NCONS, sizeof(double));
    double* fm = (double*)xcalloc(N * NCONS, sizeof(double));
    double* fps = (double*)xcalloc(N * NS, sizeof(double));
    double* fms = (double*)xcalloc(N * NS, sizeof(double));
    double* mu = (double*)xcalloc(N, sizeof(double));
    double* lam = (double*)xcalloc(N, sizeof(double));
    double* D = (double*)xcalloc(N * NS, sizeof(double));
    double* fl[3] = {fx, fy, fz};
    double* fls[3] = {fxs, fys, fzs};
    double* fld[3] = {fxd, fyd, fzd};
    zero_faces(&b, fl, NCONS);
    zero_faces(&b, fls, NS);
    if (do_visc) zero_faces(&b, fld, NS);
    ocfdo_c2prim(p, 1, S, spec, nx, ny, nz, q);
    if (do_visc) transport_q(p, &b, q, spec, mu, lam, D);
    for (int d = 0; d < 3; ++d) {
        long long FN = fN(&b, d);
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (long long c = 0; c < N; ++c) {
            double qc[8], a[5], m[5], tp, tm, tmp1;
            for (int n = 0; n < 8; ++n) qc[n] = q[n * N + c];
            sw_split(qc[QGAMA], qc, d, a, m);
            for (int n = 0; n < 5; ++n) { fp[n * N + c] = a[n]; fm[n * N + c] = m[n]; }
            spec_split_cell(qc, d, &tp, &tm, &tmp1);
            for (int n = 0; n < NS; ++n) {
                double tmp0 = spec[n * N + c] * tmp1;
                fps[n * N + c] = tmp0 * tp;
                fms[n * N + c] = tmp0 * tm;
            }
        }
#ifdef OCFDO_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
        for (int k = 0; k < nz + (d == 2); ++k)
            for (int j = 0; j < ny + (d == 1); ++j)
                for (int i = 0; i < nx + (d == 0); ++i) {
                    long long fi = fI(&b, d, i, j, k);
                    for (int n = 0; n < NCONS; ++n)
                        fl[d][n * FN + fi] = weno_face(&b, fp + n * N, fm + n * N, d, i, j, k);
                    for (int n = 0; n < NS; ++n)
                        fls[d][n * FN + fi] = weno_face(&b, fps + n * N, fms + n * N, d, i, j, k);
                }
        if (do_visc) {
#ifdef OCFDO_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
            for (int k = 0; k < nz + (d == 2); ++k)
                for (int j = 0; j < ny + (d == 1); ++j)
                    for (int i = 0; i < nx + (d == 0); ++i) {
                        long long fi = fI(&b, d, i, j, k);
                        diffusion_face(&b, q, spec, D, d, i, j, k, dxinv, fls[d] + fi, fld[d] + fi, FN);
                    }
#ifdef OCFDO_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
            for (int k = 0; k < nz + (d == 2); ++k)
                for (int j = 0; j < ny + (d == 1); ++j)
                    for (int i = 0; i < nx + (d == 0); ++i) {
                        long long fi = fI(&b, d, i, j, k);
                        double muf, lamf, hflux;
                        multi_face_props(p, &b, q, mu, lam, fld[d] + fi, FN, d, i, j, k, &muf, &lamf, &hflux);
                        visc_face(p, &b, q, d, i, j, k, dxinv, fl[d] + fi, FN, 1, muf, lamf, hflux);
                    }
        }
    }
    long long F0 = fN(&b, 0), F1 = fN(&b, 1), F2 = fN(&b, 2);
#ifdef OCFDO_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = bI(&b, i, j, k);
                long long x0 = fI(&b, 0, i, j, k), x1 = fI(&b, 0, i + 1, j, k);
                long long y0 = fI(&b, 1, i, j, k), y1 = fI(&b, 1, i, j + 1, k);
                long long z0 = fI(&b, 2, i, j, k), z1 = fI(&b, 2, i, j, k + 1);
                for (int n = 0; n < NCONS; ++n)
                    dSdt[n * BN + c] = dxinv[0] * (fx[n * F0 + x0] - fx[n * F0 + x1]) +
                                       dxinv[1] * (fy[n * F1 + y0] - fy[n * F1 + y1]) +
                                       dxinv[2] * (fz[n * F2 + z0] - fz[n * F2 + z1]);
                for (int n = 0; n < NS; ++n)
                    dSdt_spec[n * BN + c] = dxinv[0] * (fxs[n * F0 + x0] - fxs[n * F0 + x1]) +
                                            dxinv[1] * (fys[n * F1 + y0] - fys[n * F1 + y1]) +
                                            dxinv[2] * (fzs[n * F2 + z0] - fzs[n * F2 + z1]);
            }
    free(q); free(fp); free(fm); free(fps); free(fms); free(mu); free(lam); free(D);
}

/* Van Leer species flux, Source/CHEM/FlowAdvanceBox.cpp:166-223 */
static void vanleer_spec(const double* ql, const double* qr, const double* rl, const double* rr,
                         int d, double* fs) {
    double fp[NS], fm[NS];
    for (int n = 0; n < NS; ++n) { fp[n] = 0; fm[n] = 0; }
    double ul = ql[QU + d], ur = qr[QU + d];
    double cL = ql[QC], cR = qr[QC];
    double ML = ul / cL, MR = ur / cR, UL = ul, UR = ur;
    if (ML >= 1.0) {
        for (int n = 0; n < NS; ++n) fp[n] = rl[n] * UL;
    } else if (fabs(ML) < 1.0) {
        double Mp = 0.250 * (1.0 + ML) * (1.0 + ML);
        for (int n = 0; n < NS; ++n) fp[n] = rl[n] * cL * Mp;
    }
    if (fabs(MR) < 1.0) {
        double Mm = -0.250 * (MR - 1.0) * (MR - 1.0);
        for (int n = 0; n < NS; ++n) fm[n] = rr[n] * cR * Mm;
    } else if (MR <= -1.0) {
        for (int n = 0; n < NS; ++n) fm[n] = rr[n] * UR;
    }
    for (int n = 0; n < NS; ++n) fs[n] = fp[n] + fm[n];
}

void ocfdo_rhs_chem_eb(const ocfdo_parm* p, const double* S, const double* spec,
                       const uint32_t* flag, const double* vfrac, const double* apx,
                       const double* apy, const double* apz, int nx, int ny, int nz,
                       const double* dxinv, int do_visc, double* dSdt, double* dSdt_spec,
                       double* fx, double* fy, double* fz, double* fxs, double* fys,
                       double* fzs, double* fxd, double* fyd, double* fzd) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b), BN = bN(&b);
    double* q = (double*)xcalloc(N * 8, sizeof(double));
    double* mu = (double*)xcalloc(N, sizeof(double));
    double* lam = (double*)xcalloc(N, sizeof(double));
    double* D = (double*)xcalloc(N * NS, sizeof(double));
    double* divc = (double*)xcalloc(BN * NCONS, sizeof(double));
    double* fl[3] = {fx, fy, fz};
    double* fls[3] = {fxs, fys, fzs};
    double* fld[3] = {fxd, fyd, fzd};
    const double* cfl[3] = {fx, fy, fz};
    const double* cfls[3] = {fxs, fys, fzs};
    const double* ap[3] = {apx, apy, apz};
    zero_faces(&b, fl, NCONS);
    zero_faces(&b, fls, NS);
    if (do_visc) zero_faces(&b, fld, NS);
    ocfdo_c2prim(p, 1, S, spec, nx, ny, nz, q);
    if (do_visc) transport_q(p, &b, q, spec, mu, lam, D);
    for (int d = 0; d < 3; ++d) {
        long long FN = fN(&b, d);
        for (int k = 0; k < nz + (d == 2); ++k)
            for (int j = 0; j < ny + (d == 1); ++j)
                for (int i = 0; i < nx + (d == 0); ++i) {
                    double ql[8], qr[8], rl[NS], rr[NS], flx[5], fs[NS];
                    for (int n = 0; n < 8; ++n) eb_recon(&b, flag, q + n * N, d, i, j, k, &ql[n], &qr[n]);
                    for (int n = 0; n < NS; ++n) eb_recon(&b, flag, spec + n * N, d, i, j, k, &rl[n], &rr[n]);
                    vanleer(p, 1, ql, qr, d, flx);
                    vanleer_spec(ql, qr, rl, rr, d, fs);
                    long long fi = fI(&b, d, i, j, k);
                    for (int n = 0; n < NCONS; ++n) fl[d][n * FN + fi] = flx[n];
                    for (int n = 0; n < NS; ++n) fls[d][n * FN + fi] = fs[n];
                }
        if (do_visc) {
            for (int k = 0; k < nz + (d == 2); ++k)
                for (int j = 0; j < ny + (d == 1); ++j)
                    for (int i = 0; i < nx + (d == 0); ++i) {
                        long long fi = fI(&b, d, i, j, k);
                        diffusion_face(&b, q, spec, D, d, i, j, k, dxinv, fls[d] + fi, fld[d] + fi, FN);
                    }
            for (int k = 0; k < nz + (d == 2); ++k)
                for (int j = 0; j < ny + (d == 1); ++j)
                    for (int i = 0; i < nx + (d == 0); ++i) {
                        long long fi = fI(&b, d, i, j, k);
                        double muf, lamf, hflux;
                        multi_face_props(p, &b, q, mu, lam, fld[d] + fi, FN, d, i, j, k, &muf, &lamf, &hflux);
                        eb_visc_face(p, &b, flag, q, d, i, j, k, dxinv, fl[d] + fi, FN, 1, muf, lamf, hflux);
                    }
        }
    }
    /* flow divergence goes to a scratch array that is never copied back: the
     * reference leaves the divc -> dSdt copy commented out
     * (Source/CHEM/FlowAdvanceBox.cpp:500-523), so dSdt stays zero here */
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = bI(&b, i, j, k);
                eb_div_cell(p, 1, &b, flag, vfrac, ap, q, cfl, NCONS, i, j, k, dxinv, do_visc, divc + c, BN);
                for (int n = 0; n < NCONS; ++n) dSdt[n * BN + c] = 0.0;
            }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = bI(&b, i, j, k), g = gI(&b, i, j, k);
                eb_div_cell(p, 1, &b, flag, vfrac, ap, q, cfls, NS, i, j, k, dxinv, 0, dSdt_spec + c, BN);
                uint32_t f = flag[g];
                if (!is_covered(f) && !is_regular(f) && do_visc) {
                    double tmp = dxinv[0] / vfrac[g];
                    long long x0 = fI(&b, 0, i, j, k), x1 = fI(&b, 0, i + 1, j, k);
                    long long y0 = fI(&b, 1, i, j, k), y1 = fI(&b, 1, i, j + 1, k);
                    long long z0 = fI(&b, 2, i, j, k), z1 = fI(&b, 2, i, j, k + 1);
                    double axm = apx[x0], axp = apx[x1], aym = apy[y0], ayp = apy[y1], azm = apz[z0], azp = apz[z1];
                    double apnorm = sqrt((axm - axp) * (axm - axp) + (aym - ayp) * (aym - ayp) + (azm - azp) * (azm - azp));
                    double un = q[QU * N + g] * (axm - axp) + q[QV * N + g] * (aym - ayp) + q[QW * N + g] * (azm - azp);
                    double lambda0 = fabs(un) + q[QC * N + g] * apnorm;
                    double fw[NS];
                    for (int n = 0; n < NS; ++n) {
                        double sn = spec[n * N + g];
                        double fpw = 0.5 * (sn * un + lambda0 * sn);
                        double fmw = -0.5 * (sn * un + lambda0 * sn);
                        fw[n] = fpw + fmw;
                    }
                    for (int n = 0; n < NS; ++n) dSdt_spec[n * BN + c] += fw[n] * tmp;
                }
                for (int n = 0; n < NS; ++n) dSdt_spec[n * BN + c] *= -1.0;
            }
    free(q); free(mu); free(lam); free(D); free(divc);
}

void ocfdo_chem_advance(const ocfdo_parm* p, double* S, double* spec, long long ncell,
                        long long cstride, double dt) {
    /* Source/CHEM/ChemAdvance.cpp:27-82 */
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(dynamic, 256)
#endif
    for (long long c = 0; c < ncell; ++c) {
        double* sf = S + c;
        double* rh = spec + c;
        double rho = dmax(sf[URHO * cstride], p->smallr);
        double rhoinv = 1.0 / rho;
        double ux = sf[UMX * cstride] * rhoinv, uy = sf[UMY * cstride] * rhoinv, uz = sf[UMZ * cstride] * rhoinv;
        double kineng = 0.5 * (ux * ux + uy * uy + uz * uz);
        double ei = sf[UEDEN * cstride] - rho * kineng;
        double r0[NS], cc[NS], wdot[NS], Ar[NS * NS], A1[NS * NS], b1[NS], drho[NS];
        for (int n = 0; n < NS; ++n) r0[n] = rh[n * cstride];
        double T = ocfdo_get_t_given_ey(p, ei, r0);
        for (int n = 0; n < NS; n++) cc[n] = r0[n] / p->mw[n] * 1e-6;
        ocfdo_production_rate(p, cc, T, wdot, Ar);
        for (int i = 0; i < NS; ++i)
            for (int j = 0; j < NS; ++j) {
                A1[i * NS + j] = (i == j ? 1.0 : 0.0);
                A1[i * NS + j] -= Ar[i * NS + j] * p->mw[i] / p->mw[j] * dt;
            }
        for (int n = 0; n < NS; ++n) b1[n] = wdot[n] * p->mw[n] * 1e6 * dt;
        ocfdo_gauss(A1, b1, drho);
        for (int n = 0; n < NS; ++n) {
            rh[n * cstride] += drho[n];
            if (rh[n * cstride] < 0) rh[n * cstride] = 0.0;
        }
        double dei = 0;
        for (int n = 0; n < NS; ++n) dei += -p->HP[n] * p->Ru / p->mw[n] * drho[n];
        sf[UEDEN * cstride] += dei;
    }
}

void ocfdo_spec_renorm(double* S, double* spec, long long ncell, long long cstride) {
    /* Source/EBR.cpp:341-355 */
    for (long long c = 0; c < ncell; ++c) {
        double rho0 = 0;
        for (int n = 0; n < NS; ++n) {
            if (spec[c + n * cstride] < 0) spec[c + n * cstride] = 0.0;
            rho0 += spec[c + n * cstride];
        }
        double tmp = S[c + URHO * cstride] / rho0;
        for (int n = 0; n < NS; ++n) spec[c + n * cstride] *= tmp;
    }
}

/* ============================================================ ghost fill */
/* AMReX BCType codes used by Source/Setup.cpp:22-35 */
enum { BC_INT_DIR = 0, BC_EXT_DIR = 1, BC_FOEXTRAP = 2, BC_REFLECT_EVEN = 3, BC_REFLECT_ODD = 4 };
static const int SCALAR_BC[6] = {BC_INT_DIR, BC_EXT_DIR, BC_FOEXTRAP, BC_REFLECT_EVEN, BC_REFLECT_EVEN, BC_REFLECT_EVEN};
static const int NORM_VEL_BC[6] = {BC_INT_DIR, BC_EXT_DIR, BC_FOEXTRAP, BC_REFLECT_ODD, BC_REFLECT_ODD, BC_REFLECT_ODD};
static const int TANG_VEL_BC[6] = {BC_INT_DIR, BC_EXT_DIR, BC_FOEXTRAP, BC_REFLECT_EVEN, BC_REFLECT_EVEN, BC_REFLECT_ODD};

static int comp_bc(int phys, int comp, int d) {
    /* component n of the conserved state: 0 rho, 1-3 momentum, 4 energy;
     * comp >= 5 are species (scalar) */
    if (comp >= 1 && comp <= 3) return (comp - 1 == d) ? NORM_VEL_BC[phys] : TANG_VEL_BC[phys];
    return SCALAR_BC[phys];
}

/* Double Mach reflection boundary functor, Exec/1_DMR/prob_bcfill.cpp:9-59 */
static void dmr_fill(const ocfdo_bc* bc, double* S, long long N, const box_t* b, int i, int j,
                     int k, int ncomp, double time) {
    int ai = i + bc->dom_lo[0], aj = j + bc->dom_lo[1];
    double x = bc->prob_lo[0] + (ai + 0.5) * bc->dx[0];
    long long c = gI(b, i, j, k);
    double x0 = 1.0 / 6.0 + sqrt(1 / 3.0) + time * 10.0 / sin(OCFDO_PI * (1.0 / 3.0));
    if (bc->hi_bc[1] == 1 && aj > bc->dom_hi[1]) {
        const double* st = x < x0 ? bc->dmr_left : bc->dmr_right;
        for (int n = 0; n < ncomp; ++n) S[n * N + c] = st[n];
    }
    /* scalar BC of the y-lo face is reflect_even for phys codes 3, 4, 5 (Source/Setup.cpp:22-25) */
    if ((bc->lo_bc[1] == 3 || bc->lo_bc[1] == 4 || bc->lo_bc[1] == 5) && aj < 0) {
        if (x < 1.0 / 6.0)
            for (int n = 0; n < ncomp; ++n) S[n * N + c] = bc->dmr_left[n];
    }
    if (bc->lo_bc[0] == 1 && ai < 0)
        for (int n = 0; n < ncomp; ++n) S[n * N + c] = bc->dmr_left[n];
}

/* Planar jet inflow on the x-lo face (the multi-level EB workload): with s(y) =
 * (1 + tanh((w - |y - yc|) / delta)) / 2, u = u_co + (u_jet - u_co) s, rho =
 * rho_co + (rho_jet - rho_co) s, v = w = 0, uniform pressure */
static void jet_fill(const ocfdo_bc* bc, double* S, long long N, const box_t* b, int i, int j, int k,
                     int ncomp) {
    const double* pr = bc->jet;
    int aj = j + bc->dom_lo[1];
    double y = bc->prob_lo[1] + (aj + 0.5) * bc->dx[1];
    double s = 0.5 * (1.0 + tanh((pr[4] - fabs(y - pr[3])) / pr[5]));
    double u = pr[2] + (pr[1] - pr[2]) * s;
    double r = pr[7] + (pr[0] - pr[7]) * s;
    double st[5] = {r, r * u, 0.0, 0.0, pr[6] + 0.5 * r * u * u};
    long long c = gI(b, i, j, k);
    for (int n = 0; n < ncomp && n < 5; ++n) S[n * N + c] = st[n];
}

void ocfdo_fill_ghosts(const ocfdo_bc* bc, double* S, int ncomp, int nx, int ny, int nz,
                       double time) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b);
    int n3[3] = {nx, ny, nz};
    /* directions in order x, y, z; direction d covers the already-grown range of
     * the directions before it so that edges and corners end up filled */
    for (int d = 0; d < 3; ++d) {
        int lo[3], hi[3];
        for (int t = 0; t < 3; ++t) {
            lo[t] = t < d ? -NG : 0;
            hi[t] = t < d ? n3[t] + NG : n3[t];
        }
        /* transverse directions, the slower one outermost (the inner loop walks
         * the faster index; every write is a distinct ghost cell and every read
         * a cell that is not a ghost in direction d, so the order is free) */
        const int ta = (d + 1) % 3 > (d + 2) % 3 ? (d + 1) % 3 : (d + 2) % 3;
        const int tb = 3 - d - ta;
        for (int side = 0; side < 2; ++side) {
            int phys = side == 0 ? bc->lo_bc[d] : bc->hi_bc[d];
            for (int gcell = 0; gcell < NG; ++gcell) {
                int gi_d = side == 0 ? -1 - gcell : n3[d] + gcell;
                for (int n = 0; n < ncomp; ++n) {
                    int t = comp_bc(phys, n, d);
                    if (t != BC_INT_DIR && t != BC_FOEXTRAP && t != BC_REFLECT_EVEN && t != BC_REFLECT_ODD)
                        continue; /* ext_dir: left to the case functor */
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
                    for (int a = lo[ta]; a < hi[ta]; ++a)
                        for (int bb = lo[tb]; bb < hi[tb]; ++bb) {
                            int idx[3];
                            idx[d] = gi_d;
                            idx[ta] = a;
                            idx[tb] = bb;
                            int src[3] = {idx[0], idx[1], idx[2]};
                            double sign = 1.0;
                            if (t == BC_INT_DIR) {
                                src[d] = side == 0 ? gi_d + n3[d] : gi_d - n3[d];
                            } else if (t == BC_FOEXTRAP) {
                                src[d] = side == 0 ? 0 : n3[d] - 1;
                            } else {
                                src[d] = side == 0 ? -1 - gi_d : 2 * n3[d] - 1 - gi_d;
                                if (t == BC_REFLECT_ODD) sign = -1.0;
                            }
                            S[n * N + gI(&b, idx[0], idx[1], idx[2])] =
                                sign * S[n * N + gI(&b, src[0], src[1], src[2])];
                        }
                }
            }
        }
        if (bc->dirichlet_case == 3 && d == 0 && bc->lo_bc[0] == 1) {
            for (int gcell = 0; gcell < NG; ++gcell)
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
                for (int bb = lo[2]; bb < hi[2]; ++bb)
                    for (int a = lo[1]; a < hi[1]; ++a) jet_fill(bc, S, N, &b, -1 - gcell, a, bb, ncomp);
        }
        if (bc->dirichlet_case == 1) {
            for (int side = 0; side < 2; ++side)
                for (int gcell = 0; gcell < NG; ++gcell) {
                    int gi_d = side == 0 ? -1 - gcell : n3[d] + gcell;
#ifdef OCFDO_OPENMP
#pragma omp parallel for schedule(static)
#endif
                    for (int a = lo[ta]; a < hi[ta]; ++a)
                        for (int bb = lo[tb]; bb < hi[tb]; ++bb) {
                            int idx[3];
                            idx[d] = gi_d;
                            idx[ta] = a;
                            idx[tb] = bb;
                            dmr_fill(bc, S, N, &b, idx[0], idx[1], idx[2], ncomp, time);
                        }
                }
        }
    }
}

/* ============================================================ RK3 driver */
double ocfdo_advance_rk3(const ocfdo_parm* p, const ocfdo_bc* bc, double* S, int nx, int ny,
                         int nz, int do_visc, double cfl, int nsteps, int form, double* dts) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b), BN = bN(&b);
    double dxinv[3] = {1.0 / bc->dx[0], 1.0 / bc->dx[1], 1.0 / bc->dx[2]};
    double* S0 = (double*)xcalloc(N * NCONS, sizeof(double));
    double* Ss = (double*)xcalloc(N * NCONS, sizeof(double));
    double* k1 = (double*)xcalloc(BN * NCONS, sizeof(double));
    double* k2 = (double*)xcalloc(BN * NCONS, sizeof(double));
    double* k3 = (double*)xcalloc(BN * NCONS, sizeof(double));
    double* fl[3];
    for (int d = 0; d < 3; ++d) fl[d] = (double*)xcalloc(fN(&b, d) * NCONS, sizeof(double));
    double time = 0.0, dt_prev = -1.0;
    for (int s = 0; s < nsteps; ++s) {
        ocfdo_fill_ghosts(bc, S, NCONS, nx, ny, nz, time);
        double dt = cfl * ocfdo_estdt(p, S, nx, ny, nz, bc->dx);
        if (dt_prev > 0 && dt > 1.1 * dt_prev) dt = 1.1 * dt_prev;
        dt_prev = dt;
        if (dts) dts[s] = dt;
        memcpy(S0, S, sizeof(double) * N * NCONS);
        /* stage 1 */
        ocfdo_rhs_regular(p, S, nx, ny, nz, dxinv, do_visc, k1, fl[0], fl[1], fl[2]);
        memcpy(Ss, S0, sizeof(double) * N * NCONS);
#ifdef OCFDO_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
        for (int n = 0; n < NCONS; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        long long g = n * N + gI(&b, i, j, k), c = n * BN + bI(&b, i, j, k);
                        Ss[g] = S0[g] + dt * k1[c];
                    }
        ocfdo_fill_ghosts(bc, Ss, NCONS, nx, ny, nz, time + dt);
        /* stage 2 */
        ocfdo_rhs_regular(p, Ss, nx, ny, nz, dxinv, do_visc, k2, fl[0], fl[1], fl[2]);
#ifdef OCFDO_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
        for (int n = 0; n < NCONS; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        long long g = n * N + gI(&b, i, j, k), c = n * BN + bI(&b, i, j, k);
                        if (form == 0)
                            Ss[g] = S0[g] + dt * (0.25 * k1[c] + 0.25 * k2[c]);
                        else
                            Ss[g] = 0.75 * S0[g] + 0.25 * (Ss[g] + dt * k2[c]);
                    }
        ocfdo_fill_ghosts(bc, Ss, NCONS, nx, ny, nz, time + 0.5 * dt);
        /* stage 3 */
        ocfdo_rhs_regular(p, Ss, nx, ny, nz, dxinv, do_visc, k3, fl[0], fl[1], fl[2]);
#ifdef OCFDO_OPENMP
#pragma omp parallel for collapse(2) schedule(static)
#endif
        for (int n = 0; n < NCONS; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        long long g = n * N + gI(&b, i, j, k), c = n * BN + bI(&b, i, j, k);
                        if (form == 0)
                            S[g] = S0[g] + dt * ((1.0 / 6.0) * k1[c] + (1.0 / 6.0) * k2[c] + (2.0 / 3.0) * k3[c]);
                        else
                            S[g] = (1.0 / 3.0) * S0[g] + (2.0 / 3.0) * (Ss[g] + dt * k3[c]);
                    }
        time += dt;
    }
    free(S0); free(Ss); free(k1); free(k2); free(k3);
    for (int d = 0; d < 3; ++d) free(fl[d]);
    return time;
}

/* ============================================== one box's RK3 step (timing)
 * The per-box work of one SSP-RK3 step of a level (Source/Advance.cpp:182-418
 * per stage: the regular or the cut-cell right-hand side of the box; then the
 * Shu-Osher update of AmrLevel::RK(3) over the box's valid cells), without the
 * ghost exchange between stages: the CPU baseline times this on a sample of a
 * hierarchy's boxes.  flag == NULL: the regular scheme; else the cut-cell one
 * (vfrac, apx, apy, apz as for ocfdo_rhs_eb).  S is advanced in place. */
void ocfdo_box_rk3_step(const ocfdo_parm* p, double* S, const uint32_t* flag, const double* vfrac,
                        const double* apx, const double* apy, const double* apz, int nx, int ny, int nz,
                        const double* dxinv, int do_redistribute, double dt) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b), BN = bN(&b);
    double* S0 = (double*)xcalloc(N * NCONS, sizeof(double));
    double* k = (double*)xcalloc(BN * NCONS, sizeof(double));
    double* fl[3];
    for (int d = 0; d < 3; ++d) fl[d] = (double*)xcalloc(fN(&b, d) * NCONS, sizeof(double));
    memcpy(S0, S, sizeof(double) * N * NCONS);
    static const double A[3] = {0.0, 0.75, 1.0 / 3.0}, B[3] = {1.0, 0.25, 2.0 / 3.0};
    for (int st = 0; st < 3; ++st) {
        if (flag)
            ocfdo_rhs_eb(p, S, flag, vfrac, apx, apy, apz, nx, ny, nz, dxinv, 0, do_redistribute, k, fl[0],
                         fl[1], fl[2]);
        else
            ocfdo_rhs_regular(p, S, nx, ny, nz, dxinv, 0, k, fl[0], fl[1], fl[2]);
        for (int n = 0; n < NCONS; ++n)
            for (int kk = 0; kk < nz; ++kk)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        long long g = n * N + gI(&b, i, j, kk), c = n * BN + bI(&b, i, j, kk);
                        S[g] = A[st] * S0[g] + B[st] * (S[g] + dt * k[c]);
                    }
    }
    free(S0);
    free(k);
    for (int d = 0; d < 3; ++d) free(fl[d]);
}

/* ======================================================= RK2 / Euler driver
 * EBR::flow_advance, Source/Advance.cpp:115-138:
 *   Euler: FillPatch(t); S_new = 1.0 * Sborder + dt * dSdt        (LinComb)
 *   RK2:   FillPatch(t); S_new = 1.0 * Sborder + dt * dSdt        (stage 1)
 *          FillPatch(t + dt) of S_new;
 *          S_new = 0.5 * Sborder + 0.5 * S_old; S_new += 0.5 * dt * dSdt */
double ocfdo_advance_rk12(const ocfdo_parm* p, const ocfdo_bc* bc, double* S, int nx, int ny,
                          int nz, int do_visc, double cfl, int nsteps, int order, double* dts) {
    box_t b = mkbox(nx, ny, nz);
    long long N = gN(&b), BN = bN(&b);
    double dxinv[3] = {1.0 / bc->dx[0], 1.0 / bc->dx[1], 1.0 / bc->dx[2]};
    double* S0 = (double*)xcalloc(N * NCONS, sizeof(double));
    double* k1 = (double*)xcalloc(BN * NCONS, sizeof(double));
    double* fl[3];
    for (int d = 0; d < 3; ++d) fl[d] = (double*)xcalloc(fN(&b, d) * NCONS, sizeof(double));
    double time = 0.0, dt_prev = -1.0;
    for (int s = 0; s < nsteps; ++s) {
        ocfdo_fill_ghosts(bc, S, NCONS, nx, ny, nz, time);
        double dt = cfl * ocfdo_estdt(p, S, nx, ny, nz, bc->dx);
        if (dt_prev > 0 && dt > 1.1 * dt_prev) dt = 1.1 * dt_prev;
        dt_prev = dt;
        if (dts) dts[s] = dt;
        memcpy(S0, S, sizeof(double) * N * NCONS);
        ocfdo_rhs_regular(p, S, nx, ny, nz, dxinv, do_visc, k1, fl[0], fl[1], fl[2]);
        for (int n = 0; n < NCONS; ++n)
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        long long g = n * N + gI(&b, i, j, k), c = n * BN + bI(&b, i, j, k);
                        S[g] = 1.0 * S0[g] + dt * k1[c];
                    }
        if (order == 2) {
            ocfdo_fill_ghosts(bc, S, NCONS, nx, ny, nz, time + dt);
            ocfdo_rhs_regular(p, S, nx, ny, nz, dxinv, do_visc, k1, fl[0], fl[1], fl[2]);
            for (int n = 0; n < NCONS; ++n)
                for (int k = 0; k < nz; ++k)
                    for (int j = 0; j < ny; ++j)
                        for (int i = 0; i < nx; ++i) {
                            long long g = n * N + gI(&b, i, j, k), c = n * BN + bI(&b, i, j, k);
                            double v = 0.5 * S[g] + 0.5 * S0[g];
                            S[g] = v + (0.5 * dt) * k1[c];
                        }
        }
        time += dt;
    }
    free(S0); free(k1);
    for (int d = 0; d < 3; ++d) free(fl[d]);
    return time;
}
