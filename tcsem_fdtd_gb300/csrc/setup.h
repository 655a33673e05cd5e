// Host front-end of the TCSEM_FDTD path: input files, grid, index maps,
// receiver/transmitter location, source waveform, time-step schedule, the
// receiver sampling plan and the precomputed boundary operators.
//
// Everything here is FP64 host code whose results must equal the reference's
// host code (ModelingSetup.cpp, ModelGridMapping.cpp, LoadRxTxPos.cpp,
// SourceWave.cpp, logspace.cpp, main.cu:150-273, EFInterp2Rx.cu:472-585).
#pragma once
#include <string>
#include <vector>
#include <stdexcept>
#include <cstdint>

#include "tcsem.h"

namespace tcsem {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

constexpr double kPi = 3.141592653589793238;  // FTDT.h:39
constexpr int kNPad = 4;                      // FTDT.h:40

struct Transmitter {
    int ort = 0, nr = 0;
    double len = 0, x = 0, y = 0, z = 0, azi = 0, dip = 0;
    int ixa = 0, iya = 0, iza = 0, ixb = 0, iyb = 0, izb = 0, ictx = 0, icty = 0, ictz = 0;
    double len1 = 0, x1 = 0, y1 = 0, z1 = 0, azi1 = 0, dip1 = 0;
    int ixa1 = 0, iya1 = 0, iza1 = 0, ixb1 = 0, iyb1 = 0, izb1 = 0, ictx1 = 0, icty1 = 0, ictz1 = 0;
    std::vector<int> rx;  // 1-based receiver ids
};

// Plain description of a survey, as read from the four input files.
struct SurveyInput {
    double sfa1 = 0, sfa2 = 0, sita_t = 0, x0 = 0, y0 = 0, z0 = 0;
    double dxmin = 0, dymin = 0, dzmin = 0, arg1 = 0, arg2 = 0;
    int n1 = 0;
    int ALx2 = 0, ALx1 = 0, Nx = 0, ARx1 = 0, ARx2 = 0, Ay2 = 0, Ay1 = 0, Ny = 0, Az2 = 0, Az1 = 0, Nz = 0;
    std::vector<double> con;  // [N][M][L]
    double T0 = 0, Tn = 0;
    int Nt = 0, IsLog = 0, isComp[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> rx, ry, rz;  // by receiver id - 1
    std::vector<Transmitter> tx;     // by transmitter id - 1
};

SurveyInput read_survey_dir(const std::string &dir);
// the same from the host records of the in-memory open (tcsem_open)
SurveyInput survey_from_host(const tcsem_model *m, const tcsem_survey *s);

// Source injection as a set of axis-aligned segments: E component `comp`
// (0 Ex, 1 Ey, 2 Ez), fixed cell along the other two axes, `count` cells from
// `start` along the segment axis.  The per-step injected value at cell q is
// wave_n * gain * coef[q] (ElectricalFiled.cu:347-475, 531-641).
struct SourceSegment {
    int comp = 0, i = 0, j = 0, k = 0, count = 0;  // start cell (i,j,k); runs along comp's axis
    double gain = 0;
    std::vector<double> coef;
};

// Receiver sampling plan of one step (EFInterp2Rx.cu:472-585): which slot the
// current E (B) field is written to, and which samples are then produced.
struct StepActions {
    int8_t e_slot = -1, b_slot = -1;  // -1 none, 0 or 1
    int e_first = 0, e_count = 0, b_first = 0, b_count = 0;
};

struct Schedule {
    std::vector<double> dt1, dt2, lam, dtB, wave;  // per step
    std::vector<StepActions> act;
    std::vector<double> e_l1, b_l1;                // per sample index
    long nsteps = 0;
};

// Precomputed 4x4x4 receiver stencils: value = sum_abc wx[a] wy[b] wz[c] F[s3+c][s2+b][s1+a]
struct RxStencil {
    int comp = 0, s1 = 0, s2 = 0, s3 = 0;
    double wx[4], wy[4], wz[4];
};

// One strip of the boundary spline remap (Intep_BzIR2R_*, SplineGridConvIR2R.cu:180-498)
// in factored form.  The natural-spline second derivatives mb of the n source
// values y solve a fixed tridiagonal system: r_i = (y_{i+1} - y_i) g_i -
// (y_i - y_{i-1}) g_{i-1}, forward elimination r'_i = r_i - w_i r'_{i-1}, back
// substitution mb_i = (r'_i - du_i mb_{i+1}) inv_i, mb_0 = mb_{n-1} = 0.  Output
// point p then reads three consecutive nodes from k0[p]:
//   out_p = sum_j c[j][p] y_{k0+j} + c[3+j][p] mb_{k0+j}.
struct SplinePlan {
    int n = 0, npts = 0;
    std::vector<double> g, w, inv, du;  // n each
    std::vector<double> c;              // [6][npts]
    std::vector<int> k0;                // npts
};

struct Model {
    SurveyInput in;
    int L = 0, M = 0, N = 0, AnLx_New = 0, AnRx_New = 0, Any_New = 0, L1 = 0, M1 = 0, nsrc = 0;
    int NComp = 0, nefcmp = 0;
    double minsita = 0.1, mu0 = 0, mindx = 0;
    std::vector<double> dx, dy, dz, X, Y, Z, Xn, Yn;  // host grid
    std::vector<double> dxk, dyk, dzk;                // cell sizes as the kernels evaluate them
    std::vector<int> xBzNew2old, yBzNew2old, xBzold2New, yBzold2New, xoldBx2NewBz, yoldBy2NewBz;
    std::vector<int> rix, riy, riz;
    std::vector<double> times, tw, dtw, wave;

    // uniform-plane boundary operators: the four strip remaps (left, right, front, back)
    SplinePlan sl, sr, sf, sb;
    int n1 = 0, n2 = 0, n3 = 0, ox = 0, oy = 0;

    void build(SurveyInput &&in);
    Schedule schedule() const;
    std::vector<SourceSegment> sources(int itx, bool fix_dual_bipole) const;
    std::vector<RxStencil> rx_stencils(int itx) const;
};

// helpers shared with the tests through the C ABI
int search_insert(const double *A, int n, double target);
void waveform(int N, double s, double *t, double *dt, double *wave);
double spline4(const double *x, const double *y, double t);

}  // namespace tcsem
