// Host front-end: see setup.h.  Each routine names the reference code whose
// results it reproduces; the golden tests compare them with the reference's
// own host code.
#include "setup.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "tcsem.h"

namespace tcsem {

// ---------------------------------------------------------------- small helpers

int search_insert(const double *A, int n, double target) {  // logspace.cpp:30-66
    if (n < 1) return 0;
    int lo = 0, hi = n - 1, pos = 0;
    while (lo <= hi) {
        int mid = lo + (hi - lo) / 2;
        if (A[mid] == target) return mid;
        if (A[mid] > target) { hi = mid - 1; pos = mid; }
        else { lo = mid + 1; pos = mid + 1; }
    }
    return pos;
}

// SourceWave.cpp:8-58 (dt[2N] taken as 0 where the reference reads
// uninitialised memory; this reproduces the shipped testwaveform.dat)
void waveform(int N, double s, double *t, double *dt, double *wave) {
    t[0] = 0;
    for (int i = 0; i < N; i++) {
        double a = t[i] - 3 * s;
        dt[i] = -s * s * (1 - std::exp(-4.5)) / N / a / std::exp(-a * a / (2 * s * s));
        t[i + 1] = t[i] + dt[i];
    }
    if (3 * s < t[N]) t[N] = 3 * s;
    for (int i = N + 1; i < 2 * N + 1; i++) {
        t[i] = 6 * s - t[2 * N - i];
        dt[i - 1] = t[i] - t[i - 1];
    }
    dt[2 * N] = 0.0;
    for (int i = 0; i < 2 * N + 1; i++)
        wave[i] = 1 / (std::sqrt(2 * kPi) * s) * std::exp(-(t[i] - 3 * s) * (t[i] - 3 * s) / 2 / s / s);
    dt[2 * N + 1] = 0.5 * (dt[2 * N] * dt[2 * N] / dt[2 * N - 1] + dt[2 * N]);
    double prev = dt[0];
    dt[0] = 0.5 * (prev * prev / dt[1] + prev);
    for (int i = 1; i < 2 * N + 1; i++) {
        double cur = dt[i];
        dt[i] = 0.5 * (prev + dt[i]);
        prev = cur;
    }
}

// CubicSpline_1d4p, EFInterp2Rx.cu:46-57
double spline4(const double *x, const double *y, double t) {
    const double h1 = x[2] - x[1];
    const double v1 = 2.0 * (x[2] - x[0]);
    const double v2 = 2.0 * (x[3] - x[1]);
    const double u1 = 6.0 * ((y[2] - y[1]) / h1 - (y[1] - y[0]) / (x[1] - x[0]));
    const double u2 = 6.0 * ((y[3] - y[2]) / (x[3] - x[2]) - (y[2] - y[1]) / h1);
    const double z1 = (v2 * u1 - h1 * u2) / (v1 * v2 - h1 * h1);
    const double z2 = (v1 * u2 - h1 * u1) / (v1 * v2 - h1 * h1);
    return z2 / (6.0 * h1) * std::pow(t - x[1], 3) + z1 / (6.0 * h1) * std::pow(x[2] - t, 3) +
           (y[2] / h1 - z2 / 6.0 * h1) * (t - x[1]) + (y[1] / h1 - z1 / 6.0 * h1) * (x[2] - t);
}

// ---------------------------------------------------------------- input files

namespace {

std::string slurp(const std::string &path, bool binary = false) {
    std::ifstream f(path, binary ? std::ios::binary : std::ios::in);
    if (!f) throw Error(TCSEM_ERR_IO, "cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

struct Tokens {
    std::istringstream s;
    std::string what;
    explicit Tokens(const std::string &text, std::string w) : s(text), what(std::move(w)) {}
    template <class T> T get() {
        T v;
        if (!(s >> v)) throw Error(TCSEM_ERR_PARSE, "malformed " + what);
        return v;
    }
};

}  // namespace

namespace {
// The grid lines of FDTD_setup.in as the setup (ModelingSetup.cpp:100-152) uses them: strip widths
// are cell counts (>= 0), each core has at least one cell, the core spacings are positive.  Returns
// the grid's L, M, N.
void check_grid(const SurveyInput &in, long &L, long &M, long &N) {
    const int strips[] = {in.ALx2, in.ALx1, in.ARx1, in.ARx2, in.Ay2, in.Ay1, in.Az2, in.Az1};
    for (int w : strips)
        if (w < 0) throw Error(TCSEM_ERR_INVALID, "bad grid dimensions: a negative strip width");
    if (in.Nx < 1 || in.Ny < 1 || in.Nz < 1) throw Error(TCSEM_ERR_INVALID, "bad grid dimensions: an empty core");
    if (!(in.dxmin > 0) || !(in.dymin > 0) || !(in.dzmin > 0))
        throw Error(TCSEM_ERR_INVALID, "bad grid spacing: dxmin, dymin and dzmin must be positive");
    L = (long)in.ALx2 + in.ALx1 + in.ARx2 + in.ARx1 + in.Nx;
    M = 2L * (in.Ay2 + in.Ay1) + in.Ny;
    N = (long)in.Nz + in.Az2 + in.Az1;
    if (L * M * N > (1L << 33)) throw Error(TCSEM_ERR_INVALID, "bad grid dimensions");
}
}  // namespace

SurveyInput read_survey_dir(const std::string &dir) {
    SurveyInput in;
    {  // ModelingSetup.cpp:51-59
        Tokens t(slurp(dir + "/FDTD_setup.in"), "FDTD_setup.in");
        in.sfa1 = t.get<double>(); in.sfa2 = t.get<double>();
        in.n1 = t.get<int>(); in.sita_t = t.get<double>();
        in.x0 = t.get<double>(); in.y0 = t.get<double>(); in.z0 = t.get<double>();
        in.dxmin = t.get<double>(); in.dymin = t.get<double>(); in.dzmin = t.get<double>();
        in.arg1 = t.get<double>(); in.arg2 = t.get<double>();
        in.ALx2 = t.get<int>(); in.ALx1 = t.get<int>(); in.Nx = t.get<int>(); in.ARx1 = t.get<int>(); in.ARx2 = t.get<int>();
        in.Ay2 = t.get<int>(); in.Ay1 = t.get<int>(); in.Ny = t.get<int>();
        in.Az2 = t.get<int>(); in.Az1 = t.get<int>(); in.Nz = t.get<int>();
    }
    long L, M, N;
    check_grid(in, L, M, N);
    {  // Cond.bin, float64 [N][M][L] (ModelingSetup.cpp:201-209), read straight into place
        const std::string path = dir + "/Cond.bin";
        std::ifstream f(path, std::ios::binary | std::ios::ate);
        if (!f) throw Error(TCSEM_ERR_IO, "cannot open " + path);
        const size_t n = (size_t)L * M * N, bytes = (size_t)f.tellg();
        if (bytes < n * sizeof(double)) throw Error(TCSEM_ERR_PARSE, "Cond.bin shorter than N*M*L doubles");
        in.con.resize(n);
        f.seekg(0);
        if (!f.read(reinterpret_cast<char *>(in.con.data()), (std::streamsize)(n * sizeof(double))))
            throw Error(TCSEM_ERR_IO, "cannot read " + path);
    }
    {  // LoadRxTxPos.cpp:51-84
        Tokens t(slurp(dir + "/Receiver.in"), "Receiver.in");
        in.T0 = t.get<double>(); in.Tn = t.get<double>();
        in.Nt = t.get<int>(); in.IsLog = t.get<int>();
        for (int c = 0; c < 6; c++) in.isComp[c] = t.get<int>();
        int nrx = t.get<int>();
        if (nrx < 1) throw Error(TCSEM_ERR_PARSE, "Receiver.in: no receivers");
        in.rx.assign(nrx, 0); in.ry.assign(nrx, 0); in.rz.assign(nrx, 0);
        for (int r = 0; r < nrx; r++) {
            int id = t.get<int>();
            if (id < 1 || id > nrx) throw Error(TCSEM_ERR_PARSE, "Receiver.in: receiver id out of range");
            in.rx[id - 1] = t.get<double>(); in.ry[id - 1] = t.get<double>(); in.rz[id - 1] = t.get<double>();
        }
    }
    {  // LoadRxTxPos.cpp:134-200 (field order id ort BipoLen x y z ...)
        Tokens t(slurp(dir + "/Transmitter.in"), "Transmitter.in");
        int ntx = t.get<int>();
        if (ntx < 1) throw Error(TCSEM_ERR_PARSE, "Transmitter.in: no transmitters");
        in.tx.assign(ntx, Transmitter());
        for (int q = 0; q < ntx; q++) {
            int id = t.get<int>();
            if (id < 1 || id > ntx) throw Error(TCSEM_ERR_PARSE, "Transmitter.in: id out of range");
            Transmitter &T = in.tx[id - 1];
            T.ort = t.get<int>();
            T.len = t.get<double>(); T.x = t.get<double>(); T.y = t.get<double>(); T.z = t.get<double>();
            if (T.ort == 4 || T.ort == 5) {
                T.azi = t.get<double>() * kPi / 180.0;
                T.dip = t.get<double>() * kPi / 180.0;
            } else if (T.ort < 1 || T.ort > 5) {
                throw Error(TCSEM_ERR_PARSE, "Transmitter.in: illegal orientation");
            }
            if (T.ort == 5) {
                T.len1 = t.get<double>(); T.x1 = t.get<double>(); T.y1 = t.get<double>(); T.z1 = t.get<double>();
                T.azi1 = t.get<double>() * kPi / 180.0;
                T.dip1 = t.get<double>() * kPi / 180.0;
            }
            T.nr = t.get<int>();
            if (T.nr < 1) throw Error(TCSEM_ERR_PARSE, "Transmitter.in: no receivers for a transmitter");
            T.rx.resize(T.nr);
            for (int r = 0; r < T.nr; r++) {
                T.rx[r] = t.get<int>();
                if (T.rx[r] < 1 || T.rx[r] > (int)in.rx.size())
                    throw Error(TCSEM_ERR_PARSE, "Transmitter.in: receiver id out of range");
            }
        }
    }
    return in;
}

// The same SurveyInput from host records (tcsem_open): the values and checks of
// read_survey_dir, field for field, with angles converted from degrees as the
// parser does (LoadRxTxPos.cpp:151-200).
SurveyInput survey_from_host(const tcsem_model *m, const tcsem_survey *s) {
    if (!m || !s) throw Error(TCSEM_ERR_INVALID, "null model or survey");
    SurveyInput in;
    in.sfa1 = m->sfa1; in.sfa2 = m->sfa2; in.n1 = m->n1; in.sita_t = m->sita_t;
    in.x0 = m->x0; in.y0 = m->y0; in.z0 = m->z0;
    in.dxmin = m->dxmin; in.dymin = m->dymin; in.dzmin = m->dzmin;
    in.arg1 = m->arg1; in.arg2 = m->arg2;
    in.ALx2 = m->ALx2; in.ALx1 = m->ALx1; in.Nx = m->Nx; in.ARx1 = m->ARx1; in.ARx2 = m->ARx2;
    in.Ay2 = m->Ay2; in.Ay1 = m->Ay1; in.Ny = m->Ny;
    in.Az2 = m->Az2; in.Az1 = m->Az1; in.Nz = m->Nz;
    long L, M, N;
    check_grid(in, L, M, N);
    if (!m->con) throw Error(TCSEM_ERR_INVALID, "null conductivity");
    in.con.assign(m->con, m->con + (size_t)L * M * N);
    in.T0 = s->T0; in.Tn = s->Tn; in.Nt = s->Nt; in.IsLog = s->IsLog;
    for (int c = 0; c < 6; c++) in.isComp[c] = s->comps[c];
    if (s->NRx < 1 || !s->rx_xyz) throw Error(TCSEM_ERR_PARSE, "survey: no receivers");
    in.rx.resize(s->NRx); in.ry.resize(s->NRx); in.rz.resize(s->NRx);
    for (int r = 0; r < s->NRx; r++) {
        in.rx[r] = s->rx_xyz[3 * r]; in.ry[r] = s->rx_xyz[3 * r + 1]; in.rz[r] = s->rx_xyz[3 * r + 2];
    }
    if (s->NTx < 1 || !s->tx) throw Error(TCSEM_ERR_PARSE, "survey: no transmitters");
    in.tx.assign(s->NTx, Transmitter());
    for (int q = 0; q < s->NTx; q++) {
        const tcsem_transmitter &h = s->tx[q];
        Transmitter &T = in.tx[q];
        T.ort = h.ort;
        T.len = h.len; T.x = h.x; T.y = h.y; T.z = h.z;
        if (T.ort < 1 || T.ort > 5) throw Error(TCSEM_ERR_PARSE, "survey: illegal transmitter orientation");
        if (T.ort >= 4) { T.azi = h.azi * kPi / 180.0; T.dip = h.dip * kPi / 180.0; }
        if (T.ort == 5) {
            T.len1 = h.len1; T.x1 = h.x1; T.y1 = h.y1; T.z1 = h.z1;
            T.azi1 = h.azi1 * kPi / 180.0; T.dip1 = h.dip1 * kPi / 180.0;
        }
        T.nr = h.nr;
        if (T.nr < 1 || !h.rx) throw Error(TCSEM_ERR_PARSE, "survey: no receivers for a transmitter");
        T.rx.assign(h.rx, h.rx + T.nr);
        for (int id : T.rx)
            if (id < 1 || id > s->NRx) throw Error(TCSEM_ERR_PARSE, "survey: receiver id out of range");
    }
    return in;
}

// ---------------------------------------------------------------- model build

namespace {

// evaluation rule of Intep_BzIR2R_* (SplineGridConvIR2R.cu:180-498): cubic
// inside the node range, the end derivative's quadratic outside it
double spline_at(int n, const double *d, const double *xo, const double *y, const double *mb, int map, double xnew) {
    int id = std::max(map - 1, 0);
    double ma, mc;
    if (id < n - 1) {
        double h = 0.5 * d[id] + 0.5 * d[id + 1];
        ma = 1.0 / 3.0 * (mb[id + 1] - mb[id]) / h;
        mc = (y[id + 1] - y[id]) / h - 1.0 / 3.0 * (2.0 * mb[id] + mb[id + 1]) * h;
    } else {
        double h = 0.5 * d[id - 1] + 0.5 * d[id];
        ma = 1.0 / 3.0 * (mb[id] - mb[id - 1]) / h;
        mc = (y[id] - y[id - 1]) / h - 1.0 / 3.0 * (2.0 * mb[id - 1] + mb[id]) * h;
        mc += 3.0 * ma * h * h + 2.0 * mb[id - 1] * h;
        ma = 0.0;
    }
    double h = xnew - xo[id];
    int id2 = map - 1;
    if (id2 >= 0 && id2 < n - 1) return ma * h * h * h + mb[id2] * h * h + mc * h + y[id2];
    int c = std::max(id2, 0);
    return (mb[c] * h + mc) * h + y[c];
}

// factored form of one strip remap: elimination factors of the natural cubic
// spline system of SplineGridConvIR2R.cu (tridiagonal rows of fillA*,
// initialize_UpCont_gpu_resources.cu:46-144; right hand side of Fill_B_*,
// SplineGridConvIR2R.cu:70-173) and, per output point, the weights of its three-node window.  spline_at is
// linear in (y, mb) jointly, so the window weights are its values at unit
// vectors.
void spline_plan(int n, const double *d, const double *xo, int npts, const int *map, int map_shift,
                 const double *xnew, SplinePlan &P) {
    P.n = n;
    P.npts = npts;
    P.g.assign(n, 0.0); P.w.assign(n, 0.0); P.inv.assign(n, 0.0); P.du.assign(n, 0.0);
    std::vector<double> dl(n, 0.0), dd(n, 2.0), du(n, 0.0);
    for (int i = 1; i < n - 1; i++) {
        dd[i] = 2.0 / 3.0 * (d[i] + 0.5 * d[i - 1] + 0.5 * d[i + 1]);
        dl[i] = 1.0 / 3.0 * (0.5 * d[i - 1] + 0.5 * d[i]);
        du[i] = 1.0 / 3.0 * (0.5 * d[i] + 0.5 * d[i + 1]);
    }
    for (int i = 0; i + 1 < n; i++) P.g[i] = 1.0 / (0.5 * d[i] + 0.5 * d[i + 1]);
    for (int i = 1; i < n; i++) {
        P.w[i] = dl[i] / dd[i - 1];
        dd[i] -= P.w[i] * du[i - 1];
    }
    for (int i = 0; i < n; i++) { P.inv[i] = 1.0 / dd[i]; P.du[i] = du[i]; }
    P.c.assign((size_t)6 * npts, 0.0);
    P.k0.assign(npts, 0);
    std::vector<double> y(n, 0.0), mb(n, 0.0);
    for (int p = 0; p < npts; p++) {
        const int mp = map[p] - map_shift, id = std::max(mp - 1, 0);
        if (id > n - 1) throw Error(TCSEM_ERR_INVALID, "boundary remap point beyond its strip");
        const int k0 = std::min(std::max(id - 1, 0), n - 3);
        P.k0[p] = k0;
        for (int j = 0; j < 3; j++) {
            y[k0 + j] = 1.0;
            P.c[(size_t)j * npts + p] = spline_at(n, d, xo, y.data(), mb.data(), mp, xnew[p]);
            y[k0 + j] = 0.0;
            mb[k0 + j] = 1.0;
            P.c[(size_t)(3 + j) * npts + p] = spline_at(n, d, xo, y.data(), mb.data(), mp, xnew[p]);
            mb[k0 + j] = 0.0;
        }
    }
}

}  // namespace

void Model::build(SurveyInput &&src) {
    in = std::move(src);
    SurveyInput &I = in;
    if (I.Nx < 1 || I.Ny < 1 || I.Nz < 1 || I.dxmin <= 0 || I.dymin <= 0 || I.dzmin <= 0)
        throw Error(TCSEM_ERR_INVALID, "grid spacings and core sizes must be positive");
    if (I.ALx1 + I.ALx2 < 1 || I.ARx1 + I.ARx2 < 1 || I.Ay1 + I.Ay2 < 1)
        throw Error(TCSEM_ERR_INVALID, "each lateral boundary strip needs at least one cell");
    if (I.ALx1 + I.ALx2 + kNPad > 128 || I.ARx1 + I.ARx2 + kNPad > 128 || I.Ay1 + I.Ay2 + kNPad > 128)
        throw Error(TCSEM_ERR_INVALID, "boundary strips wider than 124 cells");  // initialize_UpCont_gpu_resources.cu:138
    if (I.n1 < 4) throw Error(TCSEM_ERR_INVALID, "source waveform needs n1 >= 4");
    if (I.Nt < 2) throw Error(TCSEM_ERR_INVALID, "need at least two sampling times");
    nsrc = I.n1 / 2;
    L = I.ALx2 + I.ALx1 + I.ARx2 + I.ARx1 + I.Nx;
    M = 2 * (I.Ay2 + I.Ay1) + I.Ny;
    N = I.Nz + I.Az2 + I.Az1;
    const int AL = I.ALx2 + I.ALx1, Ay = I.Ay2 + I.Ay1;

    // cell sizes and centres, ModelingSetup.cpp:100-187
    dx.assign(L, 0); dy.assign(M, 0); dz.assign(N, 0);
    for (int i = AL; i < I.Nx + AL; i++) dx[i] = I.dxmin;
    for (int i = AL - 1; i >= I.ALx2; i--) dx[i] = I.dxmin * std::pow(I.arg1, double(I.ALx1 + I.ALx2 - i));
    for (int i = I.ALx2 - 1; i >= 0; i--) dx[i] = I.dxmin * std::pow(I.arg1, double(I.ALx1)) * std::pow(I.arg2, double(I.ALx2 - i));
    for (int i = I.Nx + AL; i < I.Nx + AL + I.ARx1; i++) dx[i] = I.dxmin * std::pow(I.arg1, double(i - AL - I.Nx + 1));
    for (int i = I.Nx + AL + I.ARx1; i < L; i++)
        dx[i] = I.dxmin * std::pow(I.arg1, double(I.ARx1)) * std::pow(I.arg2, double(i - I.Nx - AL - I.ARx1 + 1));
    for (int j = Ay; j < I.Ny + Ay; j++) dy[j] = I.dymin;
    for (int j = Ay - 1; j >= I.Ay2; j--) dy[j] = dy[j + 1] * I.arg1;
    for (int j = I.Ay2 - 1; j >= 0; j--) dy[j] = dy[j + 1] * I.arg2;
    for (int j = I.Ny + Ay; j < I.Ny + I.Ay2 + 2 * I.Ay1; j++) dy[j] = dy[j - 1] * I.arg1;
    for (int j = I.Ny + I.Ay2 + 2 * I.Ay1; j < M; j++) dy[j] = dy[j - 1] * I.arg2;
    for (int k = 0; k < I.Nz; k++) dz[k] = I.dzmin;
    for (int k = I.Nz; k < I.Nz + I.Az1; k++) dz[k] = dz[k - 1] * I.arg1;
    for (int k = I.Nz + I.Az1; k < N; k++) dz[k] = dz[k - 1] * I.arg2;
    auto centres = [](const std::vector<double> &d, int core, int lead, double o, std::vector<double> &C) {
        int n = (int)d.size(), nc;
        C.assign(n, 0);
        if (core % 2 == 0) { nc = core / 2 + lead; C[nc] = 0.5 * d[nc] + o; }
        else { nc = (core - 1) / 2 + lead; C[nc] = o; }
        for (int i = nc + 1; i < n; i++) C[i] = C[i - 1] + 0.5 * d[i - 1] + 0.5 * d[i];
        for (int i = nc - 1; i >= 0; i--) C[i] = C[i + 1] - 0.5 * d[i + 1] - 0.5 * d[i];
    };
    centres(dx, I.Nx, AL, I.x0, X);
    centres(dy, I.Ny, Ay, I.y0, Y);
    Z.assign(N, 0);
    Z[0] = 0.5 * dz[0] + I.z0;
    for (int k = 1; k < N; k++) Z[k] = Z[k - 1] + 0.5 * dz[k - 1] + 0.5 * dz[k];
    const int AR0 = L - I.ARx1 - I.ARx2;
    AnLx_New = (int)std::ceil((X[AL - 1] - X[0] + dx[AL - 1] / 2 + dx[0] / 2) / I.dxmin);
    AnRx_New = (int)std::ceil((X[L - 1] - X[AR0] + dx[L - 1] / 2 + dx[AR0] / 2) / I.dxmin);
    Any_New = (int)std::ceil((Y[Ay - 1] - Y[0] + dy[Ay - 1] / 2 + dy[0] / 2) / I.dymin);
    L1 = AnLx_New + AnRx_New + I.Nx;
    M1 = 2 * Any_New + I.Ny;

    // Grid_dx/Grid_dy/Grid_dz as evaluated inside the kernels (ElectricalFiled.cu:36-86)
    dxk.assign(L, 0); dyk.assign(M, 0); dzk.assign(N, 0);
    for (int i = 0; i < L; i++) {
        if (i >= AL && i < I.Nx + AL) dxk[i] = I.dxmin;
        else if (i >= I.ALx2 && i < AL) dxk[i] = I.dxmin * std::pow(I.arg1, double(AL - i));
        else if (i < I.ALx2) dxk[i] = I.dxmin * std::pow(I.arg1, double(I.ALx1)) * std::pow(I.arg2, double(I.ALx2 - i));
        else if (i < I.Nx + I.ARx1 + AL) dxk[i] = I.dxmin * std::pow(I.arg1, double(i - I.Nx - AL + 1));
        else dxk[i] = I.dxmin * std::pow(I.arg1, double(I.ARx1)) * std::pow(I.arg2, double(i - I.Nx - I.ARx1 - AL + 1));
    }
    for (int j = 0; j < M; j++) {
        if (j >= Ay && j < I.Ny + Ay) dyk[j] = I.dymin;
        else if (j >= I.Ay2 && j < Ay) dyk[j] = I.dymin * std::pow(I.arg1, double(Ay - j));
        else if (j < I.Ay2) dyk[j] = I.dymin * std::pow(I.arg1, double(I.Ay1)) * std::pow(I.arg2, double(I.Ay2 - j));
        else if (j < I.Ny + 2 * I.Ay1 + I.Ay2) dyk[j] = I.dymin * std::pow(I.arg1, double(j - I.Ny - Ay + 1));
        else dyk[j] = I.dymin * std::pow(I.arg1, double(I.Ay1)) * std::pow(I.arg2, double(j - I.Ny - 2 * I.Ay1 - I.Ay2 + 1));
    }
    for (int k = 0; k < N; k++) {
        if (k < I.Nz) dzk[k] = I.dzmin;
        else if (k < I.Nz + I.Az1) dzk[k] = I.dzmin * std::pow(I.arg1, double(k - I.Nz + 1));
        else dzk[k] = I.dzmin * std::pow(I.arg1, double(I.Az1)) * std::pow(I.arg2, double(k - I.Nz - I.Az1 + 1));
    }

    mu0 = 4 * kPi * 1.e-7;                                      // main.cu:55
    mindx = std::min(I.dzmin, std::min(I.dxmin, I.dymin));      // main.cu:107
    minsita = 0.1;  // ModelingSetup.cpp:211-230: its filter never selects a cell, so the default stays
    tw.assign(2 * nsrc + 1, 0); dtw.assign(2 * nsrc + 2, 0); wave.assign(2 * nsrc + 1, 0);
    waveform(nsrc, I.sita_t, tw.data(), dtw.data(), wave.data());

    // uniform plane and index maps, ModelGridMapping.cpp:43-395
    const int Nx = I.Nx, Ny = I.Ny, L0 = L, M0 = M;
    Xn.assign(L1, 0); Yn.assign(M1, 0);
    for (int i = AnLx_New; i < AnLx_New + Nx; i++) Xn[i] = X[i - AnLx_New + AL];
    for (int i = AnLx_New - 1; i >= 0; i--) Xn[i] = Xn[i + 1] - I.dxmin;
    for (int i = AnLx_New + Nx; i < L1; i++) Xn[i] = Xn[i - 1] + I.dxmin;
    for (int j = Any_New; j < Any_New + Ny; j++) Yn[j] = Y[j - Any_New + Ay];
    for (int j = Any_New - 1; j >= 0; j--) Yn[j] = Yn[j + 1] - I.dymin;
    for (int j = Any_New + Ny; j < M1; j++) Yn[j] = Yn[j - 1] + I.dymin;
    // new-plane points located in the old grid: index of the first old node >= point
    auto new2old = [](const std::vector<double> &Old, const std::vector<double> &New, int core0, int ncore, int oldcore0,
                      std::vector<int> &map) {
        int n1 = (int)New.size(), n0 = (int)Old.size();
        map.assign(n1, 0);
        for (int i = core0; i < core0 + ncore; i++) map[i] = i - core0 + oldcore0;
        for (int i = core0 - 1; i >= 0; i--) {
            int j = map[i + 1];
            while (j > 0 && Old[j - 1] >= New[i]) j--;
            map[i] = j;
        }
        for (int i = core0 + ncore; i < n1; i++) {
            int j = map[i - 1] - 1;
            while (j < n0 - 1 && Old[j + 1] < New[i]) j++;
            map[i] = j + 1;
        }
    };
    new2old(X, Xn, AnLx_New, Nx, AL, xBzNew2old);
    new2old(Y, Yn, Any_New, Ny, Ay, yBzNew2old);
    // old points (optionally shifted to the staggered face) located in the new plane
    auto old2new = [](const std::vector<double> &P, const std::vector<double> &New, int core0, int ncore, int newcore0,
                      std::vector<int> &map) {
        int n0 = (int)P.size(), n1 = (int)New.size();
        map.assign(n0, 0);
        for (int i = core0; i < core0 + ncore; i++) map[i] = i - core0 + newcore0;
        for (int i = core0 - 1; i >= 0; i--) {
            int j = map[i + 1];
            while (j > 0 && New[j - 1] >= P[i]) j--;
            map[i] = j;
        }
        for (int i = core0 + ncore; i < n0; i++) {
            int j = map[i - 1];
            while (j < n1 - 1 && New[j + 1] < P[i]) j++;
            map[i] = j + 1;
        }
    };
    old2new(X, Xn, AL, Nx, AnLx_New, xBzold2New);
    old2new(Y, Yn, Ay, Ny, Any_New, yBzold2New);
    {
        std::vector<double> Px(L0 + 1), Py(M0 + 1);
        for (int i = 0; i < L0; i++) Px[i] = X[i] - 0.5 * dx[i];
        Px[L0] = X[L0 - 1] + 0.5 * dx[L0 - 1];
        for (int j = 0; j < M0; j++) Py[j] = Y[j] - 0.5 * dy[j];
        Py[M0] = Y[M0 - 1] + 0.5 * dy[M0 - 1];
        old2new(Px, Xn, AL, Nx, AnLx_New, xoldBx2NewBz);
        old2new(Py, Yn, Ay, Ny, Any_New, yoldBy2NewBz);
    }

    // receivers, LoadRxTxPos.cpp:86-123
    int nrx = (int)I.rx.size();
    rix.assign(nrx, 0); riy.assign(nrx, 0); riz.assign(nrx, 0);
    for (int r = 0; r < nrx; r++) {
        int n = search_insert(X.data(), L, I.rx[r]);
        if (n == 0 || n == L) throw Error(TCSEM_ERR_INVALID, "receiver " + std::to_string(r + 1) + " outside the model in x");
        rix[r] = n;
        n = search_insert(Y.data(), M, I.ry[r]);
        if (n == 0 || n == M) throw Error(TCSEM_ERR_INVALID, "receiver " + std::to_string(r + 1) + " outside the model in y");
        riy[r] = n;
        riz[r] = search_insert(Z.data(), N, I.rz[r]);
        // the 4-point stencils (EFInterp2Rx.cu:60-378) read nodes up to two cells either side
        if (rix[r] < 2 || rix[r] > L - 3 || riy[r] < 2 || riy[r] > M - 3 || riz[r] > N - 3)
            throw Error(TCSEM_ERR_INVALID, "receiver " + std::to_string(r + 1) + " too close to the model edge");
    }
    // transmitters, LoadRxTxPos.cpp:203-453
    auto pair_fix = [](int &a, int &b) { if (b > a) b--; else if (b < a) a--; };
    for (size_t t = 0; t < I.tx.size(); t++) {
        Transmitter &T = I.tx[t];
        auto bad = [&](const char *axis) {
            throw Error(TCSEM_ERR_INVALID, "transmitter " + std::to_string(t + 1) + " outside the model in " + axis);
        };
        const double *Xp = X.data(), *Yp = Y.data(), *Zp = Z.data();
        if (T.ort == 1) {
            T.ixa = search_insert(Xp, L, T.x - T.len / 2);
            T.ixb = search_insert(Xp, L, T.x + T.len / 2) - 1;
            if (T.ixa == 0 || T.ixb == L) bad("x");
            T.icty = search_insert(Yp, M, T.y);
            if (T.icty == 0 || T.icty == M) bad("y");
            T.ictz = search_insert(Zp, N, T.z);
        } else if (T.ort == 2) {
            T.ictx = search_insert(Xp, L, T.x);
            if (T.ictx == 0 || T.ictx == L) bad("x");
            T.iya = search_insert(Yp, M, T.y - T.len / 2);
            T.iyb = search_insert(Yp, M, T.y + T.len / 2) - 1;
            if (T.iya == 0 || T.iyb == M) bad("y");
            T.ictz = search_insert(Zp, N, T.z);
        } else if (T.ort == 3) {
            T.ictx = search_insert(Xp, L, T.x);
            if (T.ictx == 0 || T.ictx == L) bad("x");
            T.icty = search_insert(Yp, M, T.y);
            if (T.icty == 0 || T.icty == M) bad("y");
            T.iza = search_insert(Zp, N, T.z - T.len / 2);
            T.izb = search_insert(Zp, N, T.z + T.len / 2) - 1;
        } else {
            double cd = std::cos(T.dip), ca = std::cos(T.azi), sa = std::sin(T.azi), sd = std::sin(T.dip);
            T.ixa = search_insert(Xp, L, T.x - T.len * cd * ca / 2.0);
            T.ixb = search_insert(Xp, L, T.x + T.len * cd * ca / 2.0);
            pair_fix(T.ixa, T.ixb);
            if (T.ort == 5) {
                double cd1 = std::cos(T.dip1), ca1 = std::cos(T.azi1);
                T.ixa1 = search_insert(Xp, L, T.x1 - T.len1 * cd1 * ca1 / 2.0);
                T.ixb1 = search_insert(Xp, L, T.x1 + T.len1 * cd1 * ca1 / 2.0);
                pair_fix(T.ixa1, T.ixb1);
                if (T.ixa1 == 0 || T.ixb1 == L) bad("x");
            }
            if (T.ixa == 0 || T.ixb == L) bad("x");
            T.iya = search_insert(Yp, M, T.y - T.len * cd * sa / 2.0);
            T.iyb = search_insert(Yp, M, T.y + T.len * cd * sa / 2.0);
            pair_fix(T.iya, T.iyb);
            if (T.ort == 5) {
                double cd1 = std::cos(T.dip1), sa1 = std::sin(T.azi1);
                T.iya1 = search_insert(Yp, M, T.y1 - T.len1 * cd1 * sa1 / 2.0);
                T.iyb1 = search_insert(Yp, M, T.y1 + T.len1 * cd1 * sa1 / 2.0);
                pair_fix(T.iya1, T.iyb1);
                if (T.iya1 == 0 || T.iyb1 == M) bad("y");
            }
            if (T.iya == 0 || T.iyb == M) bad("y");
            T.iza = search_insert(Zp, N, T.z - T.len * sd / 2.0);
            T.izb = search_insert(Zp, N, T.z + T.len * sd / 2.0);
            pair_fix(T.iza, T.izb);
            if (T.ort == 5) {
                double sd1 = std::sin(T.dip1);
                T.iza1 = search_insert(Zp, N, T.z1 - T.len1 * sd1 / 2.0);
                T.izb1 = search_insert(Zp, N, T.z1 + T.len1 * sd1 / 2.0);
                pair_fix(T.iza1, T.izb1);
                T.ictx1 = search_insert(Xp, L, T.x1);
                T.icty1 = search_insert(Yp, M, T.y1);
                T.ictz1 = search_insert(Zp, N, T.z1);
            }
            T.ictx = search_insert(Xp, L, T.x);
            T.icty = search_insert(Yp, M, T.y);
            T.ictz = search_insert(Zp, N, T.z);
        }
        // injected cells must lie inside the update ranges of the E kernels
        auto chk = [&](bool ok) { if (!ok) throw Error(TCSEM_ERR_INVALID, "transmitter " + std::to_string(t + 1) + " touches the model edge"); };
        if (T.ort == 1 || T.ort >= 4) chk(T.icty >= 1 && T.icty < M && T.ictz < N && std::max(T.ixa, T.ixb) < L);
        if (T.ort == 2 || T.ort >= 4) chk(T.ictx >= 1 && T.ictx < L && T.ictz < N && std::max(T.iya, T.iyb) < M && std::min(T.iya, T.iyb) >= 0);
        if (T.ort == 3 || T.ort >= 4) chk(T.ictx >= 1 && T.ictx < L && T.icty >= 1 && T.icty < M && std::max(T.iza, T.izb) < N);
    }
    times.assign(I.Nt, 0);
    if (I.IsLog) {  // logspace.cpp:5-19
        if (I.T0 <= 0) throw Error(TCSEM_ERR_INVALID, "log-spaced sampling needs T0 > 0");
        double step = (std::log10(I.Tn) - std::log10(I.T0)) / (I.Nt - 1);
        for (int i = 0; i < I.Nt; i++) times[i] = exp10(std::log10(I.T0) + i * step);
    } else {
        double step = (I.Tn - I.T0) / (I.Nt - 1);
        for (int i = 0; i < I.Nt; i++) times[i] = I.T0 + i * step;
    }
    NComp = nefcmp = 0;
    for (int c = 0; c < 6; c++) NComp += I.isComp[c] ? 1 : 0;
    for (int c = 0; c < 3; c++) nefcmp += I.isComp[c] ? 1 : 0;

    // boundary remap weights (the spline remap is linear in the Bz plane)
    n1 = AL + kNPad; n2 = I.ARx1 + I.ARx2 + kNPad; n3 = Ay + kNPad;
    ox = I.Nx + AL - kNPad; oy = I.Ny + Ay - kNPad;
    if (ox < 0 || oy < 0 || n1 > L || n3 > M) throw Error(TCSEM_ERR_INVALID, "core too small for the boundary remap");
    spline_plan(n1, dx.data(), X.data(), AnLx_New, xBzNew2old.data(), 0, Xn.data(), sl);
    spline_plan(n2, dx.data() + ox, X.data() + ox, AnRx_New, xBzNew2old.data() + Nx + AnLx_New, ox,
                Xn.data() + Nx + AnLx_New, sr);
    spline_plan(n3, dy.data(), Y.data(), Any_New, yBzNew2old.data(), 0, Yn.data(), sf);
    spline_plan(n3, dy.data() + oy, Y.data() + oy, Any_New, yBzNew2old.data() + Ny + Any_New, oy,
                Yn.data() + Ny + Any_New, sb);
}

// main.cu:212-273 plus the host decisions of EFInterp2Rx.cu:472-585
Schedule Model::schedule() const {
    Schedule S;
    S.e_l1.assign(in.Nt, 0.0);
    S.b_l1.assign(in.Nt, 0.0);
    const double *T = times.data();
    const int Nt = in.Nt;
    const bool has_b = in.isComp[3] || in.isComp[4] || in.isComp[5];
    double Tp[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int ne = 0, nb = 0, n = 0;
    double toT = 0, dt1 = dtw[0], dt2 = dtw[1];
    Tp[0][1] = toT + dt1;
    Tp[1][1] = toT + dt1 + 0.5 * dt2;
    while (ne < Nt || (nb < Nt && nefcmp < NComp)) {
        if (S.nsteps > 50000000) throw Error(TCSEM_ERR_INVALID, "time window needs more than 5e7 steps");
        StepActions a;
        S.dt1.push_back(dt1);
        S.dt2.push_back(dt2);
        S.lam.push_back(7.5 * in.sfa2 * dt2 * dt1 / mu0 / mindx / mindx);
        S.dtB.push_back(0.5 * (dt1 + dt2));
        S.wave.push_back(n < 2 * nsrc ? wave[n] : 0.0);
        toT += dt1;
        dt1 = dt2;
        n++;
        if (n < 2 * nsrc) dt2 = dtw[n + 1];
        else dt2 = std::min(0.15 * in.sfa1 * std::sqrt(mu0 * toT * minsita / 8.) * mindx, 1.2 * dt1);
        const double t0 = toT + dt1;
        if (ne < Nt) {
            Tp[0][2] = t0;
            while (ne < Nt && T[ne] <= Tp[0][0]) ne++;
            if (ne < Nt && T[ne] <= Tp[0][2] && T[ne] > Tp[0][1]) {
                a.e_slot = 0;
            } else if (ne < Nt && T[ne] <= Tp[0][1] && T[ne] > Tp[0][0]) {
                a.e_slot = 1;
                a.e_first = ne;
                while (ne < Nt && T[ne] <= Tp[0][1]) {
                    S.e_l1[ne] = (T[ne] - Tp[0][0]) / (Tp[0][1] - Tp[0][0]);
                    ne++;
                }
                a.e_count = ne - a.e_first;
            }
            Tp[0][0] = Tp[0][1];
            Tp[0][1] = Tp[0][2];
        }
        if (nb < Nt && has_b) {
            Tp[1][2] = t0 + 0.5 * dt2;
            while (nb < Nt && T[nb] <= Tp[1][0]) nb++;
            if (nb < Nt && T[nb] <= Tp[1][2] && T[nb] > Tp[1][1]) {
                a.b_slot = 0;
            } else if (nb < Nt && T[nb] <= Tp[1][1] && T[nb] > Tp[1][0]) {
                a.b_slot = 1;
                a.b_first = nb;
                while (nb < Nt && T[nb] <= Tp[1][1]) {
                    S.b_l1[nb] = (T[nb] - Tp[1][0]) / (Tp[1][1] - Tp[1][0]);
                    nb++;
                }
                a.b_count = nb - a.b_first;
            }
            Tp[1][0] = Tp[1][1];
            Tp[1][1] = Tp[1][2];
        }
        S.act.push_back(a);
        S.nsteps++;
    }
    return S;
}

// Source injection of ElectricalField (ElectricalFiled.cu:347-475, 531-641)
// as segments.  With fix_dual_bipole the second bipole of ort=5 is injected at
// its own cells; otherwise at the first bipole's cells like the reference.
std::vector<SourceSegment> Model::sources(int itx, bool fix_dual_bipole) const {
    const Transmitter &T = in.tx.at(itx);
    const double *C = in.con.data();
    auto con = [&](int k, int j, int i) { return C[((size_t)k * M + j) * L + i]; };
    std::vector<SourceSegment> out;
    auto seg_x = [&](int ixa, int ixb, int icty, int ictz, int count, double gain) {
        SourceSegment s;
        s.comp = 0; s.i = std::min(ixa, ixb); s.j = icty; s.k = ictz;
        s.count = std::min(count, std::abs(ixb - ixa) + 1);
        s.gain = gain;
        for (int q = 0; q < s.count; q++) {
            int i = s.i + q;
            double sg = ictz == 0 ? con(0, icty, i) + con(0, icty - 1, i)
                                  : con(ictz, icty, i) + con(ictz, icty - 1, i) + con(ictz - 1, icty, i) + con(ictz - 1, icty - 1, i);
            s.coef.push_back(2.0 / (0.25 * sg * dyk[icty] * dzk[ictz]));
        }
        out.push_back(s);
    };
    auto seg_y = [&](int iya, int iyb, int ictx, int ictz, int count, double gain) {
        SourceSegment s;
        s.comp = 1; s.i = ictx; s.j = std::min(iya, iyb); s.k = ictz;
        s.count = std::min(count, std::abs(iyb - iya) + 1);
        s.gain = gain;
        for (int q = 0; q < s.count; q++) {
            int j = s.j + q;
            double sg = ictz == 0 ? con(0, j, ictx - 1) + con(0, j, ictx)
                                  : con(ictz, j, ictx - 1) + con(ictz, j, ictx) + con(ictz - 1, j, ictx - 1) + con(ictz - 1, j, ictx);
            s.coef.push_back(2.0 / (0.25 * sg * dxk[ictx] * dzk[ictz]));
        }
        out.push_back(s);
    };
    auto seg_z = [&](int iza, int izb, int ictx, int icty, int count, double gain) {
        SourceSegment s;
        s.comp = 2; s.i = ictx; s.j = icty; s.k = std::min(iza, izb);
        s.count = std::min(count, std::abs(izb - iza) + 1);
        s.gain = gain;
        for (int q = 0; q < s.count; q++) {
            int k = s.k + q;
            double sg = con(k, icty, ictx - 1) + con(k, icty, ictx) + con(k, icty - 1, ictx - 1) + con(k, icty - 1, ictx);
            s.coef.push_back(2.0 / (0.25 * sg * dxk[ictx] * dyk[icty]));
        }
        out.push_back(s);
    };
    const double *Xp = X.data(), *Yp = Y.data(), *Zp = Z.data(), *dxp = dx.data(), *dyp = dy.data(), *dzp = dz.data();
    switch (T.ort) {
    case 1:
        seg_x(T.ixa, T.ixb, T.icty, T.ictz, std::abs(T.ixb - T.ixa) + 1,
              1.0 / (Xp[T.ixb] - Xp[T.ixa] + dxp[T.ixb] / 2 + dxp[T.ixa] / 2));
        break;
    case 2:
        seg_y(T.iya, T.iyb, T.ictx, T.ictz, std::abs(T.iyb - T.iya) + 1,
              1.0 / (Yp[T.iyb] - Yp[T.iya] + dyp[T.iyb] / 2 + dyp[T.iya] / 2));
        break;
    case 3:
        seg_z(T.iza, T.izb, T.ictx, T.icty, std::abs(T.izb - T.iza) + 1,
              1.0 / (Zp[T.izb] - Zp[T.iza] + dzp[T.izb] / 2 + dzp[T.iza] / 2));
        break;
    default: {
        double f = T.ort == 5 ? T.len : 1.0;
        seg_x(T.ixa, T.ixb, T.icty, T.ictz, std::abs(T.ixb - T.ixa) + 1,
              std::cos(T.dip) * std::cos(T.azi) * f / (std::fabs(Xp[T.ixb] - Xp[T.ixa]) + dxp[T.ixb] / 2.0 + dxp[T.ixa] / 2.0));
        seg_y(T.iya, T.iyb, T.ictx, T.ictz, std::abs(T.iyb - T.iya) + 1,
              std::cos(T.dip) * std::sin(T.azi) * f / (std::fabs(Yp[T.iyb] - Yp[T.iya]) + dyp[T.iyb] / 2.0 + dyp[T.iya] / 2.0));
        seg_z(T.iza, T.izb, T.ictx, T.icty, std::abs(T.izb - T.iza) + 1,
              std::sin(T.dip) * f / (std::fabs(Zp[T.izb] - Zp[T.iza]) + dzp[T.izb] / 2.0 + dzp[T.iza] / 2.0));
        if (T.ort == 5) {
            double gx = std::cos(T.dip1) * std::cos(T.azi1) * T.len1 /
                        (std::fabs(Xp[T.ixb1] - Xp[T.ixa1]) + dxp[T.ixb1] / 2.0 + dxp[T.ixa1] / 2.0);
            double gy = std::cos(T.dip1) * std::sin(T.azi1) * T.len1 /
                        (std::fabs(Yp[T.iyb1] - Yp[T.iya1]) + dyp[T.iyb1] / 2.0 + dyp[T.iya1] / 2.0);
            double gz = std::sin(T.dip1) * T.len1 / (std::fabs(Zp[T.izb1] - Zp[T.iza1]) + dzp[T.izb1] / 2.0 + dzp[T.iza1] / 2.0);
            if (fix_dual_bipole) {
                seg_x(T.ixa1, T.ixb1, T.icty1, T.ictz1, std::abs(T.ixb1 - T.ixa1) + 1, gx);
                seg_y(T.iya1, T.iyb1, T.ictx1, T.ictz1, std::abs(T.iyb1 - T.iya1) + 1, gy);
                seg_z(T.iza1, T.izb1, T.ictx1, T.icty1, std::abs(T.izb1 - T.iza1) + 1, gz);
            } else {  // launch width from bipole 2, cells and guard from bipole 1 (ElectricalFiled.cu:612-635)
                seg_x(T.ixa, T.ixb, T.icty, T.ictz, std::abs(T.ixb1 - T.ixa1) + 1, gx);
                seg_y(T.iya, T.iyb, T.ictx, T.ictz, std::abs(T.iyb1 - T.iya1) + 1, gy);
                seg_z(T.iza, T.izb, T.ictx, T.icty, std::abs(T.izb1 - T.iza1) + 1, gz);
            }
        }
    }
    }
    return out;
}

// Receiver stencils of Ex..BzSpatialInterp (EFInterp2Rx.cu:60-378): the 4x4x4
// natural-spline interpolation is separable and linear in the field values, so
// it is stored as node weights per axis.
std::vector<RxStencil> Model::rx_stencils(int itx) const {
    const Transmitter &T = in.tx.at(itx);
    std::vector<RxStencil> out;
    auto half = [](const std::vector<double> &c, const std::vector<double> &d, int idx, double pos) {
        return (c[idx - 1] + 0.5 * d[idx - 1]) > pos ? idx - 2 : idx - 1;
    };
    auto weights = [](const double *nodes, double t, double *w) {
        for (int q = 0; q < 4; q++) {
            double e[4] = {0, 0, 0, 0};
            e[q] = 1.0;
            w[q] = spline4(nodes, e, t);
        }
    };
    for (int comp = 0; comp < 6; comp++) {
        if (!in.isComp[comp]) continue;
        for (int r = 0; r < T.nr; r++) {
            int ir = T.rx[r] - 1;
            double px = in.rx[ir], py = in.ry[ir], pz = in.rz[ir];
            int ix = rix[ir], iy = riy[ir], iz = riz[ir];
            // stagger of component comp: x-face (Ey,Ez,Bx), y-face (Ex,Ez,By), z-face (Ex,Ey,Bz)
            bool xf = comp == 1 || comp == 2 || comp == 3;
            bool yf = comp == 0 || comp == 2 || comp == 4;
            bool zf = comp == 0 || comp == 1 || comp == 5;
            RxStencil s;
            s.comp = comp;
            s.s1 = xf ? half(X, dx, ix, px) : ix - 2;
            s.s2 = yf ? half(Y, dy, iy, py) : iy - 2;
            int s3 = zf ? (iz >= 1 ? half(Z, dz, iz, pz) : -1) : iz - 2;
            s.s3 = std::max(s3, 0);
            double xn[4], yn[4], zn[4];
            for (int q = 0; q < 4; q++) {
                xn[q] = xf ? X[s.s1 + q] - 0.5 * dx[s.s1 + q] : X[s.s1 + q];
                yn[q] = yf ? Y[s.s2 + q] - 0.5 * dy[s.s2 + q] : Y[s.s2 + q];
                zn[q] = zf ? Z[s.s3 + q] - 0.5 * dz[s.s3 + q] : Z[s.s3 + q];
            }
            weights(xn, px, s.wx);
            weights(yn, py, s.wy);
            weights(zn, pz, s.wz);
            out.push_back(s);
        }
    }
    return out;
}

}  // namespace tcsem
