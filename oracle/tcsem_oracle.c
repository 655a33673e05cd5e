#define _GNU_SOURCE
/*
 * tcsem_oracle.c -- FP64 CPU restatement of the TCSEM_FDTD time-stepping path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA product is
 * checked against.  It is loaded by the tests, by __graft_entry__.smoke() and by
 * the CPU-baseline leg of bench.py -- never by the product library.
 *
 * Pinning: the setup half (grid, index maps, receiver/transmitter location,
 * source waveform, sampling times) is checked bit-exactly against fixtures that
 * the reference's own host code produced (tests/golden, written by
 * tests/golden/gen_ref_host_golden.py with the program oracle/build_ref.py
 * compiles from ModelingSetup.cpp, ModelGridMapping.cpp, LoadRxTxPos.cpp,
 * SourceWave.cpp, logspace.cpp), and Waveform() against the
 * reference's shipped testwaveform.dat.  The device half (E/B update, source
 * injection, spline remap, continuation, receiver interpolation) restates the
 * reference's CUDA kernels line by line; each function cites the kernel it
 * follows.
 *
 * Everything is double precision, reference array layout:
 *   Ex[N+1][M+1][L]  Ey[N+1][M][L+1]  Ez[N][M+1][L+1]
 *   Bx[N][M][L+1]    By[N][M+1][L]    Bz[N+1][M][L]    Con[N][M][L]
 *   BxAir[M][L+1]    ByAir[M+1][L]
 * (FTDT.h:62-74, prepare_free_mem.cu:63-81).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <complex.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.141592653589793238 /* FTDT.h:39 */
#define ORC_NPAD 4                 /* FTDT.h:40 */

typedef double complex cplx;

typedef struct {
    int ort, nr;
    double BipoLen, x, y, z, azi, dip;
    int ixa, iya, iza, ixb, iyb, izb, ictx, icty, ictz;
    double BipoLen1, x1, y1, z1, azi1, dip1;
    int ixa1, iya1, iza1, ixb1, iyb1, izb1, ictx1, icty1, ictz1;
    int *rxnum; /* 1-based receiver ids */
} orc_tx;

typedef struct {
    /* FDTD_setup.in (ModelingSetup.cpp:51-59) */
    double sfa1, sfa2, sita_t, x0, y0, z0, dxmin, dymin, dzmin, arg1, arg2;
    int n1, nsrc;
    int ALx2, ALx1, Nx, ARx1, ARx2, Ay2, Ay1, Ny, Az2, Az1, Nz;
    int L, M, N, AnLx_New, AnRx_New, Any_New, L1, M1;
    double minsita, mu0, mindx;
    /* host grid (ModelingSetup.cpp:100-187, ModelGridMapping.cpp) */
    double *dx, *dy, *dz, *X, *Y, *Z, *Xn, *Yn;
    /* cell sizes as the kernels recompute them (ElectricalFiled.cu:36-86) */
    double *dxk, *dyk, *dzk;
    int *xBzNew2old, *yBzNew2old, *xBzold2New, *yBzold2New, *xoldBx2NewBz, *yoldBy2NewBz;
    double *con;
    /* source waveform (SourceWave.cpp) */
    double *tw, *dtw, *wave;
    /* Receiver.in / Transmitter.in (LoadRxTxPos.cpp) */
    double T0, Tn;
    int Nt, IsLog, isComp[6], NComp, nefcmp;
    double *times;
    int NRx, NTx;
    double *rx, *ry, *rz;
    int *rix, *riy, *riz;
    orc_tx *tx;
    /* fields */
    double *Ex, *Ey, *Ez, *Bx, *By, *Bz, *BxAir, *ByAir;
    /* boundary scratch */
    double *BzAir, *FBxR, *FByR;
    cplx *FBzC, *FBxC, *FByC;
    double *semi_x00, *semi_x01, *semi_x10, *semi_x11;
    /* receiver slots ef0[2][NComp][nr] and traces efs[nr][NComp][Nt] */
    double *ef0, *efs;
    int cur_tx;
    int bug_compat_dual_bipole; /* D3: second bipole injected at the first bipole's cells */
    int padded_plane;           /* the time loop uses orc_upcontinuation_padded */
    char err[256];
} orc_sim;

static double *dalloc(size_t n) { return (double *)calloc(n ? n : 1, sizeof(double)); }
static int *ialloc(size_t n) { return (int *)calloc(n ? n : 1, sizeof(int)); }

/* ---------------------------------------------------------------- helpers */

/* logspace.cpp:5-19 (pow10 == exp10) */
static void orc_logspace(double *a, double b, double e, int n) {
    double step = (log10(e) - log10(b)) / (n - 1);
    for (int i = 0; i < n; i++) a[i] = exp10(log10(b) + i * step);
}
/* logspace.cpp:20-28 */
static void orc_linspace(double *a, double b, double e, int n) {
    double step = (e - b) / (n - 1);
    for (int i = 0; i < n; i++) a[i] = b + i * step;
}
/* logspace.cpp:30-66: binary search for the insertion position */
static int orc_search_insert(const double *A, int n, double target) {
    if (n < 1) return 0;
    int low = 0, high = n - 1, mid, pos = 0;
    while (low <= high) {
        mid = low + (high - low) / 2;
        if (A[mid] == target) return mid;
        if (A[mid] > target) { high = mid - 1; pos = mid; }
        else { low = mid + 1; pos = mid + 1; }
    }
    return pos;
}

/* SourceWave.cpp:8-58.  dt[2N] is read before it is written in the reference
 * (uninitialised heap memory); the shipped testwaveform.dat equals the value
 * obtained with 0 there, which is what is used here. */
static void orc_waveform(int N, double s, double *t, double *dt, double *wave) {
    t[0] = 0;
    for (int i = 0; i < N; i++) {
        double t0 = t[i] - 3 * s;
        dt[i] = -s * s * (1 - exp(-4.5)) / N / t0 / exp(-t0 * t0 / (2 * s * s));
        t[i + 1] = t[i] + dt[i];
    }
    if (3 * s < t[N]) t[N] = 3 * s;
    for (int i = N + 1; i < 2 * N + 1; i++) {
        t[i] = 6 * s - t[2 * N - i];
        dt[i - 1] = t[i] - t[i - 1];
    }
    dt[2 * N] = 0.0;
    for (int i = 0; i < 2 * N + 1; i++)
        wave[i] = 1 / (sqrt(2 * ORC_PI) * s) * exp(-(t[i] - 3 * s) * (t[i] - 3 * s) / 2 / s / s);
    dt[2 * N + 1] = 0.5 * (dt[2 * N] * dt[2 * N] / dt[2 * N - 1] + dt[2 * N]);
    double t0 = dt[0], t1;
    dt[0] = 0.5 * (t0 * t0 / dt[1] + t0);
    for (int i = 1; i < 2 * N + 1; i++) {
        t1 = dt[i];
        dt[i] = 0.5 * (t0 + dt[i]);
        t0 = t1;
    }
}

/* ------------------------------------------------------------------ setup */

static int read_setup(orc_sim *S, const char *dir) {
    char path[1024];
    snprintf(path, sizeof path, "%s/FDTD_setup.in", dir);
    FILE *f = fopen(path, "r");
    if (!f) { snprintf(S->err, sizeof S->err, "cannot open %s", path); return 1; }
    int ok = 1;
    ok &= fscanf(f, "%lf %lf\n", &S->sfa1, &S->sfa2) == 2;
    ok &= fscanf(f, "%d %lf\n", &S->n1, &S->sita_t) == 2;
    ok &= fscanf(f, "%lf %lf %lf\n", &S->x0, &S->y0, &S->z0) == 3;
    ok &= fscanf(f, "%lf %lf %lf\n", &S->dxmin, &S->dymin, &S->dzmin) == 3;
    ok &= fscanf(f, "%lf %lf\n", &S->arg1, &S->arg2) == 2;
    ok &= fscanf(f, "%d %d %d %d %d\n", &S->ALx2, &S->ALx1, &S->Nx, &S->ARx1, &S->ARx2) == 5;
    ok &= fscanf(f, "%d %d %d\n", &S->Ay2, &S->Ay1, &S->Ny) == 3;
    ok &= fscanf(f, "%d %d %d\n", &S->Az2, &S->Az1, &S->Nz) == 3;
    fclose(f);
    if (!ok) { snprintf(S->err, sizeof S->err, "malformed FDTD_setup.in"); return 1; }
    S->nsrc = S->n1 / 2;
    return 0;
}

/* ModelingSetup.cpp:79-195 */
static void build_grid(orc_sim *S) {
    int L = S->ALx2 + S->ALx1 + S->ARx2 + S->ARx1 + S->Nx;
    int M = 2 * (S->Ay2 + S->Ay1) + S->Ny;
    int N = S->Nz + S->Az2 + S->Az1;
    S->L = L; S->M = M; S->N = N;
    S->dx = dalloc(L); S->dy = dalloc(M); S->dz = dalloc(N);
    S->X = dalloc(L); S->Y = dalloc(M); S->Z = dalloc(N);
    int AL = S->ALx2 + S->ALx1;
    for (int i = AL; i < S->Nx + AL; i++) S->dx[i] = S->dxmin;
    for (int i = AL - 1; i >= S->ALx2; i--) S->dx[i] = S->dxmin * pow(S->arg1, (double)(S->ALx1 + S->ALx2 - i));
    for (int i = S->ALx2 - 1; i >= 0; i--)
        S->dx[i] = S->dxmin * pow(S->arg1, (double)S->ALx1) * pow(S->arg2, (double)(S->ALx2 - i));
    for (int i = S->Nx + AL; i < S->Nx + AL + S->ARx1; i++)
        S->dx[i] = S->dxmin * pow(S->arg1, (double)(i - S->ALx1 - S->ALx2 - S->Nx + 1));
    for (int i = S->Nx + AL + S->ARx1; i < L; i++)
        S->dx[i] = S->dxmin * pow(S->arg1, (double)S->ARx1) * pow(S->arg2, (double)(i - S->Nx - AL - S->ARx1 + 1));
    int Ay = S->Ay2 + S->Ay1;
    for (int j = Ay; j < S->Ny + Ay; j++) S->dy[j] = S->dymin;
    for (int j = Ay - 1; j >= S->Ay2; j--) S->dy[j] = S->dy[j + 1] * S->arg1;
    for (int j = S->Ay2 - 1; j >= 0; j--) S->dy[j] = S->dy[j + 1] * S->arg2;
    for (int j = S->Ny + Ay; j < S->Ny + S->Ay2 + 2 * S->Ay1; j++) S->dy[j] = S->dy[j - 1] * S->arg1;
    for (int j = S->Ny + S->Ay2 + 2 * S->Ay1; j < M; j++) S->dy[j] = S->dy[j - 1] * S->arg2;
    for (int k = 0; k < S->Nz; k++) S->dz[k] = S->dzmin;
    for (int k = S->Nz; k < S->Nz + S->Az1; k++) S->dz[k] = S->dz[k - 1] * S->arg1;
    for (int k = S->Nz + S->Az1; k < N; k++) S->dz[k] = S->dz[k - 1] * S->arg2;
    int nc;
    if (S->Nx % 2 == 0) { nc = S->Nx / 2 + AL; S->X[nc] = 0.5 * S->dx[nc] + S->x0; }
    else { nc = (S->Nx - 1) / 2 + AL; S->X[nc] = S->x0; }
    for (int i = nc + 1; i < L; i++) S->X[i] = S->X[i - 1] + 0.5 * S->dx[i - 1] + 0.5 * S->dx[i];
    for (int i = nc - 1; i >= 0; i--) S->X[i] = S->X[i + 1] - 0.5 * S->dx[i + 1] - 0.5 * S->dx[i];
    if (S->Ny % 2 == 0) { nc = S->Ny / 2 + Ay; S->Y[nc] = 0.5 * S->dy[nc] + S->y0; }
    else { nc = (S->Ny - 1) / 2 + Ay; S->Y[nc] = S->y0; }
    for (int j = nc + 1; j < M; j++) S->Y[j] = S->Y[j - 1] + 0.5 * S->dy[j - 1] + 0.5 * S->dy[j];
    for (int j = nc - 1; j >= 0; j--) S->Y[j] = S->Y[j + 1] - 0.5 * S->dy[j + 1] - 0.5 * S->dy[j];
    S->Z[0] = 0.5 * S->dz[0] + S->z0;
    for (int k = 1; k < N; k++) S->Z[k] = S->Z[k - 1] + 0.5 * S->dz[k - 1] + 0.5 * S->dz[k];
    S->AnLx_New = (int)ceil((S->X[AL - 1] - S->X[0] + S->dx[AL - 1] / 2 + S->dx[0] / 2) / S->dxmin);
    int AR0 = L - S->ARx1 - S->ARx2;
    S->AnRx_New = (int)ceil((S->X[L - 1] - S->X[AR0] + S->dx[L - 1] / 2 + S->dx[AR0] / 2) / S->dxmin);
    S->Any_New = (int)ceil((S->Y[Ay - 1] - S->Y[0] + S->dy[Ay - 1] / 2 + S->dy[0] / 2) / S->dymin);
    S->L1 = S->AnLx_New + S->AnRx_New + S->Nx;
    S->M1 = 2 * S->Any_New + S->Ny;

    /* Grid_dx/Grid_dy/Grid_dz as the kernels evaluate them (ElectricalFiled.cu:36-86) */
    S->dxk = dalloc(L); S->dyk = dalloc(M); S->dzk = dalloc(N);
    for (int i = 0; i < L; i++) {
        double d;
        if (i >= S->ALx2 + S->ALx1 && i < S->Nx + S->ALx1 + S->ALx2) d = S->dxmin;
        else if (i >= S->ALx2 && i < S->ALx2 + S->ALx1) d = S->dxmin * pow(S->arg1, (double)(S->ALx2 + S->ALx1 - i));
        else if (i < S->ALx2) d = S->dxmin * pow(S->arg1, (double)S->ALx1) * pow(S->arg2, (double)(S->ALx2 - i));
        else if (i >= S->Nx + S->ALx1 + S->ALx2 && i < S->Nx + S->ARx1 + S->ALx1 + S->ALx2)
            d = S->dxmin * pow(S->arg1, (double)(i - S->Nx - S->ALx1 - S->ALx2 + 1));
        else d = S->dxmin * pow(S->arg1, (double)S->ARx1) * pow(S->arg2, (double)(i - S->Nx - S->ARx1 - S->ALx1 - S->ALx2 + 1));
        S->dxk[i] = d;
    }
    for (int j = 0; j < M; j++) {
        double d;
        if (j >= S->Ay2 + S->Ay1 && j < S->Ny + S->Ay1 + S->Ay2) d = S->dymin;
        else if (j >= S->Ay2 && j < S->Ay2 + S->Ay1) d = S->dymin * pow(S->arg1, (double)(S->Ay2 + S->Ay1 - j));
        else if (j < S->Ay2) d = S->dymin * pow(S->arg1, (double)S->Ay1) * pow(S->arg2, (double)(S->Ay2 - j));
        else if (j >= S->Ny + S->Ay1 + S->Ay2 && j < S->Ny + 2 * S->Ay1 + S->Ay2)
            d = S->dymin * pow(S->arg1, (double)(j - S->Ny - S->Ay1 - S->Ay2 + 1));
        else d = S->dymin * pow(S->arg1, (double)S->Ay1) * pow(S->arg2, (double)(j - S->Ny - 2 * S->Ay1 - S->Ay2 + 1));
        S->dyk[j] = d;
    }
    for (int k = 0; k < N; k++) {
        double d;
        if (k < S->Nz) d = S->dzmin;
        else if (k < S->Nz + S->Az1) d = S->dzmin * pow(S->arg1, (double)(k - S->Nz + 1));
        else d = S->dzmin * pow(S->arg1, (double)S->Az1) * pow(S->arg2, (double)(k - S->Nz - S->Az1 + 1));
        S->dzk[k] = d;
    }
}

/* ModelGridMapping.cpp:13-395 */
static void build_mapping(orc_sim *S) {
    int L0 = S->L, M0 = S->M, L1 = S->L1, M1 = S->M1;
    int AnLx = S->ALx1 + S->ALx2, Nx = S->Nx, Any = S->Ay1 + S->Ay2, Ny = S->Ny;
    double *Xo = S->X, *Yo = S->Y, *dx = S->dx, *dy = S->dy;
    S->Xn = dalloc(L1); S->Yn = dalloc(M1);
    double *Xn = S->Xn, *Yn = S->Yn;
    for (int i = S->AnLx_New; i < S->AnLx_New + Nx; i++) Xn[i] = Xo[i - S->AnLx_New + AnLx];
    for (int i = S->AnLx_New - 1; i >= 0; i--) Xn[i] = Xn[i + 1] - S->dxmin;
    for (int i = S->AnLx_New + Nx; i < L1; i++) Xn[i] = Xn[i - 1] + S->dxmin;
    for (int j = S->Any_New; j < S->Any_New + Ny; j++) Yn[j] = Yo[j - S->Any_New + Any];
    for (int j = S->Any_New - 1; j >= 0; j--) Yn[j] = Yn[j + 1] - S->dymin;
    for (int j = S->Any_New + Ny; j < M1; j++) Yn[j] = Yn[j - 1] + S->dymin;

    int *a = S->xBzNew2old = ialloc(L1);
    for (int i = S->AnLx_New; i < S->AnLx_New + Nx; i++) a[i] = i - S->AnLx_New + AnLx;
    for (int i = S->AnLx_New - 1; i >= 0; i--) {
        int j = a[i + 1];
        while (j > 0 && Xo[j - 1] >= Xn[i]) j--;
        a[i] = j;
    }
    for (int i = S->AnLx_New + Nx; i < L1; i++) {
        int j = a[i - 1] - 1;
        while (j < L0 - 1 && Xo[j + 1] < Xn[i]) j++;
        a[i] = j + 1;
    }
    a = S->yBzNew2old = ialloc(M1);
    for (int j = S->Any_New; j < S->Any_New + Ny; j++) a[j] = j - S->Any_New + Any;
    for (int j = S->Any_New - 1; j >= 0; j--) {
        int i = a[j + 1];
        while (i > 0 && Yo[i - 1] >= Yn[j]) i--;
        a[j] = i;
    }
    for (int j = S->Any_New + Ny; j < M1; j++) {
        int i = a[j - 1] - 1;
        while (i < M0 - 1 && Yo[i + 1] < Yn[j]) i++;
        a[j] = i + 1;
    }
    a = S->xBzold2New = ialloc(L0);
    for (int i = AnLx; i < AnLx + Nx; i++) a[i] = i - AnLx + S->AnLx_New;
    for (int i = AnLx - 1; i >= 0; i--) {
        int j = a[i + 1];
        while (j > 0 && Xn[j - 1] >= Xo[i]) j--;
        a[i] = j;
    }
    for (int i = AnLx + Nx; i < L0; i++) {
        int j = a[i - 1];
        while (j < L1 - 1 && Xn[j + 1] < Xo[i]) j++;
        a[i] = j + 1;
    }
    a = S->yBzold2New = ialloc(M0);
    for (int j = Any; j < Any + Ny; j++) a[j] = j - Any + S->Any_New;
    for (int j = Any - 1; j >= 0; j--) {
        int i = a[j + 1];
        while (i > 0 && Yn[i - 1] >= Yo[j]) i--;
        a[j] = i;
    }
    for (int j = Any + Ny; j < M0; j++) {
        int i = a[j - 1];
        while (i < M1 - 1 && Yn[i + 1] < Yo[j]) i++;
        a[j] = i + 1;
    }
    a = S->xoldBx2NewBz = ialloc(L0 + 1);
    for (int i = AnLx; i < AnLx + Nx; i++) a[i] = i - AnLx + S->AnLx_New;
    for (int i = AnLx - 1; i >= 0; i--) {
        int j = a[i + 1];
        while (j > 0 && Xn[j - 1] >= Xo[i] - 0.5 * dx[i]) j--;
        a[i] = j;
    }
    for (int i = AnLx + Nx; i < L0; i++) {
        int j = a[i - 1];
        while (j < L1 - 1 && Xn[j + 1] < Xo[i] - 0.5 * dx[i]) j++;
        a[i] = j + 1;
    }
    {
        int i = L0, j = a[i - 1];
        while (j < L1 - 1 && Xn[j + 1] < Xo[i - 1] + 0.5 * dx[i - 1]) j++;
        a[i] = j + 1;
    }
    a = S->yoldBy2NewBz = ialloc(M0 + 1);
    for (int j = Any; j < Any + Ny; j++) a[j] = j - Any + S->Any_New;
    for (int j = Any - 1; j >= 0; j--) {
        int i = a[j + 1];
        while (i > 0 && Yn[i - 1] >= Yo[j] - 0.5 * dy[j]) i--;
        a[j] = i;
    }
    for (int j = Any + Ny; j < M0; j++) {
        int i = a[j - 1];
        while (i < M1 - 1 && Yn[i + 1] < Yo[j] - 0.5 * dy[j]) i++;
        a[j] = i + 1;
    }
    {
        int j = M0, i = a[j - 1];
        while (i < M1 - 1 && Yn[i + 1] < Yo[j - 1] + 0.5 * dy[j - 1]) i++;
        a[j] = i + 1;
    }
}

/* Tx location rules of LoadRxTxPos.cpp:203-453 */
static void adj_pair(int *a, int *b) {
    if (*b > *a) (*b)--;
    else if (*b < *a) (*a)--;
}
static int locate_tx(orc_sim *S, orc_tx *T) {
    int L = S->L, M = S->M, K = S->N;
    const double *X = S->X, *Y = S->Y, *Z = S->Z;
    switch (T->ort) {
    case 1:
        T->ixa = orc_search_insert(X, L, T->x - T->BipoLen / 2);
        T->ixb = orc_search_insert(X, L, T->x + T->BipoLen / 2) - 1;
        if (T->ixa == 0 || T->ixb == L) return 1;
        T->icty = orc_search_insert(Y, M, T->y);
        if (T->icty == 0 || T->icty == M) return 1;
        T->ictz = orc_search_insert(Z, K, T->z);
        break;
    case 2:
        T->ictx = orc_search_insert(X, L, T->x);
        if (T->ictx == 0 || T->ictx == L) return 1;
        T->iya = orc_search_insert(Y, M, T->y - T->BipoLen / 2);
        T->iyb = orc_search_insert(Y, M, T->y + T->BipoLen / 2) - 1;
        if (T->iya == 0 || T->iyb == M) return 1;
        T->ictz = orc_search_insert(Z, K, T->z);
        break;
    case 3:
        T->ictx = orc_search_insert(X, L, T->x);
        if (T->ictx == 0 || T->ictx == L) return 1;
        T->icty = orc_search_insert(Y, M, T->y);
        if (T->icty == 0 || T->icty == M) return 1;
        T->iza = orc_search_insert(Z, K, T->z - T->BipoLen / 2);
        T->izb = orc_search_insert(Z, K, T->z + T->BipoLen / 2) - 1;
        break;
    case 4:
    case 5: {
        double cd = cos(T->dip), ca = cos(T->azi), sa = sin(T->azi), sd = sin(T->dip);
        T->ixa = orc_search_insert(X, L, T->x - T->BipoLen * cd * ca / 2.0);
        T->ixb = orc_search_insert(X, L, T->x + T->BipoLen * cd * ca / 2.0);
        adj_pair(&T->ixa, &T->ixb);
        if (T->ort == 5) {
            double cd1 = cos(T->dip1), ca1 = cos(T->azi1);
            T->ixa1 = orc_search_insert(X, L, T->x1 - T->BipoLen1 * cd1 * ca1 / 2.0);
            T->ixb1 = orc_search_insert(X, L, T->x1 + T->BipoLen1 * cd1 * ca1 / 2.0);
            adj_pair(&T->ixa1, &T->ixb1);
            if (T->ixa1 == 0 || T->ixb1 == L) return 1;
        }
        if (T->ixa == 0 || T->ixb == L) return 1;
        T->iya = orc_search_insert(Y, M, T->y - T->BipoLen * cd * sa / 2.0);
        T->iyb = orc_search_insert(Y, M, T->y + T->BipoLen * cd * sa / 2.0);
        adj_pair(&T->iya, &T->iyb);
        if (T->ort == 5) {
            double cd1 = cos(T->dip1), sa1 = sin(T->azi1);
            T->iya1 = orc_search_insert(Y, M, T->y1 - T->BipoLen1 * cd1 * sa1 / 2.0);
            T->iyb1 = orc_search_insert(Y, M, T->y1 + T->BipoLen1 * cd1 * sa1 / 2.0);
            adj_pair(&T->iya1, &T->iyb1);
            if (T->iya1 == 0 || T->iyb1 == M) return 1;
        }
        if (T->iya == 0 || T->iyb == M) return 1;
        T->iza = orc_search_insert(Z, K, T->z - T->BipoLen * sd / 2.0);
        T->izb = orc_search_insert(Z, K, T->z + T->BipoLen * sd / 2.0);
        adj_pair(&T->iza, &T->izb);
        if (T->ort == 5) {
            double sd1 = sin(T->dip1);
            T->iza1 = orc_search_insert(Z, K, T->z1 - T->BipoLen1 * sd1 / 2.0);
            T->izb1 = orc_search_insert(Z, K, T->z1 + T->BipoLen1 * sd1 / 2.0);
            adj_pair(&T->iza1, &T->izb1);
            T->ictx1 = orc_search_insert(X, L, T->x1);
            T->icty1 = orc_search_insert(Y, M, T->y1);
            T->ictz1 = orc_search_insert(Z, K, T->z1);
        }
        T->ictx = orc_search_insert(X, L, T->x);
        T->icty = orc_search_insert(Y, M, T->y);
        T->ictz = orc_search_insert(Z, K, T->z);
        break;
    }
    default:
        return 1;
    }
    return 0;
}

static int read_rx_tx(orc_sim *S, const char *dir) {
    char path[1024];
    snprintf(path, sizeof path, "%s/Receiver.in", dir);
    FILE *f = fopen(path, "r");
    if (!f) { snprintf(S->err, sizeof S->err, "cannot open %s", path); return 1; }
    int ok = 1;
    ok &= fscanf(f, "%lf %lf\n", &S->T0, &S->Tn) == 2;
    ok &= fscanf(f, "%d %d\n", &S->Nt, &S->IsLog) == 2;
    ok &= fscanf(f, "%d %d %d %d %d %d\n", &S->isComp[0], &S->isComp[1], &S->isComp[2], &S->isComp[3], &S->isComp[4],
                 &S->isComp[5]) == 6;
    ok &= fscanf(f, "%d\n", &S->NRx) == 1;
    if (!ok || S->NRx < 1) { fclose(f); snprintf(S->err, sizeof S->err, "malformed Receiver.in"); return 1; }
    S->rx = dalloc(S->NRx); S->ry = dalloc(S->NRx); S->rz = dalloc(S->NRx);
    S->rix = ialloc(S->NRx); S->riy = ialloc(S->NRx); S->riz = ialloc(S->NRx);
    for (int r = 0; r < S->NRx; r++) {
        int id; double x, y, z;
        if (fscanf(f, "%d %lf %lf %lf\n", &id, &x, &y, &z) != 4 || id < 1 || id > S->NRx) {
            fclose(f); snprintf(S->err, sizeof S->err, "bad receiver line %d", r + 1); return 1;
        }
        S->rx[id - 1] = x; S->ry[id - 1] = y; S->rz[id - 1] = z;
    }
    fclose(f);
    for (int r = 0; r < S->NRx; r++) {
        int n = orc_search_insert(S->X, S->L, S->rx[r]);
        if (n == 0 || n == S->L) { snprintf(S->err, sizeof S->err, "receiver %d outside x", r + 1); return 1; }
        S->rix[r] = n;
        n = orc_search_insert(S->Y, S->M, S->ry[r]);
        if (n == 0 || n == S->M) { snprintf(S->err, sizeof S->err, "receiver %d outside y", r + 1); return 1; }
        S->riy[r] = n;
        S->riz[r] = orc_search_insert(S->Z, S->N, S->rz[r]);
        /* the 4-point stencils of EFInterp2Rx.cu read nodes ix-2..ix+1 (y, z
         * alike); the reference does not check this and reads out of bounds */
        if (S->rix[r] < 2 || S->rix[r] > S->L - 3 || S->riy[r] < 2 || S->riy[r] > S->M - 3 || S->riz[r] > S->N - 3) {
            snprintf(S->err, sizeof S->err, "receiver %d too close to the model edge", r + 1);
            return 1;
        }
    }
    snprintf(path, sizeof path, "%s/Transmitter.in", dir);
    f = fopen(path, "r");
    if (!f) { snprintf(S->err, sizeof S->err, "cannot open %s", path); return 1; }
    if (fscanf(f, "%d\n", &S->NTx) != 1 || S->NTx < 1) { fclose(f); snprintf(S->err, sizeof S->err, "bad Transmitter.in"); return 1; }
    S->tx = (orc_tx *)calloc(S->NTx, sizeof(orc_tx));
    for (int t = 0; t < S->NTx; t++) {
        int id, ort;
        if (fscanf(f, "%d %d", &id, &ort) != 2 || id < 1 || id > S->NTx) {
            fclose(f); snprintf(S->err, sizeof S->err, "bad transmitter line"); return 1;
        }
        orc_tx *T = &S->tx[id - 1];
        T->ort = ort;
        double azi, dip;
        if (ort < 4) {
            ok = fscanf(f, " %lf %lf %lf %lf %d", &T->BipoLen, &T->x, &T->y, &T->z, &T->nr) == 5;
        } else if (ort == 4) {
            ok = fscanf(f, " %lf %lf %lf %lf %lf %lf %d", &T->BipoLen, &T->x, &T->y, &T->z, &azi, &dip, &T->nr) == 7;
            T->azi = azi * ORC_PI / 180.0; T->dip = dip * ORC_PI / 180.0;
        } else if (ort == 5) {
            ok = fscanf(f, " %lf %lf %lf %lf %lf %lf", &T->BipoLen, &T->x, &T->y, &T->z, &azi, &dip) == 6;
            T->azi = azi * ORC_PI / 180.0; T->dip = dip * ORC_PI / 180.0;
            ok &= fscanf(f, " %lf %lf %lf %lf %lf %lf %d", &T->BipoLen1, &T->x1, &T->y1, &T->z1, &azi, &dip, &T->nr) == 7;
            T->azi1 = azi * ORC_PI / 180.0; T->dip1 = dip * ORC_PI / 180.0;
        } else ok = 0;
        if (!ok || T->nr < 1) { fclose(f); snprintf(S->err, sizeof S->err, "bad transmitter %d", id); return 1; }
        T->rxnum = ialloc(T->nr);
        for (int r = 0; r < T->nr; r++) {
            if (fscanf(f, " %d", &T->rxnum[r]) != 1 || T->rxnum[r] < 1 || T->rxnum[r] > S->NRx) {
                fclose(f); snprintf(S->err, sizeof S->err, "bad receiver id in transmitter %d", id); return 1;
            }
        }
    }
    fclose(f);
    for (int t = 0; t < S->NTx; t++)
        if (locate_tx(S, &S->tx[t])) { snprintf(S->err, sizeof S->err, "transmitter %d outside model", t + 1); return 1; }
    S->times = dalloc(S->Nt);
    if (S->IsLog) orc_logspace(S->times, S->T0, S->Tn, S->Nt);
    else orc_linspace(S->times, S->T0, S->Tn, S->Nt);
    S->NComp = 0; S->nefcmp = 0;
    for (int c = 0; c < 6; c++) if (S->isComp[c]) S->NComp++;
    for (int c = 0; c < 3; c++) if (S->isComp[c]) S->nefcmp++;
    return 0;
}

/* ------------------------------------------------------------ field index */
#define EXI(S, k, j, i) ((((size_t)(k)) * ((S)->M + 1) + (j)) * (S)->L + (i))
#define EYI(S, k, j, i) ((((size_t)(k)) * ((S)->M) + (j)) * ((S)->L + 1) + (i))
#define EZI(S, k, j, i) ((((size_t)(k)) * ((S)->M + 1) + (j)) * ((S)->L + 1) + (i))
#define BXI(S, k, j, i) ((((size_t)(k)) * ((S)->M) + (j)) * ((S)->L + 1) + (i))
#define BYI(S, k, j, i) ((((size_t)(k)) * ((S)->M + 1) + (j)) * (S)->L + (i))
#define BZI(S, k, j, i) ((((size_t)(k)) * ((S)->M) + (j)) * (S)->L + (i))
#define CI(S, k, j, i) ((((size_t)(k)) * ((S)->M) + (j)) * (S)->L + (i))

size_t orc_field_size(const orc_sim *S, int comp) {
    size_t L = S->L, M = S->M, N = S->N;
    switch (comp) {
    case 0: return L * (M + 1) * (N + 1);
    case 1: return (L + 1) * M * (N + 1);
    case 2: return (L + 1) * (M + 1) * N;
    case 3: return (L + 1) * M * N;
    case 4: return L * (M + 1) * N;
    case 5: return L * M * (N + 1);
    case 6: return (L + 1) * M;       /* BxAir */
    case 7: return L * (M + 1);       /* ByAir */
    case 8: return L * M * N;         /* Con */
    case 9: return (size_t)S->L1 * S->M1; /* BzAir */
    }
    return 0;
}
static double *field_ptr(orc_sim *S, int comp) {
    switch (comp) {
    case 0: return S->Ex; case 1: return S->Ey; case 2: return S->Ez;
    case 3: return S->Bx; case 4: return S->By; case 5: return S->Bz;
    case 6: return S->BxAir; case 7: return S->ByAir; case 8: return S->con; case 9: return S->BzAir;
    }
    return NULL;
}

/* -------------------------------------------------------------- public API */

void orc_free(orc_sim *S);

static void alloc_state(orc_sim *S) {
    S->Ex = dalloc(orc_field_size(S, 0)); S->Ey = dalloc(orc_field_size(S, 1)); S->Ez = dalloc(orc_field_size(S, 2));
    S->Bx = dalloc(orc_field_size(S, 3)); S->By = dalloc(orc_field_size(S, 4)); S->Bz = dalloc(orc_field_size(S, 5));
    S->BxAir = dalloc(orc_field_size(S, 6)); S->ByAir = dalloc(orc_field_size(S, 7));
    size_t P = (size_t)S->L1 * S->M1, H = (size_t)S->M1 * (S->L1 / 2 + 1);
    S->BzAir = dalloc(P); S->FBxR = dalloc(P); S->FByR = dalloc(P);
    S->FBzC = (cplx *)calloc(H, sizeof(cplx)); S->FBxC = (cplx *)calloc(H, sizeof(cplx)); S->FByC = (cplx *)calloc(H, sizeof(cplx));
    int n3 = S->Ay1 + S->Ay2 + ORC_NPAD;
    S->semi_x00 = dalloc((size_t)S->AnLx_New * n3); S->semi_x01 = dalloc((size_t)S->AnLx_New * n3);
    S->semi_x10 = dalloc((size_t)S->AnRx_New * n3); S->semi_x11 = dalloc((size_t)S->AnRx_New * n3);
}

/* ModelingSetup + Waveform + ModelGridMapping + LoadRxTxPos, in the order of
 * main.cu:93-146.  Returns NULL and fills errbuf on failure. */
orc_sim *orc_open(const char *dir, char *errbuf, int errlen) {
    orc_sim *S = (orc_sim *)calloc(1, sizeof(orc_sim));
    S->bug_compat_dual_bipole = 1;
    if (read_setup(S, dir)) goto fail;
    if (S->Nx < 1 || S->Ny < 1 || S->Nz < 1 || S->dxmin <= 0 || S->dymin <= 0 || S->dzmin <= 0 ||
        S->ALx1 + S->ALx2 < 1 || S->ARx1 + S->ARx2 < 1 || S->Ay1 + S->Ay2 < 1 || S->nsrc < 1) {
        snprintf(S->err, sizeof S->err, "unsupported grid split");
        goto fail;
    }
    if (S->ALx1 + S->ALx2 + ORC_NPAD > 128 || S->ARx1 + S->ARx2 + ORC_NPAD > 128 || S->Ay1 + S->Ay2 + ORC_NPAD > 128) {
        /* initialize_UpCont_gpu_resources.cu:138 */
        snprintf(S->err, sizeof S->err, "boundary strip wider than 124 cells");
        goto fail;
    }
    build_grid(S);
    {
        char path[1024];
        snprintf(path, sizeof path, "%s/Cond.bin", dir);
        FILE *f = fopen(path, "rb");
        if (!f) { snprintf(S->err, sizeof S->err, "cannot open %s", path); goto fail; }
        size_t n = (size_t)S->N * S->M * S->L;
        S->con = dalloc(n);
        if (fread(S->con, sizeof(double), n, f) != n) { fclose(f); snprintf(S->err, sizeof S->err, "short Cond.bin"); goto fail; }
        fclose(f);
    }
    S->minsita = 0.1; /* ModelingSetup.cpp:211-230: the filter never matches */
    S->mu0 = 4 * ORC_PI * 1.e-7;
    S->mindx = fmin(S->dzmin, fmin(S->dxmin, S->dymin));
    S->tw = dalloc(2 * S->nsrc + 1); S->dtw = dalloc(2 * S->nsrc + 2); S->wave = dalloc(2 * S->nsrc + 1);
    orc_waveform(S->nsrc, S->sita_t, S->tw, S->dtw, S->wave);
    build_mapping(S);
    if (read_rx_tx(S, dir)) goto fail;
    alloc_state(S);
    return S;
fail:
    if (errbuf) snprintf(errbuf, errlen, "%s", S->err);
    orc_free(S);
    return NULL;
}

void orc_free(orc_sim *S) {
    if (!S) return;
    void *p[] = {S->dx, S->dy, S->dz, S->X, S->Y, S->Z, S->Xn, S->Yn, S->dxk, S->dyk, S->dzk, S->xBzNew2old,
                 S->yBzNew2old, S->xBzold2New, S->yBzold2New, S->xoldBx2NewBz, S->yoldBy2NewBz, S->con, S->tw, S->dtw,
                 S->wave, S->times, S->rx, S->ry, S->rz, S->rix, S->riy, S->riz, S->Ex, S->Ey, S->Ez, S->Bx, S->By,
                 S->Bz, S->BxAir, S->ByAir, S->BzAir, S->FBxR, S->FByR, S->FBzC, S->FBxC, S->FByC, S->semi_x00,
                 S->semi_x01, S->semi_x10, S->semi_x11, S->ef0, S->efs};
    for (size_t i = 0; i < sizeof p / sizeof p[0]; i++) free(p[i]);
    if (S->tx) for (int t = 0; t < S->NTx; t++) free(S->tx[t].rxnum);
    free(S->tx);
    free(S);
}

/* scalar/array accessors used by the tests */
void orc_dims(const orc_sim *S, int *out /* 16 ints */) {
    int v[16] = {S->L, S->M, S->N, S->L1, S->M1, S->AnLx_New, S->AnRx_New, S->Any_New,
                 S->NRx, S->NTx, S->Nt, S->NComp, S->nefcmp, S->nsrc, S->IsLog, 0};
    memcpy(out, v, sizeof v);
}
void orc_params(const orc_sim *S, double *out /* 8 */) {
    double v[8] = {S->sfa1, S->sfa2, S->sita_t, S->minsita, S->mu0, S->mindx, S->T0, S->Tn};
    memcpy(out, v, sizeof v);
}
/* which: 0 dx 1 dy 2 dz 3 X 4 Y 5 Z 6 Xn 7 Yn 8 dxk 9 dyk 10 dzk 11 times 12 tw 13 dtw 14 wave 15 rx 16 ry 17 rz */
int orc_get_darray(const orc_sim *S, int which, double *out) {
    const double *src; size_t n;
    switch (which) {
    case 0: src = S->dx; n = S->L; break; case 1: src = S->dy; n = S->M; break; case 2: src = S->dz; n = S->N; break;
    case 3: src = S->X; n = S->L; break; case 4: src = S->Y; n = S->M; break; case 5: src = S->Z; n = S->N; break;
    case 6: src = S->Xn; n = S->L1; break; case 7: src = S->Yn; n = S->M1; break;
    case 8: src = S->dxk; n = S->L; break; case 9: src = S->dyk; n = S->M; break; case 10: src = S->dzk; n = S->N; break;
    case 11: src = S->times; n = S->Nt; break;
    case 12: src = S->tw; n = 2 * S->nsrc + 1; break; case 13: src = S->dtw; n = 2 * S->nsrc + 2; break;
    case 14: src = S->wave; n = 2 * S->nsrc + 1; break;
    case 15: src = S->rx; n = S->NRx; break; case 16: src = S->ry; n = S->NRx; break; case 17: src = S->rz; n = S->NRx; break;
    default: return -1;
    }
    memcpy(out, src, n * sizeof(double));
    return (int)n;
}
/* which: 0 xBzNew2old 1 yBzNew2old 2 xBzold2New 3 yBzold2New 4 xoldBx2NewBz 5 yoldBy2NewBz 6 rix 7 riy 8 riz */
int orc_get_iarray(const orc_sim *S, int which, int *out) {
    const int *src; size_t n;
    switch (which) {
    case 0: src = S->xBzNew2old; n = S->L1; break; case 1: src = S->yBzNew2old; n = S->M1; break;
    case 2: src = S->xBzold2New; n = S->L; break; case 3: src = S->yBzold2New; n = S->M; break;
    case 4: src = S->xoldBx2NewBz; n = S->L + 1; break; case 5: src = S->yoldBy2NewBz; n = S->M + 1; break;
    case 6: src = S->rix; n = S->NRx; break; case 7: src = S->riy; n = S->NRx; break; case 8: src = S->riz; n = S->NRx; break;
    default: return -1;
    }
    memcpy(out, src, n * sizeof(int));
    return (int)n;
}
/* transmitter record: ints[24] = ort nr ixa iya iza ixb iyb izb ictx icty ictz ixa1 iya1 iza1 ixb1 iyb1 izb1 ictx1 icty1 ictz1,
 * doubles[12] = BipoLen x y z azi dip BipoLen1 x1 y1 z1 azi1 dip1 */
int orc_get_tx(const orc_sim *S, int t, int *iv, double *dv, int *rxnum) {
    if (t < 0 || t >= S->NTx) return -1;
    const orc_tx *T = &S->tx[t];
    int a[20] = {T->ort, T->nr, T->ixa, T->iya, T->iza, T->ixb, T->iyb, T->izb, T->ictx, T->icty, T->ictz,
                 T->ixa1, T->iya1, T->iza1, T->ixb1, T->iyb1, T->izb1, T->ictx1, T->icty1, T->ictz1};
    double d[12] = {T->BipoLen, T->x, T->y, T->z, T->azi, T->dip, T->BipoLen1, T->x1, T->y1, T->z1, T->azi1, T->dip1};
    memcpy(iv, a, sizeof a); memcpy(dv, d, sizeof d);
    if (rxnum) memcpy(rxnum, T->rxnum, T->nr * sizeof(int));
    return 0;
}
int orc_get_field(orc_sim *S, int comp, double *out) {
    double *p = field_ptr(S, comp);
    if (!p) return -1;
    memcpy(out, p, orc_field_size(S, comp) * sizeof(double));
    return 0;
}
int orc_set_field(orc_sim *S, int comp, const double *in) {
    double *p = field_ptr(S, comp);
    if (!p) return -1;
    memcpy(p, in, orc_field_size(S, comp) * sizeof(double));
    return 0;
}
void orc_set_dual_bipole_compat(orc_sim *S, int on) { S->bug_compat_dual_bipole = on; }
void orc_upcontinuation_padded(orc_sim *S);
void orc_set_padded_plane(orc_sim *S, int on) { S->padded_plane = on; }

/* prepare_free_mem.cu:164-186 */
void orc_zero_fields(orc_sim *S) {
    for (int c = 0; c < 8; c++) memset(field_ptr(S, c), 0, orc_field_size(S, c) * sizeof(double));
}

/* ------------------------------------------------------------ E update */

/* UpdateEx / UpdateEy / UpdateEz, ElectricalFiled.cu:89-345 */
void orc_update_e(orc_sim *S, double lambda, double dt) {
    const int L = S->L, M = S->M, N = S->N;
    const double mu = S->mu0;
    double *Ex = S->Ex, *Ey = S->Ey, *Ez = S->Ez, *Bx = S->Bx, *By = S->By, *Bz = S->Bz, *C = S->con;
#pragma omp parallel for schedule(static)
    for (int j = 1; j < M; j++) {
        for (int i = 0; i < L; i++) {
            double dy2 = S->dyk[j - 1] + S->dyk[j];
            double sx = 0.5 * (C[CI(S, 0, j - 1, i)] + C[CI(S, 0, j, i)]), sy = 0.0;
            for (int k = 0; k < N; k++) {
                if (k > 0) { sy = sx; sx = 0.5 * (C[CI(S, k, j - 1, i)] + C[CI(S, k, j, i)]); }
                double s = 0.5 * (sx + sy);
                double t1 = (Bz[BZI(S, k, j, i)] - Bz[BZI(S, k, j - 1, i)]) / dy2;
                double byu = k == 0 ? S->ByAir[(size_t)j * L + i] : By[BYI(S, k - 1, j, i)];
                double dzs = k == 0 ? 2.0 * S->dzk[0] : S->dzk[k] + S->dzk[k - 1];
                size_t e = EXI(S, k, j, i);
                Ex[e] = (2.0 * lambda - s * dt) / (2.0 * lambda + s * dt) * Ex[e] +
                        4.0 * dt / (2.0 * lambda + s * dt) * (t1 - (By[BYI(S, k, j, i)] - byu) / dzs) / mu;
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < M; j++) {
        for (int i = 1; i < L; i++) {
            double dx2 = S->dxk[i - 1] + S->dxk[i];
            for (int k = 0; k < N; k++) {
                double s = k == 0 ? 0.25 * (C[CI(S, 0, j, i - 1)] + C[CI(S, 0, j, i)])
                                  : 0.25 * (C[CI(S, k, j, i - 1)] + C[CI(S, k, j, i)] + C[CI(S, k - 1, j, i - 1)] +
                                            C[CI(S, k - 1, j, i)]);
                double bxu = k == 0 ? S->BxAir[(size_t)j * (L + 1) + i] : Bx[BXI(S, k - 1, j, i)];
                double dzs = k == 0 ? 2.0 * S->dzk[0] : S->dzk[k] + S->dzk[k - 1];
                size_t e = EYI(S, k, j, i);
                Ey[e] = (2.0 * lambda - s * dt) / (2.0 * lambda + s * dt) * Ey[e] +
                        4.0 * dt / (2.0 * lambda + s * dt) *
                            ((Bx[BXI(S, k, j, i)] - bxu) / dzs - (Bz[BZI(S, k, j, i)] - Bz[BZI(S, k, j, i - 1)]) / dx2) / mu;
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int j = 1; j < M; j++) {
        for (int i = 1; i < L; i++) {
            double dx2 = S->dxk[i - 1] + S->dxk[i], dy2 = S->dyk[j - 1] + S->dyk[j];
            for (int k = 0; k < N; k++) {
                double s = 0.25 * (C[CI(S, k, j - 1, i - 1)] + C[CI(S, k, j - 1, i)] + C[CI(S, k, j, i - 1)] +
                                   C[CI(S, k, j, i)]);
                double t2 = Bx[BXI(S, k, j, i)] - Bx[BXI(S, k, j - 1, i)];
                size_t e = EZI(S, k, j, i);
                Ez[e] = (2.0 * lambda - s * dt) / (2.0 * lambda + s * dt) * Ez[e] +
                        4.0 * dt / (2.0 * lambda + s * dt) *
                            ((By[BYI(S, k, j, i)] - By[BYI(S, k, j, i - 1)]) / dx2 - t2 / dy2) / mu;
            }
        }
    }
}

/* AddTx_x / AddTx_y / AddTx_z, ElectricalFiled.cu:347-475.  `count` is the
 * launch width; the kernel guard uses the first bipole's extent. */
static void addtx_x(orc_sim *S, const orc_tx *T, double cur, int count) {
    int ixa = T->ixa < T->ixb ? T->ixa : T->ixb, iya = T->icty, iza = T->ictz;
    int lim = abs(T->ixb - T->ixa);
    const double *C = S->con;
    for (int ix = 0; ix < count && ix <= lim; ix++) {
        int i = ix + ixa;
        double s = iza == 0 ? C[CI(S, iza, iya, i)] + C[CI(S, iza, iya - 1, i)]
                            : C[CI(S, iza, iya, i)] + C[CI(S, iza, iya - 1, i)] + C[CI(S, iza - 1, iya, i)] +
                                  C[CI(S, iza - 1, iya - 1, i)];
        S->Ex[EXI(S, iza, iya, i)] -= 2.0 * cur / (0.25 * s * S->dyk[iya] * S->dzk[iza]);
    }
}
static void addtx_y(orc_sim *S, const orc_tx *T, double cur, int count) {
    int ixa = T->ictx, iya = T->iya < T->iyb ? T->iya : T->iyb, iza = T->ictz;
    int lim = abs(T->iyb - T->iya);
    const double *C = S->con;
    for (int iy = 0; iy < count && iy <= lim; iy++) {
        int j = iy + iya;
        double s = iza == 0 ? C[CI(S, iza, j, ixa - 1)] + C[CI(S, iza, j, ixa)]
                            : C[CI(S, iza, j, ixa - 1)] + C[CI(S, iza, j, ixa)] + C[CI(S, iza - 1, j, ixa - 1)] +
                                  C[CI(S, iza - 1, j, ixa)];
        S->Ey[EYI(S, iza, j, ixa)] -= 2.0 * cur / (0.25 * s * S->dxk[ixa] * S->dzk[iza]);
    }
}
static void addtx_z(orc_sim *S, const orc_tx *T, double cur, int count) {
    int ixa = T->ictx, iya = T->icty, iza = T->iza < T->izb ? T->iza : T->izb;
    int lim = abs(T->izb - T->iza);
    const double *C = S->con;
    for (int iz = 0; iz < count && iz <= lim; iz++) {
        int k = iz + iza;
        double s = C[CI(S, k, iya, ixa - 1)] + C[CI(S, k, iya, ixa)] + C[CI(S, k, iya - 1, ixa - 1)] +
                   C[CI(S, k, iya - 1, ixa)];
        S->Ez[EZI(S, k, iya, ixa)] -= 2.0 * cur / (0.25 * s * S->dxk[ixa] * S->dyk[iya]);
    }
}

/* host side of ElectricalField, ElectricalFiled.cu:531-641 */
void orc_add_source(orc_sim *S, int itx, double wave) {
    if (wave == 0) return;
    const orc_tx *T = &S->tx[itx];
    const double *X = S->X, *Y = S->Y, *Z = S->Z, *dx = S->dx, *dy = S->dy, *dz = S->dz;
    double cur;
    switch (T->ort) {
    case 1:
        wave /= (X[T->ixb] - X[T->ixa] + dx[T->ixb] / 2 + dx[T->ixa] / 2);
        addtx_x(S, T, wave, abs(T->ixb - T->ixa) + 1);
        break;
    case 2:
        wave /= (Y[T->iyb] - Y[T->iya] + dy[T->iyb] / 2 + dy[T->iya] / 2);
        addtx_y(S, T, wave, abs(T->iyb - T->iya) + 1);
        break;
    case 3:
        wave /= (Z[T->izb] - Z[T->iza] + dz[T->izb] / 2 + dz[T->iza] / 2);
        addtx_z(S, T, wave, abs(T->izb - T->iza) + 1);
        break;
    case 4:
    case 5: {
        double f = T->ort == 5 ? T->BipoLen : 1.0;
        if (T->ort == 4) {
            cur = wave * cos(T->dip) * cos(T->azi) / (fabs(X[T->ixb] - X[T->ixa]) + dx[T->ixb] / 2.0 + dx[T->ixa] / 2.0);
        } else {
            cur = wave * cos(T->dip) * cos(T->azi) * f / (fabs(X[T->ixb] - X[T->ixa]) + dx[T->ixb] / 2.0 + dx[T->ixa] / 2.0);
        }
        addtx_x(S, T, cur, abs(T->ixb - T->ixa) + 1);
        if (T->ort == 4)
            cur = wave * cos(T->dip) * sin(T->azi) / (fabs(Y[T->iyb] - Y[T->iya]) + dy[T->iyb] / 2.0 + dy[T->iya] / 2.0);
        else
            cur = wave * cos(T->dip) * sin(T->azi) * f / (fabs(Y[T->iyb] - Y[T->iya]) + dy[T->iyb] / 2.0 + dy[T->iya] / 2.0);
        addtx_y(S, T, cur, abs(T->iyb - T->iya) + 1);
        if (T->ort == 4)
            cur = wave * sin(T->dip) / (fabs(Z[T->izb] - Z[T->iza]) + dz[T->izb] / 2.0 + dz[T->iza] / 2.0);
        else
            cur = wave * sin(T->dip) * f / (fabs(Z[T->izb] - Z[T->iza]) + dz[T->izb] / 2.0 + dz[T->iza] / 2.0);
        addtx_z(S, T, cur, abs(T->izb - T->iza) + 1);
        if (T->ort == 5) {
            orc_tx T2 = *T;
            if (!S->bug_compat_dual_bipole) {
                T2.ixa = T->ixa1; T2.ixb = T->ixb1; T2.iya = T->iya1; T2.iyb = T->iyb1; T2.iza = T->iza1;
                T2.izb = T->izb1; T2.ictx = T->ictx1; T2.icty = T->icty1; T2.ictz = T->ictz1;
            }
            cur = wave * cos(T->dip1) * cos(T->azi1) * T->BipoLen1 /
                  (fabs(X[T->ixb1] - X[T->ixa1]) + dx[T->ixb1] / 2.0 + dx[T->ixa1] / 2.0);
            addtx_x(S, &T2, cur, abs(T->ixb1 - T->ixa1) + 1);
            cur = wave * cos(T->dip1) * sin(T->azi1) * T->BipoLen1 /
                  (fabs(Y[T->iyb1] - Y[T->iya1]) + dy[T->iyb1] / 2.0 + dy[T->iya1] / 2.0);
            addtx_y(S, &T2, cur, abs(T->iyb1 - T->iya1) + 1);
            cur = wave * sin(T->dip1) * T->BipoLen1 /
                  (fabs(Z[T->izb1] - Z[T->iza1]) + dz[T->izb1] / 2.0 + dz[T->iza1] / 2.0);
            addtx_z(S, &T2, cur, abs(T->izb1 - T->iza1) + 1);
        }
        break;
    }
    default:
        break;
    }
}

void orc_electric_field(orc_sim *S, int itx, double lambda, double dt, double wave) {
    orc_update_e(S, lambda, dt);
    orc_add_source(S, itx, wave);
}

/* ------------------------------------------------------------ B update */

/* UpdateBx / UpdateBy / UpdateBz, Bderivate.cu:79-265 */
void orc_bderivate(orc_sim *S, double dt) {
    const int L = S->L, M = S->M, N = S->N;
    double *Ex = S->Ex, *Ey = S->Ey, *Ez = S->Ez, *Bx = S->Bx, *By = S->By, *Bz = S->Bz;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < M; j++)
        for (int i = 1; i < L; i++)
            for (int k = 0; k < N; k++)
                Bx[BXI(S, k, j, i)] += ((Ey[EYI(S, k + 1, j, i)] - Ey[EYI(S, k, j, i)]) / S->dzk[k] -
                                        (Ez[EZI(S, k, j + 1, i)] - Ez[EZI(S, k, j, i)]) / S->dyk[j]) * dt;
#pragma omp parallel for schedule(static)
    for (int j = 1; j < M; j++)
        for (int i = 0; i < L; i++)
            for (int k = 0; k < N; k++)
                By[BYI(S, k, j, i)] += ((Ez[EZI(S, k, j, i + 1)] - Ez[EZI(S, k, j, i)]) / S->dxk[i] -
                                        (Ex[EXI(S, k + 1, j, i)] - Ex[EXI(S, k, j, i)]) / S->dzk[k]) * dt;
#pragma omp parallel for schedule(static)
    for (int j = 0; j < M; j++)
        for (int i = 0; i < L; i++) {
            double acc = 0.0;
            for (int k = N - 1; k >= 0; k--) {
                acc += S->dzk[k] * ((Bx[BXI(S, k, j, i + 1)] - Bx[BXI(S, k, j, i)]) / S->dxk[i] +
                                    (By[BYI(S, k, j + 1, i)] - By[BYI(S, k, j, i)]) / S->dyk[j]);
                Bz[BZI(S, k, j, i)] = acc;
            }
        }
}

/* ------------------------------------------------------- spline remap */

/* Natural-spline pieces of SplineGridConvIR2R.cu: tridiagonal rows as filled
 * by fillA0x..fillA1y (initialize_UpCont_gpu_resources.cu:46-144), right hand
 * side as in Fill_B_* (SplineGridConvIR2R.cu:70-173), solved without pivoting
 * like cusparse?gtsv2_nopivot, evaluated as in Intep_BzIR2R_* (:180-498). */
static void spline_coeffs(int n, const double *d, const double *bz, double *mb) {
    double *dl = dalloc(n), *dd = dalloc(n), *du = dalloc(n), *rhs = dalloc(n);
    for (int r = 0; r < n; r++) {
        if (r == 0 || r == n - 1) { dd[r] = 2.0; dl[r] = 0.0; du[r] = 0.0; rhs[r] = 0.0; }
        else {
            dd[r] = 2.0 / 3.0 * (d[r] + 0.5 * d[r - 1] + 0.5 * d[r + 1]);
            dl[r] = 1.0 / 3.0 * (0.5 * d[r - 1] + 0.5 * d[r]);
            du[r] = 1.0 / 3.0 * (0.5 * d[r] + 0.5 * d[r + 1]);
            rhs[r] = (bz[r + 1] - bz[r]) / (0.5 * d[r] + 0.5 * d[r + 1]) - (bz[r] - bz[r - 1]) / (0.5 * d[r - 1] + 0.5 * d[r]);
        }
    }
    /* Thomas elimination */
    for (int r = 1; r < n; r++) {
        double w = dl[r] / dd[r - 1];
        dd[r] -= w * du[r - 1];
        rhs[r] -= w * rhs[r - 1];
    }
    mb[n - 1] = rhs[n - 1] / dd[n - 1];
    for (int r = n - 2; r >= 0; r--) mb[r] = (rhs[r] - du[r] * mb[r + 1]) / dd[r];
    free(dl); free(dd); free(du); free(rhs);
}
/* evaluation at coordinate `xnew` given the insertion index `map` (already
 * shifted to local node numbering): Intep_BzIR2R_0x body. */
static double spline_eval(int n, const double *d, const double *xo, const double *bz, const double *mb, int map,
                          double xnew) {
    int id = map - 1 > 0 ? map - 1 : 0;
    double ma, mc;
    if (id < n - 1) {
        ma = 1.0 / 3.0 * (mb[id + 1] - mb[id]) / (0.5 * d[id] + 0.5 * d[id + 1]);
        mc = (bz[id + 1] - bz[id]) / (0.5 * d[id] + 0.5 * d[id + 1]) -
             1.0 / 3.0 * (2.0 * mb[id] + mb[id + 1]) * (0.5 * d[id] + 0.5 * d[id + 1]);
    } else {
        ma = 1.0 / 3.0 * (mb[id] - mb[id - 1]) / (0.5 * d[id - 1] + 0.5 * d[id]);
        mc = (bz[id] - bz[id - 1]) / (0.5 * d[id - 1] + 0.5 * d[id]) -
             1.0 / 3.0 * (2.0 * mb[id - 1] + mb[id]) * (0.5 * d[id - 1] + 0.5 * d[id]);
        mc += 3.0 * ma * (0.5 * d[id - 1] + 0.5 * d[id]) * (0.5 * d[id - 1] + 0.5 * d[id]) +
              2.0 * mb[id - 1] * (0.5 * d[id - 1] + 0.5 * d[id]);
        ma = 0.0;
    }
    double h = xnew - xo[id];
    int id2 = map - 1;
    if (id2 >= 0 && id2 < n - 1) return ma * h * h * h + mb[id2] * h * h + mc * h + bz[id2];
    int c = id2 > 0 ? id2 : 0;
    return (mb[c] * h + mc) * h + bz[c];
}

/* SplineGridConvIR2R, SplineGridConvIR2R.cu:539-752: Bz top plane -> BzAir */
void orc_spline_remap(orc_sim *S) {
    const int L = S->L, M = S->M, L1 = S->L1, NP = ORC_NPAD;
    const int AL = S->ALx1 + S->ALx2, Ay = S->Ay1 + S->Ay2;
    const int n1 = AL + NP, n2 = S->ARx1 + S->ARx2 + NP, n3 = Ay + NP;
    const int ox = S->Nx + AL - NP, oy = S->Ny + Ay - NP;
    const double *B0 = S->Bz; /* plane 0, row stride L */
    double *A = S->BzAir;
    /* centre copy (Intep_BzIR2R_cpy_center) */
    for (int iy = 0; iy < S->Ny; iy++)
        for (int ix = 0; ix < S->Nx; ix++)
            A[(size_t)(iy + S->Any_New) * L1 + ix + S->AnLx_New] = B0[(size_t)(iy + Ay) * L + ix + AL];
    /* left and right strips along x (Intep_BzIR2R_0x / _1x) */
#pragma omp parallel for schedule(static)
    for (int iy = 0; iy < M; iy++) {
        double mb[512];
        const double *row = B0 + (size_t)iy * L;
        spline_coeffs(n1, S->dx, row, mb);
        for (int ix = 0; ix < S->AnLx_New; ix++) {
            double f = spline_eval(n1, S->dx, S->X, row, mb, S->xBzNew2old[ix], S->Xn[ix]);
            if (iy < n3) S->semi_x00[(size_t)iy * S->AnLx_New + ix] = f;
            if (iy > Ay - 1 && iy < Ay + S->Ny) A[(size_t)(iy - Ay + S->Any_New) * L1 + ix] = f;
            if (iy > oy - 1) S->semi_x01[(size_t)(iy - oy) * S->AnLx_New + ix] = f;
        }
        spline_coeffs(n2, S->dx + ox, row + ox, mb);
        for (int ix = 0; ix < S->AnRx_New; ix++) {
            int c = S->Nx + S->AnLx_New + ix;
            double f = spline_eval(n2, S->dx + ox, S->X + ox, row + ox, mb, S->xBzNew2old[c] - ox, S->Xn[c]);
            if (iy < n3) S->semi_x10[(size_t)iy * S->AnRx_New + ix] = f;
            if (iy > Ay - 1 && iy < Ay + S->Ny) A[(size_t)(iy - Ay + S->Any_New) * L1 + c] = f;
            if (iy > oy - 1) S->semi_x11[(size_t)(iy - oy) * S->AnRx_New + ix] = f;
        }
    }
    /* front and back strips along y (Intep_BzIR2R_0y / _1y) */
#pragma omp parallel for schedule(static)
    for (int c = 0; c < L1; c++) {
        double bz[512], mb[512];
        for (int r = 0; r < n3; r++) {
            if (c < S->AnLx_New) bz[r] = S->semi_x00[c + (size_t)r * S->AnLx_New];
            else if (c < S->Nx + S->AnLx_New) bz[r] = B0[c - S->AnLx_New + AL + (size_t)r * L];
            else bz[r] = S->semi_x10[c - (S->Nx + S->AnLx_New) + (size_t)r * S->AnRx_New];
        }
        spline_coeffs(n3, S->dy, bz, mb);
        for (int ix = 0; ix < S->Any_New; ix++)
            A[c + (size_t)ix * L1] = spline_eval(n3, S->dy, S->Y, bz, mb, S->yBzNew2old[ix], S->Yn[ix]);
        for (int r = 0; r < n3; r++) {
            if (c < S->AnLx_New) bz[r] = S->semi_x01[c + (size_t)r * S->AnLx_New];
            else if (c < S->Nx + S->AnLx_New) bz[r] = B0[c - S->AnLx_New + AL + (size_t)(oy + r) * L];
            else bz[r] = S->semi_x11[c - (S->Nx + S->AnLx_New) + (size_t)r * S->AnRx_New];
        }
        spline_coeffs(n3, S->dy + oy, bz, mb);
        for (int ix = 0; ix < S->Any_New; ix++) {
            int rr = ix + S->Any_New + S->Ny;
            A[c + (size_t)rr * L1] = spline_eval(n3, S->dy + oy, S->Y + oy, bz, mb, S->yBzNew2old[rr] - oy, S->Yn[rr]);
        }
    }
}

/* ---------------------------------------------------------------- FFT */

/* Plain recursive mixed-radix DFT (decimation in time, any factorisation),
 * used only as the oracle's transform: X[k] = sum_n x[n] exp(sign*2*pi*i*n*k/N). */
static void fft_rec(int n, const cplx *in, int is, cplx *out, const cplx *tw, int twstep, cplx *tmp) {
    if (n == 1) { out[0] = in[0]; return; }
    int p = 2;
    while (p * p <= n && n % p) p++;
    if (n % p) p = n;
    int m = n / p;
    for (int q = 0; q < p; q++) fft_rec(m, in + (size_t)q * is, is * p, out + (size_t)q * m, tw, twstep * p, tmp);
    /* out[q*m + k] holds sub-transform q at frequency k */
    for (int k = 0; k < m; k++) {
        for (int s = 0; s < p; s++) {
            int kk = k + s * m;
            cplx acc = 0;
            for (int q = 0; q < p; q++) {
                long e = ((long)q * kk) % n;
                acc += out[(size_t)q * m + k] * tw[(size_t)e * twstep];
            }
            tmp[kk] = acc;
        }
    }
    memcpy(out, tmp, (size_t)n * sizeof(cplx));
}
static void fft1d(int n, cplx *data, int stride, int sign) {
    cplx *tw = (cplx *)malloc((size_t)n * sizeof(cplx));
    cplx *in = (cplx *)malloc((size_t)n * sizeof(cplx));
    cplx *out = (cplx *)malloc((size_t)n * sizeof(cplx));
    cplx *tmp = (cplx *)malloc((size_t)n * sizeof(cplx));
    for (int k = 0; k < n; k++) {
        double a = sign * 2.0 * ORC_PI * (double)k / (double)n;
        tw[k] = cos(a) + I * sin(a);
    }
    for (int k = 0; k < n; k++) in[k] = data[(size_t)k * stride];
    fft_rec(n, in, 1, out, tw, 1, tmp);
    for (int k = 0; k < n; k++) data[(size_t)k * stride] = out[k];
    free(tw); free(in); free(out); free(tmp);
}
/* 2-D real-to-half-complex transform of a[M1][L1] -> F[M1][L1/2+1] (cufftExecD2Z) */
static void r2c_2d(int M1, int L1, const double *a, cplx *F) {
    int H = L1 / 2 + 1;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < M1; y++) {
        cplx *row = (cplx *)malloc((size_t)L1 * sizeof(cplx));
        for (int x = 0; x < L1; x++) row[x] = a[(size_t)y * L1 + x];
        fft1d(L1, row, 1, -1);
        for (int x = 0; x < H; x++) F[(size_t)y * H + x] = row[x];
        free(row);
    }
#pragma omp parallel for schedule(static)
    for (int x = 0; x < H; x++) fft1d(M1, F + x, H, -1);
}
/* 2-D half-complex-to-real inverse, unnormalised (cufftExecZ2D).  The input
 * is taken as the half of a Hermitian spectrum: the self-conjugate columns
 * (kx = 0 and kx = L1/2 for even L1) contribute their Hermitian part. */
static void c2r_2d(int M1, int L1, const cplx *F, double *a) {
    int H = L1 / 2 + 1;
    cplx *G = (cplx *)malloc((size_t)M1 * H * sizeof(cplx));
    memcpy(G, F, (size_t)M1 * H * sizeof(cplx));
#pragma omp parallel for schedule(static)
    for (int x = 0; x < H; x++) fft1d(M1, G + x, H, +1);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < M1; y++) {
        cplx *row = (cplx *)malloc((size_t)L1 * sizeof(cplx));
        const cplx *g = G + (size_t)y * H;
        row[0] = creal(g[0]);
        for (int x = 1; x < H; x++) {
            if (2 * x == L1) row[x] = creal(g[x]);
            else { row[x] = g[x]; row[L1 - x] = conj(g[x]); }
        }
        fft1d(L1, row, 1, +1);
        for (int x = 0; x < L1; x++) a[(size_t)y * L1 + x] = creal(row[x]);
        free(row);
    }
    free(G);
}

/* FBz_to_FBxFBy, UpContinuation_gpu.cu:113-164, on an L x M transform plane */
static void continuation_multiply_on(const orc_sim *S, int L, int M, const cplx *FBz, cplx *FBx, cplx *FBy) {
    const int H = L / 2 + 1;
    for (int iy = 0; iy < M; iy++) {
        double v1 = iy < M / 2 + 1 ? (1.0 * ORC_PI * iy) / M * (S->dzmin / S->dymin)
                                   : -(1.0 * ORC_PI * (M - iy)) / M * (S->dzmin / S->dymin);
        for (int ix = 0; ix < H; ix++) {
            double u1 = (1.0 * ORC_PI * ix) / L * (S->dzmin / S->dxmin);
            cplx f = FBz[(size_t)iy * H + ix];
            cplx a = -cimag(f) + I * creal(f);
            if (ix == 0 && iy == 0) {
                FBx[0] = a; FBy[0] = a;
            } else {
                double upcc = exp(-sqrt(u1 * u1 + v1 * v1)) * (1.0 / sqrt(u1 * u1 + v1 * v1));
                FBx[(size_t)iy * H + ix] = (S->dxmin / S->dymin) * u1 * upcc * a;
                FBy[(size_t)iy * H + ix] = (S->dymin / S->dxmin) * v1 * upcc * a;
            }
        }
    }
}
static void continuation_multiply(orc_sim *S) {
    continuation_multiply_on(S, S->L1, S->M1, S->FBzC, S->FBxC, S->FByC);
}

/* Blinear_BxR2IR / Blinear_ByR2IR, UpContinuation_gpu.cu:42-110 */
static void bilinear_back_norm(orc_sim *S, double norm) {
    const int L0 = S->L, M0 = S->M, L1 = S->L1, M1 = S->M1;
    for (int iy = 0; iy < M0; iy++)
        for (int ix = 0; ix < L0 + 1; ix++) {
            int II = S->xoldBx2NewBz[ix]; II = II < 1 ? 1 : II; II = II > L1 - 1 ? L1 - 1 : II;
            int JJ = S->yBzold2New[iy]; JJ = JJ < 1 ? 1 : JJ; JJ = JJ > M1 - 1 ? M1 - 1 : JJ;
            double Xp = ix == L0 ? S->X[L0 - 1] + 0.5 * S->dx[L0 - 1] : S->X[ix] - 0.5 * S->dx[ix];
            double l1 = (Xp - S->Xn[II - 1]) / (S->Xn[II] - S->Xn[II - 1]);
            double a0 = (1.0 - l1) * S->FBxR[(size_t)(JJ - 1) * L1 + II - 1] + l1 * S->FBxR[(size_t)(JJ - 1) * L1 + II];
            double a1 = (1.0 - l1) * S->FBxR[(size_t)JJ * L1 + II - 1] + l1 * S->FBxR[(size_t)JJ * L1 + II];
            l1 = (S->Y[iy] - S->Yn[JJ - 1]) / (S->Yn[JJ] - S->Yn[JJ - 1]);
            S->BxAir[(size_t)iy * (L0 + 1) + ix] = ((1.0 - l1) * a0 + l1 * a1) / norm;
        }
    for (int iy = 0; iy < M0 + 1; iy++)
        for (int ix = 0; ix < L0; ix++) {
            int II = S->xBzold2New[ix]; II = II < 1 ? 1 : II; II = II > L1 - 1 ? L1 - 1 : II;
            int JJ = S->yoldBy2NewBz[iy]; JJ = JJ < 1 ? 1 : JJ; JJ = JJ > M1 - 1 ? M1 - 1 : JJ;
            double Yp = iy == M0 ? S->Y[M0 - 1] + 0.5 * S->dy[M0 - 1] : S->Y[iy] - 0.5 * S->dy[iy];
            double l1 = (S->X[ix] - S->Xn[II - 1]) / (S->Xn[II] - S->Xn[II - 1]);
            double a0 = (1.0 - l1) * S->FByR[(size_t)(JJ - 1) * L1 + II - 1] + l1 * S->FByR[(size_t)(JJ - 1) * L1 + II];
            double a1 = (1.0 - l1) * S->FByR[(size_t)JJ * L1 + II - 1] + l1 * S->FByR[(size_t)JJ * L1 + II];
            l1 = (Yp - S->Yn[JJ - 1]) / (S->Yn[JJ] - S->Yn[JJ - 1]);
            S->ByAir[(size_t)iy * L0 + ix] = ((1.0 - l1) * a0 + l1 * a1) / norm;
        }
}

static void bilinear_back(orc_sim *S) { bilinear_back_norm(S, (double)(S->L1 * S->M1)); }

/* UpContinuation_gpu, UpContinuation_gpu.cu:166-274 */
void orc_upcontinuation(orc_sim *S) {
    orc_spline_remap(S);
    r2c_2d(S->M1, S->L1, S->BzAir, S->FBzC);
    continuation_multiply(S);
    c2r_2d(S->M1, S->L1, S->FBxC, S->FBxR);
    c2r_2d(S->M1, S->L1, S->FByC, S->FByR);
    bilinear_back(S);
}

/* The padded variant (not the reference's arithmetic; the padding that
 * UpContinuation.cpp:21-49 sketches, with the plane sizes of
 * ModelingSetup.cpp:194-195 in mode 1): the uniform plane is centred in a
 * plane of the next powers of two above L1 and M1 (mode 1) or of the smallest
 * lengths >= L1, M1 without prime factors above 5 (mode 2; padded_plane as set
 * by orc_set_padded_plane, mode 1 when unset), each row is continued left of the grid
 * by its first value and right of it by its last value times a raised-cosine
 * taper to zero, then each column of the widened plane likewise; the
 * continuation runs on that plane and the grid part goes to the bilinear
 * remap, normalised by the padded size. */
static int orc_plane_len(int n, int mode) {
    if (mode == 1) { int p = 1; while (p <= n) p *= 2; return p; }
    if (mode == 2)
        for (int m = n;; m++) {
            int r = m;
            while (r % 2 == 0) r /= 2;
            while (r % 3 == 0) r /= 3;
            while (r % 5 == 0) r /= 5;
            if (r == 1) return m;
        }
    return n;
}
static double orc_taper(int i, int n, int nu, int d) {
    if (i < d) return 0.5 * (1.0 - cos(ORC_PI * i / d));
    return 0.5 * (1.0 - cos(ORC_PI * (n - i) / (n - nu - d + 1)));
}
void orc_upcontinuation_padded(orc_sim *S) {
    orc_spline_remap(S);
    const int mode = S->padded_plane > 0 ? S->padded_plane : 1;
    const int L1 = S->L1, M1 = S->M1, Lf = orc_plane_len(L1, mode), Mf = orc_plane_len(M1, mode);
    const int DL = (Lf - L1) / 2, DM = (Mf - M1) / 2, H = Lf / 2 + 1;
    double *P = (double *)calloc((size_t)Lf * Mf, sizeof(double));
    for (int y = 0; y < M1; y++) {
        double *row = P + (size_t)(DM + y) * Lf;
        const double *src = S->BzAir + (size_t)y * L1;
        for (int x = 0; x < L1; x++) row[DL + x] = src[x];
        for (int x = 0; x < Lf; x++)
            if (x < DL || x >= DL + L1) row[x] = orc_taper(x, Lf, L1, DL) * (x < DL ? src[0] : src[L1 - 1]);
    }
    for (int y = 0; y < Mf; y++) {
        if (y >= DM && y < DM + M1) continue;
        const double w = orc_taper(y, Mf, M1, DM);
        const double *edge = P + (size_t)(y < DM ? DM : DM + M1 - 1) * Lf;
        for (int x = 0; x < Lf; x++) P[(size_t)y * Lf + x] = w * edge[x];
    }
    cplx *Fz = (cplx *)malloc((size_t)Mf * H * sizeof(cplx));
    cplx *Fx = (cplx *)malloc((size_t)Mf * H * sizeof(cplx));
    cplx *Fy = (cplx *)malloc((size_t)Mf * H * sizeof(cplx));
    double *Rx = (double *)malloc((size_t)Lf * Mf * sizeof(double));
    double *Ry = (double *)malloc((size_t)Lf * Mf * sizeof(double));
    r2c_2d(Mf, Lf, P, Fz);
    continuation_multiply_on(S, Lf, Mf, Fz, Fx, Fy);
    c2r_2d(Mf, Lf, Fx, Rx);
    c2r_2d(Mf, Lf, Fy, Ry);
    for (int y = 0; y < M1; y++)
        for (int x = 0; x < L1; x++) {
            S->FBxR[(size_t)y * L1 + x] = Rx[(size_t)(DM + y) * Lf + DL + x];
            S->FByR[(size_t)y * L1 + x] = Ry[(size_t)(DM + y) * Lf + DL + x];
        }
    bilinear_back_norm(S, (double)Lf * (double)Mf);
    free(P); free(Fz); free(Fx); free(Fy); free(Rx); free(Ry);
}

/* ---------------------------------------------------- receiver sampling */

/* CubicSpline_1d4p, EFInterp2Rx.cu:46-57 */
static double spline4(const double *x, const double *y, double t) {
    const double h1 = x[2] - x[1];
    const double v1 = 2.0 * (x[2] - x[0]);
    const double v2 = 2.0 * (x[3] - x[1]);
    const double u1 = 6.0 * ((y[2] - y[1]) / h1 - (y[1] - y[0]) / (x[1] - x[0]));
    const double u2 = 6.0 * ((y[3] - y[2]) / (x[3] - x[2]) - (y[2] - y[1]) / h1);
    const double z1 = (v2 * u1 - h1 * u2) / (v1 * v2 - h1 * h1);
    const double z2 = (v1 * u2 - h1 * u1) / (v1 * v2 - h1 * h1);
    return z2 / (6.0 * h1) * pow(t - x[1], 3) + z1 / (6.0 * h1) * pow(x[2] - t, 3) + (y[2] / h1 - z2 / 6.0 * h1) * (t - x[1]) +
           (y[1] / h1 - z1 / 6.0 * h1) * (x[2] - t);
}

/* stencil start rule shared by the *SpatialInterp kernels: step back one more
 * node when the receiver lies in the lower half of its cell */
static int half_start(const double *c, const double *d, int idx, double pos) {
    return (c[idx - 1] + 0.5 * d[idx - 1]) > pos ? idx - 2 : idx - 1;
}

/* Ex..BzSpatialInterp, EFInterp2Rx.cu:60-378.  Returns the value of field
 * component `comp` (0..5) at receiver `ir` (0-based position index). */
double orc_rx_interp(const orc_sim *S, int comp, int ir) {
    const int L = S->L, M = S->M;
    const double *X = S->X, *Y = S->Y, *Z = S->Z, *dx = S->dx, *dy = S->dy, *dz = S->dz;
    double px = S->rx[ir], py = S->ry[ir], pz = S->rz[ir];
    int ix = S->rix[ir], iy = S->riy[ir], iz = S->riz[ir];
    int s1, s2, s3;
    double xn[4], yn[4], zn[4], Y1[4], Y2[4];
    const double *F; size_t rowlen, nrows;
    switch (comp) {
    case 0: /* Ex at (X, Y-dy/2, Z-dz/2) */
        s1 = ix - 2; s2 = half_start(Y, dy, iy, py);
        s3 = iz >= 1 ? half_start(Z, dz, iz, pz) : -1;
        if (s3 < 0) s3 = 0;
        for (int q = 0; q < 4; q++) { xn[q] = X[s1 + q]; yn[q] = Y[s2 + q] - 0.5 * dy[s2 + q]; zn[q] = Z[s3 + q] - 0.5 * dz[s3 + q]; }
        F = S->Ex; rowlen = L; nrows = M + 1; break;
    case 1: /* Ey at (X-dx/2, Y, Z-dz/2) */
        s1 = half_start(X, dx, ix, px); s2 = iy - 2;
        s3 = iz >= 1 ? half_start(Z, dz, iz, pz) : -1;
        if (s3 < 0) s3 = 0;
        for (int q = 0; q < 4; q++) { xn[q] = X[s1 + q] - 0.5 * dx[s1 + q]; yn[q] = Y[s2 + q]; zn[q] = Z[s3 + q] - 0.5 * dz[s3 + q]; }
        F = S->Ey; rowlen = L + 1; nrows = M; break;
    case 2: /* Ez at (X-dx/2, Y-dy/2, Z) */
        s1 = half_start(X, dx, ix, px); s2 = half_start(Y, dy, iy, py);
        s3 = iz - 2; if (s3 < 0) s3 = 0;
        for (int q = 0; q < 4; q++) { xn[q] = X[s1 + q] - 0.5 * dx[s1 + q]; yn[q] = Y[s2 + q] - 0.5 * dy[s2 + q]; zn[q] = Z[s3 + q]; }
        F = S->Ez; rowlen = L + 1; nrows = M + 1; break;
    case 3: /* Bx at (X-dx/2, Y, Z) */
        s1 = half_start(X, dx, ix, px); s2 = iy - 2;
        s3 = iz - 2; if (s3 < 0) s3 = 0;
        for (int q = 0; q < 4; q++) { xn[q] = X[s1 + q] - 0.5 * dx[s1 + q]; yn[q] = Y[s2 + q]; zn[q] = Z[s3 + q]; }
        F = S->Bx; rowlen = L + 1; nrows = M; break;
    case 4: /* By at (X, Y-dy/2, Z) */
        s1 = ix - 2; s2 = half_start(Y, dy, iy, py);
        s3 = iz - 2; if (s3 < 0) s3 = 0;
        for (int q = 0; q < 4; q++) { xn[q] = X[s1 + q]; yn[q] = Y[s2 + q] - 0.5 * dy[s2 + q]; zn[q] = Z[s3 + q]; }
        F = S->By; rowlen = L; nrows = M + 1; break;
    default: /* Bz at (X, Y, Z-dz/2) */
        s1 = ix - 2; s2 = iy - 2;
        s3 = iz >= 1 ? half_start(Z, dz, iz, pz) : -1;
        if (s3 < 0) s3 = 0;
        for (int q = 0; q < 4; q++) { xn[q] = X[s1 + q]; yn[q] = Y[s2 + q]; zn[q] = Z[s3 + q] - 0.5 * dz[s3 + q]; }
        F = S->Bz; rowlen = L; nrows = M; break;
    }
    for (int ik = 0; ik < 4; ik++) {
        for (int ij = 0; ij < 4; ij++) {
            size_t indx = ((size_t)(ik + s3) * nrows + ij + s2) * rowlen + s1;
            Y1[ij] = spline4(xn, F + indx, px);
        }
        Y2[ik] = spline4(yn, Y1, py);
    }
    return spline4(zn, Y2, pz);
}

/* EFXInterp / BFXInterp into slot `base` of ef0[2][NComp][nr] */
static void rx_spatial(orc_sim *S, int itx, int efield, int slot) {
    const orc_tx *T = &S->tx[itx];
    int nr = T->nr, base = slot * S->NComp * nr;
    int c0 = efield ? 0 : 3, pos = efield ? 0 : S->nefcmp;
    for (int c = c0; c < c0 + 3; c++) {
        if (!S->isComp[c]) continue;
        for (int r = 0; r < nr; r++) S->ef0[base + pos * nr + r] = orc_rx_interp(S, c, T->rxnum[r] - 1);
        pos++;
    }
}
static void rx_time(orc_sim *S, int itx, int efield, int isample, double l0, double l1) {
    const orc_tx *T = &S->tx[itx];
    int nr = T->nr, NC = S->NComp;
    int c0 = efield ? 0 : S->nefcmp, c1 = efield ? S->nefcmp : NC;
    for (int r = 0; r < nr; r++)
        for (int c = c0; c < c1; c++)
            S->efs[(size_t)r * NC * S->Nt + (size_t)c * S->Nt + isample] = l0 * S->ef0[c * nr + r] + l1 * S->ef0[NC * nr + c * nr + r];
}

/* EFInterp2Rx host state machine, EFInterp2Rx.cu:472-585 */
static void rx_step(orc_sim *S, int itx, int *ne, int *nb, double t0, double dt, double Tp[2][3]) {
    const double *T = S->times;
    const int Nt = S->Nt;
    if (*ne < Nt) {
        Tp[0][2] = t0;
        if (T[*ne] <= Tp[0][0])
            while (*ne < Nt && T[*ne] <= Tp[0][0]) (*ne)++;
        if (*ne < Nt && T[*ne] <= Tp[0][2] && T[*ne] > Tp[0][1]) {
            rx_spatial(S, itx, 1, 0);
        } else if (*ne < Nt && T[*ne] <= Tp[0][1] && T[*ne] > Tp[0][0]) {
            rx_spatial(S, itx, 1, 1);
            while (*ne < Nt && T[*ne] <= Tp[0][1]) {
                double l1 = (T[*ne] - Tp[0][0]) / (Tp[0][1] - Tp[0][0]);
                rx_time(S, itx, 1, *ne, 1.0 - l1, l1);
                (*ne)++;
            }
        }
        Tp[0][0] = Tp[0][1];
        Tp[0][1] = Tp[0][2];
    }
    if (*nb < Nt && (S->isComp[3] || S->isComp[4] || S->isComp[5])) {
        Tp[1][2] = t0 + 0.5 * dt;
        if (T[*nb] <= Tp[1][0])
            while (*nb < Nt && T[*nb] <= Tp[1][0]) (*nb)++;
        if (*nb < Nt && T[*nb] <= Tp[1][2] && T[*nb] > Tp[1][1]) {
            rx_spatial(S, itx, 0, 0);
        } else if (*nb < Nt && T[*nb] <= Tp[1][1] && T[*nb] > Tp[1][0]) {
            rx_spatial(S, itx, 0, 1);
            while (*nb < Nt && T[*nb] <= Tp[1][1]) {
                double l1 = (T[*nb] - Tp[1][0]) / (Tp[1][1] - Tp[1][0]);
                rx_time(S, itx, 0, *nb, 1.0 - l1, l1);
                (*nb)++;
            }
        }
        Tp[1][0] = Tp[1][1];
        Tp[1][1] = Tp[1][2];
    }
}

/* ------------------------------------------------------------ step loop */

/* One transmitter, main.cu:195-298, with the per-transmitter state reset that
 * the reference omits (it is only well defined for the first transmitter).
 * traces: [nr][NComp][Nt].  max_steps < 0 runs to completion.  Returns the
 * number of steps taken. */
long orc_run(orc_sim *S, int itx, double *traces, long max_steps) {
    const orc_tx *Tx = &S->tx[itx];
    size_t ntr = (size_t)Tx->nr * S->NComp * S->Nt;
    free(S->ef0); free(S->efs);
    S->ef0 = dalloc((size_t)2 * S->NComp * Tx->nr);
    S->efs = dalloc(ntr);
    orc_zero_fields(S);
    const double mu = S->mu0, mindx = S->mindx;
    double Tp[2][3] = {{0}};
    int ne = 0, nb = 0, n = 0;
    double toT = 0, dt1 = S->dtw[0], dt2 = S->dtw[1];
    Tp[0][1] = toT + dt1;
    Tp[1][1] = toT + dt1 + 0.5 * dt2;
    long steps = 0;
    while (ne < S->Nt || (nb < S->Nt && S->nefcmp < S->NComp)) {
        if (max_steps >= 0 && steps >= max_steps) break;
        double nmuda = 7.5 * S->sfa2 * dt2 * dt1 / mu / mindx / mindx;
        if (S->padded_plane > 0) orc_upcontinuation_padded(S);
        else orc_upcontinuation(S);
        orc_electric_field(S, itx, nmuda, dt1, n < 2 * S->nsrc ? S->wave[n] : 0);
        orc_bderivate(S, 0.5 * (dt1 + dt2));
        toT += dt1;
        dt1 = dt2;
        n++;
        if (n < 2 * S->nsrc) dt2 = S->dtw[n + 1];
        else dt2 = fmin(0.15 * S->sfa1 * sqrt(mu * toT * S->minsita / 8.) * mindx, 1.2 * dt1);
        rx_step(S, itx, &ne, &nb, toT + dt1, dt2, Tp);
        steps++;
    }
    if (traces) memcpy(traces, S->efs, ntr * sizeof(double));
    return steps;
}

/* The host schedule alone (no field work): per step dt1, dt2, nmuda, wave.
 * Returns the number of steps; arrays may be NULL to count only. */
long orc_schedule(orc_sim *S, double *dt1_out, double *dt2_out, double *lam_out, double *wave_out, long cap) {
    const double mu = S->mu0, mindx = S->mindx;
    double Tp[2][3] = {{0}};
    int ne = 0, nb = 0, n = 0;
    double toT = 0, dt1 = S->dtw[0], dt2 = S->dtw[1];
    Tp[0][1] = toT + dt1;
    Tp[1][1] = toT + dt1 + 0.5 * dt2;
    long steps = 0;
    /* rx_step without field work: reuse the state machine with a dummy slot buffer */
    free(S->ef0); free(S->efs);
    S->ef0 = dalloc((size_t)2 * S->NComp * S->tx[0].nr);
    S->efs = dalloc((size_t)S->tx[0].nr * S->NComp * S->Nt);
    while (ne < S->Nt || (nb < S->Nt && S->nefcmp < S->NComp)) {
        if (steps < cap) {
            if (dt1_out) dt1_out[steps] = dt1;
            if (dt2_out) dt2_out[steps] = dt2;
            if (lam_out) lam_out[steps] = 7.5 * S->sfa2 * dt2 * dt1 / mu / mindx / mindx;
            if (wave_out) wave_out[steps] = n < 2 * S->nsrc ? S->wave[n] : 0;
        }
        toT += dt1;
        dt1 = dt2;
        n++;
        if (n < 2 * S->nsrc) dt2 = S->dtw[n + 1];
        else dt2 = fmin(0.15 * S->sfa1 * sqrt(mu * toT * S->minsita / 8.) * mindx, 1.2 * dt1);
        /* state machine only: mimic rx_step without interpolation */
        const double *T = S->times; const int Nt = S->Nt;
        double t0 = toT + dt1;
        if (ne < Nt) {
            Tp[0][2] = t0;
            while (ne < Nt && T[ne] <= Tp[0][0]) ne++;
            if (ne < Nt && T[ne] <= Tp[0][2] && T[ne] > Tp[0][1]) { }
            else if (ne < Nt && T[ne] <= Tp[0][1] && T[ne] > Tp[0][0]) { while (ne < Nt && T[ne] <= Tp[0][1]) ne++; }
            Tp[0][0] = Tp[0][1]; Tp[0][1] = Tp[0][2];
        }
        if (nb < Nt && (S->isComp[3] || S->isComp[4] || S->isComp[5])) {
            Tp[1][2] = t0 + 0.5 * dt2;
            while (nb < Nt && T[nb] <= Tp[1][0]) nb++;
            if (nb < Nt && T[nb] <= Tp[1][2] && T[nb] > Tp[1][1]) { }
            else if (nb < Nt && T[nb] <= Tp[1][1] && T[nb] > Tp[1][0]) { while (nb < Nt && T[nb] <= Tp[1][1]) nb++; }
            Tp[1][0] = Tp[1][1]; Tp[1][1] = Tp[1][2];
        }
        steps++;
    }
    return steps;
}

const char *orc_version(void) { return "tcsem-oracle-1"; }

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
