/*
 * Timing driver of the reference's CPU spline remap.  TEST INFRASTRUCTURE (the CPU
 * baseline of bench.py): it links, unmodified, the reference's host setup files and
 * SplineGridConvIR2R_cpu.cpp (compiled from the reference tree by oracle/build_ref.py),
 * sets a survey up as main.cu:93-146 does, fills the top Bz plane with seeded values and
 * times `reps` calls of SplineGridConvIR2R_cpu (SplineGridConvIR2R_cpu.cpp:7-691, the
 * remap of the reference's FFTW flavour; OpenMP threads from OMP_NUM_THREADS).
 * Prints one line: "<L1> <M1> <threads> <reps> <seconds per call> <checksum>".
 * Usage: ref_cpu_remap <input-dir> <reps>   (runs inside <input-dir>)
 */
#include <omp.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unistd.h>

#include "FTDT.h"

double miu = 4 * PI * 1.e-7; /* main.cu:55 */
int MAXTHREAD = 1;

int main(int argc, char **argv) {
    if (argc != 3) { fprintf(stderr, "usage: ref_cpu_remap <dir> <reps>\n"); return 2; }
    const int reps = atoi(argv[2]);
    if (reps < 1 || chdir(argv[1])) { perror("args"); return 2; }
    MAXTHREAD = omp_get_max_threads();
    ModelPara MP; ModelGrid MG; GridConv GC;
    memset(&MP, 0, sizeof MP); memset(&MG, 0, sizeof MG); memset(&GC, 0, sizeof GC);
    double ***Con0, sfa1, sfa2, sita_t = 5e-4, minsita = 0.1; int Nsrc = 100;
    if (ModelingSetup(&Con0, &MP, &MG, &sfa1, &sfa2, &sita_t, &Nsrc, &minsita)) return 3;
    const int L = MP.L, M = MP.M;
    const int L1 = MP.AnLx_New + MP.AnRx_New + MP.Nx, M1 = 2 * MP.Any_New + MP.Ny;
    MG.X_BzNew = (double *)malloc(L1 * sizeof(double)); MG.Y_BzNew = (double *)malloc(M1 * sizeof(double));
    GC.xBzNew2old = (int *)malloc(L1 * sizeof(int)); GC.yBzNew2old = (int *)malloc(M1 * sizeof(int));
    GC.xBzold2New = (int *)malloc(L * sizeof(int)); GC.yBzold2New = (int *)malloc(M * sizeof(int));
    GC.xoldBx2NewBz = (int *)malloc((L + 1) * sizeof(int)); GC.yoldBy2NewBz = (int *)malloc((M + 1) * sizeof(int));
    ModelGridMapping(&MP, &MG, &GC);
    double **Fold = Create2DArray(M, L), **Fnew = Create2DArray(M1, L1);
    unsigned s = 12345u;
    for (int j = 0; j < M; j++)
        for (int i = 0; i < L; i++) {
            s = s * 1664525u + 1013904223u;
            Fold[j][i] = (double)(s >> 8) / 16777216.0 - 0.5;
        }
    SplineGridConvIR2R_cpu(&MP, &MG, &GC, Fold, Fnew); /* first touch */
    const double t0 = omp_get_wtime();
    for (int r = 0; r < reps; r++) SplineGridConvIR2R_cpu(&MP, &MG, &GC, Fold, Fnew);
    const double dt = (omp_get_wtime() - t0) / reps;
    double sum = 0;
    for (int j = 0; j < M1; j++)
        for (int i = 0; i < L1; i++) sum += Fnew[j][i];
    printf("%d %d %d %d %.9f %.17g\n", L1, M1, MAXTHREAD, reps, dt, sum);
    return 0;
}
