/*
 * Golden-vector driver for the reference's host setup code.  TEST
 * INFRASTRUCTURE: it links, unmodified, the reference's ModelingSetup.cpp,
 * SourceWave.cpp, ModelGridMapping.cpp, LoadRxTxPos.cpp, logspace.cpp and
 * AuxiliaryMemory.cpp (compiled from the reference tree by
 * oracle/build_ref.py) and calls them in the order of main.cu:93-146, then
 * writes every array they produce to a flat binary record file:
 *   repeated { int32 name_len; char name[name_len]; char kind ('d'|'i');
 *              int32 count; payload }
 * Usage: ref_host <input-dir> <output-file>   (runs inside <input-dir>)
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <unistd.h>
#include "FTDT.h"

double miu = 4 * PI * 1.e-7; /* main.cu:55 */
int MAXTHREAD = 1;

static FILE *g_out;
static void put(const char *name, const double *p, int n) {
    int l = (int)strlen(name);
    fwrite(&l, 4, 1, g_out); fwrite(name, 1, l, g_out);
    char k = 'd'; fwrite(&k, 1, 1, g_out); fwrite(&n, 4, 1, g_out); fwrite(p, 8, n, g_out);
}
static void puti(const char *name, const int *p, int n) {
    int l = (int)strlen(name);
    fwrite(&l, 4, 1, g_out); fwrite(name, 1, l, g_out);
    char k = 'i'; fwrite(&k, 1, 1, g_out); fwrite(&n, 4, 1, g_out); fwrite(p, 4, n, g_out);
}

int main(int argc, char **argv) {
    if (argc != 3) { fprintf(stderr, "usage: ref_host <dir> <out>\n"); return 2; }
    char outpath[4096];
    if (argv[2][0] == '/') snprintf(outpath, sizeof outpath, "%s", argv[2]);
    else { char cwd[2048]; if (!getcwd(cwd, sizeof cwd)) return 2; snprintf(outpath, sizeof outpath, "%s/%s", cwd, argv[2]); }
    if (chdir(argv[1])) { perror("chdir"); return 2; }
    ModelPara MP; ModelGrid MG; GridConv GC; RxTime tRx; RxPos xyzRx; TxPos *xyzTx; int NRx, NTx;
    memset(&MP, 0, sizeof MP); memset(&MG, 0, sizeof MG); memset(&GC, 0, sizeof GC);
    double ***Con0, sfa1, sfa2, sita_t = 5e-4, minsita = 0.1; int Nsrc = 100;
    if (ModelingSetup(&Con0, &MP, &MG, &sfa1, &sfa2, &sita_t, &Nsrc, &minsita)) return 3;
    int L = MP.L, M = MP.M, N = MP.N;
    int L1 = MP.AnLx_New + MP.AnRx_New + MP.Nx, M1 = 2 * MP.Any_New + MP.Ny;
    double *Wave = (double *)calloc(2 * Nsrc + 1, sizeof(double));
    double *dt = (double *)calloc(2 * Nsrc + 2, sizeof(double)); /* zeroed, see SourceWave.cpp:52 */
    Waveform(Nsrc, sita_t, dt, Wave);
    MG.X_BzNew = (double *)malloc(L1 * sizeof(double)); MG.Y_BzNew = (double *)malloc(M1 * sizeof(double));
    GC.xBzNew2old = (int *)malloc(L1 * sizeof(int)); GC.yBzNew2old = (int *)malloc(M1 * sizeof(int));
    GC.xBzold2New = (int *)malloc(L * sizeof(int)); GC.yBzold2New = (int *)malloc(M * sizeof(int));
    GC.xoldBx2NewBz = (int *)malloc((L + 1) * sizeof(int)); GC.yoldBy2NewBz = (int *)malloc((M + 1) * sizeof(int));
    ModelGridMapping(&MP, &MG, &GC);
    if (LoadRxTxPos(MP, MG, &tRx, &xyzRx, &xyzTx, &NRx, &NTx)) return 4;
    g_out = fopen(outpath, "wb");
    if (!g_out) { perror("open out"); return 2; }
    int dims[] = {L, M, N, L1, M1, MP.AnLx_New, MP.AnRx_New, MP.Any_New, NRx, NTx, tRx.Nt, tRx.NComp, tRx.nefcmp, Nsrc, tRx.IsLog, MP.LNx2, MP.LMy2};
    puti("dims", dims, 17);
    double par[] = {sfa1, sfa2, sita_t, minsita, miu, tRx.T0, tRx.Tn};
    put("params", par, 7);
    /* the whole ModelPara record, fields in declaration order (FTDT.h:78-110), for drivers of
     * the reference's device code */
    int mpi[] = {MP.AnLx_old, MP.AnRx_old, MP.Any_old, MP.Anz, MP.ALx1, MP.ALx2, MP.ARx1, MP.ARx2,
                 MP.Ay1, MP.Ay2, MP.Az1, MP.Az2, MP.L, MP.M, MP.N, MP.Nx, MP.Ny, MP.Nz,
                 MP.AnLx_New, MP.AnRx_New, MP.Any_New, MP.LNx2, MP.LMy2};
    puti("mp_i", mpi, 23);
    double mpd[] = {MP.dxmin, MP.dymin, MP.dzmin, MP.arg1, MP.arg2};
    put("mp_d", mpd, 5);
    put("dx", MG.dx, L); put("dy", MG.dy, M); put("dz", MG.dz, N);
    put("X", MG.X_Bzold, L); put("Y", MG.Y_Bzold, M); put("Z", MG.Z, N);
    put("Xn", MG.X_BzNew, L1); put("Yn", MG.Y_BzNew, M1);
    puti("xBzNew2old", GC.xBzNew2old, L1); puti("yBzNew2old", GC.yBzNew2old, M1);
    puti("xBzold2New", GC.xBzold2New, L); puti("yBzold2New", GC.yBzold2New, M);
    puti("xoldBx2NewBz", GC.xoldBx2NewBz, L + 1); puti("yoldBy2NewBz", GC.yoldBy2NewBz, M + 1);
    put("dtw", dt, 2 * Nsrc + 2); put("wave", Wave, 2 * Nsrc + 1);
    put("times", tRx.Times, tRx.Nt);
    puti("isComp", tRx.isComp, 6);
    put("rx", xyzRx.x, NRx); put("ry", xyzRx.y, NRx); put("rz", xyzRx.z, NRx);
    puti("rix", xyzRx.ix, NRx); puti("riy", xyzRx.iy, NRx); puti("riz", xyzRx.iz, NRx);
    for (int t = 0; t < NTx; t++) {
        TxPos *T = &xyzTx[t];
        int iv[20] = {T->ort, T->nr, T->ixa, T->iya, T->iza, T->ixb, T->iyb, T->izb, T->ictx, T->icty, T->ictz,
                      T->ixa1, T->iya1, T->iza1, T->ixb1, T->iyb1, T->izb1, T->ictx1, T->icty1, T->ictz1};
        /* indices the reference leaves unset for a given orientation are reported as -1 */
        if (T->ort == 1) { iv[3] = iv[4] = iv[6] = iv[7] = iv[8] = -1; }
        if (T->ort == 2) { iv[2] = iv[4] = iv[5] = iv[7] = iv[9] = -1; }
        if (T->ort == 3) { iv[2] = iv[3] = iv[5] = iv[6] = iv[10] = -1; }
        if (T->ort != 5) for (int q = 11; q < 20; q++) iv[q] = -1;
        double dv[12] = {T->BipoLen, T->x, T->y, T->z, T->azi, T->dip, T->BipoLen1, T->x1, T->y1, T->z1, T->azi1, T->dip1};
        if (T->ort < 4) { dv[4] = dv[5] = 0; }
        if (T->ort != 5) for (int q = 6; q < 12; q++) dv[q] = 0;
        char nm[64];
        snprintf(nm, sizeof nm, "tx%d_i", t); puti(nm, iv, 20);
        snprintf(nm, sizeof nm, "tx%d_d", t); put(nm, dv, 12);
        snprintf(nm, sizeof nm, "tx%d_rx", t); puti(nm, T->RxNum, T->nr);
    }
    fclose(g_out);
    return 0;
}
