/*
 * Driver of the reference's own CUDA kernels.  TEST INFRASTRUCTURE: it
 * produces the reference's receiver traces on a GPU so that the oracle and the
 * product can be checked against numbers the reference itself computed.
 *
 * What runs is the reference's device code, unmodified: oracle/build_ref.py
 * compiles ElectricalFiled.cu, Bderivate.cu, SplineGridConvIR2R.cu,
 * UpContinuation_gpu.cu, EFInterp2Rx.cu and initialize_UpCont_gpu_resources.cu
 * from the reference tree (FP64, the reference's default) into device-only
 * modules (oracle/_ref/*.cubin).  This file is the host side: it loads those
 * modules with the CUDA driver API and issues, in the reference's order and
 * with the reference's launch shapes, the launches and library calls of
 *   main.cu:195-273            the step loop of one transmitter,
 *   UpContinuation_gpu.cu:166-274 / SplineGridConvIR2R.cu:539-752
 *                              the air boundary (cuSPARSE gtsv2_nopivot, cuFFT),
 *   ElectricalFiled.cu:478-655 the E update and source injection,
 *   Bderivate.cu:269-316       the B update,
 *   EFInterp2Rx.cu:410-585     the receiver sampling state machine,
 * with the allocations of prepare_free_mem.cu:45-186, initialize_fft.cu:43-120
 * and initialize_UpCont_gpu_resources.cu:146-275.  Everything goes to one
 * stream in program order, which is what the reference's build does: it
 * synchronises the device after every kernel (Cuda_device.h:73-78).  The setup
 * arrays (grid, maps, receiver and transmitter cells, waveform) are the ones
 * the reference's host code produced (oracle/ref_host_driver.cpp).
 *
 * Records passed to the kernels keep the reference's field order (FTDT.h:62-262),
 * because the device code reads them by offset.
 *
 * Only the first transmitter of a survey is defined in the reference (its step
 * counters and trace buffer carry over between transmitters, main.cu:76-78,207),
 * so the caller runs one transmitter from a zero state; the trace buffer is
 * zeroed first (the reference leaves it uninitialised, main.cu:207).
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <cusparse.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

// ---------------------------------------------------------------- records
// ModelPara, FTDT.h:78-110 (MP_VER_1 layout)
struct RModelPara {
    int AnLx_old, AnRx_old, Any_old, Anz;
    int ALx1, ALx2, ARx1, ARx2, Ay1, Ay2, Az1, Az2;
    int L, M, N;
    int Nx, Ny, Nz, AnLx_New, AnRx_New, Any_New, LNx2, LMy2;
    double dxmin, dymin, dzmin, arg1, arg2;
};
// ModelGrid, FTDT.h:112-121
struct RModelGrid {
    double *dx, *dy, *dz, *Z, *X_Bzold, *Y_Bzold, *X_BzNew, *Y_BzNew;
};
// TriDiagM, FTDT.h:150-154
struct RTriDiag {
    double *dl, *du, *d;
};
// GridConv, FTDT.h:193-200
struct RGridConv {
    int *xBzNew2old, *yBzNew2old, *xBzold2New, *yBzold2New, *xoldBx2NewBz, *yoldBy2NewBz;
};
// RxPos, FTDT.h:216-223
struct RRxPos {
    double *x, *y, *z;
    int *ix, *iy, *iz;
};
// TxPos, FTDT.h:226-262
struct RTxPos {
    int ort, nr;
    double BipoLen, x, y, z, azi, dip;
    int ixa, iya, iza, ixb, iyb, izb, ictx, icty, ictz;
    double BipoLen1, x1, y1, z1, azi1, dip1;
    int ixa1, iya1, iza1, ixb1, iyb1, izb1, ictx1, icty1, ictz1;
    int *RxNum;
};

// launch shapes of the reference build, Cuda_device.h:222-226 and FTDT.h:40
constexpr int BLOCKSIZE1 = 128, BLOCKSIZE2x = 16, BLOCKSIZE2y1 = 8, BLOCKSIZE2y2 = 16, BLOCKSIZE3 = 128;
constexpr int NPAD = 4;

struct Fail {
    std::string msg;
};
[[noreturn]] void fail(const char *fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof b, fmt, ap);
    va_end(ap);
    throw Fail{b};
}
void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) fail("%s: %s", what, cudaGetErrorString(e));
}
void ckd(CUresult e, const char *what) {
    if (e != CUDA_SUCCESS) {
        const char *s = nullptr;
        cuGetErrorString(e, &s);
        fail("%s: %s", what, s ? s : "?");
    }
}
void ckf(cufftResult e, const char *what) {
    if (e != CUFFT_SUCCESS) fail("%s: cufft error %d", what, (int)e);
}
void cks(cusparseStatus_t e, const char *what) {
    if (e != CUSPARSE_STATUS_SUCCESS) fail("%s: cusparse error %d", what, (int)e);
}

// device memory owned by the run
struct Pool {
    std::vector<void *> ptrs;
    ~Pool() {
        for (void *p : ptrs) cudaFree(p);
    }
    template <class T> T *alloc(size_t n, bool zero = true) {
        void *p = nullptr;
        ck(cudaMalloc(&p, (n ? n : 1) * sizeof(T)), "cudaMalloc");
        ptrs.push_back(p);
        if (zero) ck(cudaMemset(p, 0, (n ? n : 1) * sizeof(T)), "cudaMemset");
        return static_cast<T *>(p);
    }
    template <class T> T *upload(const T *h, size_t n) {
        T *d = alloc<T>(n, false);
        if (n) ck(cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice), "upload");
        return d;
    }
};

// the reference's kernels, looked up by name in the loaded modules
struct Kernels {
    std::vector<CUmodule> mods;
    std::map<std::string, CUfunction> fn;
    ~Kernels() {
        for (CUmodule m : mods) cuModuleUnload(m);
    }
    void load(const std::string &dir, const char *file) {
        CUmodule m;
        std::string p = dir + "/" + file;
        ckd(cuModuleLoad(&m, p.c_str()), p.c_str());
        mods.push_back(m);
        unsigned n = 0;
        ckd(cuModuleGetFunctionCount(&n, m), "cuModuleGetFunctionCount");
        std::vector<CUfunction> fs(n);
        ckd(cuModuleEnumerateFunctions(fs.data(), n, m), "cuModuleEnumerateFunctions");
        for (CUfunction f : fs) {
            const char *nm = nullptr;
            ckd(cuFuncGetName(&nm, f), "cuFuncGetName");
            // Itanium-mangled "_Z<len><name>..." -> name
            std::string s(nm);
            if (s.size() > 2 && s[0] == '_' && s[1] == 'Z') {
                size_t q = 2, len = 0;
                while (q < s.size() && isdigit((unsigned char)s[q])) len = len * 10 + (s[q++] - '0');
                s = s.substr(q, len);
            }
            if (fn.count(s)) fail("kernel %s defined twice", s.c_str());
            fn[s] = f;
        }
    }
    CUfunction get(const char *name) const {
        auto it = fn.find(name);
        if (it == fn.end()) fail("kernel %s not found in the reference modules", name);
        return it->second;
    }
};

// one launch: argument values copied into a byte buffer, pointers to them passed
struct Args {
    std::vector<std::vector<unsigned char>> vals;
    template <class T> Args &operator<<(const T &v) {
        std::vector<unsigned char> b(sizeof(T));
        std::memcpy(b.data(), &v, sizeof(T));
        vals.push_back(std::move(b));
        return *this;
    }
};
void launch(const Kernels &K, const char *name, dim3 g, dim3 b, Args &a, cudaStream_t st) {
    std::vector<void *> pp;
    for (auto &v : a.vals) pp.push_back(v.data());
    ckd(cuLaunchKernel(K.get(name), g.x, g.y, g.z, b.x, b.y, b.z, 0, (CUstream)st, pp.data(), nullptr), name);
}

}  // namespace

extern "C" {

// Inputs of one run: the reference host code's setup arrays and the model.
typedef struct {
    int mp_i[23];     // ModelPara integer fields, declaration order
    double mp_d[5];   // dxmin dymin dzmin arg1 arg2
    const double *dx, *dy, *dz, *Z, *X, *Y, *Xn, *Yn;
    const int *xBzNew2old, *yBzNew2old, *xBzold2New, *yBzold2New, *xoldBx2NewBz, *yoldBy2NewBz;
    const double *con;  // [N][M][L]
    int NRx;
    const double *rx, *ry, *rz;
    const int *rix, *riy, *riz;
    int Nt, NComp, nefcmp;
    int isComp[6];
    const double *times;
    int nsrc;
    const double *dtw, *wave;  // 2 nsrc + 2 and 2 nsrc + 1 values (SourceWave.cpp)
    double sfa1, sfa2, minsita, miu;
    int tx_i[20];  // ort nr ixa iya iza ixb iyb izb ictx icty ictz ixa1 .. ictz1
    double tx_d[12];  // BipoLen x y z azi dip BipoLen1 x1 y1 z1 azi1 dip1
    const int *rxnum;  // the transmitter's receiver ids (1-based)
} refgpu_inputs;

// Runs the first `max_steps` steps (all when negative) of one transmitter with the
// reference's kernels; traces [nr][NComp][Nt].  Returns 0, or 1 with a message in err.
int refgpu_run(const char *cubin_dir, const refgpu_inputs *in, double *traces, long max_steps, long *steps_out,
               double *loop_ms, char *err, int errlen) {
    try {
        ck(cudaFree(0), "context");
        Kernels K;
        for (const char *f : {"ElectricalFiled.cubin", "Bderivate.cubin", "SplineGridConvIR2R.cubin",
                              "UpContinuation_gpu.cubin", "EFInterp2Rx.cubin", "initialize_UpCont_gpu_resources.cubin"})
            K.load(cubin_dir, f);

        RModelPara mp;
        int *mi = &mp.AnLx_old;
        for (int q = 0; q < 23; q++) mi[q] = in->mp_i[q];
        mp.dxmin = in->mp_d[0]; mp.dymin = in->mp_d[1]; mp.dzmin = in->mp_d[2];
        mp.arg1 = in->mp_d[3]; mp.arg2 = in->mp_d[4];
        const int L = mp.L, M = mp.M, N = mp.N;
        const int L1 = mp.AnLx_New + mp.AnRx_New + mp.Nx, M1 = 2 * mp.Any_New + mp.Ny;
        const int n1 = mp.ALx1 + mp.ALx2 + NPAD, n2 = mp.ARx1 + mp.ARx2 + NPAD, n3 = mp.Ay1 + mp.Ay2 + NPAD;
        if (n1 > BLOCKSIZE3 || n2 > BLOCKSIZE3 || n3 > BLOCKSIZE3) fail("boundary strips exceed BLOCKSIZE3");
        if (L < 4 || M < 4 || N < 4) fail("grid too small");

        RTxPos tx;
        std::memset(&tx, 0, sizeof tx);
        const int *ti = in->tx_i;
        auto nz = [](int v) { return v < 0 ? 0 : v; };  // fields the orientation leaves unset
        tx.ort = ti[0]; tx.nr = ti[1];
        tx.ixa = nz(ti[2]); tx.iya = nz(ti[3]); tx.iza = nz(ti[4]);
        tx.ixb = nz(ti[5]); tx.iyb = nz(ti[6]); tx.izb = nz(ti[7]);
        tx.ictx = nz(ti[8]); tx.icty = nz(ti[9]); tx.ictz = nz(ti[10]);
        tx.ixa1 = nz(ti[11]); tx.iya1 = nz(ti[12]); tx.iza1 = nz(ti[13]);
        tx.ixb1 = nz(ti[14]); tx.iyb1 = nz(ti[15]); tx.izb1 = nz(ti[16]);
        tx.ictx1 = nz(ti[17]); tx.icty1 = nz(ti[18]); tx.ictz1 = nz(ti[19]);
        const double *td = in->tx_d;
        tx.BipoLen = td[0]; tx.x = td[1]; tx.y = td[2]; tx.z = td[3]; tx.azi = td[4]; tx.dip = td[5];
        tx.BipoLen1 = td[6]; tx.x1 = td[7]; tx.y1 = td[8]; tx.z1 = td[9]; tx.azi1 = td[10]; tx.dip1 = td[11];
        const int nr = tx.nr;
        const int Nt = in->Nt, NComp = in->NComp, nefcmp = in->nefcmp;

        Pool P;
        cudaStream_t st;
        ck(cudaStreamCreate(&st), "stream");
        struct StreamGuard {
            cudaStream_t s;
            ~StreamGuard() { cudaStreamDestroy(s); }
        } sg{st};

        // ---- prepare_free_mem.cu:63-160
        double *Ex = P.alloc<double>((size_t)L * (M + 1) * (N + 1));
        double *Ey = P.alloc<double>((size_t)(L + 1) * M * (N + 1));
        double *Ez = P.alloc<double>((size_t)(L + 1) * (M + 1) * N);
        double *Bx = P.alloc<double>((size_t)(L + 1) * M * N);
        double *By = P.alloc<double>((size_t)L * (M + 1) * N);
        double *Bz = P.alloc<double>((size_t)L * M * (N + 1));
        double *BxAir = nullptr, *ByAir = nullptr;
        size_t BxPitch = 0, ByPitch = 0;
        ck(cudaMallocPitch((void **)&BxAir, &BxPitch, (L + 1) * sizeof(double), M), "BxAir");
        P.ptrs.push_back(BxAir);
        ck(cudaMallocPitch((void **)&ByAir, &ByPitch, L * sizeof(double), M + 1), "ByAir");
        P.ptrs.push_back(ByAir);
        ck(cudaMemset2D(BxAir, BxPitch, 0, (L + 1) * sizeof(double), M), "BxAir zero");
        ck(cudaMemset2D(ByAir, ByPitch, 0, L * sizeof(double), M + 1), "ByAir zero");
        double *Con = P.upload(in->con, (size_t)L * M * N);
        RRxPos rxp;
        rxp.x = P.upload(in->rx, in->NRx); rxp.y = P.upload(in->ry, in->NRx); rxp.z = P.upload(in->rz, in->NRx);
        rxp.ix = P.upload(in->rix, in->NRx); rxp.iy = P.upload(in->riy, in->NRx); rxp.iz = P.upload(in->riz, in->NRx);
        int *RxLst = P.upload(in->rxnum, nr);
        RModelGrid mg;
        mg.dx = P.upload(in->dx, L); mg.dy = P.upload(in->dy, M); mg.dz = P.upload(in->dz, N);
        mg.Z = P.upload(in->Z, N); mg.X_Bzold = P.upload(in->X, L); mg.Y_Bzold = P.upload(in->Y, M);
        mg.X_BzNew = P.upload(in->Xn, L1); mg.Y_BzNew = P.upload(in->Yn, M1);
        RGridConv gc;
        gc.xBzNew2old = P.upload(in->xBzNew2old, L1); gc.yBzNew2old = P.upload(in->yBzNew2old, M1);
        gc.xBzold2New = P.upload(in->xBzold2New, L); gc.yBzold2New = P.upload(in->yBzold2New, M);
        gc.xoldBx2NewBz = P.upload(in->xoldBx2NewBz, L + 1); gc.yoldBy2NewBz = P.upload(in->yoldBy2NewBz, M + 1);
        // the records the kernels read through pointers (the reference keeps them in
        // __constant__ memory, prepare_constants_cuda.h:92-195; the values are the same)
        RModelPara *d_mp = P.upload(&mp, 1);
        RTxPos txd = tx;
        txd.RxNum = RxLst;
        RTxPos *d_Tx = P.upload(&txd, 1);

        // ---- initialize_fft.cu:103-120
        double *FBxR = P.alloc<double>((size_t)M1 * L1), *FByR = P.alloc<double>((size_t)M1 * L1);
        double *BzAir = P.alloc<double>((size_t)M1 * L1);
        const size_t H = (size_t)(L1 / 2 + 1);
        cufftDoubleComplex *FBzC = P.alloc<cufftDoubleComplex>(M1 * H);
        cufftDoubleComplex *FBxC = P.alloc<cufftDoubleComplex>(M1 * H);
        cufftDoubleComplex *FByC = P.alloc<cufftDoubleComplex>(M1 * H);
        cufftHandle plan1, plan2, plan3;
        ckf(cufftPlan2d(&plan1, M1, L1, CUFFT_D2Z), "plan1");
        ckf(cufftPlan2d(&plan2, M1, L1, CUFFT_Z2D), "plan2");
        ckf(cufftPlan2d(&plan3, M1, L1, CUFFT_Z2D), "plan3");
        struct PlanGuard {
            cufftHandle a, b, c;
            ~PlanGuard() { cufftDestroy(a); cufftDestroy(b); cufftDestroy(c); }
        } pg{plan1, plan2, plan3};
        for (cufftHandle p : {plan1, plan2, plan3}) ckf(cufftSetStream(p, st), "cufftSetStream");

        // ---- initialize_UpCont_gpu_resources.cu:160-270
        struct Tds {
            RTriDiag A;
            double *B, *semi0, *semi1;
            void *buff;
        } t0x, t1x, t0y, t1y;
        const int sx[4] = {n1, n2, n3, n3}, nrhs[4] = {M, M, L1, L1};
        Tds *tds[4] = {&t0x, &t1x, &t0y, &t1y};
        for (int q = 0; q < 4; q++) {
            tds[q]->A.dl = P.alloc<double>(sx[q]);
            tds[q]->A.du = P.alloc<double>(sx[q]);
            tds[q]->A.d = P.alloc<double>(sx[q]);
            tds[q]->B = P.alloc<double>((size_t)nrhs[q] * sx[q]);
            tds[q]->semi0 = tds[q]->semi1 = nullptr;
        }
        t0x.semi0 = P.alloc<double>((size_t)mp.AnLx_New * n3);
        t0x.semi1 = P.alloc<double>((size_t)mp.AnLx_New * n3);
        t1x.semi0 = P.alloc<double>((size_t)mp.AnRx_New * n3);
        t1x.semi1 = P.alloc<double>((size_t)mp.AnRx_New * n3);
        cusparseHandle_t sp;
        cks(cusparseCreate(&sp), "cusparseCreate");
        struct SpGuard {
            cusparseHandle_t h;
            ~SpGuard() { cusparseDestroy(h); }
        } spg{sp};
        cks(cusparseSetStream(sp, st), "cusparseSetStream");
        for (int q = 0; q < 4; q++) {
            size_t bs = 0;
            cks(cusparseDgtsv2_nopivot_bufferSizeExt(sp, sx[q], nrhs[q], tds[q]->A.dl, tds[q]->A.d, tds[q]->A.du,
                                                     tds[q]->B, sx[q], &bs),
                "gtsv2 buffer size");
            tds[q]->buff = P.alloc<unsigned char>(bs);
        }
        {
            const char *fills[4] = {"fillA0x", "fillA1x", "fillA0y", "fillA1y"};
            for (int q = 0; q < 4; q++) {
                Args a;
                a << tds[q]->A << d_mp << mg;
                launch(K, fills[q], dim3((sx[q] + BLOCKSIZE3 - 1) / BLOCKSIZE3), dim3(BLOCKSIZE3), a, st);
            }
        }

        double *efs = P.alloc<double>((size_t)nr * NComp * Nt);
        double *ef0 = P.alloc<double>((size_t)nr * NComp * 2);

        // ---- boundary, UpContinuation_gpu.cu:166-274 with SplineGridConvIR2R.cu:539-752
        auto upcontinuation = [&]() {
            const dim3 t16(BLOCKSIZE2x, BLOCKSIZE2y2);
            {
                Args a;
                a << Bz << BzAir << d_mp;
                launch(K, "Intep_BzIR2R_cpy_center", dim3((mp.Nx + 15) / 16, (mp.Ny + 15) / 16), t16, a, st);
            }
            {
                Args a;
                a << Bz << t0x.B << d_mp << mg;
                launch(K, "Fill_B_0x", dim3(M), dim3(n1 <= BLOCKSIZE3 / 2 ? BLOCKSIZE3 / 2 : BLOCKSIZE3), a, st);
            }
            {
                Args a;
                a << Bz << t1x.B << d_mp << mg;
                launch(K, "Fill_B_1x", dim3(M), dim3(n2 <= BLOCKSIZE3 / 2 ? BLOCKSIZE3 / 2 : BLOCKSIZE3), a, st);
            }
            cks(cusparseDgtsv2_nopivot(sp, n1, M, t0x.A.dl, t0x.A.d, t0x.A.du, t0x.B, n1, t0x.buff), "gtsv 0x");
            cks(cusparseDgtsv2_nopivot(sp, n2, M, t1x.A.dl, t1x.A.d, t1x.A.du, t1x.B, n2, t1x.buff), "gtsv 1x");
            {
                Args a;
                a << Bz << t0x.semi0 << BzAir << t0x.semi1 << t0x.B << d_mp << mg << gc.xBzNew2old;
                launch(K, "Intep_BzIR2R_0x", dim3((mp.AnLx_New + 2 * BLOCKSIZE3 - 1) / (2 * BLOCKSIZE3), M),
                       dim3(2 * BLOCKSIZE3), a, st);
            }
            {
                Args a;
                a << Bz << t1x.semi0 << BzAir << t1x.semi1 << t1x.B << d_mp << mg << gc.xBzNew2old;
                launch(K, "Intep_BzIR2R_1x", dim3((mp.AnRx_New + 2 * BLOCKSIZE3 - 1) / (2 * BLOCKSIZE3), M),
                       dim3(2 * BLOCKSIZE3), a, st);
            }
            const dim3 b3(n3 <= BLOCKSIZE3 / 2 ? BLOCKSIZE3 / 2 : BLOCKSIZE3);
            {
                Args a;
                a << Bz << t0x.semi0 << t1x.semi0 << t0y.B << d_mp << mg;
                launch(K, "Fill_B_0y", dim3(L1), b3, a, st);
            }
            {
                Args a;
                a << Bz << t0x.semi1 << t1x.semi1 << t1y.B << d_mp << mg;
                launch(K, "Fill_B_1y", dim3(L1), b3, a, st);
            }
            cks(cusparseDgtsv2_nopivot(sp, n3, L1, t0y.A.dl, t0y.A.d, t0y.A.du, t0y.B, n3, t0y.buff), "gtsv 0y");
            cks(cusparseDgtsv2_nopivot(sp, n3, L1, t1y.A.dl, t1y.A.d, t1y.A.du, t1y.B, n3, t1y.buff), "gtsv 1y");
            const dim3 g0y((mp.Any_New + 2 * BLOCKSIZE3 - 1) / (2 * BLOCKSIZE3), L1);
            {
                Args a;
                a << Bz << t0x.semi0 << BzAir << t1x.semi0 << t0y.B << d_mp << mg << gc.yBzNew2old;
                launch(K, "Intep_BzIR2R_0y", g0y, dim3(2 * BLOCKSIZE3), a, st);
            }
            {
                Args a;
                a << Bz << t0x.semi1 << BzAir << t1x.semi1 << t1y.B << d_mp << mg << gc.yBzNew2old;
                launch(K, "Intep_BzIR2R_1y", g0y, dim3(2 * BLOCKSIZE3), a, st);
            }
            ckf(cufftExecD2Z(plan1, BzAir, FBzC), "D2Z");
            {
                Args a;
                a << FBzC << FBxC << FByC << d_mp;
                launch(K, "FBz_to_FBxFBy", dim3((L1 / 2 + 1 + 15) / 16, (M1 + 15) / 16), t16, a, st);
            }
            ckf(cufftExecZ2D(plan2, FBxC, FBxR), "Z2D x");
            ckf(cufftExecZ2D(plan3, FByC, FByR), "Z2D y");
            {
                Args a;
                a << BxAir << BxPitch << FBxR << d_mp << mg << gc;
                launch(K, "Blinear_BxR2IR", dim3((L + 1 + 15) / 16, (M + 15) / 16), t16, a, st);
            }
            {
                Args a;
                a << ByAir << ByPitch << FByR << d_mp << mg << gc;
                launch(K, "Blinear_ByR2IR", dim3((L + 15) / 16, (M + 1 + 15) / 16), t16, a, st);
            }
        };

        // ---- ElectricalFiled.cu:478-641
        const double *Xh = in->X, *Yh = in->Y, *Zh = in->Z, *dxh = in->dx, *dyh = in->dy, *dzh = in->dz;
        auto add_tx = [&](const char *k, double *E, int nthreads, double current) {
            Args a;
            a << E << Con << d_mp << d_Tx << current;
            launch(K, k, dim3(1), dim3(nthreads), a, st);
        };
        auto electric_field = [&](double lambda, double dt, double wave) {
            {
                Args a;
                a << Ex << By << Bz << Con << ByAir << ByPitch << d_mp << dt << lambda;
                launch(K, "UpdateEx", dim3((L + BLOCKSIZE1 - 1) / BLOCKSIZE1, M - 1), dim3(BLOCKSIZE1), a, st);
            }
            {
                Args a;
                a << Ey << Bx << Bz << Con << BxAir << BxPitch << d_mp << dt << lambda;
                launch(K, "UpdateEy", dim3((L - 1 + BLOCKSIZE1 - 1) / BLOCKSIZE1, M), dim3(BLOCKSIZE1), a, st);
            }
            {
                Args a;
                a << Ez << Bx << By << Con << d_mp << dt << lambda;
                launch(K, "UpdateEz", dim3((L - 1 + BLOCKSIZE1 - 1) / BLOCKSIZE1, M - 1), dim3(BLOCKSIZE1), a, st);
            }
            if (wave == 0) return;
            const int nxs = std::abs(tx.ixb - tx.ixa) + 1, nys = std::abs(tx.iyb - tx.iya) + 1,
                      nzs = std::abs(tx.izb - tx.iza) + 1;
            const double wx = std::fabs(Xh[tx.ixb] - Xh[tx.ixa]) + dxh[tx.ixb] / 2.0 + dxh[tx.ixa] / 2.0;
            const double wy = std::fabs(Yh[tx.iyb] - Yh[tx.iya]) + dyh[tx.iyb] / 2.0 + dyh[tx.iya] / 2.0;
            const double wz = std::fabs(Zh[tx.izb] - Zh[tx.iza]) + dzh[tx.izb] / 2.0 + dzh[tx.iza] / 2.0;
            switch (tx.ort) {
            case 1:
                add_tx("AddTx_x", Ex, nxs, wave / (Xh[tx.ixb] - Xh[tx.ixa] + dxh[tx.ixb] / 2 + dxh[tx.ixa] / 2));
                break;
            case 2:
                add_tx("AddTx_y", Ey, nys, wave / (Yh[tx.iyb] - Yh[tx.iya] + dyh[tx.iyb] / 2 + dyh[tx.iya] / 2));
                break;
            case 3:
                add_tx("AddTx_z", Ez, nzs, wave / (Zh[tx.izb] - Zh[tx.iza] + dzh[tx.izb] / 2 + dzh[tx.iza] / 2));
                break;
            case 4:
                add_tx("AddTx_x", Ex, nxs, wave * cos(tx.dip) * cos(tx.azi) / wx);
                add_tx("AddTx_y", Ey, nys, wave * cos(tx.dip) * sin(tx.azi) / wy);
                add_tx("AddTx_z", Ez, nzs, wave * sin(tx.dip) / wz);
                break;
            case 5: {
                add_tx("AddTx_x", Ex, nxs, wave * cos(tx.dip) * cos(tx.azi) * tx.BipoLen / wx);
                add_tx("AddTx_y", Ey, nys, wave * cos(tx.dip) * sin(tx.azi) * tx.BipoLen / wy);
                add_tx("AddTx_z", Ez, nzs, wave * sin(tx.dip) * tx.BipoLen / wz);
                // second bipole: its own extents set the thread counts and currents; the
                // kernels read the first bipole's cells from the record (ElectricalFiled.cu:612-635)
                const int mx = std::abs(tx.ixb1 - tx.ixa1) + 1, my = std::abs(tx.iyb1 - tx.iya1) + 1,
                          mz = std::abs(tx.izb1 - tx.iza1) + 1;
                const double vx = std::fabs(Xh[tx.ixb1] - Xh[tx.ixa1]) + dxh[tx.ixb1] / 2.0 + dxh[tx.ixa1] / 2.0;
                const double vy = std::fabs(Yh[tx.iyb1] - Yh[tx.iya1]) + dyh[tx.iyb1] / 2.0 + dyh[tx.iya1] / 2.0;
                const double vz = std::fabs(Zh[tx.izb1] - Zh[tx.iza1]) + dzh[tx.izb1] / 2.0 + dzh[tx.iza1] / 2.0;
                add_tx("AddTx_x", Ex, mx, wave * cos(tx.dip1) * cos(tx.azi1) * tx.BipoLen1 / vx);
                add_tx("AddTx_y", Ey, my, wave * cos(tx.dip1) * sin(tx.azi1) * tx.BipoLen1 / vy);
                add_tx("AddTx_z", Ez, mz, wave * sin(tx.dip1) * tx.BipoLen1 / vz);
                break;
            }
            default:
                fail("transmitter orientation %d", tx.ort);
            }
        };

        // ---- Bderivate.cu:269-316
        auto bderivate = [&](double dt) {
            const dim3 t16(BLOCKSIZE2x, BLOCKSIZE2y2);
            {
                Args a;
                a << Bx << Ey << Ez << d_mp << dt;
                launch(K, "UpdateBx", dim3((L - 1 + 15) / 16, (M + 15) / 16), t16, a, st);
            }
            {
                Args a;
                a << By << Ex << Ez << d_mp << dt;
                launch(K, "UpdateBy", dim3((L + 15) / 16, (M - 1 + 15) / 16), t16, a, st);
            }
            {
                Args a;
                a << Bz << Bx << By << d_mp;
                launch(K, "UpdateBz", dim3((L + BLOCKSIZE2x - 1) / BLOCKSIZE2x, (M + BLOCKSIZE2y1 - 1) / BLOCKSIZE2y1),
                       dim3(BLOCKSIZE2x, BLOCKSIZE2y1), a, st);
            }
        };

        // ---- EFInterp2Rx.cu:410-470: spatial interpolation of the E or B components into ef0 + base
        const int *isc = in->isComp;
        auto fx_interp = [&](bool efield, int base) {
            const dim3 g((nr + BLOCKSIZE1 - 1) / BLOCKSIZE1), b(BLOCKSIZE1);
            const char *names[6] = {"ExSpatialInterp", "EySpatialInterp", "EzSpatialInterp",
                                    "BxSpatialInterp", "BySpatialInterp", "BzSpatialInterp"};
            double *fields[6] = {Ex, Ey, Ez, Bx, By, Bz};
            int pos = efield ? 0 : nefcmp;
            for (int c = efield ? 0 : 3; c < (efield ? 3 : 6); c++) {
                if (!isc[c]) continue;
                Args a;
                a << fields[c] << d_mp << mg << rxp << RxLst << ef0 << nr << (base + pos * nr);
                launch(K, names[c], g, b, a, st);
                pos++;
            }
        };
        auto time_interp = [&](bool efield, int sample, double l0, double l1) {
            Args a;
            a << ef0 << efs << nr << Nt << sample << nefcmp << NComp << l0 << l1;
            launch(K, efield ? "EFTimeInterp" : "BFTimeInterp", dim3((nr + BLOCKSIZE1 - 1) / BLOCKSIZE1),
                   dim3(BLOCKSIZE1), a, st);
        };
        // the state machine of EFInterp2Rx.cu:472-585 (E times at the step, B times half a step later)
        const double *T = in->times;
        auto rx_sample = [&](int &ne, int &nb, double t0, double dt, double Tp[2][3]) {
            if (ne < Nt) {
                Tp[0][2] = t0;
                if (T[ne] <= Tp[0][0])
                    while (ne < Nt && T[ne] <= Tp[0][0]) ne++;
                if (ne < Nt && T[ne] <= Tp[0][2] && T[ne] > Tp[0][1]) {
                    fx_interp(true, 0);
                } else if (ne < Nt && T[ne] <= Tp[0][1] && T[ne] > Tp[0][0]) {
                    fx_interp(true, NComp * nr);
                    while (ne < Nt && T[ne] <= Tp[0][1]) {
                        const double l1 = (T[ne] - Tp[0][0]) / (Tp[0][1] - Tp[0][0]);
                        time_interp(true, ne, 1.0 - l1, l1);
                        ne++;
                    }
                }
                Tp[0][0] = Tp[0][1];
                Tp[0][1] = Tp[0][2];
            }
            if (nb < Nt && (isc[3] || isc[4] || isc[5])) {
                Tp[1][2] = t0 + 0.5 * dt;
                if (T[nb] <= Tp[1][0])
                    while (nb < Nt && T[nb] <= Tp[1][0]) nb++;
                if (nb < Nt && T[nb] <= Tp[1][2] && T[nb] > Tp[1][1]) {
                    fx_interp(false, 0);
                } else if (nb < Nt && T[nb] <= Tp[1][1] && T[nb] > Tp[1][0]) {
                    fx_interp(false, NComp * nr);
                    while (nb < Nt && T[nb] <= Tp[1][1]) {
                        const double l1 = (T[nb] - Tp[1][0]) / (Tp[1][1] - Tp[1][0]);
                        time_interp(false, nb, 1.0 - l1, l1);
                        nb++;
                    }
                }
                Tp[1][0] = Tp[1][1];
                Tp[1][1] = Tp[1][2];
            }
        };

        // ---- main.cu:195-273, one transmitter from a zero state
        const double miu = in->miu, sfa1 = in->sfa1, sfa2 = in->sfa2, minsita = in->minsita;
        const double mindx = std::min(mp.dzmin, std::min(mp.dxmin, mp.dymin));
        const int nsrc = in->nsrc;
        const double *dtw = in->dtw, *Wave = in->wave;
        double Tp[2][3] = {{0, 0, 0}, {0, 0, 0}};
        int ne = 0, nb = 0, n = 0;
        double toT = 0, dt1 = dtw[0], dt2 = dtw[1];
        Tp[0][1] = toT + dt1;
        Tp[1][1] = toT + dt1 + 0.5 * dt2;
        long steps = 0;
        cudaEvent_t e0, e1;
        ck(cudaEventCreate(&e0), "event");
        ck(cudaEventCreate(&e1), "event");
        ck(cudaStreamSynchronize(st), "setup");
        ck(cudaEventRecord(e0, st), "event");
        while (ne < Nt || (nb < Nt && nefcmp < NComp)) {
            if (max_steps >= 0 && steps >= max_steps) break;
            const double nmuda = 7.5 * sfa2 * dt2 * dt1 / miu / mindx / mindx;
            upcontinuation();
            electric_field(nmuda, dt1, n < 2 * nsrc ? Wave[n] : 0.0);
            bderivate(0.5 * (dt1 + dt2));
            toT += dt1;
            dt1 = dt2;
            n++;
            if (n < 2 * nsrc) dt2 = dtw[n + 1];
            else dt2 = std::min(0.15 * sfa1 * std::sqrt(miu * toT * minsita / 8.) * mindx, 1.2 * dt1);
            rx_sample(ne, nb, toT + dt1, dt2, Tp);
            steps++;
        }
        ck(cudaEventRecord(e1, st), "event");
        ck(cudaStreamSynchronize(st), "step loop");
        float ms = 0;
        ck(cudaEventElapsedTime(&ms, e0, e1), "event time");
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ck(cudaMemcpy(traces, efs, sizeof(double) * nr * NComp * Nt, cudaMemcpyDeviceToHost), "traces");
        if (steps_out) *steps_out = steps;
        if (loop_ms) *loop_ms = ms;
        return 0;
    } catch (const Fail &f) {
        if (err && errlen > 0) snprintf(err, errlen, "%s", f.msg.c_str());
        return 1;
    }
}

}  // extern "C"
