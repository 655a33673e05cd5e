// Test helper: runs cufftExecZ2D (the call of UpContinuation_gpu.cu:244-248)
// on seeded half spectra that are not Hermitian-consistent, so the test can
// check the oracle's model of that call (Hermitian part of the self-conjugate
// bins) against the library.  Usage: cufft_c2r_probe <outdir> M1 L1 [M1 L1 ...]
#include <cufft.h>
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdlib>
#include <vector>
static unsigned long long s = 88172645463325252ull;
static double rnd() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return (double)(s >> 11) / 9007199254740992.0 - 0.5; }
int main(int argc, char **argv) {
    if (argc < 4) return 2;
    for (int a = 2; a + 1 < argc; a += 2) {
        int M1 = std::atoi(argv[a]), L1 = std::atoi(argv[a + 1]), H = L1 / 2 + 1;
        std::vector<cufftDoubleComplex> X((size_t)M1 * H);
        for (auto &c : X) { c.x = rnd(); c.y = rnd(); }
        cufftDoubleComplex *dX = nullptr;
        double *dY = nullptr;
        if (cudaMalloc(&dX, X.size() * sizeof(cufftDoubleComplex)) != cudaSuccess) return 1;
        if (cudaMalloc(&dY, (size_t)M1 * L1 * sizeof(double)) != cudaSuccess) return 1;
        cudaMemcpy(dX, X.data(), X.size() * sizeof(cufftDoubleComplex), cudaMemcpyHostToDevice);
        cufftHandle p;
        if (cufftPlan2d(&p, M1, L1, CUFFT_Z2D) != CUFFT_SUCCESS) return 1;
        if (cufftExecZ2D(p, dX, dY) != CUFFT_SUCCESS) return 1;
        std::vector<double> Y((size_t)M1 * L1);
        if (cudaMemcpy(Y.data(), dY, Y.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
        char name[1024];
        std::snprintf(name, sizeof name, "%s/c2r_%d_%d.bin", argv[1], M1, L1);
        FILE *f = std::fopen(name, "wb");
        if (!f) return 1;
        int hdr[2] = {M1, L1};
        std::fwrite(hdr, 4, 2, f);
        std::fwrite(X.data(), sizeof(cufftDoubleComplex), X.size(), f);
        std::fwrite(Y.data(), sizeof(double), Y.size(), f);
        std::fclose(f);
        cufftDestroy(p);
        cudaFree(dX);
        cudaFree(dY);
    }
    return 0;
}
