// Device view of the boundary pipeline (see boundary.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include "kernels.cuh"

namespace tcsem {

// mixed-radix factorisation of one transform length
struct FFTPlan {
    int n, nst;
    int radix[32];
};

template <typename T> struct C2 { T x, y; };

template <typename T> struct BoundaryDev {
    // plane geometry
    int L1, M1, H, M;          // H = L1/2 + 1 kept x-frequencies
    int AnLx, Nx, AL, ox, n1, n2;
    int Any, Ny, Ay, oy, n3;
    FFTPlan px, py;
    const C2<T> *twx, *twy;    // forward twiddles exp(-2 pi i k / n)
    // spline remap weights
    const T *Wl, *Wr, *Wf, *Wb;
    // projected continuation filters, [H][M1], applied as i*g*F
    const T *Gx, *Gy;
    // rows of the uniform plane that the bilinear remap samples
    int S;
    const int *rows;
    // scratch
    C2<T> *FT, *VX, *VY, *Z;
    // bilinear tables (indices already clamped as in the reference)
    const int *bxc_II, *bxr_a, *bxr_b, *byc_II, *byr_a, *byr_b;
    const T *bxc_l, *bxr_l, *byc_l, *byr_l;
    T inv_norm;
};

}  // namespace tcsem

namespace tcsem {
template <typename T> size_t boundary_smem_need(const BoundaryDev<T> &bd, int L);
template <typename T> cudaError_t boundary_configure(const BoundaryDev<T> &bd, int L);
template <typename T>
void launch_boundary(const BoundaryDev<T> &bd, const Geom &g, const T *bz, const T *tot, int nch, T *bx, T *by,
                     StepGate gate, cudaStream_t st);
template <typename T>
cudaError_t launch_fft_rows(const FFTPlan &P, const void *tw, const void *in, void *out, int rows, int inv,
                            cudaStream_t st);
}  // namespace tcsem
