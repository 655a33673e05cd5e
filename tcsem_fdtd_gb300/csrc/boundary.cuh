// Device view of the boundary pipeline (see boundary.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include "kernels.cuh"
#include "async.cuh"

namespace tcsem {

// mixed-radix factorisation of one transform length
struct FFTPlan {
    int n, nst;
    int radix[32];
};

template <typename T> struct C2 { T x, y; };

// one strip of the spline remap in factored form (host side: SplinePlan)
struct StripPlan {
    int n, npts;  // source nodes, output points
    int src, dst; // first source node in the line, first output index on the uniform line
    int f;        // offset of the factors g, w, inv, du (n values each) in the table
    int c;        // offset of the window weights, [6][npts]
    int k;        // offset of the window starts in the int table
};

// the two strips of one axis, their factor/weight table and its size
template <typename T> struct AxisRemap {
    StripPlan s[2];
    int nT, nI, nmax;
    const T *tabT;
    const int *tabI;
};

template <typename T> struct BoundaryDev {
    // plane geometry: the transforms have L1 x M1 points; the uniform grid (Lu x Mu points)
    // sits at offset (DL, DM) in them.  Without padding Lu = L1, Mu = M1, DL = DM = 0; with
    // padding the points outside the grid taper each row (column) from its edge values to
    // zero with the weights padx[L1] (pady[M1]), zero inside the grid.
    int L1, M1, H, M;          // H = L1/2 + 1 kept x-frequencies
    int Lu, Mu, DL, DM;
    const T *padx, *pady;
    int AnLx, Nx, AL;
    int Any, Ny, Ay;
    int Mp, M1p, Hp;           // padded strides of FT, Gx/Gy and VX/VY (16-byte rows)
    FFTPlan px, py;
    const C2<T> *twx, *twy;    // forward twiddles exp(-2 pi i k / n)
    // spline remaps of the x strips (left, right) and y strips (front, back)
    AxisRemap<T> rx, ry;
    // projected continuation filters, [H][M1p], applied as i*g*F
    const T *Gx, *Gy;
    // rows of the uniform plane that the bilinear remap samples
    int S;
    const int *rows;
    // scratch
    C2<T> *FT, *VX, *VY, *Z;  // FT is [H][Mp]; VX, VY are [S][Hp]; Z is [S][Lu]
    int *err;                 // device error word (a bounded wait gave up)
    // bilinear tables (indices already clamped as in the reference)
    const int *bxc_II, *bxr_a, *bxr_b, *byc_II, *byr_a, *byr_b;
    const T *bxc_l, *bxr_l, *byc_l, *byr_l;
    T inv_norm;
};

// one slot of a batched boundary step (device memory)
template <typename T> struct BoundarySlot {
    BoundaryDev<T> bd;
    Geom g;
    const T *bz, *tot;  // plane 0 of Bz and the chunk totals of the current field set
    int nch;
    T *bx, *by;         // plane -1 of Bx/By of the current field set
    const int *step_base;
    long nsteps;
};
// blocks and dynamic shared memory of the four boundary kernels for one survey
struct BoundaryBlocks {
    int rows_fwd, cols, rows_inv, bilinear;
    size_t smem_rows, smem_cols, smem_inv;
};

}  // namespace tcsem

namespace tcsem {
template <typename T> size_t boundary_smem_need(const BoundaryDev<T> &bd, int L);
template <typename T> cudaError_t boundary_configure(const BoundaryDev<T> &bd, int L);
// pdl: the last three kernels may start while their predecessor finishes (programmatic
// dependent launch); off where the chain runs beside a long sweep whose CTAs need the slots
template <typename T>
void launch_boundary(const BoundaryDev<T> &bd, const Geom &g, const T *bz, const T *tot, int nch, T *bx, T *by,
                     StepGate gate, cudaStream_t st, bool pdl = true);
template <typename T> BoundaryBlocks boundary_blocks(const BoundaryDev<T> &bd, const Geom &g);
// idx[4] and smem[3]: the block lists of rows_fwd, cols, rows_inv, bilinear and the largest shared memory
template <typename T>
cudaError_t launch_boundary_batched(const BoundarySlot<T> *slots, const BatchIndex *idx, const size_t *smem, int s,
                                    cudaStream_t st);
template <typename T> cudaError_t boundary_configure_batched(const size_t *smem);
}  // namespace tcsem
