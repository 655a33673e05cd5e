// Air-interface boundary pipeline: Bz on the top plane (non-uniform) ->
// uniform L1 x M1 plane -> 2-D FFT -> upward-continuation filters -> inverse
// FFT -> bilinear remap back to the staggered BxAir / ByAir planes.
//
// The reference (UpContinuation_gpu.cu:166-274, SplineGridConvIR2R.cu:539-752)
// materialises the whole uniform plane three times per step (cuSPARSE spline
// solves, one R2C and two C2R cuFFT calls).  Every stage of that chain is
// linear and the spline remap is separable, BzAir = Py . Bz . Px^T, so this
// pipeline instead
//   1. remaps each of the M old rows to L1 uniform points with dense spline
//      weights (precomputed from the same natural-spline rule) and FFTs it
//      along x -- M rows, not M1, two real rows packed in one complex
//      transform;
//   2. per x-frequency column: applies Py in the x-frequency domain, FFTs
//      along y, multiplies by the two continuation filters, inverse-FFTs
//      along y and keeps only the rows the final bilinear remap samples;
//   3. inverse-FFTs those rows along x with Bx and By packed as the real and
//      imaginary parts of one complex transform;
//   4. bilinearly remaps into plane k = -1 of the Bx/By buffers.
// All transforms are in-shared-memory mixed-radix Stockham FFTs of arbitrary
// length written here (no cuFFT).
#include "boundary_body.cuh"

namespace tcsem {


// ---- single-survey kernels
template <typename T>
__global__ void __launch_bounds__(kBndThreads) k_rows_fwd(BoundaryDev<T> bd, const T *__restrict__ bz,
                                                          const T *__restrict__ tot, int nch, Geom g,
                                                          StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    rows_fwd_cta<T>(bd, bz, tot, nch, g, blockIdx.x);
}
template <typename T> __global__ void __launch_bounds__(kBndThreads) k_cols(BoundaryDev<T> bd, StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    cols_cta<T>(bd, blockIdx.x);
}
template <typename T> __global__ void __launch_bounds__(kBndThreads) k_rows_inv(BoundaryDev<T> bd, StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    rows_inv_cta<T>(bd, blockIdx.x);
}
template <typename T> __global__ void k_bilinear(BoundaryDev<T> bd, T *bx, T *by, Geom g, StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    bilinear_cta<T>(bd, bx, by, g, blockIdx.x, gridDim.x);
}

// ---- batched kernels: block b works for slot idx.slot_of(b)
template <typename T>
__device__ __forceinline__ const BoundarySlot<T> *bnd_slot(const BoundarySlot<T> *slots, const BatchIndex &idx,
                                                           int s, int &lb) {
    const int q = idx.slot_of(blockIdx.x);
    const BoundarySlot<T> *d = slots + q;
    if ((long)*d->step_base + s >= d->nsteps) return nullptr;
    lb = blockIdx.x - idx.off[q];
    return d;
}
template <typename T>
__global__ void __launch_bounds__(kBndThreads)
    k_rows_fwd_b(const BoundarySlot<T> *__restrict__ slots, const __grid_constant__ BatchIndex idx, int s) {
    int lb;
    const BoundarySlot<T> *d = bnd_slot(slots, idx, s, lb);
    if (d) rows_fwd_cta<T>(d->bd, d->bz, d->tot, d->nch, d->g, lb);
}
template <typename T>
__global__ void __launch_bounds__(kBndThreads)
    k_cols_b(const BoundarySlot<T> *__restrict__ slots, const __grid_constant__ BatchIndex idx, int s) {
    int lb;
    const BoundarySlot<T> *d = bnd_slot(slots, idx, s, lb);
    if (d) cols_cta<T>(d->bd, lb);
}
template <typename T>
__global__ void __launch_bounds__(kBndThreads)
    k_rows_inv_b(const BoundarySlot<T> *__restrict__ slots, const __grid_constant__ BatchIndex idx, int s) {
    int lb;
    const BoundarySlot<T> *d = bnd_slot(slots, idx, s, lb);
    if (d) rows_inv_cta<T>(d->bd, lb);
}
template <typename T>
__global__ void k_bilinear_b(const BoundarySlot<T> *__restrict__ slots, const __grid_constant__ BatchIndex idx, int s) {
    int lb;
    const BoundarySlot<T> *d = bnd_slot(slots, idx, s, lb);
    if (d) {
        const int q = idx.slot_of(blockIdx.x);
        bilinear_cta<T>(d->bd, d->bx, d->by, d->g, lb, idx.off[q + 1] - idx.off[q]);
    }
}

template <typename T> static size_t smem_rows(const BoundaryDev<T> &bd, int L) { return rows_fwd_layout(bd, L).total; }
template <typename T> static size_t smem_cols(const BoundaryDev<T> &bd) { return cols_layout(bd).total; }
template <typename T> static size_t smem_inv(const BoundaryDev<T> &bd) { return rows_inv_layout(bd).total; }

template <typename T> size_t boundary_smem_need(const BoundaryDev<T> &bd, int L) {
    size_t a = smem_rows(bd, L), b = smem_cols(bd), c = smem_inv(bd);
    return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

template <typename T> cudaError_t boundary_configure(const BoundaryDev<T> &bd, int L) {
    cudaError_t e;
    e = cudaFuncSetAttribute(k_rows_fwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_rows(bd, L));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_cols<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_cols(bd));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_rows_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_inv(bd));
}

template <typename T> BoundaryBlocks boundary_blocks(const BoundaryDev<T> &bd, const Geom &g) {
    BoundaryBlocks b;
    b.rows_fwd = (g.M + 1) / 2;
    b.cols = bd.H;
    b.rows_inv = bd.S;
    b.bilinear = ((g.L + 1) * g.M + g.L * (g.M + 1) + 255) / 256;
    b.smem_rows = smem_rows(bd, g.L);
    b.smem_cols = smem_cols(bd);
    b.smem_inv = smem_inv(bd);
    return b;
}

template <typename T> cudaError_t boundary_configure_batched(const size_t *smem) {
    cudaError_t e;
    e = cudaFuncSetAttribute(k_rows_fwd_b<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem[0]);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cols_b<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem[1]);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rows_inv_b<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem[2]);
    return e;
}

// a launch that may begin while the previous kernel on the stream is still running
// (programmatic dependent launch; the kernel waits with pdl_wait_prev before its reads)
template <typename... P, typename... A>
static void launch_after(bool pdl, void (*k)(P...), int grid, int block, size_t smem, cudaStream_t st, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k, static_cast<P>(args)...);
}

template <typename T>
cudaError_t launch_boundary_batched(const BoundarySlot<T> *slots, const BatchIndex *idx, const size_t *smem, int s,
                                    cudaStream_t st) {
    if (idx[0].total()) k_rows_fwd_b<T><<<idx[0].total(), kBndThreads, smem[0], st>>>(slots, idx[0], s);
    if (idx[1].total()) launch_after(true, k_cols_b<T>, idx[1].total(), kBndThreads, smem[1], st, slots, idx[1], s);
    if (idx[2].total()) launch_after(true, k_rows_inv_b<T>, idx[2].total(), kBndThreads, smem[2], st, slots, idx[2], s);
    if (idx[3].total()) launch_after(true, k_bilinear_b<T>, idx[3].total(), 256, (size_t)0, st, slots, idx[3], s);
    return cudaGetLastError();
}

template <typename T>
void launch_boundary(const BoundaryDev<T> &bd, const Geom &g, const T *bz, const T *tot, int nch, T *bx, T *by,
                     StepGate gate, cudaStream_t st, bool pdl) {
    k_rows_fwd<T><<<(g.M + 1) / 2, kBndThreads, smem_rows(bd, g.L), st>>>(bd, bz, tot, nch, g, gate);
    // The column stage starts early only where the caller asks (beside a long sweep its early CTAs
    // would take slots the sweep's single wave needs at the start of a step); the last two stages
    // always do: by then the sweep's CTAs are all resident.
    launch_after(pdl, k_cols<T>, bd.H, kBndThreads, smem_cols(bd), st, bd, gate);
    launch_after(true, k_rows_inv<T>, bd.S, kBndThreads, smem_inv(bd), st, bd, gate);
    int n = (g.L + 1) * g.M + g.L * (g.M + 1);
    launch_after(true, k_bilinear<T>, (n + 255) / 256, 256, (size_t)0, st, bd, bx, by, g, gate);
}

#define INST(T)                                                                                            \
    template size_t boundary_smem_need<T>(const BoundaryDev<T> &, int);                                   \
    template cudaError_t boundary_configure<T>(const BoundaryDev<T> &, int);                              \
    template void launch_boundary<T>(const BoundaryDev<T> &, const Geom &, const T *, const T *, int, T *, T *,  \
                                     StepGate, cudaStream_t, bool);                                       \
    template BoundaryBlocks boundary_blocks<T>(const BoundaryDev<T> &, const Geom &);                     \
    template cudaError_t launch_boundary_batched<T>(const BoundarySlot<T> *, const BatchIndex *, const size_t *, int, \
                                                    cudaStream_t);                                        \
    template cudaError_t boundary_configure_batched<T>(const size_t *);
INST(float)
INST(double)
#undef INST

}  // namespace tcsem
