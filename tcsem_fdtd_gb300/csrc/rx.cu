// Receiver sampling (EFInterp2Rx.cu): 4x4x4 natural-spline interpolation of
// the staggered components to the receivers, stored into one of two slots,
// and linear interpolation in time between the slots at the sampling times.
//
// The host decides, per step, which slot the current E (B) field goes to and
// which samples are produced (EFInterp2Rx.cu:472-585); that plan is a device
// table here so the kernel can run inside captured step blocks.  A sample
// produced in a step uses slot 0 (written in an earlier step) and the slot-1
// value being computed, so the time interpolation is fused into the spatial
// pass and needs no grid-wide synchronisation.
#include "rx_body.cuh"

namespace tcsem {

template <typename T>
__global__ void k_rx(RxDev<T> rd, FieldSet<T> f, const T *tot, ZChunks zc, Geom g, StepGate gate, RxAction act) {
    if (gate.base) {
        const long st = gate.step();
        if (st >= gate.nsteps) return;
        act = step_action(rd, st);
    }
    rx_thread(rd, f, tot, zc, g, act, blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T>
__global__ void k_rx_b(const RxSlot<T> *__restrict__ slots, const __grid_constant__ BatchIndex idx, int s) {
    const int q = idx.slot_of(blockIdx.x);
    const RxSlot<T> &d = slots[q];
    const long st = (long)*d.step_base + s;
    if (st >= d.nsteps) return;
    rx_thread(d.rd, d.f, d.tot, d.zc, d.g, step_action(d.rd, st), (blockIdx.x - idx.off[q]) * blockDim.x + threadIdx.x);
}

template <typename T>
__global__ void k_advance(int *base, int by) {
    *base += by;
}

__global__ void k_advance_all(int *counters, int n, int by) {
    if ((int)threadIdx.x < n) counters[threadIdx.x] += by;
}

template <typename T>
void launch_rx(const RxDev<T> &rd, FieldSet<T> f, const T *tot, const ZChunks &zc, const Geom &g, StepGate gate,
               RxAction act, cudaStream_t st, bool early) {
    int n = rd.NComp * rd.nr;
    if (n == 0) return;
    // early: programmatic dependent launch after the previous kernel on the stream, for receivers
    // that read nothing that kernel writes (they do not wait for it; its launch latency is saved)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(rx_blocks(n));
    cfg.blockDim = dim3(kRxThreads);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = early ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_rx<T>, rd, f, tot, zc, g, gate, act);
}

void launch_advance(int *base, int by, cudaStream_t st) { k_advance<float><<<1, 1, 0, st>>>(base, by); }
void launch_advance_all(int *counters, int n, int by, cudaStream_t st) { k_advance_all<<<1, kMaxSlots, 0, st>>>(counters, n, by); }

int rx_blocks(int nstencils) { return (nstencils + kRxThreads - 1) / kRxThreads; }

template <typename T> void launch_rx_batched(const RxSlot<T> *slots, const BatchIndex &idx, int s, cudaStream_t st) {
    if (idx.total()) k_rx_b<T><<<idx.total(), kRxThreads, 0, st>>>(slots, idx, s);
}

template void launch_rx<float>(const RxDev<float> &, FieldSet<float>, const float *, const ZChunks &, const Geom &,
                               StepGate, RxAction, cudaStream_t, bool);
template void launch_rx<double>(const RxDev<double> &, FieldSet<double>, const double *, const ZChunks &, const Geom &,
                                StepGate, RxAction, cudaStream_t, bool);
template void launch_rx_batched<float>(const RxSlot<float> *, const BatchIndex &, int, cudaStream_t);
template void launch_rx_batched<double>(const RxSlot<double> *, const BatchIndex &, int, cudaStream_t);

}  // namespace tcsem
