// Device view of the receiver sampling (see rx.cu).
#pragma once
#include <cuda_runtime.h>
#include "kernels.cuh"

namespace tcsem {

struct StepEntryActs {
    int e_slot, e_first, e_count, b_slot, b_first, b_count;
};

struct RxAction {
    int e_slot, e_first, e_count, b_slot, b_first, b_count;
};

template <typename T> struct RxDev {
    int nr, NComp, nefcmp, Nt;
    const long long *base;      // per stencil [NComp][nr]: padded index of the (s1, s2, s3) corner
    const int *comp;            // per stencil: field component 0..5
    const T *w;                 // per stencil: wx[4], wy[4], wz[4]
    T *ef0;                     // [2][NComp][nr]
    T *efs;                     // [nr][NComp][Nt]
    const T *e_l1, *b_l1;       // per sample: time-interpolation weight
    const StepEntryActs *acts;  // per step
    int *err;                   // device error word (bounds-checked builds)
};

template <typename T>
void launch_rx(const RxDev<T> &rd, FieldSet<T> f, const T *tot, const ZChunks &zc, const Geom &g, StepGate gate,
               RxAction act, cudaStream_t st, bool early = false);
void launch_advance(int *base, int by, cudaStream_t st);

constexpr int kRxThreads = 128;
int rx_blocks(int nstencils);
// one slot of a batched receiver step (device memory)
template <typename T> struct RxSlot {
    RxDev<T> rd;
    FieldSet<T> f;  // the new fields
    const T *tot;   // their chunk totals
    ZChunks zc;
    Geom g;
    const int *step_base;
    long nsteps;
};
template <typename T> void launch_rx_batched(const RxSlot<T> *slots, const BatchIndex &idx, int s, cudaStream_t st);
void launch_advance_all(int *counters, int n, int by, cudaStream_t st);

}  // namespace tcsem
