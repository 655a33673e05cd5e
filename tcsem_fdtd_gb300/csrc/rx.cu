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
#include "check.cuh"
#include "kernels.cuh"
#include "rx.cuh"

namespace tcsem {

template <typename T>
__device__ __forceinline__ T stencil_value(const RxDev<T> &rd, const FieldSet<T> &f, int s, const Geom &g,
                                           const T *tot, const ZChunks &zc) {
    const int comp = rd.comp[s];
    const T *F = comp == 0 ? f.ex : comp == 1 ? f.ey : comp == 2 ? f.ez : comp == 3 ? f.bx : comp == 4 ? f.by : f.bz;
    const T *w = rd.w + (size_t)s * 12;
    const long long base = rd.base[s];
    T v = T(0);
    // chunk-partial Bz: add the totals of the chunks below each plane
    const long long plane = (long long)(g.M + 2) * g.XP;
    const long long col = (base % g.PS);
    const int k3 = (int)(base / g.PS) - 1;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        T vy = T(0);
        int cz = 0;
        if (comp == 5 && zc.n > 1)
            while (cz + 1 < zc.n && k3 + c >= zc.kb[cz + 1]) cz++;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const long long o = base + (long long)c * g.PS + (long long)b * g.XP;
            if (!TCSEM_IN(o, g.total(), rd.err) || !TCSEM_IN(o + 3, g.total(), rd.err)) continue;
            const T *row = F + o;
            T r0 = row[0], r1 = row[1], r2 = row[2], r3 = row[3];
            if (comp == 5 && zc.n > 1) {
                const long long cb = col + (long long)b * g.XP;
                for (int q = cz + 1; q < zc.n; q++) {
                    if (!TCSEM_IN(q * plane + cb + 3, zc.n * plane, rd.err)) continue;
                    const T *t = tot + q * plane + cb;
                    r0 += t[0]; r1 += t[1]; r2 += t[2]; r3 += t[3];
                }
            }
            T vx = w[0] * r0 + w[1] * r1 + w[2] * r2 + w[3] * r3;
            vy += w[4 + b] * vx;
        }
        v += w[8 + c] * vy;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ void rx_thread(const RxDev<T> &rd, const FieldSet<T> &f, const T *tot, const ZChunks &zc,
                                          const Geom &g, RxAction act, int idx) {
    const int nr = rd.nr, NC = rd.NComp, ne = rd.nefcmp;
    if (idx >= NC * nr) return;
    const int p = idx / nr, r = idx % nr;  // slot image position [p][r]
    const bool efield = p < ne;
    const int slot = efield ? act.e_slot : act.b_slot;
    if (slot < 0) return;
    const T v = stencil_value(rd, f, idx, g, tot, zc);
    if (!TCSEM_IN((long long)slot * NC * nr + idx, 2LL * NC * nr, rd.err)) return;
    rd.ef0[(size_t)slot * NC * nr + idx] = v;
    const int first = efield ? act.e_first : act.b_first, count = efield ? act.e_count : act.b_count;
    const T *l1 = efield ? rd.e_l1 : rd.b_l1;
    if (slot == 1) {  // EFTimeInterp / BFTimeInterp, EFInterp2Rx.cu:380-407
        const T v0 = rd.ef0[idx];
        for (int s = first; s < first + count; s++)
            if (TCSEM_IN(((long long)r * NC + p) * rd.Nt + s, (long long)nr * NC * rd.Nt, rd.err))
                rd.efs[((size_t)r * NC + p) * rd.Nt + s] = (T(1) - l1[s]) * v0 + l1[s] * v;
    }
}

template <typename T> __device__ __forceinline__ RxAction step_action(const RxDev<T> &rd, long st) {
    const StepEntryActs &a = rd.acts[st];
    return RxAction{a.e_slot, a.e_first, a.e_count, a.b_slot, a.b_first, a.b_count};
}

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
               RxAction act, cudaStream_t st) {
    int n = rd.NComp * rd.nr;
    if (n == 0) return;
    k_rx<T><<<rx_blocks(n), kRxThreads, 0, st>>>(rd, f, tot, zc, g, gate, act);
}

void launch_advance(int *base, int by, cudaStream_t st) { k_advance<float><<<1, 1, 0, st>>>(base, by); }
void launch_advance_all(int *counters, int n, int by, cudaStream_t st) { k_advance_all<<<1, kMaxSlots, 0, st>>>(counters, n, by); }

int rx_blocks(int nstencils) { return (nstencils + kRxThreads - 1) / kRxThreads; }

template <typename T> void launch_rx_batched(const RxSlot<T> *slots, const BatchIndex &idx, int s, cudaStream_t st) {
    if (idx.total()) k_rx_b<T><<<idx.total(), kRxThreads, 0, st>>>(slots, idx, s);
}

template void launch_rx<float>(const RxDev<float> &, FieldSet<float>, const float *, const ZChunks &, const Geom &,
                               StepGate, RxAction, cudaStream_t);
template void launch_rx<double>(const RxDev<double> &, FieldSet<double>, const double *, const ZChunks &, const Geom &,
                                StepGate, RxAction, cudaStream_t);
template void launch_rx_batched<float>(const RxSlot<float> *, const BatchIndex &, int, cudaStream_t);
template void launch_rx_batched<double>(const RxSlot<double> *, const BatchIndex &, int, cudaStream_t);

}  // namespace tcsem
