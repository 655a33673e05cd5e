// The per-thread body of the receiver kernel, shared by the single-survey
// kernel, the batched kernel and the persistent batch scheduler.
#pragma once
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

}  // namespace tcsem
