// Volume kernels: DuFort-Frankel E update, source injection and B update on
// the staggered non-uniform grid.
//
// Two forms:
//  * reference-structured kernels (k_update_e, k_source, k_update_bxy,
//    k_update_bz) that update one field set in place, stage by stage, as
//    ElectricalField/Bderivate do (ElectricalFiled.cu:89-475, Bderivate.cu:79-265);
//  * the production fused sweep (k_sweep): one pass over the volume per
//    time step that reads the old E/B/sigma planes and writes the new E and B
//    into the other buffer of a ping-pong pair.  It marches z bottom-up so the
//    div B = 0 prefix for Bz (Bderivate.cu:202-265) runs in a register, and each
//    CTA recomputes the one-cell halo of E/B it needs instead of waiting for
//    its neighbours.  Algorithmic traffic: 7 words read + 6 written per cell.
#include "kernels.cuh"
#include "async.cuh"
#include "check.cuh"
#include "sweep.cuh"

namespace tcsem {

// ------------------------------------------------------------------ helpers

template <typename T> __device__ __forceinline__ T recip(T x) { return T(1) / x; }

// DuFort-Frankel update of one E component (ElectricalFiled.cu:138-139):
//   E <- (2g - s dt)/(2g + s dt) E + 4 dt/(2g + s dt) curl / mu0
template <typename T>
__device__ __forceinline__ T df_update(const StepScalars<T> &s, T sigma, T e_old, T curl) {
    T sdt = sigma * s.dt;
    T r = recip(s.lam2 + sdt);
    return (s.lam2 - sdt) * r * e_old + s.c4 * r * curl;
}

// ----------------------------------------------------- reference-structured

template <typename T>
__global__ void k_update_e(Geom g, FieldSet<T> f, const T *__restrict__ con, Axis<T> ax, StepScalars<T> s, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.L || j >= g.M) return;
    const long long PS = g.PS, XP = g.XP;
    const bool vx = j >= 1, vy = i >= 1, vz = vx && vy;
    const T rdy2 = vx ? ax.rdy2[j] : T(0), rdx2 = vy ? ax.rdx2[i] : T(0);
    long long c = g.at(i, j, 0);
    for (int k = 0; k < g.N; k++, c += PS) {
        if (!TCSEM_IN(c + PS, g.total(), err) || !TCSEM_IN(c - PS - XP - 1, g.total(), err)) continue;
        const T rzs = ax.rdzs[k];
        if (vx) {  // UpdateEx, ElectricalFiled.cu:89-175
            T sg = T(0.5) * (T(0.5) * (con[c - XP] + con[c]) + T(0.5) * (con[c - PS - XP] + con[c - PS]));
            T curl = (f.bz[c] - f.bz[c - XP]) * rdy2 - (f.by[c] - f.by[c - PS]) * rzs;
            f.ex[c] = df_update(s, sg, f.ex[c], curl);
        }
        if (vy) {  // UpdateEy, :178-274
            T sg = T(0.25) * (con[c - 1] + con[c] + con[c - PS - 1] + con[c - PS]);
            T curl = (f.bx[c] - f.bx[c - PS]) * rzs - (f.bz[c] - f.bz[c - 1]) * rdx2;
            f.ey[c] = df_update(s, sg, f.ey[c], curl);
        }
        if (vz) {  // UpdateEz, :277-345
            T sg = T(0.25) * (con[c - XP - 1] + con[c - XP] + con[c - 1] + con[c]);
            T curl = (f.by[c] - f.by[c - 1]) * rdx2 - (f.bx[c] - f.bx[c - XP]) * rdy2;
            f.ez[c] = df_update(s, sg, f.ez[c], curl);
        }
    }
}

// AddTx_x/_y/_z (ElectricalFiled.cu:347-475): one thread per injected cell
template <typename T>
__global__ void k_source(Geom g, FieldSet<T> f, SourceTable<T> src, T wave, int *err) {
    for (int sgi = 0; sgi < src.nseg; sgi++) {
        for (int q = threadIdx.x; q < src.count[sgi]; q += blockDim.x) {
            int i = src.i[sgi], j = src.j[sgi], k = src.k[sgi];
            T *e = src.comp[sgi] == 0 ? f.ex : src.comp[sgi] == 1 ? f.ey : f.ez;
            if (src.comp[sgi] == 0) i += q; else if (src.comp[sgi] == 1) j += q; else k += q;
            if (TCSEM_IN(g.at(i, j, k), g.total(), err)) e[g.at(i, j, k)] -= wave * src.coef[src.off[sgi] + q];
        }
        __syncthreads();
    }
}

// UpdateBx/UpdateBy, Bderivate.cu:79-200
template <typename T>
__global__ void k_update_bxy(Geom g, FieldSet<T> f, Axis<T> ax, T dtb, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.L || j >= g.M) return;
    const long long PS = g.PS, XP = g.XP;
    const T rdy = ax.rdy[j], rdx = ax.rdx[i];
    long long c = g.at(i, j, 0);
    for (int k = 0; k < g.N; k++, c += PS) {
        if (!TCSEM_IN(c + PS, g.total(), err) || !TCSEM_IN(c, g.total(), err)) continue;
        const T rdz = ax.rdz[k];
        if (i >= 1) f.bx[c] += ((f.ey[c + PS] - f.ey[c]) * rdz - (f.ez[c + XP] - f.ez[c]) * rdy) * dtb;
        if (j >= 1) f.by[c] += ((f.ez[c + 1] - f.ez[c]) * rdx - (f.ex[c + PS] - f.ex[c]) * rdz) * dtb;
    }
}

// UpdateBz, Bderivate.cu:202-265: div B = 0, integrated from the bottom up
template <typename T>
__global__ void k_update_bz(Geom g, FieldSet<T> f, Axis<T> ax, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.L || j >= g.M) return;
    const long long PS = g.PS, XP = g.XP;
    const T rdx = ax.rdx[i], rdy = ax.rdy[j];
    long long c = g.at(i, j, g.N - 1);
    T acc = T(0);
    for (int k = g.N - 1; k >= 0; k--, c -= PS) {
        if (!TCSEM_IN(c + XP, g.total(), err) || !TCSEM_IN(c, g.total(), err)) continue;
        acc += ax.dzk[k] * ((f.bx[c + 1] - f.bx[c]) * rdx + (f.by[c + XP] - f.by[c]) * rdy);
        f.bz[c] = acc;
    }
}

template <typename T>
void launch_update_e(const Geom &g, FieldSet<T> f, const T *con, const Axis<T> &ax, StepScalars<T> s,
                     const SourceTable<T> &src, int *err, cudaStream_t st) {
    dim3 blk(32, 8), grd((g.L + 31) / 32, (g.M + 7) / 8);
    k_update_e<T><<<grd, blk, 0, st>>>(g, f, con, ax, s, err);
    if (src.nseg > 0 && s.wave != T(0)) k_source<T><<<1, 128, 0, st>>>(g, f, src, s.wave, err);
}

template <typename T>
void launch_bderivate(const Geom &g, FieldSet<T> f, const Axis<T> &ax, T dtb, int *err, cudaStream_t st) {
    dim3 blk(32, 8), grd((g.L + 31) / 32, (g.M + 7) / 8);
    k_update_bxy<T><<<grd, blk, 0, st>>>(g, f, ax, dtb, err);
    k_update_bz<T><<<grd, blk, 0, st>>>(g, f, ax, err);
}


template <typename T>
__global__ void __launch_bounds__(fs3::NT, sizeof(T) == 4 ? 2 : 1)
    k_sweep(const __grid_constant__ SweepMaps maps, Geom g, FieldSet<T> out, const T *__restrict__ tin,
            T *__restrict__ tout, Axis<T> ax, StepScalars<T> sdir, const StepScalars<T> *__restrict__ table,
            StepGate gate, SourceTable<T> src, ZChunks zc, int cbase, int rev, int *err) {
    StepScalars<T> s = sdir;
    if (gate.base) {
        const long st = gate.step();
        if (st >= gate.nsteps) return;
        s = table[st];
    }
    const int c = cbase + (int)(rev ? gridDim.z - 1 - blockIdx.z : blockIdx.z);
    sweep_cta<T>(maps, g, out, tin, tout, ax, s, src, zc, blockIdx.x, blockIdx.y, c, err);
}

// every slot of a batch in one launch: block b belongs to the slot whose range of idx holds it
template <typename T>
__global__ void __launch_bounds__(fs3::NT, sizeof(T) == 4 ? 2 : 1)
    k_sweep_batched(const SweepSlot<T> *__restrict__ slots, const __grid_constant__ BatchIndex idx, int s, int c0) {
    const int q = idx.slot_of(blockIdx.x);
    const SweepSlot<T> &d = slots[q];
    const long st = (long)*d.step_base + s;
    if (st >= d.nsteps) return;
    const int lb = blockIdx.x - idx.off[q];
    const int bx = lb % d.tiles_x, rest = lb / d.tiles_x, by = rest % d.tiles_y, c = c0 + rest / d.tiles_y;
    sweep_cta<T>(d.maps, d.g, d.out, d.tin, d.tout, d.ax, d.table[st], d.src, d.zc, bx, by, c, d.err);
}

template <typename T>
void launch_fused_sweep(const SweepMaps &maps, const Geom &g, FieldSet<T> out, const T *tin, T *tout,
                        const Axis<T> &ax, StepScalars<T> s, const StepScalars<T> *table, StepGate gate,
                        const SourceTable<T> &src, const ZChunks &zc, int c0, int c1, bool rev, int *err,
                        cudaStream_t st, bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((g.L + fs3::TX - 1) / fs3::TX, (g.M + fs3::BY - 1) / fs3::BY, c1 - c0);
    cfg.blockDim = dim3(fs3::NT);
    cfg.dynamicSmemBytes = fs3::smem_bytes_n<T>(g.N);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_sweep<T>, maps, g, out, tin, tout, ax, s, table, gate, src, zc, c0, rev ? 1 : 0, err);
}

template <typename T>
void launch_sweep_batched(const SweepSlot<T> *slots, const BatchIndex &idx, int s, int c0, int N_max, cudaStream_t st) {
    if (idx.total() == 0) return;
    k_sweep_batched<T><<<idx.total(), fs3::NT, fs3::smem_bytes_n<T>(N_max), st>>>(slots, idx, s, c0);
}
int sweep_tiles_x(int L) { return (L + fs3::TX - 1) / fs3::TX; }
int sweep_tiles_y(int M) { return (M + fs3::BY - 1) / fs3::BY; }

template <typename T> cudaError_t sweep_configure(int N) {
    const int sm = (int)fs3::smem_bytes_n<T>(N);
    cudaError_t e = cudaFuncSetAttribute(k_sweep<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_sweep_batched<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
}
template <typename T> size_t sweep_smem_bytes(int N) { return fs3::smem_bytes_n<T>(N); }
template <typename T> int sweep_blocks_per_sm(int N) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_sweep<T>, fs3::NT, fs3::smem_bytes_n<T>(N)) != cudaSuccess)
        return 1;
    return nb > 0 ? nb : 1;
}
int sweep_box_x() { return fs3::BXW; }
int sweep_box_y() { return fs3::BYH; }

// materialise Bz = P + O_c in place and clear the chunk totals
template <typename T>
__global__ void k_bz_consolidate(Geom g, T *bz, T *tot, ZChunks zc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i > g.L || j > g.M || zc.n <= 1) return;
    const int XP = g.XP, PS = (int)g.PS, plane = (g.M + 2) * XP;
    const int col = (j + 1) * XP + (i + 4);
    T o = T(0);
    for (int c = zc.n - 1; c >= 0; c--) {
        for (int k = zc.kb[c]; k < zc.kb[c + 1]; k++) bz[col + (k + 1) * PS] += o;
        o += tot[c * plane + col];
        tot[c * plane + col] = T(0);
    }
}

template <typename T> void launch_bz_consolidate(const Geom &g, T *bz, T *tot, const ZChunks &zc, cudaStream_t st) {
    if (zc.n <= 1) return;
    dim3 blk(32, 8), grd((g.L + 1 + 31) / 32, (g.M + 1 + 7) / 8);
    k_bz_consolidate<T><<<grd, blk, 0, st>>>(g, bz, tot, zc);
}

#define INST(T)                                                                                                    \
    template void launch_update_e<T>(const Geom &, FieldSet<T>, const T *, const Axis<T> &, StepScalars<T>,        \
                                     const SourceTable<T> &, int *, cudaStream_t);                                 \
    template void launch_bderivate<T>(const Geom &, FieldSet<T>, const Axis<T> &, T, int *, cudaStream_t);         \
    template void launch_fused_sweep<T>(const SweepMaps &, const Geom &, FieldSet<T>, const T *, T *,             \
                                        const Axis<T> &, StepScalars<T>, const StepScalars<T> *, StepGate,         \
                                        const SourceTable<T> &, const ZChunks &, int, int, bool, int *, cudaStream_t,  \
                                        bool);                                                                     \
    template cudaError_t sweep_configure<T>(int);                                                                  \
    template size_t sweep_smem_bytes<T>(int);                                                                      \
    template int sweep_blocks_per_sm<T>(int);                                                                      \
    template void launch_bz_consolidate<T>(const Geom &, T *, T *, const ZChunks &, cudaStream_t);             \
    template void launch_sweep_batched<T>(const SweepSlot<T> *, const BatchIndex &, int, int, int, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace tcsem
