// Device-side data layout and kernel entry points of the TCSEM path.
//
// HBM layout.  All seven volume arrays (Ex, Ey, Ez, Bx, By, Bz and the
// conductivity) share one padded geometry so that a single index expression
// addresses any of them and neighbouring components line up in memory:
//   x (fastest): i in [-4, XP-4), row pitch XP = round_up(L + 6, 32) elements,
//                so i = 0 starts on a 128-byte boundary;
//   y          : j in [-1, M]    (YP = M + 2 rows per plane);
//   z          : k in [-1, N]    (N + 2 planes).
// Cells outside a component's update range stay zero for the life of the run.
// Plane k = -1 of Bx and By holds the air-interface fields BxAir/ByAir that
// the boundary pipeline writes each step, plane k = -1 of the conductivity is
// the air (0 S/m), and plane N of Ex/Ey/Bz is the zero bottom -- so the
// kernels need no special case for the top or bottom plane.
#pragma once
#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>
#include <cstdint>

namespace tcsem {

struct Geom {
    int L, M, N;
    int XP, YP;
    long long PS;  // plane stride XP*YP
    __host__ __device__ long long at(int i, int j, int k) const {
        return ((long long)(k + 1) * YP + (j + 1)) * XP + (i + 4);
    }
    __host__ __device__ long long total() const { return PS * (long long)(N + 2); }
};

inline Geom make_geom(int L, int M, int N) {
    Geom g;
    g.L = L; g.M = M; g.N = N;
    g.XP = ((L + 6 + 31) / 32) * 32;
    g.YP = M + 2;
    g.PS = (long long)g.XP * g.YP;
    return g;
}

// per-axis tables: sizes and reciprocals of sizes / summed sizes
template <typename T> struct Axis {
    const T *dxk, *dyk, *dzk;  // cell sizes as the reference kernels evaluate them
    const T *rdx, *rdy, *rdz;  // 1/dxk ...
    const T *rdx2, *rdy2;      // 1/(dxk[i-1]+dxk[i]), 1/(dyk[j-1]+dyk[j]) (index 0 unused)
    const T *rdzs;             // 1/(dzk[k-1]+dzk[k]), k=0: 1/(2 dzk[0])
};

template <typename T> struct FieldSet {
    T *ex, *ey, *ez, *bx, *by, *bz;
};

// scalars of one time step
template <typename T> struct StepScalars {
    T lam2;  // 2*lambda (gamma term of DuFort-Frankel)
    T dt;    // E step dt1
    T c4;    // 4*dt/mu0
    T dtb;   // B step 0.5*(dt1+dt2)
    T wave;  // source amplitude of this step (0 once the source is off)
};

// source segments (at most kMaxSeg per transmitter), see setup.h
constexpr int kMaxSeg = 6;
template <typename T> struct SourceTable {
    int nseg;
    int comp[kMaxSeg], i[kMaxSeg], j[kMaxSeg], k[kMaxSeg], count[kMaxSeg], off[kMaxSeg];
    const T *coef;  // gain already folded in: value = wave * coef[off + q]
};

// which step of a captured block a kernel belongs to: step = *base + off;
// kernels do nothing once step >= nsteps.  base == nullptr: always run.
struct StepGate {
    const int *base;
    int off;
    long nsteps;
    __device__ __forceinline__ long step() const { return (long)*base + off; }
};

// z-chunks of the fused sweep: chunk c covers planes [kb[c], kb[c+1]); the
// top chunk may be shorter than the others (it runs after the boundary)
constexpr int kMaxChunks = 16;
struct ZChunks {
    int n;
    int kb[kMaxChunks + 1];
    // kb[c] for a run-time c without indexing the array (it may live in the
    // kernel's parameter space)
    __host__ __device__ __forceinline__ int plane(int c) const {
        int v = 0;
#pragma unroll
        for (int q = 0; q <= kMaxChunks; q++) v = q == c ? kb[q] : v;
        return v;
    }
};

// ----------------------------------------------------------------- launchers
// volume.cu
template <typename T>
void launch_update_e(const Geom &g, FieldSet<T> f, const T *con, const Axis<T> &ax, StepScalars<T> s,
                     const SourceTable<T> &src, int *err, cudaStream_t st);
template <typename T>
void launch_bderivate(const Geom &g, FieldSet<T> f, const Axis<T> &ax, T dtb, int *err, cudaStream_t st);
// TMA descriptors of the fused sweep's inputs: ex ey ez bx by bz of one field set, then sigma
struct SweepMaps {
    CUtensorMap m[7];
};
// chunks c0 .. c1-1 in one launch; rev = the last chunk's blocks first (consecutive
// steps alternate, so a step starts on the planes the previous one wrote last,
// which may still be in L2); pdl = programmatic dependent launch after the previous
// kernel on the stream (the CTAs wait for it before loading the air plane k = -1)
template <typename T>
void launch_fused_sweep(const SweepMaps &maps, const Geom &g, FieldSet<T> out, const T *tin, T *tout,
                        const Axis<T> &ax, StepScalars<T> s, const StepScalars<T> *table, StepGate gate,
                        const SourceTable<T> &src, const ZChunks &zc, int c0, int c1, bool rev, int *err,
                        cudaStream_t st, bool pdl = false);
template <typename T> cudaError_t sweep_configure(int N);
template <typename T> size_t sweep_smem_bytes(int N);
template <typename T> int sweep_blocks_per_sm(int N);  // resident sweep CTAs per SM (after sweep_configure)
int sweep_box_x();
int sweep_box_y();
template <typename T> void launch_bz_consolidate(const Geom &g, T *bz, T *tot, const ZChunks &zc, cudaStream_t st);

// ------------------------------------------------------------------ batches
// Several simulations advanced by one launch per kernel: block b of a batched
// launch belongs to slot q with off[q] <= b < off[q+1] (the list is passed by
// value, so a block finds its slot in a few constant-cache reads).
constexpr int kMaxSlots = 64;
struct BatchIndex {
    int n;                   // slots
    int off[kMaxSlots + 1];  // first block of each slot, off[n] = total
    __host__ __device__ int total() const { return off[n]; }
    __device__ __forceinline__ int slot_of(int b) const {
        int lo = 0, hi = n;  // off[lo] <= b < off[hi]; empty slots are skipped
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (off[mid] <= b) lo = mid; else hi = mid;
        }
        return lo;
    }
};

// everything one step of the fused sweep needs for one slot (device memory)
template <typename T> struct SweepSlot {
    SweepMaps maps;
    Geom g;
    FieldSet<T> out;
    const T *tin;
    T *tout;
    Axis<T> ax;
    const StepScalars<T> *table;  // per step of the slot's run
    const int *step_base;         // the slot's step counter; step = *step_base + s
    long nsteps;
    SourceTable<T> src;
    ZChunks zc;
    int *err;
    int tiles_x, tiles_y;
};
// the blocks of each slot cover its chunks c0, c0+1, ... (tiles_x * tiles_y blocks per chunk)
template <typename T>
void launch_sweep_batched(const SweepSlot<T> *slots, const BatchIndex &idx, int s, int c0, int N_max, cudaStream_t st);
int sweep_tiles_x(int L);
int sweep_tiles_y(int M);

}  // namespace tcsem
