// Volume kernels: DuFort-Frankel E update, source injection and B update on
// the staggered non-uniform grid.
//
// Two forms:
//  * reference-structured kernels (k_update_e, k_source, k_update_bxy,
//    k_update_bz) that update one field set in place, stage by stage, as
//    ElectricalField/Bderivate do (ElectricalFiled.cu:89-475, Bderivate.cu:79-265);
//  * the production fused sweep (k_fused_sweep): one pass over the volume per
//    time step that reads the old E/B/sigma planes and writes the new E and B
//    into the other buffer of a ping-pong pair.  It marches z bottom-up so the
//    div B = 0 prefix for Bz (Bderivate.cu:202-265) runs in a register, and each
//    CTA recomputes the one-cell halo of E/B it needs instead of waiting for
//    its neighbours.  Algorithmic traffic: 7 words read + 6 written per cell.
#include "kernels.cuh"

namespace tcsem {

// ------------------------------------------------------------------ helpers

template <typename T> __device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

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
__global__ void k_update_e(Geom g, FieldSet<T> f, const T *__restrict__ con, Axis<T> ax, StepScalars<T> s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.L || j >= g.M) return;
    const long long PS = g.PS, XP = g.XP;
    const bool vx = j >= 1, vy = i >= 1, vz = vx && vy;
    const T rdy2 = vx ? ax.rdy2[j] : T(0), rdx2 = vy ? ax.rdx2[i] : T(0);
    long long c = g.at(i, j, 0);
    for (int k = 0; k < g.N; k++, c += PS) {
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
__global__ void k_source(Geom g, FieldSet<T> f, SourceTable<T> src, T wave) {
    for (int sgi = 0; sgi < src.nseg; sgi++) {
        for (int q = threadIdx.x; q < src.count[sgi]; q += blockDim.x) {
            int i = src.i[sgi], j = src.j[sgi], k = src.k[sgi];
            T *e = src.comp[sgi] == 0 ? f.ex : src.comp[sgi] == 1 ? f.ey : f.ez;
            if (src.comp[sgi] == 0) i += q; else if (src.comp[sgi] == 1) j += q; else k += q;
            e[g.at(i, j, k)] -= wave * src.coef[src.off[sgi] + q];
        }
        __syncthreads();
    }
}

// UpdateBx/UpdateBy, Bderivate.cu:79-200
template <typename T>
__global__ void k_update_bxy(Geom g, FieldSet<T> f, Axis<T> ax, T dtb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.L || j >= g.M) return;
    const long long PS = g.PS, XP = g.XP;
    const T rdy = ax.rdy[j], rdx = ax.rdx[i];
    long long c = g.at(i, j, 0);
    for (int k = 0; k < g.N; k++, c += PS) {
        const T rdz = ax.rdz[k];
        if (i >= 1) f.bx[c] += ((f.ey[c + PS] - f.ey[c]) * rdz - (f.ez[c + XP] - f.ez[c]) * rdy) * dtb;
        if (j >= 1) f.by[c] += ((f.ez[c + 1] - f.ez[c]) * rdx - (f.ex[c + PS] - f.ex[c]) * rdz) * dtb;
    }
}

// UpdateBz, Bderivate.cu:202-265: div B = 0, integrated from the bottom up
template <typename T>
__global__ void k_update_bz(Geom g, FieldSet<T> f, Axis<T> ax) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.L || j >= g.M) return;
    const long long PS = g.PS, XP = g.XP;
    const T rdx = ax.rdx[i], rdy = ax.rdy[j];
    long long c = g.at(i, j, g.N - 1);
    T acc = T(0);
    for (int k = g.N - 1; k >= 0; k--, c -= PS) {
        acc += ax.dzk[k] * ((f.bx[c + 1] - f.bx[c]) * rdx + (f.by[c + XP] - f.by[c]) * rdy);
        f.bz[c] = acc;
    }
}

template <typename T>
void launch_update_e(const Geom &g, FieldSet<T> f, const T *con, const Axis<T> &ax, StepScalars<T> s,
                     const SourceTable<T> &src, cudaStream_t st) {
    dim3 blk(32, 8), grd((g.L + 31) / 32, (g.M + 7) / 8);
    k_update_e<T><<<grd, blk, 0, st>>>(g, f, con, ax, s);
    if (src.nseg > 0 && s.wave != T(0)) k_source<T><<<1, 128, 0, st>>>(g, f, src, s.wave);
}

template <typename T>
void launch_bderivate(const Geom &g, FieldSet<T> f, const Axis<T> &ax, T dtb, cudaStream_t st) {
    dim3 blk(32, 8), grd((g.L + 31) / 32, (g.M + 7) / 8);
    k_update_bxy<T><<<grd, blk, 0, st>>>(g, f, ax, dtb);
    k_update_bz<T><<<grd, blk, 0, st>>>(g, f, ax);
}

// ------------------------------------------------------------- fused sweep

namespace fs {
constexpr int TX = 32, TY = 8;           // owned tile (x, y)
constexpr int NT = TX * TY;              // threads per CTA
constexpr int SX = 40, SY = TY + 2;      // shared plane: i in [i0-4, i0+36), j in [j0-1, j0+TY]
constexpr int SP = SX * SY;
constexpr int RW = TX + 2, RH = TY + 2;  // loaded region: i in [i0-1, i0+TX], j in [j0-1, j0+TY]
constexpr int RN = RW * RH;              // 340 elements
constexpr int EW = TX + 1, EH = TY + 1;  // E work region: i in [i0, i0+TX], j in [j0, j0+TY]
constexpr int EN = EW * EH;              // 297 items
static_assert(RN <= 2 * NT && EN <= 2 * NT, "two items per thread");
__device__ __forceinline__ int sidx(int li, int lj) { return (lj + 1) * SX + li + 4; }  // li = i-i0, lj = j-j0
}  // namespace fs

template <typename T>
__global__ void __launch_bounds__(fs::NT) k_fused_sweep(Geom g, FieldSet<T> in, FieldSet<T> out,
                                                       const T *__restrict__ con, Axis<T> ax, StepScalars<T> sdir,
                                                       const StepScalars<T> *__restrict__ table, StepGate gate,
                                                       SourceTable<T> src) {
    using namespace fs;
    StepScalars<T> s = sdir;
    if (gate.base) {
        const long st = gate.step();
        if (st >= gate.nsteps) return;
        s = table[st];
    }
    __shared__ T s_bx[2][SP], s_by[2][SP], s_sg[2][SP], s_bz[SP];
    __shared__ T s_ex[2][SP], s_ey[2][SP], s_ez[SP], s_bxn[SP], s_byn[SP];

    const int tid = threadIdx.x;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int L = g.L, M = g.M, N = g.N;
    const long long PS = g.PS, XP = g.XP;

    // region elements handled by this thread (load phase)
    int rs[2];
    long long rg[2];
    bool rv[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        int e = tid + q * NT;
        int li = e % RW - 1, lj = e / RW - 1;
        int i = i0 + li, j = j0 + lj;
        rv[q] = e < RN && i <= L && j <= M;
        rs[q] = e < RN ? sidx(li, lj) : 0;
        rg[q] = g.at(i, j, 0);
    }
    // E work items handled by this thread
    int es[2], ei[2], ej[2];
    long long eg[2];
    bool ev[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        int e = tid + q * NT;
        int li = e % EW, lj = e / EW;
        ei[q] = i0 + li; ej[q] = j0 + lj;
        ev[q] = e < EN;
        es[q] = ev[q] ? sidx(li, lj) : 0;
        eg[q] = g.at(ei[q], ej[q], 0);
    }
    const bool own = true;  // every thread owns exactly one cell of the TX x TY tile
    const int oi = i0 + (tid % TX), oj = j0 + (tid / TX);
    const int os = sidx(tid % TX, tid / TX);
    const bool oin = oi < L && oj < M;
    const long long og = g.at(oi, oj, 0);
    const T o_rdx = oin ? ax.rdx[oi] : T(0), o_rdy = oin ? ax.rdy[oj] : T(0);

    // zero the E(k+1) slot (plane N of Ex/Ey is the zero bottom)
    for (int e = tid; e < SP; e += NT) { s_ex[1][e] = T(0); s_ey[1][e] = T(0); }
    // prologue: B_old and sigma of the bottom plane straight into the "cur" slot
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (tid + q * NT < RN) {
            long long p = rg[q] + (long long)(N - 1) * PS;
            s_bx[0][rs[q]] = rv[q] ? ldg(in.bx + p) : T(0);
            s_by[0][rs[q]] = rv[q] ? ldg(in.by + p) : T(0);
            s_sg[0][rs[q]] = rv[q] ? ldg(con + p) : T(0);
        }
    }
    // registers: region prefetch (Bx/By/sigma of plane k-1, Bz of plane k), E_old of plane k
    T pbx[2], pby[2], psg[2], pbz[2], pex[2], pey[2], pez[2];
    auto prefetch = [&](int k) {  // data for iteration k
#pragma unroll
        for (int q = 0; q < 2; q++) {
            long long pm = rg[q] + (long long)(k - 1) * PS, pk = rg[q] + (long long)k * PS;
            pbx[q] = rv[q] ? ldg(in.bx + pm) : T(0);
            pby[q] = rv[q] ? ldg(in.by + pm) : T(0);
            psg[q] = rv[q] ? ldg(con + pm) : T(0);
            pbz[q] = rv[q] ? ldg(in.bz + pk) : T(0);
            bool ok = ev[q] && ei[q] <= L && ej[q] <= M;
            long long pe = eg[q] + (long long)k * PS;
            pex[q] = ok ? ldg(in.ex + pe) : T(0);
            pey[q] = ok ? ldg(in.ey + pe) : T(0);
            pez[q] = ok ? ldg(in.ez + pe) : T(0);
        }
    };
    prefetch(N - 1);

    T acc = T(0);
    int cur = 0, ecur = 0;
    for (int k = N - 1; k >= 0; k--) {
        const int nxt = cur ^ 1, eprev = ecur ^ 1;
        // phase 1: publish the prefetched planes, keep E_old(k), prefetch k-1
        T cex[2], cey[2], cez[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (tid + q * NT < RN) {
                s_bx[nxt][rs[q]] = pbx[q];
                s_by[nxt][rs[q]] = pby[q];
                s_sg[nxt][rs[q]] = psg[q];
                s_bz[rs[q]] = pbz[q];
            }
            cex[q] = pex[q]; cey[q] = pey[q]; cez[q] = pez[q];
        }
        if (k > 0) prefetch(k - 1);
        __syncthreads();

        // phase 2: E(k) on the (TX+1) x (TY+1) work region
        const T rzs = ax.rdzs[k];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (!ev[q]) continue;
            const int i = ei[q], j = ej[q], c = es[q];
            T ex = cex[q], ey = cey[q], ez = cez[q];
            const bool inx = i < L, iny = j < M;
            if (inx && iny && j >= 1) {
                T sg = T(0.5) * (T(0.5) * (s_sg[cur][c - SX] + s_sg[cur][c]) + T(0.5) * (s_sg[nxt][c - SX] + s_sg[nxt][c]));
                T curl = (s_bz[c] - s_bz[c - SX]) * ax.rdy2[j] - (s_by[cur][c] - s_by[nxt][c]) * rzs;
                ex = df_update(s, sg, ex, curl);
            }
            if (inx && iny && i >= 1) {
                T sg = T(0.25) * (s_sg[cur][c - 1] + s_sg[cur][c] + s_sg[nxt][c - 1] + s_sg[nxt][c]);
                T curl = (s_bx[cur][c] - s_bx[nxt][c]) * rzs - (s_bz[c] - s_bz[c - 1]) * ax.rdx2[i];
                ey = df_update(s, sg, ey, curl);
            }
            if (inx && iny && i >= 1 && j >= 1) {
                T sg = T(0.25) * (s_sg[cur][c - SX - 1] + s_sg[cur][c - SX] + s_sg[cur][c - 1] + s_sg[cur][c]);
                T curl = (s_by[cur][c] - s_by[cur][c - 1]) * ax.rdx2[i] - (s_bx[cur][c] - s_bx[cur][c - SX]) * ax.rdy2[j];
                ez = df_update(s, sg, ez, curl);
            }
            if (s.wave != T(0)) {  // AddTx_*: subtract after the update of the cell
                for (int sgi = 0; sgi < src.nseg; sgi++) {
                    const int cp = src.comp[sgi];
                    int q0;
                    if (cp == 0) { if (j != src.j[sgi] || k != src.k[sgi]) continue; q0 = i - src.i[sgi]; }
                    else if (cp == 1) { if (i != src.i[sgi] || k != src.k[sgi]) continue; q0 = j - src.j[sgi]; }
                    else { if (i != src.i[sgi] || j != src.j[sgi]) continue; q0 = k - src.k[sgi]; }
                    if (q0 < 0 || q0 >= src.count[sgi]) continue;
                    T v = s.wave * src.coef[src.off[sgi] + q0];
                    if (cp == 0) ex -= v; else if (cp == 1) ey -= v; else ez -= v;
                }
            }
            s_ex[ecur][c] = ex; s_ey[ecur][c] = ey; s_ez[c] = ez;
            if (i - i0 < TX && j - j0 < TY && inx && iny) {
                long long p = eg[q] + (long long)k * PS;
                out.ex[p] = ex; out.ey[p] = ey; out.ez[p] = ez;
            }
        }
        __syncthreads();

        // phase 3: Bx on [i0, i0+TX] x [j0, j0+TY), By on [i0, i0+TX) x [j0, j0+TY]
        const T rdz = ax.rdz[k], dtb = s.dtb;
        for (int e = tid; e < (TX + 1) * TY + TX * (TY + 1); e += NT) {
            if (e < (TX + 1) * TY) {
                int li = e % (TX + 1), lj = e / (TX + 1), i = i0 + li, j = j0 + lj, c = sidx(li, lj);
                T b = s_bx[cur][c];
                if (i >= 1 && i < L && j < M)
                    b += ((s_ey[eprev][c] - s_ey[ecur][c]) * rdz - (s_ez[c + SX] - s_ez[c]) * ax.rdy[j]) * dtb;
                s_bxn[c] = b;
                if (li < TX && i < L && j < M) out.bx[g.at(i, j, k)] = b;
            } else {
                int e2 = e - (TX + 1) * TY;
                int li = e2 % TX, lj = e2 / TX, i = i0 + li, j = j0 + lj, c = sidx(li, lj);
                T b = s_by[cur][c];
                if (j >= 1 && j < M && i < L)
                    b += ((s_ez[c + 1] - s_ez[c]) * ax.rdx[i] - (s_ex[eprev][c] - s_ex[ecur][c]) * rdz) * dtb;
                s_byn[c] = b;
                if (lj < TY && i < L && j < M) out.by[g.at(i, j, k)] = b;
            }
        }
        __syncthreads();

        // phase 4: Bz(k) = Bz(k+1) + dz (dBx/dx + dBy/dy), owned cells
        if (own) {
            acc += ax.dzk[k] * ((s_bxn[os + 1] - s_bxn[os]) * o_rdx + (s_byn[os + SX] - s_byn[os]) * o_rdy);
            if (oin) out.bz[og + (long long)k * PS] = acc;
        }
        cur = nxt;
        ecur = eprev;
    }
}

template <typename T>
void launch_fused_sweep(const Geom &g, FieldSet<T> in, FieldSet<T> out, const T *con, const Axis<T> &ax,
                        StepScalars<T> s, const StepScalars<T> *table, StepGate gate,
                        const SourceTable<T> &src, cudaStream_t st) {
    dim3 grd((g.L + fs::TX - 1) / fs::TX, (g.M + fs::TY - 1) / fs::TY);
    k_fused_sweep<T><<<grd, fs::NT, 0, st>>>(g, in, out, con, ax, s, table, gate, src);
}

#define INST(T)                                                                                                    \
    template void launch_update_e<T>(const Geom &, FieldSet<T>, const T *, const Axis<T> &, StepScalars<T>,        \
                                     const SourceTable<T> &, cudaStream_t);                                        \
    template void launch_bderivate<T>(const Geom &, FieldSet<T>, const Axis<T> &, T, cudaStream_t);                \
    template void launch_fused_sweep<T>(const Geom &, FieldSet<T>, FieldSet<T>, const T *, const Axis<T> &,        \
                                        StepScalars<T>, const StepScalars<T> *, StepGate,                          \
                                        const SourceTable<T> &, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace tcsem
