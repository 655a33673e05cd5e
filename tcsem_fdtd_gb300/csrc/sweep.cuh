// The fused E/B sweep as a per-CTA body, shared by the single-survey kernel,
// the batched kernel and the persistent batch scheduler.
#pragma once
#include "async.cuh"
#include "check.cuh"
#include "kernels.cuh"

namespace tcsem {

// ------------------------------------------------------------- fused sweep
//
// One pass per time step over the volume: old E/B/sigma planes stream into a
// shared-memory ring through TMA bulk-tensor copies (cp.async.bulk.tensor,
// mbarrier completion), the new E and B go to the other buffer of the
// ping-pong pair.  Tiles are 64 x 8 columns, aligned so every TMA box starts
// on a 16-byte boundary; each thread owns two columns of a row (x = lane and
// lane + 32) and marches them z bottom-up through one
// z-chunk.  Warps 0..7 own the tile rows, warp 8 recomputes the +y halo row
// and warp 9 the +x halo column (E and the B components the tile's Bz needs),
// so no CTA waits for another; the -x/-y halo is plain old data in the TMA box.
// Neighbour values of the new fields go through double-buffered shared planes
// with one __syncthreads per z-plane:
//   iteration k:  B(k+1)  ->  E(k)  ->  publish Ez(k), B(k+1)  ->  sync
//                 ->  TMA of plane k-4 into the freed slot  ->  Bz(k+1)
//
// Bz within a chunk is the partial sum P(k) = sum_{k'=k}^{k1-1} dz div_xy B(k');
// the true Bz(k) = P(k) + O_c with O_c = sum of the chunk totals T_c' of the
// chunks below (c' > c).  Readers add O_c; T has one plane per chunk.

namespace fs3 {
constexpr int NC = 2;                  // cells per thread along x: lane and lane + 32
constexpr int TX = 32 * NC, BY = 8;    // owned tile 64 x 8
constexpr int NW = 10;                 // warps 0..7 own the tile rows, 8: +y halo row, 9: +x halo column
constexpr int NT = 32 * NW;
constexpr int BXW = TX + 8, BYH = BY + 2;  // TMA box 72 x 10: x in [i0-4, i0+68), y in [j0-1, j0+9)
constexpr int BOX = BXW * BYH;
constexpr int NARR = 7;                // ex ey ez bx by bz sigma
// ring stride of one box: rounded up to 128 bytes so every TMA destination is 128-byte aligned
template <typename T> __host__ __device__ constexpr int boxs() { return (int)(((BOX * sizeof(T) + 127) / 128) * 128 / sizeof(T)); }
constexpr int RING = 4;                // planes in flight
constexpr int XR = BY + 2, XC = TX + 2;  // exchange planes of the new fields
enum { AEX = 0, AEY, AEZ, ABX, ABY, ABZ, ASG };
// byte offset of the RING mbarriers: after the ring, the three exchange planes and the two offset boxes
template <typename T> __host__ __device__ constexpr size_t bars_offset() {
    return (size_t)RING * NARR * boxs<T>() * sizeof(T) + 3 * 2 * XR * XC * sizeof(T) + 2 * BOX * sizeof(T);
}
template <typename T> __host__ __device__ constexpr size_t smem_bytes() { return bars_offset<T>() + RING * 8 + 16; }
template <typename T> size_t smem_bytes_n(int N) {  // plus the z tables
    return ((smem_bytes<T>() + 3 * (size_t)(N + 3) * sizeof(T)) + 15) / 16 * 16;
}
}  // namespace fs3

// reciprocal used by the E update: one MUFU op in FP32 (about 1 ulp), exact division in FP64
template <typename T> __device__ __forceinline__ T rcp_fast(T x);
template <> __device__ __forceinline__ float rcp_fast<float>(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
template <> __device__ __forceinline__ double rcp_fast<double>(double x) { return 1.0 / x; }

// the three reciprocals of the E update: three MUFU ops in FP32; in FP64, where a division
// costs about ten FP64 pipe operations and the pipe bounds the sweep, one division of the
// product and five multiplies (1/a = bc / abc, ...), a few ulp from three divisions
__device__ __forceinline__ void recip3(float a, float b, float c, float &ra, float &rb, float &rc) {
    ra = rcp_fast(a);
    rb = rcp_fast(b);
    rc = rcp_fast(c);
}
__device__ __forceinline__ void recip3(double a, double b, double c, double &ra, double &rb, double &rc) {
    const double ab = a * b, r = 1.0 / (ab * c), rab = c * r;
    rc = ab * r;
    ra = b * rab;
    rb = a * rab;
}

// per-thread state of the sweep (NC cells per thread); sweep_plane<PH>() advances
// one z-plane with PH = (ktop - k) mod 4, so ring slots and exchange parities
// are compile-time constants
template <typename T> struct SweepThread {
    T *ring, *x_ez, *x_bxn, *x_byn;
    uint64_t *bars;
    int *s_flag;
    const CUtensorMap *maps;
    unsigned plane_bytes;
    int j, PS, N, k0, k1, klow, ktop, tid, i0, j0;
    int role;  // 0: a row of the tile, 1: the +y halo row, 2: the +x halo column (warp-uniform; FP64)
    int total;  // elements of each field array (bounds-checked builds)
    int *err;
    T rdy2, rdy, fy;  // per row: 1/(dy[j-1]+dy[j]), 1/dy[j], dtb/dy[j]
    // per cell
    int so[fs3::NC], xo[fs3::NC], i[fs3::NC], col[fs3::NC];
    bool own[fs3::NC], vEx[fs3::NC], vEy[fs3::NC], vEz[fs3::NC];
    T rdx2[fs3::NC], rdx[fs3::NC], fx[fs3::NC];
    T oc0[fs3::NC], oci[fs3::NC], ocj[fs3::NC];  // Bz chunk offsets of the plane being updated: at, left of, below the cell
    T ex1[fs3::NC], ey1[fs3::NC], exn[fs3::NC], eyn[fs3::NC], ezn[fs3::NC];
    T bxo1[fs3::NC], byo1[fs3::NC], bxn[fs3::NC], byn[fs3::NC], acc[fs3::NC];
    T sxk[fs3::NC], syk[fs3::NC], szk[fs3::NC], bxk[fs3::NC], byk[fs3::NC];  // sigma sums and own B of plane k
};

template <typename T, int PH, int ROLE>
__device__ __forceinline__ bool sweep_plane(SweepThread<T> &t, int k, unsigned rp, const StepScalars<T> &s,
                                            const T *__restrict__ zt, const FieldSet<T> &out,
                                            const SourceTable<T> &src, bool src_tile) {
    using namespace fs3;
    constexpr int BS = boxs<T>();
    constexpr int S0 = PH, S1 = (PH + 1) & 3;
    constexpr int QE = PH & 1, QB = (PH + 1) & 1;
    constexpr int XP2 = XR * XC;
    const int zi = k - t.klow;  // z tables: rdz, rdzs, dzk of plane klow + zi
    // Roles (one compiled copy each, FP64 only): the row warps update and store every component; the
    // +y halo row warp only produces what the tile's last row reads from it (Ex and Ez for By there,
    // By for Bz), the +x halo column warp what the tile's last column reads (Ey and Ez for Bx there,
    // Bx for Bz).  Every copy passes the one barrier per plane in the same order.
    constexpr bool rX = ROLE != 2, rY = ROLE != 1, rR = ROLE == 0;
    // ---- B_new(k+1) from E_new(k+1) (own + neighbours) and E_new(k+2)
    const bool doB = k + 1 < t.k1;
    if (doB) {
        const T fz = zt[3 * (zi + 1)] * s.dtb;  // dtb / dz(k+1)
#pragma unroll
        for (int c = 0; c < NC; c++) {
            if constexpr (rY) {
                const T ezj = t.x_ez[QB * XP2 + t.xo[c] + XC];
                const T bx = t.bxo1[c] + (t.ey1[c] - t.eyn[c]) * fz - (ezj - t.ezn[c]) * t.fy;
                t.bxn[c] = t.vEy[c] ? bx : t.bxo1[c];
            }
            if constexpr (rX) {
                const T ezi = t.x_ez[QB * XP2 + t.xo[c] + 1];
                const T by = t.byo1[c] + (ezi - t.ezn[c]) * t.fx[c] - (t.ex1[c] - t.exn[c]) * fz;
                t.byn[c] = t.vEx[c] ? by : t.byo1[c];
            }
            if (rR && t.own[c] && TCSEM_IN(t.col[c] + (k + 2) * t.PS, t.total, t.err)) {
                const int o = t.col[c] + (k + 2) * t.PS;
                out.bx[o] = t.bxn[c];
                out.by[o] = t.byn[c];
            }
        }
    }
    // ---- E_new(k)
#pragma unroll
    for (int c = 0; c < NC; c++) {
        t.ex1[c] = t.exn[c];
        t.ey1[c] = t.eyn[c];
    }
    if (k >= t.k0) {
        const bool upd = k < t.N, lo = k < t.k1;
        const T rzs = zt[3 * zi + 1];
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const T *p0 = t.ring + S0 * NARR * BS + t.so[c], *p1 = t.ring + S1 * NARR * BS + t.so[c];
            const T a1 = p1[ASG * BS], b1 = p1[ASG * BS - 1], c1 = p1[ASG * BS - BXW], d1 = p1[ASG * BS - BXW - 1];
            const T bym = p1[ABY * BS], bxm = p1[ABX * BS];
            const T sx1 = a1 + c1, sy1 = a1 + b1, sz1 = sx1 + b1 + d1;
            const T ezo = p0[AEZ * BS];
            T exo = T(0), eyo = T(0);
            if constexpr (rX) exo = p0[AEX * BS];
            if constexpr (rY) eyo = p0[AEY * BS];
            if (upd) {
                const T bz = p0[ABZ * BS] + t.oc0[c];
                const T byi = p0[ABY * BS - 1], bxj = p0[ABX * BS - BXW];
                // DuFort-Frankel update (ElectricalFiled.cu:89-345) of the three components, computed for
                // every cell and kept where the component is updated; s.dt carries the 1/4 of the sigma sums
                const T sdx = (t.sxk[c] + sx1) * s.dt, sdy = (t.syk[c] + sy1) * s.dt, sdz = t.szk[c] * s.dt;
                const T cz = (t.byk[c] - byi) * t.rdx2[c] - (t.bxk[c] - bxj) * t.rdy2;
                if constexpr (sizeof(T) == 8) {
                    // FP64, bound by the FP64 pipe: with D = lam2 + sigma dt, the update
                    // (lam2 - sigma dt)/D E + c4/D curl is written (2 lam2 E + c4 curl)/D - E -- three
                    // operations per component after 1/D instead of five.  (In FP32, where 1/D is an
                    // approximate reciprocal, the same form raised the trace error of a long whole run on
                    // 142 x 36 x 25 cells to 1.02 % of its peak, and saved 0.3 % of the step time.)
                    T rx, ry, rz;
                    recip3(s.lam2 + sdx, s.lam2 + sdy, s.lam2 + sdz, rx, ry, rz);
                    const T l2 = s.lam2 + s.lam2;
                    if constexpr (rX) {
                        const T bzj = p0[ABZ * BS - BXW] + t.ocj[c];
                        const T cx = (bz - bzj) * t.rdy2 - (t.byk[c] - bym) * rzs;
                        const T ex = fma(fma(s.c4, cx, l2 * exo), rx, -exo);
                        t.exn[c] = t.vEx[c] ? ex : exo;
                    }
                    if constexpr (rY) {
                        const T bzi = p0[ABZ * BS - 1] + t.oci[c];
                        const T cy = (t.bxk[c] - bxm) * rzs - (bz - bzi) * t.rdx2[c];
                        const T ey = fma(fma(s.c4, cy, l2 * eyo), ry, -eyo);
                        t.eyn[c] = t.vEy[c] ? ey : eyo;
                    }
                    const T ez = fma(fma(s.c4, cz, l2 * ezo), rz, -ezo);
                    t.ezn[c] = t.vEz[c] ? ez : ezo;
                } else {
                    if constexpr (rX) {
                        const T bzj = p0[ABZ * BS - BXW] + t.ocj[c];
                        const T cx = (bz - bzj) * t.rdy2 - (t.byk[c] - bym) * rzs;
                        const T rx = rcp_fast(s.lam2 + sdx);
                        const T ex = ((s.lam2 - sdx) * rx) * exo + (s.c4 * rx) * cx;
                        t.exn[c] = t.vEx[c] ? ex : exo;
                    }
                    if constexpr (rY) {
                        const T bzi = p0[ABZ * BS - 1] + t.oci[c];
                        const T cy = (t.bxk[c] - bxm) * rzs - (bz - bzi) * t.rdx2[c];
                        const T ry = rcp_fast(s.lam2 + sdy);
                        const T ey = ((s.lam2 - sdy) * ry) * eyo + (s.c4 * ry) * cy;
                        t.eyn[c] = t.vEy[c] ? ey : eyo;
                    }
                    const T rz = rcp_fast(s.lam2 + sdz);
                    const T ez = ((s.lam2 - sdz) * rz) * ezo + (s.c4 * rz) * cz;
                    t.ezn[c] = t.vEz[c] ? ez : ezo;
                }
            } else {
                t.exn[c] = exo;
                t.eyn[c] = eyo;
                t.ezn[c] = ezo;
            }
            t.bxo1[c] = t.bxk[c];  // B_old(k) for the next plane's B update
            t.byo1[c] = t.byk[c];
            t.bxk[c] = bxm;
            t.byk[c] = bym;
            t.sxk[c] = sx1;
            t.syk[c] = sy1;
            t.szk[c] = sz1;
        }
        // AddTx_*: subtracted after the update of the cell, on the planes where a segment meets the tile
        if (upd && src_tile && s.wave != T(0) && k >= t.s_flag[1] && k <= t.s_flag[2]) {
#pragma unroll
            for (int c = 0; c < NC; c++) {
                if (!(t.vEx[c] || t.vEy[c])) continue;
                for (int q = 0; q < src.nseg; q++) {
                    const int cp = src.comp[q];
                    int d;
                    if (cp == 0) { if (t.j != src.j[q] || k != src.k[q]) continue; d = t.i[c] - src.i[q]; }
                    else if (cp == 1) { if (t.i[c] != src.i[q] || k != src.k[q]) continue; d = t.j - src.j[q]; }
                    else { if (t.i[c] != src.i[q] || t.j != src.j[q]) continue; d = k - src.k[q]; }
                    if (d < 0 || d >= src.count[q]) continue;
                    const T v = s.wave * src.coef[src.off[q] + d];
                    if (cp == 0) t.exn[c] -= v; else if (cp == 1) t.eyn[c] -= v; else t.ezn[c] -= v;
                }
            }
        }
#pragma unroll
        for (int c = 0; c < NC; c++) {
            if (rR && upd && lo && t.own[c] && TCSEM_IN(t.col[c] + (k + 1) * t.PS, t.total, t.err)) {
                const int o = t.col[c] + (k + 1) * t.PS;
                out.ex[o] = t.exn[c];
                out.ey[o] = t.eyn[c];
                out.ez[o] = t.ezn[c];
            }
            t.x_ez[QE * XP2 + t.xo[c]] = t.ezn[c];  // publish Ez_new(k)
        }
    }
    if (doB) {  // publish B_new(k+1): Bx where Bz reads it (rows, +x column), By likewise (rows, +y row)
#pragma unroll
        for (int c = 0; c < NC; c++) {
            if constexpr (rY) t.x_bxn[QB * XP2 + t.xo[c]] = t.bxn[c];
            if constexpr (rX) t.x_byn[QB * XP2 + t.xo[c]] = t.byn[c];
        }
    }
    // plane k-2 is read by the next plane
    if (k - 2 >= t.klow && !mbar_wait_bounded(t.bars + ((PH + 2) & 3), rp ^ (unsigned)((PH + 2) >> 2))) *t.s_flag = 1;
    __syncthreads();
    if (*t.s_flag) {  // a copy did not arrive: let the copies still in flight (planes k-2, k-3) land first
        if (t.tid == 0) {
            if (k - 2 >= t.klow) mbar_wait_bounded(t.bars + ((PH + 2) & 3), rp ^ (unsigned)((PH + 2) >> 2));
            if (k - 3 >= t.klow) mbar_wait_bounded(t.bars + ((PH + 3) & 3), rp ^ (unsigned)((PH + 3) >> 2));
        }
        return false;
    }
    // plane k is no longer read: its ring slot takes plane k-4
    if (t.tid == 0 && k - RING >= t.klow && k >= t.k0) {
        if (k - RING < 0) pdl_wait_prev();  // the air plane is the boundary's output (no-op without the launch attribute)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        uint64_t *b = t.bars + S0;
        mbar_expect_tx(b, t.plane_bytes);
#pragma unroll
        for (int a = 0; a < NARR; a++) tma_load_3d(t.ring + (S0 * NARR + a) * BS, t.maps + a, t.i0, t.j0, k - RING + 1, b);
    }
    // ---- Bz(k+1) = Bz(k+2) + dz (dBx/dx + dBy/dy), for the tile's own rows
    if (doB && rR) {
        const T dz = zt[3 * (zi + 1) + 2];
#pragma unroll
        for (int c = 0; c < NC; c++) {
            t.acc[c] += dz * ((t.x_bxn[QB * XP2 + t.xo[c] + 1] - t.bxn[c]) * t.rdx[c] +
                              (t.x_byn[QB * XP2 + t.xo[c] + XC] - t.byn[c]) * t.rdy);
            if (t.own[c] && TCSEM_IN(t.col[c] + (k + 2) * t.PS, t.total, t.err)) out.bz[t.col[c] + (k + 2) * t.PS] = t.acc[c];
        }
    }
    return true;
}

// the z-march of one warp through the chunk, in the copy of the plane code for its role
template <typename T, int ROLE>
__device__ __forceinline__ bool sweep_march(SweepThread<T> &t, const StepScalars<T> &s, const T *__restrict__ s_z,
                                            const FieldSet<T> &out, const SourceTable<T> &src, bool src_tile,
                                            const T *s_oc);

// the cells' Bz chunk offsets from one of the two offset boxes
template <typename T> __device__ __forceinline__ void set_offsets(SweepThread<T> &t, const T *box) {
#pragma unroll
    for (int q = 0; q < fs3::NC; q++) {
        t.oc0[q] = box[t.so[q]];
        t.oci[q] = box[t.so[q] - 1];
        t.ocj[q] = box[t.so[q] - fs3::BXW];
    }
}

template <typename T, int ROLE>
__device__ __forceinline__ bool sweep_march(SweepThread<T> &t, const StepScalars<T> &s, const T *__restrict__ s_z,
                                            const FieldSet<T> &out, const SourceTable<T> &src, bool src_tile,
                                            const T *s_oc) {
    using namespace fs3;
    bool ok = true;
    unsigned rp = 0;  // parity of the ring round
    const int ktop = t.ktop;
    for (int k = ktop; ok && k >= t.k0 - 1; k -= RING, rp ^= 1u) {
        ok = sweep_plane<T, 0, ROLE>(t, k, rp, s, s_z, out, src, src_tile);
        if (k == ktop) set_offsets(t, s_oc);
        if (!ok || k - 1 < t.k0 - 1) break;
        ok = sweep_plane<T, 1, ROLE>(t, k - 1, rp, s, s_z, out, src, src_tile);
        if (!ok || k - 2 < t.k0 - 1) break;
        ok = sweep_plane<T, 2, ROLE>(t, k - 2, rp, s, s_z, out, src, src_tile);
        if (!ok || k - 3 < t.k0 - 1) break;
        ok = sweep_plane<T, 3, ROLE>(t, k - 3, rp, s, s_z, out, src, src_tile);
    }
    return ok;
}

// one CTA of the sweep: tile (bx, by) of z-chunk c with the step scalars s.  FRESH: the chunk
// totals tin may have been written by another CTA of the same launch (persistent schedule).
template <typename T, bool FRESH = false>
__device__ __forceinline__ void sweep_cta(const SweepMaps &maps, const Geom &g, const FieldSet<T> &out,
                                          const T *__restrict__ tin, T *__restrict__ tout, const Axis<T> &ax,
                                          StepScalars<T> s, const SourceTable<T> &src, const ZChunks &zc, int bx,
                                          int by, int c, int *err) {
    using namespace fs3;
    constexpr int BS = boxs<T>();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SweepThread<T> t;
    t.ring = reinterpret_cast<T *>(smem_raw);
    t.x_ez = t.ring + RING * NARR * BS;  // [2][XR][XC]
    t.x_bxn = t.x_ez + 2 * XR * XC;
    t.x_byn = t.x_bxn + 2 * XR * XC;
    T *s_oc = t.x_byn + 2 * XR * XC;  // [BYH][BXW] chunk offsets of Bz for planes < k1
    T *s_oc1 = s_oc + BOX;            // ... for plane k1
    t.bars = reinterpret_cast<uint64_t *>(s_oc1 + BOX);  // 8-byte aligned: every region above has an even size
    static_assert(bars_offset<T>() % 8 == 0, "mbarriers need 8-byte alignment");
    t.s_flag = reinterpret_cast<int *>(t.bars + RING);
    T *s_z = reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(t.bars) + RING * 8 + 16);  // [N+3][3]
    t.maps = maps.m;

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    t.tid = tid;
    t.i0 = bx * TX;
    t.j0 = by * BY;
    const int L = g.L, M = g.M, N = g.N, XP = g.XP;
    t.N = N;
    t.PS = (int)g.PS;
    t.total = (int)g.total();
    t.err = err;
    t.k0 = zc.plane(c);
    t.k1 = zc.plane(c + 1);
    const int ty = w < 9 ? w : lane;
    t.role = w < 8 ? 0 : (w == 8 ? 1 : 2);
    t.j = t.j0 + ty;
    const bool rowok = w < 9 || lane <= BY;
    t.rdy2 = (rowok && t.j >= 1 && t.j < M) ? ax.rdy2[t.j] : T(0);
    t.rdy = (rowok && t.j < M) ? ax.rdy[t.j] : T(0);
    t.fy = t.rdy * s.dtb;
#pragma unroll
    for (int q = 0; q < NC; q++) {
        const int tx = w < 9 ? lane + 32 * q : TX;
        const bool act = w < 9 || (q == 0 && lane <= BY);
        const int i = t.i0 + tx;
        t.i[q] = i;
        t.own[q] = act && ty < BY && tx < TX && i < L && t.j < M;
        t.col[q] = (t.j + 1) * XP + (i + 4);
        t.so[q] = act ? (ty + 1) * BXW + (tx + 4) : BXW + 4;
        t.xo[q] = act ? ty * XC + tx : XR * XC - 1;  // inactive slots publish into a cell nobody reads
        t.vEx[q] = act && t.j >= 1 && t.j < M && i < L;
        t.vEy[q] = act && i >= 1 && i < L && t.j < M;
        t.vEz[q] = t.vEx[q] && i >= 1;
        t.rdx2[q] = t.vEy[q] ? ax.rdx2[i] : T(0);
        t.rdx[q] = (act && i < L) ? ax.rdx[i] : T(0);
        t.fx[q] = t.rdx[q] * s.dtb;
    }
    t.ktop = t.k1 < N ? t.k1 : N;  // first plane: the chunk's halo plane below, or the zero bottom
    t.klow = t.k0 - 1 >= -1 ? t.k0 - 1 : -1;
    t.plane_bytes = (unsigned)(NARR * BOX * sizeof(T));
    const int ktop = t.ktop, klow = t.klow;
    s.dt *= T(0.25);  // the sweep forms sigma sums of four cells: 0.25 * sum * dt
    for (int e = tid; e <= ktop + 1 - klow; e += NT) {
        const int k = klow + e;
        const bool in = k >= 0 && k < N;
        s_z[3 * e] = in ? ax.rdz[k] : T(0);
        s_z[3 * e + 1] = in ? ax.rdzs[k] : T(0);
        s_z[3 * e + 2] = in ? ax.dzk[k] : T(0);
    }

    bool src_tile = false;  // tile-uniform: does any source segment touch this tile, and on which planes?
    int sk0 = N, sk1 = -1;
    for (int q = 0; q < src.nseg; q++) {
        int a0 = src.i[q], a1 = src.i[q], b0 = src.j[q], b1 = src.j[q], c1 = src.k[q];
        if (src.comp[q] == 0) a1 += src.count[q] - 1;
        if (src.comp[q] == 1) b1 += src.count[q] - 1;
        if (src.comp[q] == 2) c1 += src.count[q] - 1;
        if (a1 >= t.i0 && a0 <= t.i0 + TX && b1 >= t.j0 && b0 <= t.j0 + BY) {
            src_tile = true;
            sk0 = min(sk0, src.k[q]);
            sk1 = max(sk1, c1);
        }
    }
    if (tid == 0) {
        for (int r = 0; r < RING; r++) mbar_init(t.bars + r, 1);
        mbar_init_fence();
        t.s_flag[0] = 0;
        t.s_flag[1] = sk0;  // read by the source epilogue, after the barrier below
        t.s_flag[2] = sk1;
    }
    __syncthreads();
    if (tid == 0)  // planes ktop .. ktop-3 into slots 0..3
        for (int p = ktop, q = 0; q < RING && p >= klow; p--, q++) {
            // the air plane (k = -1) is the boundary's output: a top chunk launched early (programmatic
            // dependent launch after the boundary's last stage) stages its other planes first
            if (p < 0) pdl_wait_prev();
            uint64_t *b = t.bars + q;
            mbar_expect_tx(b, t.plane_bytes);
            for (int a = 0; a < NARR; a++) tma_load_3d(t.ring + (q * NARR + a) * BS, t.maps + a, t.i0, t.j0, p + 1, b);
        }
    // chunk offsets of Bz over the box (zero without chunking)
    for (int e = tid; e < BOX; e += NT) {
        T o = T(0), o1 = T(0);
        if (zc.n > 1) {
            const int gy = t.j0 + e / BXW, gx = t.i0 + e % BXW;  // padded coordinates
            if (gy < g.YP && gx < XP) {
                const int pc = gy * XP + gx;
                T pv[kMaxChunks];  // all loads in flight together
#pragma unroll
                for (int q = 1; q < kMaxChunks; q++)
                    pv[q] = q > c && q < zc.n && TCSEM_IN(q * t.PS + pc, zc.n * t.PS, err) ? ld_in<FRESH>(tin + q * t.PS + pc) : T(0);
                const T first = c + 1 < zc.n ? ld_in<FRESH>(tin + (c + 1) * t.PS + pc) : T(0);
#pragma unroll
                for (int q = 1; q < kMaxChunks; q++)
                    if (q > c && q < zc.n) o += pv[q];
                o1 = c + 1 < zc.n ? o - first : T(0);
            }
        }
        s_oc[e] = o;
        s_oc1[e] = o1;
    }
    {  // every thread observes the completion of the first two planes
        bool ok = mbar_wait_bounded(t.bars + 0, 0u);
        ok = ok && mbar_wait_bounded(t.bars + 1, 0u);
        if (!ok) *t.s_flag = 1;
    }
    __syncthreads();
    if (*t.s_flag) {  // record it, let the first planes land, leave together
        if (tid == 0) {
            atomicExch(err, 1);
            for (int q = 0; q < RING && ktop - q >= klow; q++) mbar_wait_bounded(t.bars + q, 0u);
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < NC; q++) {
        const int so = t.so[q];
        const T *p0 = t.ring + so;  // carried values of plane ktop (slot 0)
        const T a = p0[ASG * BS], b = p0[ASG * BS - 1], cc = p0[ASG * BS - BXW], d = p0[ASG * BS - BXW - 1];
        t.sxk[q] = a + cc;
        t.syk[q] = a + b;
        t.szk[q] = a + cc + b + d;
        t.bxk[q] = p0[ABX * BS];
        t.byk[q] = p0[ABY * BS];
        t.ex1[q] = t.ey1[q] = t.exn[q] = t.eyn[q] = t.ezn[q] = T(0);
        t.bxo1[q] = t.byo1[q] = t.bxn[q] = t.byn[q] = t.acc[q] = T(0);
    }

    // Bz offsets of the first plane: ktop is the halo plane k1 of the chunk below (its offsets) or the
    // zero bottom; every later plane lies in this chunk
    set_offsets(t, ktop < N ? s_oc1 : s_oc);
    // FP64 (bound by the FP64 pipe): the halo warps run their reduced copies of the plane code
    // (5 % faster).  FP32 runs one copy in every warp: three copies of its issue-bound loop made the
    // sweep 40 % slower (measured; presumably the larger loop no longer fits the instruction cache).
    bool ok;
    if constexpr (sizeof(T) == 8)
        ok = t.role == 0 ? sweep_march<T, 0>(t, s, s_z, out, src, src_tile, s_oc)
             : t.role == 1 ? sweep_march<T, 1>(t, s, s_z, out, src, src_tile, s_oc)
                           : sweep_march<T, 2>(t, s, s_z, out, src, src_tile, s_oc);
    else
        ok = sweep_march<T, 0>(t, s, s_z, out, src, src_tile, s_oc);
    if (!ok) {  // a copy did not arrive (the copies in flight were drained in sweep_plane)
        if (tid == 0) atomicExch(err, 1);
        return;
    }
    if (zc.n > 1) {
#pragma unroll
        for (int q = 0; q < NC; q++)
            if (t.own[q] && TCSEM_IN(c * t.PS + t.col[q], zc.n * t.PS, err)) tout[c * t.PS + t.col[q]] = t.acc[q];
    }
}

}  // namespace tcsem
