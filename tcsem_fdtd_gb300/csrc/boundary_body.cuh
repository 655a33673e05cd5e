// The per-CTA bodies of the four boundary stages, shared by the single-survey
// kernels, the batched kernels and the persistent batch scheduler.
#pragma once
#include "async.cuh"
#include "check.cuh"
#include "kernels.cuh"
#include "boundary.cuh"
#include "fft.cuh"

namespace tcsem {

constexpr int kBndThreads = 256;

// Programmatic dependent launch.  Each kernel of the chain lets the next one start once
// its own transforms are done (the next one's blocks stage their tables while this one
// writes its results); the next one waits for this grid's completion and memory before
// it reads what this grid wrote.  Without the launch attribute the wait returns at once.
// Releasing the next kernel only after the transforms keeps its waiting blocks from holding
// SM resources that the sweep running beside the boundary needs.  The last stage releases
// the top z-chunk of the sweep at its start: by then the sweep's blocks are all resident.

// Natural-spline second derivatives mb[0..n) of the line y[0..n) (stride ys) from
// the precomputed elimination factors tab = g | w | inv | du (n values each): the
// forward elimination of the tridiagonal system and the back substitution.
// One warp solves a line: both sweeps are first-order linear recurrences,
// rp_i = s_i - w_i rp_{i-1} forward and m_i = inv_i mb_i - inv_i du_i m_{i+1} backward,
// so each lane composes the affine maps of a segment of at most ceil((n-2)/32)
// nodes, a shuffle scan composes the segments, and each lane replays its segment
// from its start value -- about 40 dependent steps instead of 2n.
template <typename T>
__device__ void spline_solve_warp(const T *tab, int n, const T *y, int ys, T *mb) {
    const T *g = tab, *w = tab + n, *inv = tab + 2 * n, *du = tab + 3 * n;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, per = (n - 2 + 31) / 32;
    const int i0 = 1 + lane * per, i1 = min(i0 + per, n - 1);  // this lane's unknowns [i0, i1)
    auto fwd = [&](int i, T &a, T &b) {
        a = -w[i];
        b = (y[(i + 1) * ys] - y[i * ys]) * g[i] - (y[i * ys] - y[(i - 1) * ys]) * g[i - 1];
    };
    T A = T(1), B = T(0), a, b;
    for (int i = i0; i < i1; i++) {
        fwd(i, a, b);
        B = a * B + b;
        A = a * A;
    }
    for (int off = 1; off < 32; off <<= 1) {  // maps of lanes <= this one, the earlier ones first
        const T Ap = __shfl_up_sync(full, A, off), Bp = __shfl_up_sync(full, B, off);
        if (lane >= off) {
            B = A * Bp + B;
            A = A * Ap;
        }
    }
    T x = __shfl_up_sync(full, B, 1);  // rp at i0 - 1 (rp_0 = 0)
    if (lane == 0) x = T(0);
    for (int i = i0; i < i1; i++) {
        fwd(i, a, b);
        x = a * x + b;
        mb[i] = x;
    }
    if (lane == 0) {
        mb[0] = T(0);
        mb[n - 1] = T(0);
    }
    __syncwarp();
    A = T(1);
    B = T(0);
    for (int i = i1 - 1; i >= i0; i--) {
        a = -inv[i] * du[i];
        b = inv[i] * mb[i];
        B = a * B + b;
        A = a * A;
    }
    for (int off = 1; off < 32; off <<= 1) {  // maps of lanes >= this one, the later ones first
        const T An = __shfl_down_sync(full, A, off), Bn = __shfl_down_sync(full, B, off);
        if (lane + off < 32) {
            B = A * Bn + B;
            A = A * An;
        }
    }
    x = __shfl_down_sync(full, B, 1);  // m at i1 (m_{n-1} = 0)
    if (lane == 31) x = T(0);
    for (int i = i1 - 1; i >= i0; i--) {
        x = inv[i] * mb[i] - inv[i] * du[i] * x;
        mb[i] = x;
    }
}

// one remapped point from its three-node window (y and mb start at the window)
template <typename T>
__device__ __forceinline__ T spline_out(const T *c, int npts, const T *y, int ys, const T *mb) {
    return c[0] * y[0] + c[npts] * y[ys] + c[2 * npts] * y[2 * ys] + c[3 * npts] * mb[0] + c[4 * npts] * mb[1] +
           c[5 * npts] * mb[2];
}

// Shared-memory layouts (byte offsets from a 128-byte aligned base), used by
// the kernels and by the host for the launch size.  Every region starts on a
// 16-byte boundary so the bulk copies can land in it.
struct RowsFwdLayout { size_t bar, tw, tab, tabi, row, a, b, mb, total; };
struct ColsLayout { size_t bar, tw, tab, tabi, col, gx, gy, a, b, mb, total; };
struct RowsInvLayout { size_t bar, tw, vx, vy, a, b, total; };

template <typename T> __host__ __device__ inline RowsFwdLayout rows_fwd_layout(const BoundaryDev<T> &bd, int L) {
    RowsFwdLayout l{};
    size_t o = 0;
    l.bar = o; o += 16;
    l.tw = o; o += rnd16(bd.L1 * sizeof(C2<T>));
    l.tab = o; o += rnd16(bd.rx.nT * sizeof(T));
    l.tabi = o; o += rnd16(bd.rx.nI * sizeof(int));
    l.row = o; o += rnd16(2 * (size_t)L * sizeof(T));
    l.a = o; o += rnd16(bd.L1 * sizeof(C2<T>));
    l.b = o; o += rnd16(bd.L1 * sizeof(C2<T>));
    l.mb = o; o += rnd16(4 * (size_t)bd.rx.nmax * sizeof(T));
    l.total = o;
    return l;
}
template <typename T> __host__ __device__ inline ColsLayout cols_layout(const BoundaryDev<T> &bd) {
    ColsLayout l{};
    size_t o = 0;
    l.bar = o; o += 16;
    l.tw = o; o += rnd16(bd.M1 * sizeof(C2<T>));
    l.tab = o; o += rnd16(bd.ry.nT * sizeof(T));
    l.tabi = o; o += rnd16(bd.ry.nI * sizeof(int));
    l.col = o; o += rnd16(bd.M * sizeof(C2<T>));
    l.gx = o; o += rnd16(bd.M1 * sizeof(T));
    l.gy = o; o += rnd16(bd.M1 * sizeof(T));
    l.a = o; o += rnd16(2 * (size_t)bd.M1 * sizeof(C2<T>));
    l.b = o; o += rnd16(2 * (size_t)bd.M1 * sizeof(C2<T>));
    l.mb = o; o += rnd16(4 * (size_t)bd.ry.nmax * sizeof(T));
    l.total = o;
    return l;
}
template <typename T> __host__ __device__ inline RowsInvLayout rows_inv_layout(const BoundaryDev<T> &bd) {
    RowsInvLayout l{};
    size_t o = 0;
    l.bar = o; o += 16;
    l.tw = o; o += rnd16(bd.L1 * sizeof(C2<T>));
    l.vx = o; o += rnd16(bd.H * sizeof(C2<T>));
    l.vy = o; o += rnd16(bd.H * sizeof(C2<T>));
    l.a = o; o += rnd16(bd.L1 * sizeof(C2<T>));
    l.b = o; o += rnd16(bd.L1 * sizeof(C2<T>));
    l.total = o;
    return l;
}

// every thread observes the bulk copies of phase 0 on bar; false (after
// recording the error and letting the copies land) if any thread gave up
__device__ __forceinline__ bool staged(uint64_t *bar, int *err) {
    const bool ok = mbar_wait_bounded(bar, 0u);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            mbar_wait_bounded(bar, 0u);
        }
        return false;
    }
    return true;
}

// Padded plane: the n - nu points outside the grid [d, d + nu) of a line of n points are the
// first grid value times w[i] left of the grid (i < d) and the last one times w[i] right of it.
template <typename T>
__device__ __forceinline__ void pad_line(C2<T> *a, int n, int nu, int d, const T *__restrict__ w) {
    const C2<T> lo = a[d], hi = a[d + nu - 1];
    for (int i = threadIdx.x; i < n - nu; i += blockDim.x) {
        const int p = i < d ? i : i + nu;  // the pad points in order, skipping the grid
        const T f = w[p];
        const C2<T> e = p < d ? lo : hi;
        a[p] = {f * e.x, f * e.y};
    }
}

// ---- stage 1: x-remap of the M old rows + forward FFT along x.  Rows j0 and
// j0+1 travel as the real and imaginary parts of one complex transform and are
// separated in the spectrum: X1 = (Z[k] + conj Z[-k]) / 2, X2 = (Z[k] - conj Z[-k]) / 2i.
// Output FT is stored x-frequency major, FT[kx][j].
template <typename T, bool FRESH = false>  // FRESH: bz and tot may come from this launch (persistent schedule)
__device__ __forceinline__ void rows_fwd_cta(const BoundaryDev<T> &bd, const T *__restrict__ bz,
                                             const T *__restrict__ tot, int nch, const Geom &g, int blk) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int L1 = bd.L1, L = g.L;
    const AxisRemap<T> &R = bd.rx;
    const RowsFwdLayout ly = rows_fwd_layout(bd, L);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + ly.bar);
    C2<T> *tw = reinterpret_cast<C2<T> *>(smem_raw + ly.tw);
    T *tab = reinterpret_cast<T *>(smem_raw + ly.tab);
    int *tabi = reinterpret_cast<int *>(smem_raw + ly.tabi);
    T *row = reinterpret_cast<T *>(smem_raw + ly.row);  // [2][L]
    C2<T> *a = reinterpret_cast<C2<T> *>(smem_raw + ly.a);
    C2<T> *b = reinterpret_cast<C2<T> *>(smem_raw + ly.b);
    T *mbuf = reinterpret_cast<T *>(smem_raw + ly.mb);  // [strip][row][nmax]
    if (threadIdx.x == 0) {  // twiddles and remap tables in one bulk phase
        const unsigned btw = (unsigned)rnd16(L1 * sizeof(C2<T>)), bt = (unsigned)rnd16(R.nT * sizeof(T)),
                       bi = (unsigned)rnd16(R.nI * sizeof(int));
        mbar_init(bar, 1);
        mbar_init_fence();
        mbar_expect_tx(bar, btw + bt + bi);
        bulk_load(tw, bd.twx, btw, bar);
        bulk_load(tab, R.tabT, bt, bar);
        bulk_load(tabi, R.tabI, bi, bar);
    }
    const int j0 = 2 * blk, nr = min(2, g.M - j0);
    const long long plane = (long long)(g.M + 2) * g.XP;
    for (int e = threadIdx.x; e < 2 * L; e += blockDim.x) {
        const int r = e >= L ? 1 : 0, i = e - r * L;
        T v = T(0);
        if (r < nr && TCSEM_IN(plane + (long long)(j0 + r + 1) * g.XP + 4 + i, g.total(), bd.err) &&
            TCSEM_IN((long long)(nch - 1) * plane + (j0 + r + 1) * g.XP + 4 + i, (long long)nch * plane, bd.err)) {
            // plane 0 of Bz is chunk-partial: add the totals of the chunks below
            const long long o = (long long)(j0 + r + 1) * g.XP + 4 + i;
            T p[kMaxChunks];
#pragma unroll
            for (int c = 1; c < kMaxChunks; c++) p[c] = c < nch ? ld_in<FRESH>(tot + c * plane + o) : T(0);
            v = ld_in<FRESH>(bz + plane + o);
#pragma unroll
            for (int c = 1; c < kMaxChunks; c++)
                if (c < nch) v += p[c];
        }
        row[e] = v;
    }
    __syncthreads();  // the barrier is initialised, the rows are in place
    if (!staged(bar, bd.err)) return;
    // left strip (Intep_BzIR2R_0x), core copy (Intep_BzIR2R_cpy_center), right strip (Intep_BzIR2R_1x)
    const T *r0 = row, *r1 = row + L;
    if (threadIdx.x < 128) {  // warps 0..3: strip (warp / 2) of row (warp & 1)
        const int wq = threadIdx.x >> 5;
        const StripPlan S = wq < 2 ? R.s[0] : R.s[1];
        spline_solve_warp(tab + S.f, S.n, row + (wq & 1) * L + S.src, 1, mbuf + wq * R.nmax);
    }
    const int anl = bd.AnLx + bd.DL, AL = bd.AL;
    for (int c = threadIdx.x; c < bd.Nx; c += blockDim.x) a[anl + c] = {r0[AL + c], r1[AL + c]};
    __syncthreads();
    const int np0 = R.s[0].npts, np = np0 + R.s[1].npts;
    for (int e = threadIdx.x; e < np; e += blockDim.x) {
        const int s = e >= np0 ? 1 : 0, q = e - s * np0;
        const StripPlan S = s ? R.s[1] : R.s[0];
        const int k0 = tabi[S.k + q];
        const T *c = tab + S.c + q, *m0 = mbuf + 2 * s * R.nmax + k0;
        a[bd.DL + S.dst + q] = {spline_out(c, S.npts, r0 + S.src + k0, 1, m0),
                                spline_out(c, S.npts, r1 + S.src + k0, 1, m0 + R.nmax)};
    }
    __syncthreads();
    if (L1 != bd.Lu) {  // padded plane: taper the row from its edge values to zero
        pad_line(a, L1, bd.Lu, bd.DL, bd.padx);
        __syncthreads();
    }
    const C2<T> *Z = fft::run<false, 1>(a, b, bd.px, tw);
    pdl_allow_next();
    for (int kx = threadIdx.x; kx < bd.H; kx += blockDim.x) {
        const C2<T> zk = Z[kx], zm = Z[kx == 0 ? 0 : L1 - kx];
        if (!TCSEM_IN((long long)kx * bd.Mp + j0 + nr - 1, (long long)bd.H * bd.Mp, bd.err)) continue;
        C2<T> *dst = bd.FT + (size_t)kx * bd.Mp + j0;
        dst[0] = {T(0.5) * (zk.x + zm.x), T(0.5) * (zk.y - zm.y)};
        if (nr == 2) dst[1] = {T(0.5) * (zk.y + zm.y), T(0.5) * (zm.x - zk.x)};
    }
}

// ---- stage 2: y-remap in the x-frequency domain, FFT_y, the two filters and
// both inverse FFT_y batched in one pass
template <typename T>
__device__ __forceinline__ void cols_cta(const BoundaryDev<T> &bd, int blk) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int M1 = bd.M1, M = bd.M, kx = blk;
    const AxisRemap<T> &R = bd.ry;
    const ColsLayout ly = cols_layout(bd);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + ly.bar);
    C2<T> *tw = reinterpret_cast<C2<T> *>(smem_raw + ly.tw);
    T *tab = reinterpret_cast<T *>(smem_raw + ly.tab);
    int *tabi = reinterpret_cast<int *>(smem_raw + ly.tabi);
    C2<T> *col = reinterpret_cast<C2<T> *>(smem_raw + ly.col);
    T *gx = reinterpret_cast<T *>(smem_raw + ly.gx);
    T *gy = reinterpret_cast<T *>(smem_raw + ly.gy);
    C2<T> *a = reinterpret_cast<C2<T> *>(smem_raw + ly.a);  // 2*M1
    C2<T> *b = reinterpret_cast<C2<T> *>(smem_raw + ly.b);  // 2*M1
    T *mbuf = reinterpret_cast<T *>(smem_raw + ly.mb);      // [strip][re/im][nmax]
    if (threadIdx.x == 0) {
        const unsigned btw = (unsigned)rnd16(M1 * sizeof(C2<T>)), bt = (unsigned)rnd16(R.nT * sizeof(T)),
                       bi = (unsigned)rnd16(R.nI * sizeof(int)), bc = (unsigned)rnd16(M * sizeof(C2<T>)),
                       bg = (unsigned)rnd16(M1 * sizeof(T));
        // a refused copy (bounds-checked builds) is left out of the expected bytes
        const bool okc = TCSEM_IN((long long)kx * bd.Mp + bc / sizeof(C2<T>) - 1, (long long)bd.H * bd.Mp, bd.err);
        mbar_init(bar, 1);
        mbar_init_fence();
        mbar_expect_tx(bar, btw + bt + bi + (okc ? bc : 0u) + 2 * bg);
        bulk_load(tw, bd.twy, btw, bar);
        bulk_load(tab, R.tabT, bt, bar);
        bulk_load(tabi, R.tabI, bi, bar);
        bulk_load(gx, bd.Gx + (size_t)kx * bd.M1p, bg, bar);
        bulk_load(gy, bd.Gy + (size_t)kx * bd.M1p, bg, bar);
        pdl_wait_prev();  // FT is the previous kernel's output
        if (okc) bulk_load(col, bd.FT + (size_t)kx * bd.Mp, bc, bar);
    }
    __syncthreads();
    if (!staged(bar, bd.err)) return;
    // front strip (Intep_BzIR2R_0y), core copy, back strip (Intep_BzIR2R_1y); the real and
    // imaginary parts of the column are independent lines
    if (threadIdx.x < 128) {  // warps 0..3: strip (warp / 2), real / imaginary part (warp & 1)
        const int wq = threadIdx.x >> 5;
        const StripPlan S = wq < 2 ? R.s[0] : R.s[1];
        spline_solve_warp(tab + S.f, S.n, reinterpret_cast<const T *>(col + S.src) + (wq & 1), 2,
                          mbuf + wq * R.nmax);
    }
    const int any = bd.Any + bd.DM, Ay = bd.Ay;
    for (int r = threadIdx.x; r < bd.Ny; r += blockDim.x) a[any + r] = col[Ay + r];
    __syncthreads();
    const int np0 = R.s[0].npts, np = np0 + R.s[1].npts;
    for (int e = threadIdx.x; e < np; e += blockDim.x) {
        const int s = e >= np0 ? 1 : 0, q = e - s * np0;
        const StripPlan S = s ? R.s[1] : R.s[0];
        const int k0 = tabi[S.k + q];
        const T *c = tab + S.c + q, *m0 = mbuf + 2 * s * R.nmax + k0;
        const T *yb = reinterpret_cast<const T *>(col + S.src + k0);
        a[bd.DM + S.dst + q] = {spline_out(c, S.npts, yb, 2, m0), spline_out(c, S.npts, yb + 1, 2, m0 + R.nmax)};
    }
    __syncthreads();
    if (M1 != bd.Mu) {  // padded plane: taper the column (x-frequency domain; the taper is linear)
        pad_line(a, M1, bd.Mu, bd.DM, bd.pady);
        __syncthreads();
    }
    C2<T> *F = fft::run<false, 1>(a, b, bd.py, tw);
    // FBx = i*gx*F, FBy = i*gy*F (FBz_to_FBxFBy, UpContinuation_gpu.cu:113-164) side by side
    C2<T> *in = F == a ? b : a;
    for (int r = threadIdx.x; r < M1; r += blockDim.x) {
        const C2<T> f = F[r];
        const T ux = gx[r], uy = gy[r];
        in[r] = {-f.y * ux, f.x * ux};
        in[M1 + r] = {-f.y * uy, f.x * uy};
    }
    __syncthreads();
    const C2<T> *out = fft::run<true, 2>(in, F, bd.py, tw);
    pdl_allow_next();
    for (int s = threadIdx.x; s < bd.S; s += blockDim.x) {
        const int rr = bd.rows[s];
        if (!TCSEM_IN((long long)s * bd.Hp + kx, (long long)bd.S * bd.Hp, bd.err)) continue;
        bd.VX[(size_t)s * bd.Hp + kx] = out[rr];
        bd.VY[(size_t)s * bd.Hp + kx] = out[M1 + rr];
    }
}

// ---- stage 3: packed inverse FFT along x of the sampled rows
template <typename T>
__device__ __forceinline__ void rows_inv_cta(const BoundaryDev<T> &bd, int blk) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int L1 = bd.L1, H = bd.H, s = blk;
    const RowsInvLayout ly = rows_inv_layout(bd);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + ly.bar);
    C2<T> *tw = reinterpret_cast<C2<T> *>(smem_raw + ly.tw);
    C2<T> *vx = reinterpret_cast<C2<T> *>(smem_raw + ly.vx);
    C2<T> *vy = reinterpret_cast<C2<T> *>(smem_raw + ly.vy);
    C2<T> *a = reinterpret_cast<C2<T> *>(smem_raw + ly.a);
    C2<T> *b = reinterpret_cast<C2<T> *>(smem_raw + ly.b);
    if (threadIdx.x == 0) {
        const unsigned btw = (unsigned)rnd16(L1 * sizeof(C2<T>)), bv = (unsigned)rnd16(H * sizeof(C2<T>));
        // a refused pair of copies (bounds-checked builds) is left out of the expected bytes
        const bool okv = TCSEM_IN((long long)s * bd.Hp + bv / sizeof(C2<T>) - 1, (long long)bd.S * bd.Hp, bd.err);
        mbar_init(bar, 1);
        mbar_init_fence();
        mbar_expect_tx(bar, btw + (okv ? 2 * bv : 0u));
        bulk_load(tw, bd.twx, btw, bar);
        pdl_wait_prev();  // VX and VY are the previous kernel's output
        if (okv) {
            bulk_load(vx, bd.VX + (size_t)s * bd.Hp, bv, bar);
            bulk_load(vy, bd.VY + (size_t)s * bd.Hp, bv, bar);
        }
    }
    __syncthreads();
    if (!staged(bar, bd.err)) return;
    for (int kx = threadIdx.x; kx < H; kx += blockDim.x) {
        const C2<T> X = vx[kx], Y = vy[kx];
        if (kx == 0 || 2 * kx == L1) {  // self-conjugate bins carry their real parts
            a[kx] = {X.x, Y.x};
        } else {
            a[kx] = {X.x - Y.y, X.y + Y.x};        // X + iY
            a[L1 - kx] = {X.x + Y.y, -X.y + Y.x};  // conj(X) + i conj(Y)
        }
    }
    __syncthreads();
    const C2<T> *res = fft::run<true, 1>(a, b, bd.px, tw);
    pdl_allow_next();
    C2<T> *dst = bd.Z + (size_t)s * bd.Lu;
    for (int x = threadIdx.x; x < bd.Lu; x += blockDim.x)
        if (TCSEM_IN((long long)s * bd.Lu + x, (long long)bd.S * bd.Lu, bd.err)) dst[x] = res[bd.DL + x];
}

// ---- stage 4: bilinear remap (Blinear_BxR2IR / Blinear_ByR2IR, UpContinuation_gpu.cu:42-110)
template <typename T>
__device__ __forceinline__ void bilinear_cta(const BoundaryDev<T> &bd, T *bx, T *by, const Geom &g, int blk, int nblk) {
    const int L = g.L, M = g.M;
    const int nbx = (L + 1) * M, nby = L * (M + 1);
    const T norm = bd.inv_norm;
    pdl_allow_next();  // the top z-chunk of the sweep may stage its planes; it waits for this grid before the air plane
    pdl_wait_prev();   // Z is the previous kernel's output
    for (int e = blk * blockDim.x + threadIdx.x; e < nbx + nby; e += nblk * blockDim.x) {
        if (e < nbx) {
            const int j = e / (L + 1), i = e % (L + 1);
            const int II = bd.bxc_II[i];
            if (!TCSEM_IN((long long)bd.bxr_a[j] * bd.Lu + II - 1, (long long)bd.S * bd.Lu, bd.err) ||
                !TCSEM_IN((long long)bd.bxr_b[j] * bd.Lu + II, (long long)bd.S * bd.Lu, bd.err) ||
                !TCSEM_IN(g.at(i, j, -1), g.total(), bd.err))
                continue;
            const T lx = bd.bxc_l[i];
            const C2<T> *ra = bd.Z + (size_t)bd.bxr_a[j] * bd.Lu, *rb = bd.Z + (size_t)bd.bxr_b[j] * bd.Lu;
            T a0 = (T(1) - lx) * ra[II - 1].x + lx * ra[II].x;
            T a1 = (T(1) - lx) * rb[II - 1].x + lx * rb[II].x;
            T ly = bd.bxr_l[j];
            bx[g.at(i, j, -1)] = ((T(1) - ly) * a0 + ly * a1) * norm;
        } else {
            const int e2 = e - nbx, j = e2 / L, i = e2 % L;
            const int II = bd.byc_II[i];
            if (!TCSEM_IN((long long)bd.byr_a[j] * bd.Lu + II - 1, (long long)bd.S * bd.Lu, bd.err) ||
                !TCSEM_IN((long long)bd.byr_b[j] * bd.Lu + II, (long long)bd.S * bd.Lu, bd.err) ||
                !TCSEM_IN(g.at(i, j, -1), g.total(), bd.err))
                continue;
            const T lx = bd.byc_l[i];
            const C2<T> *ra = bd.Z + (size_t)bd.byr_a[j] * bd.Lu, *rb = bd.Z + (size_t)bd.byr_b[j] * bd.Lu;
            T a0 = (T(1) - lx) * ra[II - 1].y + lx * ra[II].y;
            T a1 = (T(1) - lx) * rb[II - 1].y + lx * rb[II].y;
            T ly = bd.byr_l[j];
            by[g.at(i, j, -1)] = ((T(1) - ly) * a0 + ly * a1) * norm;
        }
    }
}

}  // namespace tcsem
