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
//      along x -- M rows, not M1;
//   2. per x-frequency column: applies Py in the x-frequency domain, FFTs
//      along y, multiplies by the two continuation filters, inverse-FFTs
//      along y and keeps only the rows the final bilinear remap samples;
//   3. inverse-FFTs those rows along x with Bx and By packed as the real and
//      imaginary parts of one complex transform;
//   4. bilinearly remaps into plane k = -1 of the Bx/By buffers.
// All transforms are in-shared-memory mixed-radix Stockham FFTs of arbitrary
// length written here (no cuFFT).
#include "kernels.cuh"
#include "boundary.cuh"

namespace tcsem {

template <typename T> __device__ __forceinline__ C2<T> cmul(C2<T> a, C2<T> b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T> __device__ __forceinline__ C2<T> cadd(C2<T> a, C2<T> b) { return {a.x + b.x, a.y + b.y}; }

// twiddle W_n^e = exp(-+2 pi i e / n) from the forward table
template <typename T> __device__ __forceinline__ C2<T> twid(const C2<T> *tw, int e, bool inv) {
    C2<T> w = tw[e];
    if (inv) w.y = -w.y;
    return w;
}

// Stockham autosort FFT of length P.n held in shared memory.  Radices up to 8
// run one butterfly per thread; larger prime radices compute each output
// directly.  Returns the buffer that holds the result.
template <typename T>
__device__ C2<T> *fft_smem(C2<T> *a, C2<T> *b, const FFTPlan &P, const C2<T> *__restrict__ tw, bool inv) {
    const int n = P.n, tid = threadIdx.x, nth = blockDim.x;
    int Ns = 1;
    for (int s = 0; s < P.nst; s++) {
        const int p = P.radix[s], m = n / p, step = n / (Ns * p);
        if (p <= 8) {
            for (int r = tid; r < m; r += nth) {
                const int lo = r % Ns, base = (r / Ns) * Ns * p + lo, st = step * lo;
                C2<T> v[8];
#pragma unroll
                for (int q = 0; q < 8; q++)
                    if (q < p) v[q] = a[r + q * m];
#pragma unroll
                for (int q = 1; q < 8; q++)
                    if (q < p) v[q] = cmul(v[q], twid(tw, (q * st) % n, inv));
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    if (u >= p) break;
                    C2<T> acc = v[0];
#pragma unroll
                    for (int q = 1; q < 8; q++)
                        if (q < p) acc = cadd(acc, cmul(v[q], twid(tw, ((q * u) % p) * m, inv)));
                    b[base + u * Ns] = acc;
                }
            }
        } else {
            for (int o = tid; o < n; o += nth) {
                const int hi = o / (Ns * p), rem = o % (Ns * p), u = rem / Ns, lo = rem % Ns, r = hi * Ns + lo;
                const int st = ((lo + u * Ns) * step) % n;
                C2<T> acc = {T(0), T(0)};
                int e = 0;
                for (int q = 0; q < p; q++) {
                    acc = cadd(acc, cmul(a[r + q * m], twid(tw, e, inv)));
                    e += st;
                    if (e >= n) e -= n;
                }
                b[o] = acc;
            }
        }
        __syncthreads();
        C2<T> *t = a; a = b; b = t;
        Ns *= p;
    }
    return a;
}

// ---- stage 1: x-remap of the M old rows + forward FFT along x
template <typename T>
__global__ void k_rows_fwd(BoundaryDev<T> bd, const T *__restrict__ bz, const T *__restrict__ tot, int nch, Geom g,
                           StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    extern __shared__ unsigned char smem_raw[];
    C2<T> *a = reinterpret_cast<C2<T> *>(smem_raw);
    C2<T> *b = a + bd.L1;
    T *row = reinterpret_cast<T *>(b + bd.L1);
    const int j = blockIdx.x, L = g.L;
    const T *src = bz + g.at(0, j, 0);  // plane 0 of Bz (chunk-partial: add the totals of the chunks below)
    const long long plane = (long long)(g.M + 2) * g.XP, col0 = (long long)(j + 1) * g.XP + 4;
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        T v = src[i];
        for (int c = 1; c < nch; c++) v += tot[c * plane + col0 + i];
        row[i] = v;
    }
    __syncthreads();
    const int anl = bd.AnLx, nx = bd.Nx, AL = bd.AL;
    for (int c = threadIdx.x; c < bd.L1; c += blockDim.x) {
        T v;
        if (c < anl) {  // left strip (Intep_BzIR2R_0x)
            const T *w = bd.Wl + (size_t)c * bd.n1;
            v = T(0);
            for (int m = 0; m < bd.n1; m++) v += w[m] * row[m];
        } else if (c < anl + nx) {  // core (Intep_BzIR2R_cpy_center)
            v = row[c - anl + AL];
        } else {  // right strip (Intep_BzIR2R_1x)
            const T *w = bd.Wr + (size_t)(c - anl - nx) * bd.n2;
            v = T(0);
            for (int m = 0; m < bd.n2; m++) v += w[m] * row[bd.ox + m];
        }
        a[c] = {v, T(0)};
    }
    __syncthreads();
    C2<T> *res = fft_smem(a, b, bd.px, bd.twx, false);
    C2<T> *dst = bd.FT + (size_t)j * bd.H;
    for (int kx = threadIdx.x; kx < bd.H; kx += blockDim.x) dst[kx] = res[kx];
}

// ---- stage 2: y-remap in the x-frequency domain, FFT_y, filters, IFFT_y
template <typename T>
__global__ void k_cols(BoundaryDev<T> bd, StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    extern __shared__ unsigned char smem_raw[];
    const int M1 = bd.M1, M = bd.M;
    C2<T> *a = reinterpret_cast<C2<T> *>(smem_raw);
    C2<T> *b = a + M1;
    C2<T> *F = b + M1;
    C2<T> *col = F + M1;
    const int kx = blockIdx.x;
    for (int m = threadIdx.x; m < M; m += blockDim.x) col[m] = bd.FT[(size_t)m * bd.H + kx];
    __syncthreads();
    const int any = bd.Any, ny = bd.Ny, Ay = bd.Ay;
    for (int r = threadIdx.x; r < M1; r += blockDim.x) {
        C2<T> v = {T(0), T(0)};
        if (r < any) {  // front strip (Intep_BzIR2R_0y)
            const T *w = bd.Wf + (size_t)r * bd.n3;
            for (int m = 0; m < bd.n3; m++) { v.x += w[m] * col[m].x; v.y += w[m] * col[m].y; }
        } else if (r < any + ny) {
            v = col[r - any + Ay];
        } else {  // back strip (Intep_BzIR2R_1y)
            const T *w = bd.Wb + (size_t)(r - any - ny) * bd.n3;
            for (int m = 0; m < bd.n3; m++) { v.x += w[m] * col[bd.oy + m].x; v.y += w[m] * col[bd.oy + m].y; }
        }
        a[r] = v;
    }
    __syncthreads();
    C2<T> *res = fft_smem(a, b, bd.py, bd.twy, false);
    for (int r = threadIdx.x; r < M1; r += blockDim.x) F[r] = res[r];
    __syncthreads();
    // FBx = i*gx*F, FBy = i*gy*F (FBz_to_FBxFBy, UpContinuation_gpu.cu:113-164), then IFFT_y
    for (int pass = 0; pass < 2; pass++) {
        const T *gf = (pass == 0 ? bd.Gx : bd.Gy) + (size_t)kx * M1;
        for (int r = threadIdx.x; r < M1; r += blockDim.x) {
            C2<T> f = F[r];
            T gv = gf[r];
            a[r] = {-f.y * gv, f.x * gv};
        }
        __syncthreads();
        C2<T> *out = fft_smem(a, b, bd.py, bd.twy, true);
        C2<T> *dst = pass == 0 ? bd.VX : bd.VY;
        for (int s = threadIdx.x; s < bd.S; s += blockDim.x) dst[(size_t)s * bd.H + kx] = out[bd.rows[s]];
        __syncthreads();
    }
}

// ---- stage 3: packed inverse FFT along x of the sampled rows
template <typename T>
__global__ void k_rows_inv(BoundaryDev<T> bd, StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    extern __shared__ unsigned char smem_raw[];
    const int L1 = bd.L1, H = bd.H;
    C2<T> *a = reinterpret_cast<C2<T> *>(smem_raw);
    C2<T> *b = a + L1;
    const int s = blockIdx.x;
    const C2<T> *vx = bd.VX + (size_t)s * H, *vy = bd.VY + (size_t)s * H;
    for (int kx = threadIdx.x; kx < H; kx += blockDim.x) {
        C2<T> X = vx[kx], Y = vy[kx];
        if (kx == 0 || 2 * kx == L1) {  // self-conjugate bins carry their real parts
            a[kx] = {X.x, Y.x};
        } else {
            a[kx] = {X.x - Y.y, X.y + Y.x};           // X + iY
            a[L1 - kx] = {X.x + Y.y, -X.y + Y.x};     // conj(X) + i conj(Y)
        }
    }
    __syncthreads();
    C2<T> *res = fft_smem(a, b, bd.px, bd.twx, true);
    C2<T> *dst = bd.Z + (size_t)s * L1;
    for (int x = threadIdx.x; x < L1; x += blockDim.x) dst[x] = res[x];
}

// ---- stage 4: bilinear remap (Blinear_BxR2IR / Blinear_ByR2IR, UpContinuation_gpu.cu:42-110)
template <typename T>
__global__ void k_bilinear(BoundaryDev<T> bd, T *bx, T *by, Geom g, StepGate gate) {
    if (gate.base && gate.step() >= gate.nsteps) return;
    const int L = g.L, M = g.M;
    const int nbx = (L + 1) * M, nby = L * (M + 1);
    const T norm = bd.inv_norm;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nbx + nby; e += gridDim.x * blockDim.x) {
        if (e < nbx) {
            const int j = e / (L + 1), i = e % (L + 1);
            const int II = bd.bxc_II[i];
            const T lx = bd.bxc_l[i];
            const C2<T> *ra = bd.Z + (size_t)bd.bxr_a[j] * bd.L1, *rb = bd.Z + (size_t)bd.bxr_b[j] * bd.L1;
            T a0 = (T(1) - lx) * ra[II - 1].x + lx * ra[II].x;
            T a1 = (T(1) - lx) * rb[II - 1].x + lx * rb[II].x;
            T ly = bd.bxr_l[j];
            bx[g.at(i, j, -1)] = ((T(1) - ly) * a0 + ly * a1) * norm;
        } else {
            const int e2 = e - nbx, j = e2 / L, i = e2 % L;
            const int II = bd.byc_II[i];
            const T lx = bd.byc_l[i];
            const C2<T> *ra = bd.Z + (size_t)bd.byr_a[j] * bd.L1, *rb = bd.Z + (size_t)bd.byr_b[j] * bd.L1;
            T a0 = (T(1) - lx) * ra[II - 1].y + lx * ra[II].y;
            T a1 = (T(1) - lx) * rb[II - 1].y + lx * rb[II].y;
            T ly = bd.byr_l[j];
            by[g.at(i, j, -1)] = ((T(1) - ly) * a0 + ly * a1) * norm;
        }
    }
}

template <typename T> static size_t smem_rows(const BoundaryDev<T> &bd, int L) {
    return 2 * (size_t)bd.L1 * sizeof(C2<T>) + (size_t)L * sizeof(T);
}
template <typename T> static size_t smem_cols(const BoundaryDev<T> &bd) {
    return (3 * (size_t)bd.M1 + bd.M) * sizeof(C2<T>);
}
template <typename T> static size_t smem_inv(const BoundaryDev<T> &bd) { return 2 * (size_t)bd.L1 * sizeof(C2<T>); }

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

template <typename T>
void launch_boundary(const BoundaryDev<T> &bd, const Geom &g, const T *bz, const T *tot, int nch, T *bx, T *by,
                     StepGate gate, cudaStream_t st) {
    k_rows_fwd<T><<<g.M, 256, smem_rows(bd, g.L), st>>>(bd, bz, tot, nch, g, gate);
    k_cols<T><<<bd.H, 256, smem_cols(bd), st>>>(bd, gate);
    k_rows_inv<T><<<bd.S, 256, smem_inv(bd), st>>>(bd, gate);
    int n = (g.L + 1) * g.M + g.L * (g.M + 1);
    k_bilinear<T><<<(n + 255) / 256, 256, 0, st>>>(bd, bx, by, g, gate);
}

// stand-alone FFT of `count` rows (used by the tests through the C ABI)
template <typename T>
__global__ void k_fft_rows(FFTPlan P, const C2<T> *tw, const C2<T> *in, C2<T> *out, int inv) {
    extern __shared__ unsigned char smem_raw[];
    C2<T> *a = reinterpret_cast<C2<T> *>(smem_raw);
    C2<T> *b = a + P.n;
    const C2<T> *src = in + (size_t)blockIdx.x * P.n;
    for (int x = threadIdx.x; x < P.n; x += blockDim.x) a[x] = src[x];
    __syncthreads();
    C2<T> *res = fft_smem(a, b, P, tw, inv != 0);
    for (int x = threadIdx.x; x < P.n; x += blockDim.x) out[(size_t)blockIdx.x * P.n + x] = res[x];
}

template <typename T>
cudaError_t launch_fft_rows(const FFTPlan &P, const void *tw, const void *in, void *out, int rows, int inv,
                            cudaStream_t st) {
    size_t sm = 2 * (size_t)P.n * sizeof(C2<T>);
    cudaError_t e = cudaFuncSetAttribute(k_fft_rows<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_fft_rows<T><<<rows, 256, sm, st>>>(P, (const C2<T> *)tw, (const C2<T> *)in, (C2<T> *)out, inv);
    return cudaGetLastError();
}

#define INST(T)                                                                                            \
    template size_t boundary_smem_need<T>(const BoundaryDev<T> &, int);                                   \
    template cudaError_t boundary_configure<T>(const BoundaryDev<T> &, int);                              \
    template void launch_boundary<T>(const BoundaryDev<T> &, const Geom &, const T *, const T *, int, T *, T *,  \
                                     StepGate,                                                            \
                                     cudaStream_t);                                                       \
    template cudaError_t launch_fft_rows<T>(const FFTPlan &, const void *, const void *, void *, int, int, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace tcsem
