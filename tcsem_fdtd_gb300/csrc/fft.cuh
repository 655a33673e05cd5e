// Stockham mixed-radix FFT of one or two short transforms held in shared
// memory, executed by one thread block.
//
// The continuation plane of the air boundary has arbitrary lengths (the
// reference picks them from the grid: 736 = 2^5 * 23, 435 = 3 * 5 * 29, ...),
// so every stage is one of
//   * a radix 2, 3, 4, 5 or 8 butterfly computed in registers, one butterfly
//     per thread, with the DFT written out by hand;
//   * an odd prime radix p >= 7 computed in two passes: the twiddled inputs of
//     each butterfly are folded in place into sums S_q = v_q + v_{p-q} and
//     differences D_q = v_q - v_{p-q}, then each thread forms one output pair
//     X_u, X_{p-u} = A -+ iB with A = v_0 + sum_q S_q cos(2 pi q u / p) and
//     B = sum_q D_q sin(2 pi q u / p) -- half the multiplies of a direct DFT
//     and p/2 independent tasks per butterfly.
// Twiddles come from a table exp(-2 pi i k / n), k < n, that the caller has
// staged in shared memory; the inverse transform uses its conjugate.  All
// index divisions by run-time divisors use a multiply-high reciprocal, exact
// for dividend * divisor < 2^32.
#pragma once
#include "boundary.cuh"

namespace tcsem {
namespace fft {

template <typename T> __device__ __forceinline__ C2<T> add(C2<T> a, C2<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T> __device__ __forceinline__ C2<T> sub(C2<T> a, C2<T> b) { return {a.x - b.x, a.y - b.y}; }
template <typename T> __device__ __forceinline__ C2<T> scale(C2<T> a, T s) { return {a.x * s, a.y * s}; }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename T> __device__ __forceinline__ C2<T> rot(C2<T> a) {
    return INV ? C2<T>{-a.y, a.x} : C2<T>{a.y, -a.x};
}
// a * w (forward) or a * conj(w) (inverse), w from the forward table
template <bool INV, typename T> __device__ __forceinline__ C2<T> mulw(C2<T> a, C2<T> w) {
    return INV ? C2<T>{a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y}
               : C2<T>{a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x};
}

// floor(x / d) for x * d < 2^32 with mag = magic(d)
__device__ __forceinline__ unsigned magic(unsigned d) { return d > 1 ? 0xFFFFFFFFu / d + 1u : 0u; }
__device__ __forceinline__ int fdiv(int x, int d, unsigned mag) {
    return d > 1 ? (int)__umulhi((unsigned)x, mag) : x;
}

// DFT of P points in natural order, in place
template <int P, bool INV, typename T> __device__ __forceinline__ void dft(C2<T> *v) {
    if constexpr (P == 2) {
        const C2<T> t = v[0];
        v[0] = add(t, v[1]);
        v[1] = sub(t, v[1]);
    } else if constexpr (P == 3) {
        const T s3 = T(0.86602540378443864676);  // sin(2 pi / 3)
        const C2<T> t1 = add(v[1], v[2]), t2 = sub(v[1], v[2]);
        const C2<T> m = {v[0].x - T(0.5) * t1.x, v[0].y - T(0.5) * t1.y};
        v[0] = add(v[0], t1);
        const C2<T> r = rot<INV>(scale(t2, s3));
        v[1] = add(m, r);
        v[2] = sub(m, r);
    } else if constexpr (P == 4) {
        const C2<T> t0 = add(v[0], v[2]), t1 = sub(v[0], v[2]), t2 = add(v[1], v[3]);
        const C2<T> t3 = rot<INV>(sub(v[1], v[3]));
        v[0] = add(t0, t2);
        v[2] = sub(t0, t2);
        v[1] = add(t1, t3);
        v[3] = sub(t1, t3);
    } else if constexpr (P == 5) {
        const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);  // cos(2 pi/5), cos(4 pi/5)
        const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);   // sin(2 pi/5), sin(4 pi/5)
        const C2<T> S1 = add(v[1], v[4]), D1 = sub(v[1], v[4]), S2 = add(v[2], v[3]), D2 = sub(v[2], v[3]);
        const C2<T> A1 = {v[0].x + c1 * S1.x + c2 * S2.x, v[0].y + c1 * S1.y + c2 * S2.y};
        const C2<T> A2 = {v[0].x + c2 * S1.x + c1 * S2.x, v[0].y + c2 * S1.y + c1 * S2.y};
        const C2<T> B1 = {s1 * D1.x + s2 * D2.x, s1 * D1.y + s2 * D2.y};
        const C2<T> B2 = {s2 * D1.x - s1 * D2.x, s2 * D1.y - s1 * D2.y};
        v[0] = add(v[0], add(S1, S2));
        const C2<T> r1 = rot<INV>(B1), r2 = rot<INV>(B2);
        v[1] = add(A1, r1);
        v[4] = sub(A1, r1);
        v[2] = add(A2, r2);
        v[3] = sub(A2, r2);
    } else if constexpr (P == 8) {
        const T h = T(0.70710678118654752440);  // sqrt(1/2)
        C2<T> e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
        dft<4, INV>(e);
        dft<4, INV>(o);
        // o_u * W8^u: W8 = (h, -h) forward, (h, h) inverse; W8^2 = rot, W8^3 = rot * W8
        const C2<T> o1 = INV ? C2<T>{(o[1].x - o[1].y) * h, (o[1].x + o[1].y) * h}
                             : C2<T>{(o[1].x + o[1].y) * h, (o[1].y - o[1].x) * h};
        const C2<T> w3 = INV ? C2<T>{(o[3].x - o[3].y) * h, (o[3].x + o[3].y) * h}
                             : C2<T>{(o[3].x + o[3].y) * h, (o[3].y - o[3].x) * h};
        const C2<T> o2 = rot<INV>(o[2]), o3 = rot<INV>(w3);
        v[0] = add(e[0], o[0]);
        v[4] = sub(e[0], o[0]);
        v[1] = add(e[1], o1);
        v[5] = sub(e[1], o1);
        v[2] = add(e[2], o2);
        v[6] = sub(e[2], o2);
        v[3] = add(e[3], o3);
        v[7] = sub(e[3], o3);
    }
}

// one Stockham stage of radix P (register butterflies) over NB transforms of
// length n stored back to back
template <int P, bool INV, int NB, typename T>
__device__ __forceinline__ void stage_small(const C2<T> *__restrict__ a, C2<T> *__restrict__ b,
                                            const C2<T> *__restrict__ tw, int n, int Ns, int m, int step) {
    const unsigned mag = magic(Ns);
    for (int w = threadIdx.x; w < NB * m; w += blockDim.x) {
        int t = 0, r = w;
        if (NB == 2 && r >= m) { t = 1; r -= m; }
        const int hi = fdiv(r, Ns, mag), lo = r - hi * Ns;
        const C2<T> *src = a + t * n + r;
        C2<T> *dst = b + t * n + hi * Ns * P + lo;
        C2<T> v[P];
#pragma unroll
        for (int q = 0; q < P; q++) v[q] = src[q * m];
        if (lo) {
            const int st = step * lo;
#pragma unroll
            for (int q = 1; q < P; q++) v[q] = mulw<INV>(v[q], tw[q * st]);
        }
        dft<P, INV>(v);
#pragma unroll
        for (int u = 0; u < P; u++) dst[u * Ns] = v[u];
    }
}

// one Stockham stage of odd prime radix p >= 7 (folded two-pass form);
// overwrites a
template <bool INV, int NB, typename T>
__device__ void stage_prime(C2<T> *__restrict__ a, C2<T> *__restrict__ b, const C2<T> *__restrict__ tw, int n,
                            int p, int Ns, int m, int step) {
    const int h = (p - 1) >> 1, nm = NB * m;
    const unsigned magNs = magic(Ns), magNM = magic(nm);
    for (int w = threadIdx.x; w < nm * h; w += blockDim.x) {
        const int q = fdiv(w, nm, magNM) + 1;
        int t = 0, r = w - (q - 1) * nm;
        if (NB == 2 && r >= m) { t = 1; r -= m; }
        const int lo = r - fdiv(r, Ns, magNs) * Ns;
        C2<T> *x = a + t * n + r;
        C2<T> v1 = x[q * m], v2 = x[(p - q) * m];
        if (lo) {
            const int st = step * lo;
            v1 = mulw<INV>(v1, tw[q * st]);
            v2 = mulw<INV>(v2, tw[(p - q) * st]);
        }
        x[q * m] = add(v1, v2);
        x[(p - q) * m] = sub(v1, v2);
    }
    __syncthreads();
    for (int w = threadIdx.x; w < nm * (h + 1); w += blockDim.x) {
        const int u = fdiv(w, nm, magNM);
        int t = 0, r = w - u * nm;
        if (NB == 2 && r >= m) { t = 1; r -= m; }
        const int hi = fdiv(r, Ns, magNs), lo = r - hi * Ns;
        const C2<T> *x = a + t * n + r;
        C2<T> *dst = b + t * n + hi * Ns * p + lo;
        C2<T> A = x[0];
        if (u == 0) {
            for (int q = 1; q <= h; q++) A = add(A, x[q * m]);
            dst[0] = A;
        } else {
            C2<T> B = {T(0), T(0)};
            const int du = u * m;  // tw[q u m] = exp(-2 pi i q u / p)
            int e = du;
            for (int q = 1; q <= h; q++) {
                const C2<T> c = tw[e], S = x[q * m], D = x[(p - q) * m];
                A.x += S.x * c.x;
                A.y += S.y * c.x;
                B.x -= D.x * c.y;
                B.y -= D.y * c.y;
                e += du;
                if (e >= n) e -= n;
            }
            const C2<T> r2 = rot<INV>(B);
            dst[u * Ns] = add(A, r2);
            dst[(p - u) * Ns] = sub(A, r2);
        }
    }
}

// NB transforms of length P.n in a[0 .. NB*n); b is scratch of the same size.
// Entry: a and tw written and the block synchronised.  Returns the buffer
// holding the result (a or b); the other one is clobbered.
template <bool INV, int NB, typename T>
__device__ C2<T> *run(C2<T> *a, C2<T> *b, const FFTPlan &P, const C2<T> *tw) {
    const int n = P.n;
    int Ns = 1;
    for (int s = 0; s < P.nst; s++) {
        const int p = P.radix[s], m = n / p, step = m / Ns;
        switch (p) {
        case 2: stage_small<2, INV, NB>(a, b, tw, n, Ns, m, step); break;
        case 3: stage_small<3, INV, NB>(a, b, tw, n, Ns, m, step); break;
        case 4: stage_small<4, INV, NB>(a, b, tw, n, Ns, m, step); break;
        case 5: stage_small<5, INV, NB>(a, b, tw, n, Ns, m, step); break;
        case 8: stage_small<8, INV, NB>(a, b, tw, n, Ns, m, step); break;
        default: stage_prime<INV, NB>(a, b, tw, n, p, Ns, m, step); break;
        }
        __syncthreads();
        C2<T> *t = a;
        a = b;
        b = t;
        Ns *= p;
    }
    return a;
}

}  // namespace fft
}  // namespace tcsem
