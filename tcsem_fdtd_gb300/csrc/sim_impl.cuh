#pragma once
// Simulation state of one survey on one GPU (used by sim.cu and batch.cu).
//
// A handle owns, on one device and one stream (plus a high-priority side stream
// that the steps fork onto and join back from):
//   * two field sets (ping-pong) in the padded layout of kernels.cuh, plus the
//     conductivity -- 13 volume arrays;
//   * the boundary pipeline's operators and scratch (boundary.cuh);
//   * the per-step table (scalars + receiver plan) of the whole run, so a
//     block of steps is one CUDA graph that is captured once and replayed;
//   * the receiver stencils, slots and traces of the selected transmitter.
// The step loop of main.cu:219-273 becomes: graph launch per block of
// `graph_steps` steps, each step = boundary (4 kernels) -> fused sweep ->
// receiver kernel, followed by one counter advance per block.  With z-chunks
// only the top chunk reads the air plane the boundary writes, so by default a
// step forks: [boundary -> sweep of chunk 0] on the side stream beside [sweep
// of chunks 1..n-1] on the main stream, joined before the receiver kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "boundary.cuh"
#include "check.cuh"
#include "kernels.cuh"
#include "rx.cuh"
#include "setup.h"
#include "tcsem.h"

namespace tcsem {

#define CK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            throw Error(e_ == cudaErrorMemoryAllocation ? TCSEM_ERR_NOMEM : TCSEM_ERR_CUDA,             \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                            \
    } while (0)

struct DevMem {
    void *p = nullptr;
    size_t n = 0;
    DevMem() = default;
    DevMem(const DevMem &) = delete;
    DevMem &operator=(const DevMem &) = delete;
    ~DevMem() { if (p) cudaFree(p); }
    void alloc(size_t bytes) {
        if (p) { cudaFree(p); p = nullptr; }
        n = bytes;
        if (bytes) CK(cudaMalloc(&p, bytes));
    }
    template <class U> U *as() const { return reinterpret_cast<U *>(p); }
};

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link-time dependency on libcuda)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !p)
            throw Error(TCSEM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

inline FFTPlan make_plan(int n) {
    FFTPlan P{};
    P.n = n;
    int m = n;
    while (m % 8 == 0) { P.radix[P.nst++] = 8; m /= 8; }
    while (m % 4 == 0) { P.radix[P.nst++] = 4; m /= 4; }
    while (m % 2 == 0) { P.radix[P.nst++] = 2; m /= 2; }
    for (int p = 3; m > 1; p += 2)
        while (m % p == 0) { P.radix[P.nst++] = p; m /= p; }
    return P;
}

// Tx<k>.bout of main.cu:280-292: int32 nr, NComp, Nt then float64 [nr][NComp][Nt]
inline void write_bout_file(const Model &m, int itx, const double *t, const char *path) {
    if (itx < 0 || itx >= (int)m.in.tx.size()) throw Error(TCSEM_ERR_INVALID, "transmitter index out of range");
    int hdr[3] = {m.in.tx[itx].nr, m.NComp, m.in.Nt};
    FILE *f = std::fopen(path, "wb");
    if (!f) throw Error(TCSEM_ERR_IO, std::string("cannot write ") + path);
    size_t n = (size_t)hdr[0] * hdr[1] * hdr[2];
    bool ok = std::fwrite(hdr, sizeof(int), 3, f) == 3 && std::fwrite(t, sizeof(double), n, f) == n;
    ok &= std::fclose(f) == 0;
    if (!ok) throw Error(TCSEM_ERR_IO, std::string("short write to ") + path);
}

// ---------------------------------------------------------------- base class
struct SimBase {
    Model model;
    Schedule sched;
    tcsem_opts opts{};
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    int itx = -1;
    bool begun = false;
    long step = 0;
    size_t dev_bytes = 0;
    size_t uploaded_bytes = 0;  // host-to-device bytes of the setup (tables, conductivity)
    int launches_per_step = 0;
    int chunks_used = 0, top_used = 0;  // z-chunk layout of the sweep in use (top_used 0: an even split)
    int tot_chunks_min = 0;             // chunk totals to allocate room for at least (a batch's tuner)
    virtual ~SimBase() {}
    virtual void init() = 0;
    virtual void select(int itx) = 0;
    virtual void begin(int itx) = 0;
    virtual void advance(long n, int *done) = 0;
    virtual void traces(double *out) = 0;
    virtual void upcontinuation() = 0;
    virtual void upcontinuation_in(void *scratch, size_t bytes) = 0;
    virtual void electric_field(double lam, double dt, double wave) = 0;
    virtual void bderivate(double dt) = 0;
    virtual void fused_step(double lam, double dt, double dtb, double wave) = 0;
    virtual void rx_sample(int efield, int slot, double *values) = 0;
    virtual void get_field(int comp, double *h) = 0;
    virtual void set_field(int comp, const double *h) = 0;
    virtual void time_steps(int itx, long n, double *tot, double *sweep, double *bnd) = 0;
    virtual void timed_advance(long n, double *ms) = 0;
    virtual void check_error() = 0;
    virtual void save_state(const char *path) = 0;
    virtual void load_state(const char *path) = 0;
    size_t field_count(int comp) const {
        size_t L = model.L, M = model.M, N = model.N;
        switch (comp) {
        case TCSEM_EX: return L * (M + 1) * (N + 1);
        case TCSEM_EY: return (L + 1) * M * (N + 1);
        case TCSEM_EZ: return (L + 1) * (M + 1) * N;
        case TCSEM_BX: return (L + 1) * M * N;
        case TCSEM_BY: return L * (M + 1) * N;
        case TCSEM_BZ: return L * M * (N + 1);
        case TCSEM_BXAIR: return (L + 1) * M;
        case TCSEM_BYAIR: return L * (M + 1);
        case TCSEM_CON: return L * M * N;
        }
        throw Error(TCSEM_ERR_INVALID, "unknown field component");
    }
    // extents (nx, ny, nz, z0) of a component in the reference layout
    void extents(int comp, int &nx, int &ny, int &nz, int &z0) const {
        int L = model.L, M = model.M, N = model.N;
        z0 = 0;
        switch (comp) {
        case TCSEM_EX: nx = L; ny = M + 1; nz = N + 1; break;
        case TCSEM_EY: nx = L + 1; ny = M; nz = N + 1; break;
        case TCSEM_EZ: nx = L + 1; ny = M + 1; nz = N; break;
        case TCSEM_BX: nx = L + 1; ny = M; nz = N; break;
        case TCSEM_BY: nx = L; ny = M + 1; nz = N; break;
        case TCSEM_BZ: nx = L; ny = M; nz = N + 1; break;
        case TCSEM_BXAIR: nx = L + 1; ny = M; nz = 1; z0 = -1; break;
        case TCSEM_BYAIR: nx = L; ny = M + 1; nz = 1; z0 = -1; break;
        case TCSEM_CON: nx = L; ny = M; nz = N; break;
        default: throw Error(TCSEM_ERR_INVALID, "unknown field component");
        }
    }
};

// ---------------------------------------------------------------- typed impl
template <typename T> struct SimImpl : SimBase {
    Geom g{};
    DevMem fld[2][6], con, tot[2];  // two field sets + conductivity; per-set chunk totals of Bz
    ZChunks zc{};
    SweepMaps maps[2];              // TMA descriptors of each field set (+ conductivity)
    DevMem errw;                    // device error word (a bounded wait gave up)
    DevMem axis_mem;
    Axis<T> ax{};
    // boundary
    DevMem twx, twy, remT[2], remI[2], Gx, Gy, rows, FT, VX, VY, Zs, padx, pady;
    DevMem bxc_II, bxr_a, bxr_b, byc_II, byr_a, byr_b, bxc_l, bxr_l, byc_l, byr_l;
    BoundaryDev<T> bd{};
    // step tables
    DevMem steps, acts, gate_base;
    // transmitter dependent
    DevMem src_coef, rx_base, rx_comp, rx_w, ef0, efs, e_l1, b_l1;
    SourceTable<T> src{};
    RxDev<T> rd{};
    int cur = 0;  // buffer holding the current state
    // graph cache
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // indexed by the starting buffer
    int gsteps = 0;

    // the boundary pipeline and the top z-chunk run on `side` beside the lower chunks
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // overlapped order: the receivers of a step still to be launched (field set, step gate)
    int rx_pending = -1;
    StepGate rx_gate{};
    bool overlap = false;
    bool overlap_pdl = false;  // programmatic dependent launch inside the boundary chain of the overlapped step

    ~SimImpl() override {
        for (auto &e : gexec) if (e) cudaGraphExecDestroy(e);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }

    FieldSet<T> fs(int b) {
        return {fld[b][0].as<T>(), fld[b][1].as<T>(), fld[b][2].as<T>(), fld[b][3].as<T>(), fld[b][4].as<T>(),
                fld[b][5].as<T>()};
    }

    // Copies between the host and the handle's memory go through the handle's stream and
    // finish before returning: the kernels run on non-blocking streams, which a copy on the
    // legacy default stream would not be ordered against (and a pageable host-to-device
    // cudaMemcpy may return before its DMA lands).
    void h2d(void *dst, const void *src, size_t n) {
        if (!n) return;
        CK(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
    }
    void d2h(void *dst, const void *src, size_t n) {
        if (!n) return;
        CK(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
    }
    void dzero(void *dst, size_t n) {
        if (n) CK(cudaMemsetAsync(dst, 0, n, stream));
    }
    template <class U> void upload(DevMem &m, const std::vector<U> &v) {
        m.alloc(v.size() * sizeof(U));
        dev_bytes += m.n;
        uploaded_bytes += m.n;
        h2d(m.p, v.data(), m.n);
    }
    template <class U> std::vector<T> conv(const std::vector<U> &v) { return std::vector<T>(v.begin(), v.end()); }

    void init() override {
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        const Model &m = model;
        g = make_geom(m.L, m.M, m.N);
        const size_t vol = (size_t)g.total() * sizeof(T);
        for (int b = 0; b < 2; b++)
            for (int c = 0; c < 6; c++) {
                fld[b][c].alloc(vol);
                dev_bytes += vol;
                CK(cudaMemsetAsync(fld[b][c].p, 0, vol, stream));
            }
        {  // conductivity in the padded layout, plane -1 (air) and padding zero; planes split over threads
            std::vector<T> h((size_t)g.total(), T(0));
            auto planes = [&](int k0, int k1) {
                for (int k = k0; k < k1; k++)
                    for (int j = 0; j < m.M; j++) {
                        const double *src = m.in.con.data() + ((size_t)k * m.M + j) * m.L;
                        T *dst = h.data() + g.at(0, j, k);
                        for (int i = 0; i < m.L; i++) dst[i] = (T)src[i];
                    }
            };
            const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
            std::vector<std::thread> pool;
            for (int q = 0; q < nt; q++) pool.emplace_back(planes, (int)((long)q * m.N / nt), (int)((long)(q + 1) * m.N / nt));
            for (auto &th : pool) th.join();
            upload(con, h);
        }
        {  // axis tables
            std::vector<T> t;
            auto put = [&](const std::vector<double> &v) { size_t o = t.size(); for (double x : v) t.push_back((T)x); return o; };
            std::vector<double> rdx(m.L), rdy(m.M), rdz(m.N), rdx2(m.L, 0), rdy2(m.M, 0), rdzs(m.N);
            for (int i = 0; i < m.L; i++) { rdx[i] = 1.0 / m.dxk[i]; if (i) rdx2[i] = 1.0 / (m.dxk[i - 1] + m.dxk[i]); }
            for (int j = 0; j < m.M; j++) { rdy[j] = 1.0 / m.dyk[j]; if (j) rdy2[j] = 1.0 / (m.dyk[j - 1] + m.dyk[j]); }
            for (int k = 0; k < m.N; k++) { rdz[k] = 1.0 / m.dzk[k]; rdzs[k] = k ? 1.0 / (m.dzk[k] + m.dzk[k - 1]) : 1.0 / (2.0 * m.dzk[0]); }
            size_t o[9];
            o[0] = put(m.dxk); o[1] = put(m.dyk); o[2] = put(m.dzk); o[3] = put(rdx); o[4] = put(rdy); o[5] = put(rdz);
            o[6] = put(rdx2); o[7] = put(rdy2); o[8] = put(rdzs);
            upload(axis_mem, t);
            const T *b = axis_mem.as<T>();
            ax = {b + o[0], b + o[1], b + o[2], b + o[3], b + o[4], b + o[5], b + o[6], b + o[7], b + o[8]};
        }
        init_chunks();
        init_maps();
        init_boundary();
        init_steps();
        // the top chunk's air plane is the only input of the sweep that the boundary writes
        overlap = zc.n > 1 && !opts.serial_boundary;
        if (overlap) {
            int lo = 0, hi = 0;
            CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
            CK(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi));
            CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        }
        launches_per_step = 4 + (overlap ? 2 : 1) + 1;
        CK(cudaStreamSynchronize(stream));
        if (overlap) choose_overlap_pdl();
        if (overlap && opts.zchunks < 0 && sched.nsteps >= 64) tune_layout();
        chunks_used = zc.n;
        top_used = overlap ? zc.kb[1] : 0;
    }

    // Beside the sweep, the boundary kernels launched early (programmatic dependent launch)
    // take SM space that the sweep's single wave still needs when the sweep is the longer
    // branch; they shorten the step when the boundary chain is the longer one.  Decided
    // from one timed sweep and one timed boundary pass on the zero state (the choice
    // changes timing only, never results).
    void choose_overlap_pdl() {
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        auto timed = [&](auto &&fn) {
            fn();  // untimed first launch
            CK(cudaEventRecord(e0, stream));
            fn();
            CK(cudaEventRecord(e1, stream));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            return ms;
        };
        if (itx < 0) select(0);
        const StepScalars<T> s = scal(sched.lam[0], sched.dt1[0], sched.dtB[0], 0.0);
        const float t_sweep = timed([&] { sweep(0, s, nullptr, StepGate{nullptr, 0, 0}); });
        const float t_bnd = timed([&] {
            FieldSet<T> f = fs(0);
            launch_boundary<T>(bd, g, f.bz, tot[0].as<T>(), zc.n, f.bx, f.by, StepGate{nullptr, 0, 0}, stream, false);
        });
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        CK(cudaGetLastError());
        overlap_pdl = t_bnd >= 0.5f * t_sweep;
        zero_state();
    }

    // The layout autotuner (tcsem_opts.zchunks = -1): times a captured block of 8 steps for
    // each layout near the rule of init_chunks -- one to five lower chunks around it, a
    // one-plane or an even top chunk -- and keeps the fastest.  The Bz prefix is summed per
    // chunk, so the layout decides the order of some FP additions: with the tuner the last
    // bits may differ between runs whose timings chose differently.
    int rule_lower = 1;  // lower chunks the rule of init_chunks chose
    void tune_layout() {
        if (itx < 0) select(0);
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        struct Cand { int n, top; };
        std::vector<Cand> cands;
        for (int lower = std::max(1, rule_lower - 2); lower <= rule_lower + 2 && lower + 1 <= max_chunks(); lower++)
            for (int top : {1, 0}) cands.push_back({lower + 1, top});
        const int keep = gsteps;
        gsteps = 8;
        float best = 1e30f;
        Cand pick = {zc.n, zc.n > 1 && zc.kb[1] == 1 ? 1 : 0};
        for (const Cand &c : cands) {
            set_chunks(c.n, c.top);
            for (auto &e : gexec) if (e) { cudaGraphExecDestroy(e); e = nullptr; }
            zero_state();
            cudaGraphExec_t ge = graph_for(cur);
            CK(cudaGraphLaunch(ge, stream));  // untimed
            CK(cudaEventRecord(e0, stream));
            CK(cudaGraphLaunch(ge, stream));
            CK(cudaGraphLaunch(ge, stream));
            CK(cudaEventRecord(e1, stream));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) { best = ms; pick = c; }
        }
        gsteps = keep;
        for (auto &e : gexec) if (e) { cudaGraphExecDestroy(e); e = nullptr; }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        set_chunks(pick.n, pick.top);
        zero_state();
        CK(cudaStreamSynchronize(stream));
    }

    // z-chunk layout: n chunks, the top one `top` planes deep (top <= 0: an even split)
    void set_chunks(int n, int top) {
        const int N = model.N;
        zc.n = n;
        for (int c = 0; c <= n; c++) zc.kb[c] = (int)(((long)c * N) / n);
        if (n > 1 && top > 0) {
            top = std::max(1, std::min(top, N - (n - 1)));
            for (int c = 1; c <= n; c++) zc.kb[c] = top + (int)(((long)(c - 1) * (N - top)) / (n - 1));
        }
    }
    // most chunks a layout may have: every chunk keeps at least 8 planes
    int max_chunks() const { return std::max(1, std::min(kMaxChunks, model.N / 8)); }
    // z-chunks of the fused sweep.  Overlapped step: a one-plane top chunk (the only part of
    // the sweep that waits for the boundary) and lower chunks whose CTAs fit in one wave;
    // deeper chunks also mean fewer halo planes.  In FP32 the sweep is bound by memory and
    // the wave leaves about 15 % of the CTA slots to the boundary kernels running beside it;
    // in FP64 it is bound by the FP64 pipes and the wave fills the slots as far as it can.
    // Serial step: enough CTAs to fill the GPU several times over, split evenly.
    void init_chunks() {
        const Model &m = model;
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        CK(sweep_configure<T>(m.N));
        const long tiles = (long)sweep_tiles_x(m.L) * sweep_tiles_y(m.M);
        const long slots = (long)sms * sweep_blocks_per_sm<T>(m.N);
        int n, top = 0;
        if (opts.serial_boundary) {
            n = (int)std::min<long>(kMaxChunks, std::max<long>(1, (7L * sms + tiles - 1) / tiles));
        } else {
            const long want = slots * 85 / 100;
            long lower = std::max<long>(1, want / tiles);
            if (sizeof(T) == 8 && (lower + 1) * tiles <= slots) lower++;
            n = 1 + (int)lower;
            top = 1;
        }
        n = std::min(n, max_chunks());
        rule_lower = n - 1;
        if (opts.zchunks > 0) n = std::min(std::min(opts.zchunks, kMaxChunks), m.N);
        if (opts.top_planes != 0) top = opts.top_planes;  // > 0: that many planes, < 0: an even split
        set_chunks(n, top);
        // the autotuner may pick up to two more lower chunks than the rule
        int nalloc = opts.zchunks < 0 ? std::max(n, std::min(rule_lower + 3, max_chunks())) : n;
        nalloc = std::max(nalloc, std::min(tot_chunks_min, max_chunks()));
        const size_t tb = (size_t)nalloc * g.PS * sizeof(T);
        for (int b = 0; b < 2; b++) {
            tot[b].alloc(tb);
            dev_bytes += tb;
            CK(cudaMemsetAsync(tot[b].p, 0, tb, stream));
        }
    }
    void init_maps() {
        if (g.total() >= (1LL << 31)) throw Error(TCSEM_ERR_INVALID, "grid too large for 32-bit offsets");
        EncodeTiledFn enc = encode_tiled();
        const cuuint64_t dims[3] = {(cuuint64_t)g.XP, (cuuint64_t)g.YP, (cuuint64_t)(g.N + 2)};
        const cuuint64_t strides[2] = {(cuuint64_t)g.XP * sizeof(T), (cuuint64_t)g.PS * sizeof(T)};
        const cuuint32_t box[3] = {(cuuint32_t)sweep_box_x(), (cuuint32_t)sweep_box_y(), 1};
        const cuuint32_t estr[3] = {1, 1, 1};
        const CUtensorMapDataType dt = sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
        auto make = [&](void *ptr, CUtensorMap *m) {
            CUresult r = enc(m, dt, 3, ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) throw Error(TCSEM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        };
        for (int b = 0; b < 2; b++) {
            for (int a = 0; a < 6; a++) make(fld[b][a].p, &maps[b].m[a]);
            make(con.p, &maps[b].m[6]);
        }
        errw.alloc(sizeof(int));
        dev_bytes += sizeof(int);
        dzero(errw.p, sizeof(int));
        CK(sweep_configure<T>(g.N));
    }
    void check_error() override { check_device_error(); }
    void check_device_error() {
        int h = 0;
        d2h(&h, errw.p, sizeof(int));
        if (h) {
            dzero(errw.p, sizeof(int));
            if (h == TCSEM_CHECK_CODE)
                throw Error(TCSEM_ERR_CUDA, "a kernel index fell outside its array (bounds-checked build)");
            throw Error(TCSEM_ERR_CUDA, "a bounded wait in a kernel gave up (a bulk copy did not arrive)");
        }
    }
    void sweep(int b, StepScalars<T> s, const StepScalars<T> *table, StepGate gate, int c0 = 0, int c1 = -1,
               cudaStream_t st = nullptr, bool pdl = false) {
        if (c1 < 0) c1 = zc.n;
        // Block order: consecutive steps alternate the chunk order (a step starts on the planes
        // the previous one wrote last), except in a launch that includes a top chunk shorter than
        // the others -- its blocks go last, so its short CTAs take the slots the single wave of
        // the others leaves free instead of delaying them (measured: 119.0 µs for the whole
        // 256 x 256 x 160 sweep against 121.8 alternating and 125.4 with the top chunk first)
        const bool short_top = c0 == 0 && c1 - c0 > 1 && zc.kb[1] - zc.kb[0] < zc.kb[2] - zc.kb[1];
        launch_fused_sweep<T>(maps[b], g, fs(b ^ 1), tot[b].as<T>(), tot[b ^ 1].as<T>(), ax, s, table, gate, src, zc,
                              c0, c1, short_top || (b & 1) != 0, errw.as<int>(), st ? st : stream, pdl);
    }
    void consolidate(int b) { launch_bz_consolidate<T>(g, fs(b).bz, tot[b].as<T>(), zc, stream); }

    // transform length of a uniform line of n points: n itself (mode 0), the power of two
    // above it (mode 1, the LNx2/LMy2 sizes of ModelingSetup.cpp:194-195), or the smallest
    // length >= n with no prime factor above 5 (mode 2: only the FFT-friendly size)
    static int plane_len(int n, int mode) {
        if (mode == 1) {
            int p = 1;
            while (p <= n) p *= 2;
            return p;
        }
        if (mode == 2)
            for (int m = n;; m++) {
                int r = m;
                for (int f : {2, 3, 5})
                    while (r % f == 0) r /= f;
                if (r == 1) return m;
            }
        return n;
    }
    // raised-cosine weights of the padded points of a line of n transform points around a grid
    // of nu points at offset d (the taper UpContinuation.cpp:21-49 sketches), zero on the grid
    static std::vector<double> pad_weights(int n, int nu, int d) {
        std::vector<double> w(n + 4, 0.0);  // 4 spare entries keep the upload a multiple of 16 bytes
        const int r = n - nu - d;
        for (int i = 0; i < d; i++) w[i] = 0.5 * (1.0 - std::cos(kPi * i / d));
        for (int i = d + nu; i < n; i++) w[i] = 0.5 * (1.0 - std::cos(kPi * (n - i) / (r + 1)));
        return w;
    }
    void init_boundary() {
        const Model &m = model;
        const int mode = opts.padded_plane;
        if (mode < 0 || mode > 2) throw Error(TCSEM_ERR_INVALID, "padded_plane must be 0, 1 or 2");
        const int Lu = m.L1, Mu = m.M1;                                 // the uniform grid
        const int L1 = plane_len(Lu, mode), M1 = plane_len(Mu, mode);  // the transforms
        const int H = L1 / 2 + 1, DL = (L1 - Lu) / 2, DM = (M1 - Mu) / 2;
        auto tw = [&](int n, DevMem &d) {
            std::vector<C2<T>> h(n + 1, C2<T>{T(0), T(0)});  // one spare entry: 16-byte bulk copies
            for (int k = 0; k < n; k++) {
                double a = -2.0 * kPi * (double)k / (double)n;
                h[k] = {(T)std::cos(a), (T)std::sin(a)};
            }
            upload(d, h);
        };
        tw(L1, twx);
        tw(M1, twy);
        // factored spline remaps, one table per axis: per strip g, w, inv, du, then [6][npts] window weights
        auto pack = [&](int axis, const SplinePlan &p0, const SplinePlan &p1, int src1, int dst1, AxisRemap<T> &R) {
            std::vector<double> t;
            std::vector<int> ti;
            const SplinePlan *ps[2] = {&p0, &p1};
            R.nmax = 0;
            for (int k = 0; k < 2; k++) {
                const SplinePlan &P = *ps[k];
                StripPlan &S = R.s[k];
                S.n = P.n; S.npts = P.npts;
                S.src = k ? src1 : 0;
                S.dst = k ? dst1 : 0;
                S.f = (int)t.size();
                for (const auto *v : {&P.g, &P.w, &P.inv, &P.du}) t.insert(t.end(), v->begin(), v->end());
                S.c = (int)t.size();
                t.insert(t.end(), P.c.begin(), P.c.end());
                S.k = (int)ti.size();
                ti.insert(ti.end(), P.k0.begin(), P.k0.end());
                R.nmax = std::max(R.nmax, P.n);
            }
            R.nT = (int)t.size();
            R.nI = (int)ti.size();
            t.resize(t.size() + 4, 0.0);  // the bulk copies round up to 16 bytes
            ti.resize(ti.size() + 4, 0);
            upload(remT[axis], conv(t));
            upload(remI[axis], ti);
            R.tabT = remT[axis].as<T>();
            R.tabI = remI[axis].as<int>();
        };
        // continuation filters of FBz_to_FBxFBy (UpContinuation_gpu.cu:113-164) as i*g; the two
        // self-conjugate columns keep their Hermitian part so the inverse transform is real
        const int M1p = (M1 + 3) & ~3;  // filter rows padded to 16 bytes
        std::vector<double> gx((size_t)H * M1p, 0.0), gy((size_t)H * M1p, 0.0);
        const double dxm = m.in.dxmin, dym = m.in.dymin, dzm = m.in.dzmin;
        for (int kx = 0; kx < H; kx++)
            for (int ky = 0; ky < M1; ky++) {
                double v1 = ky < M1 / 2 + 1 ? (1.0 * kPi * ky) / M1 * (dzm / dym) : -(1.0 * kPi * (M1 - ky)) / M1 * (dzm / dym);
                double u1 = (1.0 * kPi * kx) / L1 * (dzm / dxm);
                double a, b;
                if (kx == 0 && ky == 0) { a = 1.0; b = 1.0; }
                else {
                    double w = std::sqrt(u1 * u1 + v1 * v1);
                    double upcc = std::exp(-w) * (1.0 / w);
                    a = (dxm / dym) * u1 * upcc;
                    b = (dym / dxm) * v1 * upcc;
                }
                gx[(size_t)kx * M1p + ky] = a;
                gy[(size_t)kx * M1p + ky] = b;
            }
        for (int kx = 0; kx < H; kx++) {
            if (!(kx == 0 || 2 * kx == L1)) continue;
            std::vector<double> ox(gx.begin() + (size_t)kx * M1p, gx.begin() + (size_t)kx * M1p + M1);
            std::vector<double> oy(gy.begin() + (size_t)kx * M1p, gy.begin() + (size_t)kx * M1p + M1);
            for (int ky = 0; ky < M1; ky++) {
                int mk = (M1 - ky) % M1;
                gx[(size_t)kx * M1p + ky] = 0.5 * (ox[ky] - ox[mk]);
                gy[(size_t)kx * M1p + ky] = 0.5 * (oy[ky] - oy[mk]);
            }
        }
        upload(Gx, conv(gx));
        upload(Gy, conv(gy));
        // rows of the uniform plane that the bilinear remap reads, and its tables
        auto clampi = [](int v, int lo, int hi) { return std::min(std::max(v, lo), hi); };
        std::vector<int> need;
        for (int j = 0; j < m.M; j++) { int J = clampi(m.yBzold2New[j], 1, Mu - 1); need.push_back(J - 1); need.push_back(J); }
        for (int j = 0; j <= m.M; j++) { int J = clampi(m.yoldBy2NewBz[j], 1, Mu - 1); need.push_back(J - 1); need.push_back(J); }
        std::sort(need.begin(), need.end());
        need.erase(std::unique(need.begin(), need.end()), need.end());
        std::vector<int> slot(Mu, -1);
        for (size_t s = 0; s < need.size(); s++) slot[need[s]] = (int)s;
        std::vector<int> rows_t(need);  // rows of the transform plane
        for (int &r : rows_t) r += DM;
        upload(rows, rows_t);
        std::vector<int> hbxcII(m.L + 1), hbxra(m.M), hbxrb(m.M), hbycII(m.L), hbyra(m.M + 1), hbyrb(m.M + 1);
        std::vector<double> hbxcl(m.L + 1), hbxrl(m.M), hbycl(m.L), hbyrl(m.M + 1);
        for (int i = 0; i <= m.L; i++) {
            int II = clampi(m.xoldBx2NewBz[i], 1, Lu - 1);
            double Xp = i == m.L ? m.X[m.L - 1] + 0.5 * m.dx[m.L - 1] : m.X[i] - 0.5 * m.dx[i];
            hbxcII[i] = II;
            hbxcl[i] = (Xp - m.Xn[II - 1]) / (m.Xn[II] - m.Xn[II - 1]);
        }
        for (int j = 0; j < m.M; j++) {
            int J = clampi(m.yBzold2New[j], 1, Mu - 1);
            hbxra[j] = slot[J - 1]; hbxrb[j] = slot[J];
            hbxrl[j] = (m.Y[j] - m.Yn[J - 1]) / (m.Yn[J] - m.Yn[J - 1]);
        }
        for (int i = 0; i < m.L; i++) {
            int II = clampi(m.xBzold2New[i], 1, Lu - 1);
            hbycII[i] = II;
            hbycl[i] = (m.X[i] - m.Xn[II - 1]) / (m.Xn[II] - m.Xn[II - 1]);
        }
        for (int j = 0; j <= m.M; j++) {
            int J = clampi(m.yoldBy2NewBz[j], 1, Mu - 1);
            double Yp = j == m.M ? m.Y[m.M - 1] + 0.5 * m.dy[m.M - 1] : m.Y[j] - 0.5 * m.dy[j];
            hbyra[j] = slot[J - 1]; hbyrb[j] = slot[J];
            hbyrl[j] = (Yp - m.Yn[J - 1]) / (m.Yn[J] - m.Yn[J - 1]);
        }
        upload(bxc_II, hbxcII); upload(bxr_a, hbxra); upload(bxr_b, hbxrb);
        upload(byc_II, hbycII); upload(byr_a, hbyra); upload(byr_b, hbyrb);
        upload(bxc_l, conv(hbxcl)); upload(bxr_l, conv(hbxrl)); upload(byc_l, conv(hbycl)); upload(byr_l, conv(hbyrl));
        const int S = (int)need.size();
        // rows of FT and VX/VY start on 16-byte boundaries (bulk copies)
        const int cpr = (int)(16 / sizeof(C2<T>));
        const int Mp = (m.M + cpr - 1) / cpr * cpr, Hp = (H + cpr - 1) / cpr * cpr;
        FT.alloc((size_t)H * Mp * sizeof(C2<T>)); dev_bytes += FT.n;
        VX.alloc((size_t)S * Hp * sizeof(C2<T>)); dev_bytes += VX.n;
        VY.alloc((size_t)S * Hp * sizeof(C2<T>)); dev_bytes += VY.n;
        Zs.alloc((size_t)S * Lu * sizeof(C2<T>)); dev_bytes += Zs.n;
        upload(padx, conv(pad_weights(L1, Lu, DL)));
        upload(pady, conv(pad_weights(M1, Mu, DM)));
        BoundaryDev<T> &B = bd;
        B.L1 = L1; B.M1 = M1; B.H = H; B.M = m.M;
        B.Lu = Lu; B.Mu = Mu; B.DL = DL; B.DM = DM;
        B.padx = padx.as<T>(); B.pady = pady.as<T>();
        B.AnLx = m.AnLx_New; B.Nx = m.in.Nx; B.AL = m.in.ALx1 + m.in.ALx2;
        B.Any = m.Any_New; B.Ny = m.in.Ny; B.Ay = m.in.Ay1 + m.in.Ay2;
        pack(0, m.sl, m.sr, m.ox, m.AnLx_New + m.in.Nx, B.rx);
        pack(1, m.sf, m.sb, m.oy, m.Any_New + m.in.Ny, B.ry);
        B.px = make_plan(L1); B.py = make_plan(M1);
        B.twx = twx.as<C2<T>>(); B.twy = twy.as<C2<T>>();
        B.Gx = Gx.as<T>(); B.Gy = Gy.as<T>();
        B.S = S; B.rows = rows.as<int>();
        B.Mp = Mp; B.M1p = M1p; B.Hp = Hp;
        B.err = errw.as<int>();
        B.FT = FT.as<C2<T>>(); B.VX = VX.as<C2<T>>(); B.VY = VY.as<C2<T>>(); B.Z = Zs.as<C2<T>>();
        B.bxc_II = bxc_II.as<int>(); B.bxr_a = bxr_a.as<int>(); B.bxr_b = bxr_b.as<int>();
        B.byc_II = byc_II.as<int>(); B.byr_a = byr_a.as<int>(); B.byr_b = byr_b.as<int>();
        B.bxc_l = bxc_l.as<T>(); B.bxr_l = bxr_l.as<T>(); B.byc_l = byc_l.as<T>(); B.byr_l = byr_l.as<T>();
        B.inv_norm = (T)(1.0 / (double)(L1 * M1));
        size_t need_smem = boundary_smem_need(B, m.L);
        int maxsm = 0;
        CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        if (need_smem > (size_t)maxsm)
            throw Error(TCSEM_ERR_INVALID, "continuation plane too large for the shared-memory FFT (" +
                                               std::to_string(L1) + " x " + std::to_string(M1) + ")");
        CK(boundary_configure(B, m.L));
    }

    void init_steps() {
        const Schedule &S = sched;
        std::vector<StepScalars<T>> st(S.nsteps);
        std::vector<StepEntryActs> ac(S.nsteps);
        for (long n = 0; n < S.nsteps; n++) {
            st[n].lam2 = (T)(2.0 * S.lam[n]);
            st[n].dt = (T)S.dt1[n];
            st[n].c4 = (T)(4.0 * S.dt1[n] / model.mu0);
            st[n].dtb = (T)S.dtB[n];
            st[n].wave = (T)S.wave[n];
            const StepActions &a = S.act[n];
            ac[n] = {a.e_slot, a.e_first, a.e_count, a.b_slot, a.b_first, a.b_count};
        }
        upload(steps, st);
        upload(acts, ac);
        upload(e_l1, conv(S.e_l1));
        upload(b_l1, conv(S.b_l1));
        gate_base.alloc(sizeof(int));
        dev_bytes += sizeof(int);
        gsteps = opts.graph_steps > 0 ? opts.graph_steps : 64;
        if (gsteps % 2) gsteps++;
    }

    void select(int t) override {
        if (t < 0 || t >= (int)model.in.tx.size()) throw Error(TCSEM_ERR_INVALID, "transmitter index out of range");
        if (t == itx) return;
        CK(cudaStreamSynchronize(stream));  // steps still in flight read the tables replaced below
        const Model &m = model;
        // sources
        std::vector<SourceSegment> segs = m.sources(t, opts.fix_dual_bipole != 0);
        if ((int)segs.size() > kMaxSeg) throw Error(TCSEM_ERR_INVALID, "too many source segments");
        std::vector<T> coef;
        src = SourceTable<T>{};
        src.nseg = (int)segs.size();
        for (int q = 0; q < src.nseg; q++) {
            const SourceSegment &s = segs[q];
            src.comp[q] = s.comp; src.i[q] = s.i; src.j[q] = s.j; src.k[q] = s.k; src.count[q] = s.count;
            src.off[q] = (int)coef.size();
            for (double c : s.coef) coef.push_back((T)(s.gain * c));
        }
        upload(src_coef, coef);
        src.coef = src_coef.as<T>();
        // receivers
        std::vector<RxStencil> sts = m.rx_stencils(t);
        const int nr = m.in.tx[t].nr;
        std::vector<long long> base(sts.size());
        std::vector<int> comp(sts.size());
        std::vector<T> w(sts.size() * 12);
        for (size_t q = 0; q < sts.size(); q++) {
            base[q] = g.at(sts[q].s1, sts[q].s2, sts[q].s3);
            comp[q] = sts[q].comp;
            for (int a = 0; a < 4; a++) { w[q * 12 + a] = (T)sts[q].wx[a]; w[q * 12 + 4 + a] = (T)sts[q].wy[a]; w[q * 12 + 8 + a] = (T)sts[q].wz[a]; }
        }
        upload(rx_base, base); upload(rx_comp, comp); upload(rx_w, w);
        ef0.alloc((size_t)2 * m.NComp * nr * sizeof(T));
        efs.alloc((size_t)nr * m.NComp * m.in.Nt * sizeof(T));
        rd.nr = nr; rd.NComp = m.NComp; rd.nefcmp = m.nefcmp; rd.Nt = m.in.Nt;
        rd.base = rx_base.as<long long>(); rd.comp = rx_comp.as<int>(); rd.w = rx_w.as<T>();
        rd.ef0 = ef0.as<T>(); rd.efs = efs.as<T>(); rd.e_l1 = e_l1.as<T>(); rd.b_l1 = b_l1.as<T>();
        rd.acts = acts.as<StepEntryActs>();
        rd.err = errw.as<int>();
        itx = t;
        for (auto &e : gexec) if (e) { cudaGraphExecDestroy(e); e = nullptr; }
    }

    void zero_state() {
        for (int b = 0; b < 2; b++)
            for (int c = 0; c < 6; c++) CK(cudaMemsetAsync(fld[b][c].p, 0, fld[b][c].n, stream));
        if (ef0.n) CK(cudaMemsetAsync(ef0.p, 0, ef0.n, stream));
        if (efs.n) CK(cudaMemsetAsync(efs.p, 0, efs.n, stream));
        CK(cudaMemsetAsync(gate_base.p, 0, sizeof(int), stream));
        for (int b = 0; b < 2; b++) CK(cudaMemsetAsync(tot[b].p, 0, tot[b].n, stream));
        cur = 0;
        step = 0;
    }

    void begin(int t) override {
        select(t);
        zero_state();
        begun = true;
    }

    // Overlapped order: the receivers of step s (which read the field set step s wrote) are
    // launched on the main stream of step s+1, after its lower z-chunks: step s+1 only reads
    // that set, and its lower chunks finish well before the boundary branch they join, so the
    // receivers run in that slack instead of beside the next boundary chain (marine3d_256x256x160:
    // 133.4 against 138.4 us per step with them on a stream of their own).  A run of steps
    // opens with nothing pending and closes by launching the receivers of its last step (the
    // step counter advance comes after them).
    void rx_open() { rx_pending = -1; }
    void rx_close(bool early = false) {
        if (overlap && rx_pending >= 0) {
            launch_rx<T>(rd, fs(rx_pending), tot[rx_pending].as<T>(), zc, g, rx_gate, RxAction{-1, 0, 0, -1, 0, 0},
                         stream, early);
            rx_pending = -1;
        }
    }

    // one step of main.cu:219-273 on the buffers starting at `b`
    void enqueue_step(int b, StepGate gate) {
        FieldSet<T> in = fs(b), out = fs(b ^ 1);
        const StepScalars<T> *table = steps.as<StepScalars<T>>();
        if (overlap) {  // fork: boundary -> top chunk on `side`; chunks 1.., then the previous step's receivers, on `stream`
            CK(cudaEventRecord(ev_fork, stream));
            CK(cudaStreamWaitEvent(side, ev_fork, 0));
            launch_boundary<T>(bd, g, in.bz, tot[b].as<T>(), zc.n, in.bx, in.by, gate, side, overlap_pdl);
            // the top chunk directly after the boundary's last stage, launched early: it stages its planes
            // while the bilinear remap runs and waits for it only before the air plane
            sweep(b, StepScalars<T>{}, table, gate, 0, 1, side, true);
            sweep(b, StepScalars<T>{}, table, gate, 1, zc.n, stream);
            // set b, which this step only reads (receiver stencils never reach the air plane); launched as
            // a programmatic dependent of the lower chunks, whose output it does not read
            rx_close(true);
            CK(cudaEventRecord(ev_join, side));
            CK(cudaStreamWaitEvent(stream, ev_join, 0));
            rx_pending = b ^ 1;
            rx_gate = gate;
            return;
        } else {
            launch_boundary<T>(bd, g, in.bz, tot[b].as<T>(), zc.n, in.bx, in.by, gate, stream);
            sweep(b, StepScalars<T>{}, table, gate);
        }
        launch_rx<T>(rd, out, tot[b ^ 1].as<T>(), zc, g, gate, RxAction{-1, 0, 0, -1, 0, 0}, stream);
    }

    cudaGraphExec_t graph_for(int b) {
        if (gexec[b]) return gexec[b];
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        rx_open();
        for (int s = 0; s < gsteps; s++) enqueue_step(b ^ (s & 1), StepGate{gate_base.as<int>(), s, sched.nsteps});
        rx_close();
        launch_advance(gate_base.as<int>(), gsteps, stream);
        cudaError_t e = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess) throw Error(TCSEM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiateWithFlags(&gexec[b], graph, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) throw Error(TCSEM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        return gexec[b];
    }

    void advance(long n, int *done) override {
        if (!begun) throw Error(TCSEM_ERR_STATE, "tcsem_begin must precede tcsem_advance");
        long todo = std::min(sched.nsteps - step, std::max(0L, n));
        // whole captured blocks (an even number of steps returns the state to `cur`)
        while (todo >= gsteps) {
            CK(cudaGraphLaunch(graph_for(cur), stream));
            step += gsteps;
            todo -= gsteps;
        }
        // remainder: the same kernels launched one by one, gated on the same counter
        if (todo > 0) {
            rx_open();
            for (long q = 0; q < todo; q++)
                enqueue_step(cur ^ (int)(q & 1), StepGate{gate_base.as<int>(), (int)q, sched.nsteps});
            rx_close();
            launch_advance(gate_base.as<int>(), (int)todo, stream);
            if (todo & 1) cur ^= 1;
            step += todo;
        }
        CK(cudaGetLastError());
        if (done) *done = step >= sched.nsteps;
    }

    void traces(double *out) override {
        CK(cudaStreamSynchronize(stream));
        check_device_error();
        std::vector<T> h(efs.n / sizeof(T));
        d2h(h.data(), efs.p, efs.n);
        bool finite = true;
        for (size_t q = 0; q < h.size(); q++) { out[q] = (double)h[q]; finite &= std::isfinite(out[q]); }
        if (!finite) throw Error(TCSEM_ERR_NUMERIC, "non-finite receiver samples");
    }

    // ---- batches: the descriptors of one step that reads field set b and writes b ^ 1
    void batch_slot(int b, const int *counter, SweepSlot<T> &sw, BoundarySlot<T> &bs, RxSlot<T> &rs) {
        FieldSet<T> in = fs(b), out = fs(b ^ 1);
        sw.maps = maps[b]; sw.g = g; sw.out = out; sw.tin = tot[b].as<T>(); sw.tout = tot[b ^ 1].as<T>();
        sw.ax = ax; sw.table = steps.as<StepScalars<T>>(); sw.step_base = counter; sw.nsteps = sched.nsteps;
        sw.src = src; sw.zc = zc; sw.err = errw.as<int>();
        sw.tiles_x = sweep_tiles_x(g.L); sw.tiles_y = sweep_tiles_y(g.M);
        bs.bd = bd; bs.g = g; bs.bz = in.bz; bs.tot = tot[b].as<T>(); bs.nch = zc.n; bs.bx = in.bx; bs.by = in.by;
        bs.step_base = counter; bs.nsteps = sched.nsteps;
        rs.rd = rd; rs.f = out; rs.tot = tot[b ^ 1].as<T>(); rs.zc = zc; rs.g = g;
        rs.step_base = counter; rs.nsteps = sched.nsteps;
    }
    int sweep_blocks() const { return sweep_tiles_x(g.L) * sweep_tiles_y(g.M) * zc.n; }
    int rx_stencils() const { return rd.NComp * rd.nr; }
    // an upper bound of the device memory init() allocates, from the host model alone
    static size_t estimate_bytes(const Model &m, long nsteps, int padded_plane) {
        const Geom gg = make_geom(m.L, m.M, m.N);
        const size_t vol = (size_t)gg.total() * sizeof(T), L1 = plane_len(m.L1, padded_plane),
                     M1 = plane_len(m.M1, padded_plane);
        const size_t H = L1 / 2 + 2;
        size_t b = 13 * vol + 2 * (size_t)kMaxChunks * gg.PS * sizeof(T);
        b += (H * (m.M + 2) + 2 * M1 * H + M1 * L1) * 2 * sizeof(T) + 2 * H * (M1 + 4) * sizeof(T);
        b += (size_t)nsteps * (sizeof(StepScalars<T>) + sizeof(StepEntryActs)) + ((size_t)4 << 20);
        return b;
    }

    // ---- per-stage seam
    void upcontinuation() override {
        FieldSet<T> f = fs(cur);
        launch_boundary<T>(bd, g, f.bz, tot[cur].as<T>(), zc.n, f.bx, f.by, StepGate{nullptr, 0, 0}, stream);
        CK(cudaGetLastError());
    }
    // the same pipeline with its four work arrays carved from caller-provided scratch
    void upcontinuation_in(void *scratch, size_t bytes) override {
        const size_t sz[4] = {FT.n, VX.n, VY.n, Zs.n};
        size_t off[4], need = 0;
        for (int k = 0; k < 4; k++) {
            off[k] = need;
            need += (sz[k] + 255) & ~(size_t)255;
        }
        if (need > bytes)
            throw Error(TCSEM_ERR_INVALID, "the continuation plane (" + std::to_string(model.L1) + " x " +
                                               std::to_string(model.M1) + ") needs " + std::to_string(need) +
                                               " bytes of scratch; the static scratch holds " +
                                               std::to_string(bytes));
        BoundaryDev<T> b2 = bd;
        unsigned char *p = static_cast<unsigned char *>(scratch);
        b2.FT = reinterpret_cast<C2<T> *>(p + off[0]);
        b2.VX = reinterpret_cast<C2<T> *>(p + off[1]);
        b2.VY = reinterpret_cast<C2<T> *>(p + off[2]);
        b2.Z = reinterpret_cast<C2<T> *>(p + off[3]);
        FieldSet<T> f = fs(cur);
        launch_boundary<T>(b2, g, f.bz, tot[cur].as<T>(), zc.n, f.bx, f.by, StepGate{nullptr, 0, 0}, stream);
        CK(cudaGetLastError());
    }
    StepScalars<T> scal(double lam, double dt, double dtb, double wave) {
        StepScalars<T> s;
        s.lam2 = (T)(2.0 * lam); s.dt = (T)dt; s.c4 = (T)(4.0 * dt / model.mu0); s.dtb = (T)dtb; s.wave = (T)wave;
        return s;
    }
    void need_tx() { if (itx < 0) select(0); }
    void electric_field(double lam, double dt, double wave) override {
        need_tx();
        consolidate(cur);
        launch_update_e<T>(g, fs(cur), con.as<T>(), ax, scal(lam, dt, 0, wave), src, errw.as<int>(), stream);
        CK(cudaGetLastError());
    }
    void bderivate(double dtb) override {
        consolidate(cur);
        launch_bderivate<T>(g, fs(cur), ax, (T)dtb, errw.as<int>(), stream);
        CK(cudaGetLastError());
    }
    void fused_step(double lam, double dt, double dtb, double wave) override {
        need_tx();
        // the sweep writes every updated cell of the other buffer; the air plane must follow the state
        T *dst_bx = fs(cur ^ 1).bx, *dst_by = fs(cur ^ 1).by;
        sweep(cur, scal(lam, dt, dtb, wave), nullptr, StepGate{nullptr, 0, 0});
        CK(cudaMemcpyAsync(dst_bx, fs(cur).bx, g.PS * sizeof(T), cudaMemcpyDeviceToDevice, stream));
        CK(cudaMemcpyAsync(dst_by, fs(cur).by, g.PS * sizeof(T), cudaMemcpyDeviceToDevice, stream));
        CK(cudaGetLastError());
        cur ^= 1;
    }
    void rx_sample(int efield, int slot, double *values) override {
        need_tx();
        if (slot < 0 || slot > 1) throw Error(TCSEM_ERR_INVALID, "slot must be 0 or 1");
        RxAction a{-1, 0, 0, -1, 0, 0};
        if (efield) a.e_slot = slot; else a.b_slot = slot;
        launch_rx<T>(rd, fs(cur), tot[cur].as<T>(), zc, g, StepGate{nullptr, 0, 0}, a, stream);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(stream));
        size_t n = (size_t)model.NComp * rd.nr;
        std::vector<T> h(n);
        d2h(h.data(), ef0.as<T>() + (size_t)slot * n, n * sizeof(T));
        for (size_t q = 0; q < n; q++) values[q] = (double)h[q];
    }

    // ---- field access in the reference layout
    DevMem &field_mem(int comp, int b) {
        if (comp == TCSEM_CON) return con;
        if (comp == TCSEM_BXAIR) return fld[b][3];
        if (comp == TCSEM_BYAIR) return fld[b][4];
        return fld[b][comp];
    }
    void get_field(int comp, double *h) override {
        int nx, ny, nz, z0;
        extents(comp, nx, ny, nz, z0);
        if (comp == TCSEM_BZ) consolidate(cur);
        CK(cudaStreamSynchronize(stream));
        DevMem &dm = field_mem(comp, cur);
        std::vector<T> buf((size_t)g.total());
        d2h(buf.data(), dm.p, buf.size() * sizeof(T));
        size_t q = 0;
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) h[q++] = (double)buf[g.at(i, j, k + z0)];
    }
    void set_field(int comp, const double *h) override {
        int nx, ny, nz, z0;
        extents(comp, nx, ny, nz, z0);
        CK(cudaStreamSynchronize(stream));
        DevMem &dm = field_mem(comp, cur);
        std::vector<T> buf((size_t)g.total());
        d2h(buf.data(), dm.p, buf.size() * sizeof(T));
        size_t q = 0;
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) buf[g.at(i, j, k + z0)] = (T)h[q++];
        h2d(dm.p, buf.data(), buf.size() * sizeof(T));
        if (comp != TCSEM_CON) {  // keep the other buffer consistent for the fused sweep's untouched cells
            DevMem &other = field_mem(comp, cur ^ 1);
            h2d(other.p, buf.data(), buf.size() * sizeof(T));
        }
        if (comp == TCSEM_BZ)  // a plain Bz plane: no chunk offsets
            for (int b = 0; b < 2; b++) dzero(tot[b].p, tot[b].n);
    }

    // ---- checkpoint of a run in progress: what one step hands the next (the field set the
    // next step reads, its Bz chunk totals, the receiver slots and traces so far, the step)
    // version 2 adds what changes the physics of the continuing run: the continuation plane
    // (L1 x M1 and the padded-plane mode), the dual-bipole option and the schedule's length
    struct StateHeader {
        char magic[8];
        int version, tsize, L, M, N, itx, cur, nch;
        int kb[kMaxChunks + 1];
        long long step, field_bytes, tot_bytes, ef0_bytes, efs_bytes;
        int L1, M1, padded_plane, fix_dual_bipole;
        long long nsteps;
    };
    void save_state(const char *path) override {
        if (!begun) throw Error(TCSEM_ERR_STATE, "tcsem_begin must precede tcsem_save_state");
        CK(cudaStreamSynchronize(stream));
        check_device_error();
        StateHeader h{};
        std::memcpy(h.magic, "TCSEMST", 8);
        h.version = 2; h.tsize = (int)sizeof(T); h.L = model.L; h.M = model.M; h.N = model.N;
        h.L1 = model.L1; h.M1 = model.M1; h.padded_plane = opts.padded_plane;
        h.fix_dual_bipole = opts.fix_dual_bipole != 0; h.nsteps = sched.nsteps;
        h.itx = itx; h.cur = cur; h.nch = zc.n;
        for (int c = 0; c <= kMaxChunks; c++) h.kb[c] = zc.kb[c];
        h.step = step;
        h.field_bytes = (long long)fld[cur][0].n;
        h.tot_bytes = (long long)zc.n * g.PS * (long long)sizeof(T);
        h.ef0_bytes = (long long)ef0.n;
        h.efs_bytes = (long long)efs.n;
        std::FILE *f = std::fopen(path, "wb");
        if (!f) throw Error(TCSEM_ERR_IO, std::string("cannot write ") + path);
        std::vector<unsigned char> buf;
        bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
        auto put = [&](const void *dev, size_t n) {
            buf.resize(n);
            d2h(buf.data(), dev, n);
            ok = ok && std::fwrite(buf.data(), 1, n, f) == n;
        };
        try {
            for (int c = 0; c < 6; c++) put(fld[cur][c].p, (size_t)h.field_bytes);
            put(tot[cur].p, (size_t)h.tot_bytes);
            put(ef0.p, (size_t)h.ef0_bytes);
            put(efs.p, (size_t)h.efs_bytes);
        } catch (...) {
            std::fclose(f);
            throw;
        }
        ok = (std::fclose(f) == 0) && ok;
        if (!ok) throw Error(TCSEM_ERR_IO, std::string("cannot write ") + path);
    }
    // into a handle of the same survey, precision and z-chunk layout; the run continues with advance
    void load_state(const char *path) override {
        std::FILE *f = std::fopen(path, "rb");
        if (!f) throw Error(TCSEM_ERR_IO, std::string("cannot open ") + path);
        StateHeader h{};
        std::vector<unsigned char> buf;
        bool ok = std::fread(&h, sizeof h, 1, f) == 1;
        auto fail = [&](tcsem_status st, const std::string &m) {
            std::fclose(f);
            throw Error(st, m);
        };
        if (!ok || std::memcmp(h.magic, "TCSEMST", 8) != 0 || h.version != 2) fail(TCSEM_ERR_PARSE, std::string(path) + " is not a saved run state");
        bool same = h.tsize == (int)sizeof(T) && h.L == model.L && h.M == model.M && h.N == model.N && h.nch == zc.n &&
                    h.field_bytes == (long long)fld[0][0].n && h.tot_bytes == (long long)zc.n * g.PS * (long long)sizeof(T) &&
                    (h.cur == 0 || h.cur == 1) && h.step >= 0 && h.step <= sched.nsteps && h.itx >= 0 &&
                    h.itx < (int)model.in.tx.size() && h.L1 == model.L1 && h.M1 == model.M1 &&
                    h.padded_plane == opts.padded_plane && h.fix_dual_bipole == (opts.fix_dual_bipole != 0) &&
                    h.nsteps == sched.nsteps;
        for (int c = 0; c <= zc.n && same; c++) same = h.kb[c] == zc.kb[c];
        const std::string other = std::string(path) + " was saved by a different survey, precision, z-chunk layout, "
                                                      "continuation plane or dual-bipole option";
        if (!same) fail(TCSEM_ERR_INVALID, other);
        try {
            begin(h.itx);  // the transmitter's tables (receiver buffers) and a zero state, then the saved arrays
            // the zeroing runs on the handle's (non-blocking) stream: let it finish before the copies
            CK(cudaStreamSynchronize(stream));
        } catch (...) {
            std::fclose(f);
            throw;
        }
        if (h.ef0_bytes != (long long)ef0.n || h.efs_bytes != (long long)efs.n) fail(TCSEM_ERR_INVALID, other);
        auto get = [&](void *dev, size_t n) {
            buf.resize(n);
            ok = ok && std::fread(buf.data(), 1, n, f) == n;
            if (ok) h2d(dev, buf.data(), n);
        };
        try {
            for (int c = 0; c < 6; c++) get(fld[h.cur][c].p, (size_t)h.field_bytes);
            get(tot[h.cur].p, (size_t)h.tot_bytes);
            get(ef0.p, (size_t)h.ef0_bytes);
            get(efs.p, (size_t)h.efs_bytes);
        } catch (...) {
            std::fclose(f);
            throw;
        }
        std::fclose(f);
        if (!ok) {
            zero_state();
            throw Error(TCSEM_ERR_IO, std::string(path) + " is truncated");
        }
        const int s = (int)h.step;
        h2d(gate_base.p, &s, sizeof(int));
        cur = h.cur;
        step = h.step;
    }

    void timed_advance(long n, double *ms_out) override {
        if (!begun) throw Error(TCSEM_ERR_STATE, "tcsem_begin must precede tcsem_timed_advance");
        graph_for(cur);  // capture (once) outside the timed region
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        CK(cudaStreamSynchronize(stream));
        CK(cudaEventRecord(e0, stream));
        advance(n, nullptr);
        CK(cudaEventRecord(e1, stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (ms_out) *ms_out = ms;
    }

    void time_steps(int t, long n, double *ms_tot, double *ms_sweep, double *bnd) override {
        begin(t);
        n = std::min(n, sched.nsteps);
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        graph_for(cur);  // capture outside the timed region
        graph_for(cur ^ 1);
        CK(cudaStreamSynchronize(stream));
        CK(cudaEventRecord(e0, stream));
        advance(n, nullptr);
        CK(cudaEventRecord(e1, stream));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms_tot) *ms_tot = ms;
        const int reps = 20;
        if (ms_sweep) {
            StepScalars<T> s = scal(sched.lam[0], sched.dt1[0], sched.dtB[0], 0.0);
            CK(cudaEventRecord(e0, stream));
            for (int r = 0; r < reps; r++)
                sweep(r & 1, s, nullptr, StepGate{nullptr, 0, 0});
            CK(cudaEventRecord(e1, stream));
            CK(cudaEventSynchronize(e1));
            CK(cudaEventElapsedTime(&ms, e0, e1));
            *ms_sweep = ms / reps;
        }
        if (bnd) {
            CK(cudaEventRecord(e0, stream));
            for (int r = 0; r < reps; r++) {
                FieldSet<T> f = fs(r & 1);
                launch_boundary<T>(bd, g, f.bz, tot[r & 1].as<T>(), zc.n, f.bx, f.by, StepGate{nullptr, 0, 0}, stream);
            }
            CK(cudaEventRecord(e1, stream));
            CK(cudaEventSynchronize(e1));
            CK(cudaEventElapsedTime(&ms, e0, e1));
            *bnd = ms / reps;
        }
        CK(cudaGetLastError());
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        begun = false;
    }
};

}  // namespace tcsem
