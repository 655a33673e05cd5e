// C ABI of include/tcsem.h for single surveys (the batch entry points are in
// batch.cu); the simulation state itself is in sim_impl.cuh.
#include <mutex>

#include <nvtx3/nvToolsExt.h>

#include "async.cuh"
#include "sim_impl.cuh"

namespace tcsem {
// NVTX range over one entry point (visible in Nsight tools, free without one attached)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

// One CTA waits on an mbarrier that nothing completes: every thread gives up after `polls`
// polls and the CTA records it in the error word, as the production kernels do when a
// bulk copy does not arrive.
__global__ void k_wait_selftest(int *err, int polls) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0u, polls);
    __syncthreads();
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
}
}  // namespace tcsem

// ================================================================== C ABI
using namespace tcsem;

struct tcsem_sim {
    std::unique_ptr<SimBase> impl;
};

static thread_local std::string g_open_err;

template <class F> static tcsem_status guard(tcsem_sim_t *s, F &&f) {
    if (!s || !s->impl) return TCSEM_ERR_INVALID;
    try {
        CK(cudaSetDevice(s->impl->device));
        f(*s->impl);
        return TCSEM_OK;
    } catch (const Error &e) {
        s->impl->err = e.what();
        return (tcsem_status)e.code;
    } catch (const std::bad_alloc &) {
        s->impl->err = "host allocation failed";
        return TCSEM_ERR_NOMEM;
    } catch (const std::exception &e) {
        s->impl->err = e.what();
        return TCSEM_ERR_INVALID;
    }
}

// the survey of `read` (files or host records) set up on the device
template <class F> static tcsem_status open_impl(F &&read, const tcsem_opts *opts, tcsem_sim_t **out) {
    *out = nullptr;
    tcsem_opts o;
    tcsem_default_opts(&o);
    if (opts) o = *opts;
    if (o.precision == 0) o.precision = TCSEM_FP32;
    if (o.precision != TCSEM_FP32 && o.precision != TCSEM_FP64) { g_open_err = "precision must be 32 or 64"; return TCSEM_ERR_INVALID; }
    try {
        std::unique_ptr<SimBase> impl;
        if (o.precision == TCSEM_FP64) impl.reset(new SimImpl<double>());
        else impl.reset(new SimImpl<float>());
        impl->opts = o;
        impl->device = o.device;
        impl->model.build(read());
        impl->sched = impl->model.schedule();
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= o.device || o.device < 0)
            throw Error(TCSEM_ERR_CUDA, "no usable CUDA device");
        impl->init();
        tcsem_sim_t *s = new tcsem_sim;
        s->impl = std::move(impl);
        *out = s;
        return TCSEM_OK;
    } catch (const Error &e) {
        g_open_err = e.what();
        return (tcsem_status)e.code;
    } catch (const std::bad_alloc &) {
        g_open_err = "host allocation failed";
        return TCSEM_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_open_err = e.what();
        return TCSEM_ERR_INVALID;
    }
}

extern "C" {

void tcsem_default_opts(tcsem_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->precision = TCSEM_FP32;
}

tcsem_status tcsem_open_dir(const char *dir, const tcsem_opts *opts, tcsem_sim_t **out) {
    NvtxRange nr("tcsem_open_dir");
    if (!dir || !out) { g_open_err = "null argument"; return TCSEM_ERR_INVALID; }
    return open_impl([&] { return read_survey_dir(dir); }, opts, out);
}

tcsem_status tcsem_open(const tcsem_model *model, const tcsem_survey *survey, const tcsem_opts *opts,
                        tcsem_sim_t **out) {
    NvtxRange nr("tcsem_open");
    if (!model || !survey || !out) { g_open_err = "null argument"; return TCSEM_ERR_INVALID; }
    return open_impl([&] { return survey_from_host(model, survey); }, opts, out);
}

const char *tcsem_open_error(void) { return g_open_err.c_str(); }

tcsem_status tcsem_close(tcsem_sim_t *s) {
    if (!s) return TCSEM_ERR_INVALID;
    if (s->impl) cudaSetDevice(s->impl->device);
    delete s;
    return TCSEM_OK;
}

const char *tcsem_last_error(const tcsem_sim_t *s) { return s && s->impl ? s->impl->err.c_str() : "invalid handle"; }

tcsem_status tcsem_get_info(const tcsem_sim_t *s, tcsem_info *o) {
    if (!s || !s->impl || !o) return TCSEM_ERR_INVALID;
    const SimBase &b = *s->impl;
    const Model &m = b.model;
    o->L = m.L; o->M = m.M; o->N = m.N; o->L1 = m.L1; o->M1 = m.M1;
    o->NRx = (int)m.in.rx.size(); o->NTx = (int)m.in.tx.size(); o->Nt = m.in.Nt; o->NComp = m.NComp; o->nefcmp = m.nefcmp;
    o->nsteps = b.sched.nsteps;
    o->precision = b.opts.precision;
    o->device_bytes = b.dev_bytes;
    o->launches_per_step = b.launches_per_step;
    o->zchunks = b.chunks_used;
    o->top_planes = b.top_used;
    o->uploaded_bytes = b.uploaded_bytes;
    return TCSEM_OK;
}

tcsem_status tcsem_begin(tcsem_sim_t *s, int itx) { return guard(s, [&](SimBase &b) { b.begin(itx); }); }
tcsem_status tcsem_advance(tcsem_sim_t *s, long n, int *done) {
    NvtxRange nr("tcsem_advance");
    return guard(s, [&](SimBase &b) { b.advance(n, done); });
}
tcsem_status tcsem_get_traces(tcsem_sim_t *s, double *t) {
    return guard(s, [&](SimBase &b) {
        if (!t) throw Error(TCSEM_ERR_INVALID, "null trace buffer");
        if (b.itx < 0) throw Error(TCSEM_ERR_STATE, "no transmitter selected");
        b.traces(t);
    });
}
tcsem_status tcsem_save_state(tcsem_sim_t *s, const char *path) {
    return guard(s, [&](SimBase &b) {
        if (!path) throw Error(TCSEM_ERR_INVALID, "null path");
        b.save_state(path);
    });
}
tcsem_status tcsem_load_state(tcsem_sim_t *s, const char *path) {
    return guard(s, [&](SimBase &b) {
        if (!path) throw Error(TCSEM_ERR_INVALID, "null path");
        b.load_state(path);
    });
}
tcsem_status tcsem_synchronize(tcsem_sim_t *s) {
    return guard(s, [&](SimBase &b) {
        CK(cudaStreamSynchronize(b.stream));
        b.check_error();
    });
}
tcsem_status tcsem_run(tcsem_sim_t *s, int itx, double *t) {
    NvtxRange nr("tcsem_run");
    return guard(s, [&](SimBase &b) {
        if (!t) throw Error(TCSEM_ERR_INVALID, "null trace buffer");
        b.begin(itx);
        int done = 0;
        b.advance(b.sched.nsteps, &done);
        b.traces(t);
    });
}

tcsem_status tcsem_selftest_bounded_wait(int device, int polls, int *gave_up) {
    if (!gave_up || polls < 1) return TCSEM_ERR_INVALID;
    *gave_up = 0;
    int *err = nullptr;
    if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(&err, sizeof(int)) != cudaSuccess) return TCSEM_ERR_CUDA;
    tcsem_status st = TCSEM_OK;
    int h = 0;
    if (cudaMemset(err, 0, sizeof(int)) != cudaSuccess) st = TCSEM_ERR_CUDA;
    if (st == TCSEM_OK) {
        k_wait_selftest<<<1, 64>>>(err, polls);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            st = TCSEM_ERR_CUDA;
    }
    cudaFree(err);
    *gave_up = h;
    return st;
}

tcsem_status tcsem_write_bout(tcsem_sim_t *s, int itx, const double *t, const char *path) {
    return guard(s, [&](SimBase &b) {
        if (!t || !path) throw Error(TCSEM_ERR_INVALID, "null argument");
        write_bout_file(b.model, itx, t, path);
    });
}

tcsem_status tcsem_select_tx(tcsem_sim_t *s, int itx) { return guard(s, [&](SimBase &b) { b.select(itx); }); }
tcsem_status tcsem_upcontinuation(tcsem_sim_t *s) { return guard(s, [&](SimBase &b) { b.upcontinuation(); }); }

// Scratch of tcsem_upcontinuation_noalloc: static device memory of the
// library's module, one instance per device; its address is looked up once per
// device with that device current.
static __device__ __align__(256) unsigned char g_noalloc_scratch[TCSEM_NOALLOC_SCRATCH_BYTES];

static void *noalloc_scratch(int device) {
    constexpr int kMaxDevices = 64;
    static std::mutex mu;
    static void *addr[kMaxDevices] = {};
    if (device < 0 || device >= kMaxDevices) throw Error(TCSEM_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) throw Error(TCSEM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        addr[device] = p;
    }
    return addr[device];
}

tcsem_status tcsem_upcontinuation_noalloc(tcsem_sim_t *s) {
    return guard(s, [&](SimBase &b) { b.upcontinuation_in(noalloc_scratch(b.device), TCSEM_NOALLOC_SCRATCH_BYTES); });
}
tcsem_status tcsem_electric_field(tcsem_sim_t *s, double lam, double dt, double wave) {
    return guard(s, [&](SimBase &b) { b.electric_field(lam, dt, wave); });
}
tcsem_status tcsem_bderivate(tcsem_sim_t *s, double dt) { return guard(s, [&](SimBase &b) { b.bderivate(dt); }); }
tcsem_status tcsem_fused_step(tcsem_sim_t *s, double lam, double dt, double dtb, double wave) {
    return guard(s, [&](SimBase &b) { b.fused_step(lam, dt, dtb, wave); });
}
tcsem_status tcsem_rx_sample(tcsem_sim_t *s, int efield, int slot, double *v) {
    return guard(s, [&](SimBase &b) {
        if (!v) throw Error(TCSEM_ERR_INVALID, "null output");
        b.rx_sample(efield, slot, v);
    });
}
tcsem_status tcsem_get_field(tcsem_sim_t *s, int comp, double *h) {
    return guard(s, [&](SimBase &b) {
        if (!h) throw Error(TCSEM_ERR_INVALID, "null output");
        b.get_field(comp, h);
    });
}
tcsem_status tcsem_set_field(tcsem_sim_t *s, int comp, const double *h) {
    return guard(s, [&](SimBase &b) {
        if (!h) throw Error(TCSEM_ERR_INVALID, "null input");
        b.set_field(comp, h);
    });
}
tcsem_status tcsem_field_size(const tcsem_sim_t *s, int comp, size_t *n) {
    if (!s || !s->impl || !n) return TCSEM_ERR_INVALID;
    try {
        *n = s->impl->field_count(comp);
    } catch (const Error &e) {
        return (tcsem_status)e.code;
    }
    return TCSEM_OK;
}
tcsem_status tcsem_get_schedule(const tcsem_sim_t *s, double *dt1, double *dt2, double *lam, double *wave, long cap) {
    if (!s || !s->impl) return TCSEM_ERR_INVALID;
    const Schedule &S = s->impl->sched;
    long n = std::min(cap, S.nsteps);
    for (long q = 0; q < n; q++) {
        if (dt1) dt1[q] = S.dt1[q];
        if (dt2) dt2[q] = S.dt2[q];
        if (lam) lam[q] = S.lam[q];
        if (wave) wave[q] = S.wave[q];
    }
    return TCSEM_OK;
}
tcsem_status tcsem_get_waveform(const tcsem_sim_t *s, int *nsrc, double *t, double *dt, double *wave) {
    if (!s || !s->impl) return TCSEM_ERR_INVALID;
    const Model &m = s->impl->model;
    if (nsrc) *nsrc = m.nsrc;
    size_t n = 2 * (size_t)m.nsrc + 1;
    if (t) std::memcpy(t, m.tw.data(), n * sizeof(double));
    if (dt) std::memcpy(dt, m.dtw.data(), n * sizeof(double));
    if (wave) std::memcpy(wave, m.wave.data(), n * sizeof(double));
    return TCSEM_OK;
}
tcsem_status tcsem_timed_advance(tcsem_sim_t *s, long n, double *ms) {
    return guard(s, [&](SimBase &b) { b.timed_advance(n, ms); });
}
tcsem_status tcsem_time_steps(tcsem_sim_t *s, int itx, long n, double *tot, double *sw, double *bn) {
    return guard(s, [&](SimBase &b) { b.time_steps(itx, n, tot, sw, bn); });
}

}  // extern "C"
