// Batches: many surveys (slots) of different sizes advanced together, one
// launch per kernel per time step for all of them.
//
// Each slot is a full single-survey state (sim_impl.cuh: its own field sets,
// boundary plan, step table, receivers and step counter); the batch keeps, per
// step parity, a device table of the slots' kernel arguments and a list of the
// blocks each slot owns in every batched launch (BatchIndex).  One captured
// CUDA graph runs `graph_steps` steps of every slot.  A step forks like the
// single-survey step: on a high-priority side stream the four boundary
// kernels and then the sweep of every slot's top z-chunk (the only chunk that
// reads the air plane), on the main stream the sweep of all lower chunks;
// both join before the receiver kernel.  Each of these is one launch over all
// slots.  One advance of all step counters ends the block.  A slot whose
// run has ended is gated off inside the kernels; slots join (tcsem_batch_add)
// and leave (tcsem_batch_remove) between graph launches, which rebuilds the
// tables and re-captures the graph.  Admission is by device memory: a slot is
// accepted when the estimate of its allocation fits in the batch's budget.
#include <nvtx3/nvToolsExt.h>

#include "persist.cuh"
#include "sim_impl.cuh"

namespace tcsem {

struct BatchBase {
    tcsem_opts opts{};
    int device = 0;
    size_t budget = 0;  // 0: no limit
    std::string err;
    virtual ~BatchBase() {}
    virtual void init() = 0;
    virtual int add(const char *dir, int itx) = 0;
    virtual void advance(long nsteps) = 0;
    virtual int poll(int *ids, int cap) = 0;
    virtual void slot_info(int id, tcsem_info *info, long *steps_done) = 0;
    virtual void traces(int id, double *out) = 0;
    virtual void write_bout(int id, const char *path) = 0;
    virtual void remove(int id) = 0;
    virtual void stats(int *slots, int *running, size_t *bytes) = 0;
};

template <typename T> struct BatchImpl : BatchBase {
    struct Slot {
        int id = 0;
        std::unique_ptr<SimImpl<T>> sim;
        long done = 0;  // steps enqueued for this slot (capped at its run length)
        size_t bytes = 0;
        bool finished() const { return done >= sim->sched.nsteps; }
    };
    std::vector<Slot> slots;
    std::vector<int> running;  // positions in `slots` of the slots in the current graph, in table order
    int next_id = 1;
    size_t used = 0;
    cudaStream_t stream = nullptr;
    DevMem counters, dsw[2], dbs[2], drs[2];
    BatchIndex itop{}, ilow{}, irs{}, ibs[4]{};  // sweep: chunk 0 of every slot, chunks 1.. of every slot
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    size_t smem_bnd[3] = {0, 0, 0};
    int nmax = 0;
    int lps = 6;  // launches per step for all slots (a seventh when some slot has lower z-chunks)
    cudaGraphExec_t gexec = nullptr;
    int gsteps = 64;
    bool dirty = true;
    // layout autotuner (opts.zchunks = -1): at the first advance every slot's z-chunk layout
    // is timed for a few candidates on one graph block and the fastest is kept, also for
    // slots added later
    static constexpr int kTuneChunks = 3;
    bool tune_pending = false;
    int lay_n = 1, lay_top = 0;
    // persistent schedule (opts.persistent_batch): one launch per block, items from a device queue
    bool persistent = false;
    DevMem pq, pctl, perr;
    PersistArgs<T> pa{};
    int pgrid = 0;
    size_t psmem = 0;
    static constexpr long long kQueueWaitNs = 2000000000LL;  // a CTA waits at most 2 s for a ready stage

    ~BatchImpl() override {
        if (stream) cudaStreamSynchronize(stream);
        if (gexec) cudaGraphExecDestroy(gexec);
        slots.clear();
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }

    void init() override {
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        int lo = 0, hi = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        CK(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi));
        CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        counters.alloc(kMaxSlots * sizeof(int));
        CK(cudaMemsetAsync(counters.p, 0, counters.n, stream));
        CK(cudaStreamSynchronize(stream));
        for (int p = 0; p < 2; p++) {
            dsw[p].alloc(kMaxSlots * sizeof(SweepSlot<T>));
            dbs[p].alloc(kMaxSlots * sizeof(BoundarySlot<T>));
            drs[p].alloc(kMaxSlots * sizeof(RxSlot<T>));
        }
        gsteps = opts.graph_steps > 0 ? opts.graph_steps : 64;
        if (gsteps % 2) gsteps++;
        tune_pending = opts.zchunks < 0;
        persistent = opts.persistent_batch != 0;
        if (persistent) {  // queue capacity: every stage of every slot for a block (the tuner's blocks are 8 steps)
            pq.alloc((size_t)kMaxSlots * kStages * std::max(gsteps, 8) * sizeof(QueueEntry));
            pctl.alloc(kQWords * sizeof(int));
            perr.alloc(sizeof(int));
            CK(cudaMemsetAsync(perr.p, 0, sizeof(int), stream));
            CK(cudaStreamSynchronize(stream));
        }
    }

    Slot &find(int id) {
        for (auto &s : slots)
            if (s.id == id) return s;
        throw Error(TCSEM_ERR_INVALID, "no slot " + std::to_string(id) + " in the batch");
    }

    int add(const char *dir, int itx) override {
        if ((int)slots.size() >= kMaxSlots) throw Error(TCSEM_ERR_NOMEM, "the batch holds 64 slots");
        auto sim = std::make_unique<SimImpl<T>>();
        sim->opts = opts;
        // the slots fill the GPU together: one z-chunk each unless set (no halo planes; the
        // boundary kernels of all slots run as wide launches before the sweep) or tuned
        const bool tuned = opts.zchunks < 0;
        if (sim->opts.zchunks <= 0) sim->opts.zchunks = 1;
        if (tuned) sim->tot_chunks_min = kTuneChunks;
        sim->device = device;
        sim->model.build(read_survey_dir(dir));
        sim->sched = sim->model.schedule();
        const size_t est = SimImpl<T>::estimate_bytes(sim->model, sim->sched.nsteps, sim->opts.padded_plane);
        if (budget && used + est > budget)
            throw Error(TCSEM_ERR_NOMEM, "device budget: the survey needs about " + std::to_string(est) +
                                             " bytes, " + std::to_string(budget - std::min(budget, used)) + " are free");
        sim->init();
        if (tuned && !tune_pending) sim->set_chunks(std::min(lay_n, sim->max_chunks()), lay_top);
        sim->begin(itx);
        CK(cudaStreamSynchronize(sim->stream));
        Slot s;
        s.id = next_id++;
        s.bytes = sim->dev_bytes;
        s.sim = std::move(sim);
        used += s.bytes;
        slots.push_back(std::move(s));
        dirty = true;
        return slots.back().id;
    }

    // tables, block lists and graph for the slots still running
    void rebuild() {
        CK(cudaStreamSynchronize(stream));  // the tables are read by launches in flight
        if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
        running.clear();
        for (int q = 0; q < (int)slots.size(); q++)
            if (!slots[q].finished()) running.push_back(q);
        // the slots whose CTAs march the most planes first (longest processing time first: the
        // sweep's last wave is then made of short CTAs; 16 generated surveys 698 -> 672 us/step)
        auto depth = [&](int q) {
            const ZChunks &z = slots[q].sim->zc;
            int d = 0;
            for (int c = 0; c < z.n; c++) d = std::max(d, z.kb[c + 1] - z.kb[c]);
            return d;
        };
        std::stable_sort(running.begin(), running.end(), [&](int a, int b) { return depth(a) > depth(b); });
        const int n = (int)running.size();
        std::vector<SweepSlot<T>> hsw[2];
        std::vector<BoundarySlot<T>> hbs[2];
        std::vector<RxSlot<T>> hrs[2];
        std::vector<int> hc(kMaxSlots, 0);
        itop = BatchIndex{}; ilow = BatchIndex{}; irs = BatchIndex{};
        for (auto &b : ibs) b = BatchIndex{};
        itop.n = ilow.n = irs.n = n;
        for (auto &b : ibs) b.n = n;
        smem_bnd[0] = smem_bnd[1] = smem_bnd[2] = 0;
        nmax = 0;
        int *cnt = counters.as<int>();
        pa = PersistArgs<T>{};
        for (int r = 0; r < n; r++) {
            Slot &s = slots[running[r]];
            SimImpl<T> &m = *s.sim;
            for (int p = 0; p < 2; p++) {
                hsw[p].emplace_back(); hbs[p].emplace_back(); hrs[p].emplace_back();
                m.batch_slot(p, cnt + r, hsw[p].back(), hbs[p].back(), hrs[p].back());
            }
            hc[r] = (int)s.done;
            const BoundaryBlocks bb = boundary_blocks(m.bd, m.g);
            const int per_chunk = m.sweep_blocks() / m.zc.n;
            itop.off[r + 1] = itop.off[r] + per_chunk;
            ilow.off[r + 1] = ilow.off[r] + per_chunk * (m.zc.n - 1);
            ibs[0].off[r + 1] = ibs[0].off[r] + bb.rows_fwd;
            ibs[1].off[r + 1] = ibs[1].off[r] + bb.cols;
            ibs[2].off[r + 1] = ibs[2].off[r] + bb.rows_inv;
            ibs[3].off[r + 1] = ibs[3].off[r] + bb.bilinear;
            irs.off[r + 1] = irs.off[r] + rx_blocks(m.rx_stencils());
            const int it[kStages] = {bb.rows_fwd, bb.cols, bb.rows_inv, (m.g.L + 1) * m.g.M + m.g.L * (m.g.M + 1),
                                     m.sweep_blocks(), m.rx_stencils()};
            for (int q = 0; q < kStages; q++) pa.nitems[r][q] = it[q];
            smem_bnd[0] = std::max(smem_bnd[0], bb.smem_rows);
            smem_bnd[1] = std::max(smem_bnd[1], bb.smem_cols);
            smem_bnd[2] = std::max(smem_bnd[2], bb.smem_inv);
            nmax = std::max(nmax, m.g.N);
        }
        // on the batch's (non-blocking) stream, finished before the next launch reads the tables
        for (int p = 0; p < 2 && n; p++) {
            CK(cudaMemcpyAsync(dsw[p].p, hsw[p].data(), n * sizeof(SweepSlot<T>), cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(dbs[p].p, hbs[p].data(), n * sizeof(BoundarySlot<T>), cudaMemcpyHostToDevice, stream));
            CK(cudaMemcpyAsync(drs[p].p, hrs[p].data(), n * sizeof(RxSlot<T>), cudaMemcpyHostToDevice, stream));
        }
        CK(cudaMemcpyAsync(counters.p, hc.data(), kMaxSlots * sizeof(int), cudaMemcpyHostToDevice, stream));
        CK(cudaStreamSynchronize(stream));
        dirty = false;
        lps = 6 + (ilow.total() > 0 ? 1 : 0);
        if (!n) return;
        CK(sweep_configure<T>(nmax));
        CK(boundary_configure_batched<T>(smem_bnd));
        int maxsm = 0;
        CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
        if (std::max({smem_bnd[0], smem_bnd[1], smem_bnd[2], sweep_smem_bytes<T>(nmax)}) > (size_t)maxsm)
            throw Error(TCSEM_ERR_INVALID, "a slot needs more shared memory than a block can have");
        if (persistent) {  // no graph: the tables above and one launch per block
            for (int p = 0; p < 2; p++) {
                pa.sw[p] = dsw[p].as<SweepSlot<T>>();
                pa.bs[p] = dbs[p].as<BoundarySlot<T>>();
                pa.rs[p] = drs[p].as<RxSlot<T>>();
            }
            pa.q = pq.as<QueueEntry>();
            pa.ctl = pctl.as<int>();
            pa.err = perr.as<int>();
            pa.nslots = n;
            pa.wait_ns = kQueueWaitNs;
            const size_t body = rnd16(std::max({smem_bnd[0], smem_bnd[1], smem_bnd[2], sweep_smem_bytes<T>(nmax)}));
            pa.ctl_off = (int)body;
            psmem = body + 32;  // the CTA's scheduling words after every body's layout
            if (psmem > (size_t)maxsm)
                throw Error(TCSEM_ERR_INVALID, "a slot needs more shared memory than a block can have");
            CK(persist_configure<T>(psmem));
            pgrid = persist_blocks<T>(psmem);
            if (pgrid <= 0) throw Error(TCSEM_ERR_CUDA, "the persistent batch kernel does not fit on the device");
            // Claims of the boundary stages: about as many per stage as the CTAs each slot has on
            // average (at least 8), so that a claim carries several rows or columns when many slots
            // share the GPU; tiles and receiver blocks are claimed one at a time.
            const int pt = persist_threads(), target = std::max(8, pgrid / n);
            for (int r = 0; r < n; r++) {
                for (int q = 0; q < kStages; q++) {
                    const int ni = pa.nitems[r][q];
                    int per = 1, units = ni;
                    if (q < 3) per = (ni + target - 1) / target, units = per ? (ni + per - 1) / per : 0;
                    if (q == 3) units = std::min((ni + pt - 1) / pt, target);  // output points split evenly
                    if (q == 5) units = (ni + pt - 1) / pt;
                    pa.per[r][q] = per;
                    pa.units[r][q] = units;
                }
            }
            return;
        }
        // steps alternate the field sets: every slot starts a block in set 0 (blocks have an even length)
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        for (int s = 0; s < gsteps; s++) {
            const int p = s & 1;
            CK(cudaEventRecord(ev_fork, stream));
            CK(cudaStreamWaitEvent(side, ev_fork, 0));
            launch_boundary_batched<T>(dbs[p].as<BoundarySlot<T>>(), ibs, smem_bnd, s, side);
            launch_sweep_batched<T>(dsw[p].as<SweepSlot<T>>(), itop, s, 0, nmax, side);
            launch_sweep_batched<T>(dsw[p].as<SweepSlot<T>>(), ilow, s, 1, nmax, stream);
            CK(cudaEventRecord(ev_join, side));
            CK(cudaStreamWaitEvent(stream, ev_join, 0));
            launch_rx_batched<T>(drs[p].as<RxSlot<T>>(), irs, s, stream);
        }
        launch_advance_all(counters.as<int>(), n, gsteps, stream);
        cudaError_t e = cudaStreamEndCapture(stream, &graph);
        if (e != cudaSuccess) throw Error(TCSEM_ERR_CUDA, std::string("batch graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiateWithFlags(&gexec, graph, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) throw Error(TCSEM_ERR_CUDA, std::string("batch graph instantiate: ") + cudaGetErrorString(e));
    }

    // time one graph block of 8 steps per candidate layout on the slots as admitted, then put
    // every slot back to its zero state at step 0 with the fastest layout
    void tune() {
        struct Cand { int n, top; };
        const Cand cands[] = {{1, 0}, {2, 0}, {2, 1}, {3, 0}, {3, 1}};
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        float best = 1e30f;
        Cand pick = cands[0];
        auto layout = [&](const Cand &c) {
            CK(cudaStreamSynchronize(stream));
            for (auto &s : slots) {
                s.sim->set_chunks(std::min(c.n, s.sim->max_chunks()), c.top);
                s.sim->zero_state();  // the slot's transmitter stays selected
                CK(cudaStreamSynchronize(s.sim->stream));
                s.done = 0;
            }
            dirty = true;
        };
        const int keep = gsteps;
        gsteps = 8;
        for (const Cand &c : cands) {
            layout(c);
            rebuild();
            if (running.empty()) break;
            launch_block();  // untimed
            CK(cudaEventRecord(e0, stream));
            launch_block();
            CK(cudaEventRecord(e1, stream));
            CK(cudaEventSynchronize(e1));
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best) { best = ms; pick = c; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        gsteps = keep;
        lay_n = pick.n;
        lay_top = pick.top;
        layout(pick);
    }

    void advance(long nsteps) override {
        if (tune_pending && !slots.empty()) {
            tune_pending = false;
            tune();
        }
        if (dirty) rebuild();
        if (running.empty()) return;
        for (long k = 0; k < nsteps; k += gsteps) {
            launch_block();
            for (int q : running) {
                Slot &s = slots[q];
                const bool was = s.finished();
                s.done = std::min<long>(s.done + gsteps, s.sim->sched.nsteps);
                if (!was && s.finished()) dirty = true;  // drop it from the next graph
            }
        }
    }

    // one block of gsteps steps of every running slot
    void launch_block() {
        if (!persistent) {
            CK(cudaGraphLaunch(gexec, stream));
            return;
        }
        const int n = (int)running.size();
        int nq = 0;
        for (int r = 0; r < n; r++) {
            const Slot &s = slots[running[r]];
            pa.steps[r] = (int)std::max<long>(0, std::min<long>(gsteps, s.sim->sched.nsteps - s.done));
            int ns = 0;
            for (int q = 0; q < kStages; q++) ns += pa.units[r][q] > 0 ? 1 : 0;
            nq += pa.steps[r] * ns;
        }
        pa.nq = nq;
        if (nq) CK(launch_persistent<T>(pa, pgrid, psmem, stream));
        launch_advance_all(counters.as<int>(), n, gsteps, stream);
        CK(cudaGetLastError());
    }

    // a wait of the persistent schedule that gave up (its slots' error words are set too)
    void check_schedule() {
        if (!persistent) return;
        int h = 0;
        CK(cudaMemcpyAsync(&h, perr.p, sizeof h, cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        if (h) {
            CK(cudaMemsetAsync(perr.p, 0, sizeof(int), stream));
            CK(cudaStreamSynchronize(stream));
            throw Error(TCSEM_ERR_CUDA, "a wait of the persistent batch schedule gave up");
        }
    }

    int poll(int *ids, int cap) override {
        CK(cudaStreamSynchronize(stream));
        check_schedule();
        int c = 0;
        for (auto &s : slots)
            if (s.finished()) {
                if (ids && c < cap) ids[c] = s.id;
                c++;
            }
        return c;
    }

    void slot_info(int id, tcsem_info *o, long *steps_done) override {
        Slot &s = find(id);
        const Model &m = s.sim->model;
        if (o) {
            o->L = m.L; o->M = m.M; o->N = m.N; o->L1 = m.L1; o->M1 = m.M1;
            o->NRx = (int)m.in.rx.size(); o->NTx = (int)m.in.tx.size(); o->Nt = m.in.Nt;
            o->NComp = m.NComp; o->nefcmp = m.nefcmp;
            o->nsteps = s.sim->sched.nsteps;
            o->precision = s.sim->opts.precision;
            o->device_bytes = s.bytes;
            o->launches_per_step = persistent ? 0 : lps;
            const ZChunks &zc = s.sim->zc;
            o->zchunks = zc.n;
            o->top_planes = zc.n > 1 && zc.kb[1] != (int)(s.sim->model.N / zc.n) ? zc.kb[1] : 0;
            o->uploaded_bytes = s.sim->uploaded_bytes;
        }
        if (steps_done) *steps_done = s.done;
    }

    void traces(int id, double *out) override {
        Slot &s = find(id);
        CK(cudaStreamSynchronize(stream));
        s.sim->traces(out);
    }

    void write_bout(int id, const char *path) override {
        Slot &s = find(id);
        const Model &m = s.sim->model;
        std::vector<double> t((size_t)m.in.rx.size() * m.NComp * m.in.Nt);
        traces(id, t.data());
        write_bout_file(m, s.sim->itx, t.data(), path);
    }

    void remove(int id) override {
        CK(cudaStreamSynchronize(stream));
        for (size_t q = 0; q < slots.size(); q++)
            if (slots[q].id == id) {
                used -= slots[q].bytes;
                slots.erase(slots.begin() + q);
                dirty = true;
                return;
            }
        throw Error(TCSEM_ERR_INVALID, "no slot " + std::to_string(id) + " in the batch");
    }

    void stats(int *n, int *run, size_t *bytes) override {
        int r = 0;
        for (auto &s : slots) r += s.finished() ? 0 : 1;
        if (n) *n = (int)slots.size();
        if (run) *run = r;
        if (bytes) *bytes = used;
    }
};

}  // namespace tcsem

// ================================================================== C ABI
using namespace tcsem;

struct tcsem_batch {
    std::unique_ptr<BatchBase> impl;
};

static thread_local std::string g_batch_err;

template <class F> static tcsem_status bguard(tcsem_batch_t *b, F &&f) {
    if (!b || !b->impl) return TCSEM_ERR_INVALID;
    try {
        CK(cudaSetDevice(b->impl->device));
        f(*b->impl);
        return TCSEM_OK;
    } catch (const Error &e) {
        b->impl->err = e.what();
        return (tcsem_status)e.code;
    } catch (const std::bad_alloc &) {
        b->impl->err = "host allocation failed";
        return TCSEM_ERR_NOMEM;
    } catch (const std::exception &e) {
        b->impl->err = e.what();
        return TCSEM_ERR_INVALID;
    }
}

extern "C" {

tcsem_status tcsem_batch_create(const tcsem_opts *opts, size_t device_budget, tcsem_batch_t **out) {
    if (!out) { g_batch_err = "null argument"; return TCSEM_ERR_INVALID; }
    *out = nullptr;
    tcsem_opts o;
    tcsem_default_opts(&o);
    if (opts) o = *opts;
    if (o.precision == 0) o.precision = TCSEM_FP32;
    if (o.precision != TCSEM_FP32 && o.precision != TCSEM_FP64) { g_batch_err = "precision must be 32 or 64"; return TCSEM_ERR_INVALID; }
    try {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= o.device || o.device < 0)
            throw Error(TCSEM_ERR_CUDA, "no usable CUDA device");
        std::unique_ptr<BatchBase> impl;
        if (o.precision == TCSEM_FP64) impl.reset(new BatchImpl<double>());
        else impl.reset(new BatchImpl<float>());
        impl->opts = o;
        impl->device = o.device;
        impl->budget = device_budget;
        impl->init();
        tcsem_batch_t *b = new tcsem_batch;
        b->impl = std::move(impl);
        *out = b;
        return TCSEM_OK;
    } catch (const Error &e) {
        g_batch_err = e.what();
        return (tcsem_status)e.code;
    } catch (const std::exception &e) {
        g_batch_err = e.what();
        return TCSEM_ERR_INVALID;
    }
}

const char *tcsem_batch_error(const tcsem_batch_t *b) {
    return b && b->impl ? b->impl->err.c_str() : g_batch_err.c_str();
}

tcsem_status tcsem_batch_destroy(tcsem_batch_t *b) {
    if (!b) return TCSEM_ERR_INVALID;
    delete b;
    return TCSEM_OK;
}

tcsem_status tcsem_batch_add(tcsem_batch_t *b, const char *dir, int itx, int *slot) {
    nvtxRangePushA("tcsem_batch_add");
    struct Pop { ~Pop() { nvtxRangePop(); } } pop;
    if (!dir) return TCSEM_ERR_INVALID;
    return bguard(b, [&](BatchBase &x) {
        const int id = x.add(dir, itx);
        if (slot) *slot = id;
    });
}

tcsem_status tcsem_batch_advance(tcsem_batch_t *b, long nsteps) {
    nvtxRangePushA("tcsem_batch_advance");
    struct Pop { ~Pop() { nvtxRangePop(); } } pop;
    return bguard(b, [&](BatchBase &x) { x.advance(nsteps); });
}

tcsem_status tcsem_batch_poll(tcsem_batch_t *b, int *slots, int cap, int *count) {
    return bguard(b, [&](BatchBase &x) {
        const int c = x.poll(slots, cap);
        if (count) *count = c;
    });
}

tcsem_status tcsem_batch_slot_info(tcsem_batch_t *b, int slot, tcsem_info *info, long *steps_done) {
    return bguard(b, [&](BatchBase &x) { x.slot_info(slot, info, steps_done); });
}

tcsem_status tcsem_batch_traces(tcsem_batch_t *b, int slot, double *traces) {
    if (!traces) return TCSEM_ERR_INVALID;
    return bguard(b, [&](BatchBase &x) { x.traces(slot, traces); });
}

tcsem_status tcsem_batch_write_bout(tcsem_batch_t *b, int slot, const char *path) {
    if (!path) return TCSEM_ERR_INVALID;
    return bguard(b, [&](BatchBase &x) { x.write_bout(slot, path); });
}

tcsem_status tcsem_batch_remove(tcsem_batch_t *b, int slot) {
    return bguard(b, [&](BatchBase &x) { x.remove(slot); });
}

tcsem_status tcsem_batch_stats(tcsem_batch_t *b, int *slots, int *running, size_t *device_bytes) {
    return bguard(b, [&](BatchBase &x) { x.stats(slots, running, device_bytes); });
}

// The persistent batch kernel on one CTA with a queue whose first stage nothing publishes:
// its wait for a ready stage gives up after wait_ns and sets the schedule's error word.
tcsem_status tcsem_selftest_queue_wait(int device, long long wait_ns, int *gave_up) {
    if (!gave_up || wait_ns < 1) return TCSEM_ERR_INVALID;
    *gave_up = 0;
    int *words = nullptr;
    QueueEntry *q = nullptr;
    if (cudaSetDevice(device) != cudaSuccess || cudaMalloc(&words, (kQWords + 1) * sizeof(int)) != cudaSuccess)
        return TCSEM_ERR_CUDA;
    tcsem_status st = TCSEM_OK;
    if (cudaMalloc(&q, sizeof(QueueEntry)) != cudaSuccess) st = TCSEM_ERR_CUDA;
    int h = 0;
    if (st == TCSEM_OK) {
        PersistArgs<float> a{};
        a.q = q;
        a.ctl = words;
        a.err = words + kQWords;
        a.nq = 1;       // one stage expected ...
        a.nslots = 0;   // ... and no slot to publish it
        a.wait_ns = wait_ns;
        a.ctl_off = 0;  // no body runs: the scheduling words alone
        const size_t smem = 64;
        if (cudaMemset(a.err, 0, sizeof(int)) != cudaSuccess || persist_configure<float>(smem) != cudaSuccess ||
            launch_persistent<float>(a, 1, smem, nullptr) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(&h, a.err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            st = TCSEM_ERR_CUDA;
    }
    cudaFree(q);
    cudaFree(words);
    *gave_up = h;
    return st;
}

}  // extern "C"
