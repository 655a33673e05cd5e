// Persistent batch schedule (see persist.cuh): one cooperative launch per graph block whose
// CTAs take their items from a device queue of ready stages.
//
// Memory ordering.  A CTA finishes an item with a CTA barrier, then its thread 0 fences
// (gpu scope, and the async proxy) and counts the item done with an atomic add; the CTA
// whose add completes the stage fences again -- it has now observed every item of the
// stage -- and publishes the slot's next stage with a release store of the entry's ready
// word.  A CTA that takes an item acquires that word, fences (gpu scope and the async
// proxy, for the bulk-tensor copies of the sweep) and releases its threads with a CTA
// barrier.  The chain of a slot is therefore ordered exactly as the per-kernel launches
// order it, and the items read what the earlier stages wrote with plain or L2-only loads
// and bulk copies (no read-only-cache loads of data this launch writes).
#include "boundary_body.cuh"
#include "persist.cuh"
#include "rx_body.cuh"
#include "sweep.cuh"

namespace tcsem {

namespace {

// scheduling words of a CTA in shared memory
enum { kShEntry = 0, kShItem, kShSlot, kShStep, kShStage, kShCount, kShWords = 8 };

template <typename T> __device__ void give_up(const PersistArgs<T> &a) {
    atomicExch(a.ctl + kQAbort, 1);
    atomicExch(a.err, 1);
    for (int r = 0; r < a.nslots; r++) atomicExch(a.sw[0][r].err, 1);
}

// thread 0: the next unit into sh (sh[kShEntry] < 0: leave).  First the entry of this CTA's
// previous unit, which often has more (same slot, step and stage; its inputs were acquired
// with that unit), then the oldest ready entry of the queue.
template <typename T> __device__ void take_item(const PersistArgs<T> &a, int *sh) {
    if (sh[kShEntry] >= 0) {
        const int i = atomicAdd(&a.q[sh[kShEntry]].claimed, 1);
        if (i < sh[kShCount]) {
            sh[kShItem] = i;
            return;
        }
    }
    unsigned long long t0 = globaltimer_ns();
    for (;;) {
        if (ld_acquire(a.ctl + kQAbort)) break;
        const int h = ld_acquire(a.ctl + kQHead);
        if (h >= a.nq) break;  // every stage of the launch has been handed out
        QueueEntry *e = a.q + h;
        if (ld_acquire(&e->ready)) {
            const int i = atomicAdd(&e->claimed, 1);
            if (i < e->count) {
                sh[kShEntry] = h;
                sh[kShItem] = i;
                sh[kShSlot] = e->slot;
                sh[kShStep] = e->step;
                sh[kShStage] = e->stage;
                sh[kShCount] = e->count;
                fence_acq_rel_gpu();
                fence_proxy_async_global();
                return;
            }
            atomicCAS(a.ctl + kQHead, h, h + 1);  // exhausted: the next entry becomes the oldest
            t0 = globaltimer_ns();
            continue;
        }
        if (globaltimer_ns() - t0 > (unsigned long long)a.wait_ns) {
            give_up(a);
            break;
        }
        __nanosleep(128);
    }
    sh[kShEntry] = -1;
}

// thread 0, after the CTA barrier that ends a unit: count it; the last unit of a stage
// appends the slot's next stage that has units (in the same step or the next one)
template <typename T> __device__ void finish_item(const PersistArgs<T> &a, const int *sh) {
    fence_proxy_async_global();
    fence_acq_rel_gpu();  // release: the CTA's writes (ordered before by the barrier) ...
    QueueEntry *e = a.q + sh[kShEntry];
    if (atomicAdd(&e->done, 1) != sh[kShCount] - 1) return;  // ... with this add
    fence_acq_rel_gpu();  // acquire: the other units of the stage are now visible to this thread
    const int r = sh[kShSlot];
    int step = sh[kShStep], stage = sh[kShStage];
    do {
        if (++stage == kStages) { stage = 0; step++; }
    } while (step < a.steps[r] && a.units[r][stage] == 0);
    if (step >= a.steps[r]) return;  // the slot's last stage of this launch
    const int p = atomicAdd(a.ctl + kQTail, 1);
    if (p >= a.nq) {  // more stages than the host counted: cannot happen with consistent tables
        give_up(a);
        return;
    }
    QueueEntry *n = a.q + p;
    n->slot = r;
    n->step = step;
    n->stage = stage;
    n->count = a.units[r][stage];
    st_release(&n->ready, 1);
}

// every thread of the CTA: one unit.  Returns the mbarriers the unit leaves initialised:
// 0 none (receivers, bilinear stage, or a gated slot), 1 the boundary stages' one, 2 the sweep's ring
template <typename T> __device__ int run_item(const PersistArgs<T> &a, const int *sh) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int r = sh[kShSlot], step = sh[kShStep], stage = sh[kShStage], u = sh[kShItem], p = step & 1;
    switch (stage) {
    case 0: case 1: case 2: case 3: {
        const BoundarySlot<T> *d = a.bs[p] + r;
        if ((long)*d->step_base + step >= d->nsteps) return 0;
        if (stage == 3) {
            bilinear_cta<T>(d->bd, d->bx, d->by, d->g, u, sh[kShCount]);
            return 0;
        }
        const int lo = u * a.per[r][stage], hi = min(lo + a.per[r][stage], a.nitems[r][stage]);
        for (int b = lo; b < hi; b++) {
            if (b > lo) {  // the previous item is done with shared memory: retire its barrier
                __syncthreads();
                if (threadIdx.x == 0) mbar_inval(reinterpret_cast<uint64_t *>(smem_raw));
            }
            if (stage == 0) rows_fwd_cta<T, true>(d->bd, d->bz, d->tot, d->nch, d->g, b);
            else if (stage == 1) cols_cta<T>(d->bd, b);
            else rows_inv_cta<T>(d->bd, b);
        }
        return 1;
    }
    case 4: {
        const SweepSlot<T> &d = a.sw[p][r];
        const long st = (long)*d.step_base + step;
        if (st >= d.nsteps) return 0;
        const int bx = u % d.tiles_x, rest = u / d.tiles_x, by = rest % d.tiles_y, c = rest / d.tiles_y;
        sweep_cta<T, true>(d.maps, d.g, d.out, d.tin, d.tout, d.ax, d.table[st], d.src, d.zc, bx, by, c, d.err);
        return 2;
    }
    default: {
        const RxSlot<T> &d = a.rs[p][r];
        const long st = (long)*d.step_base + step;
        if (st >= d.nsteps) return 0;
        rx_thread(d.rd, d.f, d.tot, d.zc, d.g, step_action(d.rd, st), u * (int)blockDim.x + (int)threadIdx.x);
        return 0;
    }
    }
}

}  // namespace

template <typename T>
__global__ void __launch_bounds__(fs3::NT, sizeof(T) == 4 ? 2 : 1) k_persistent(const __grid_constant__ PersistArgs<T> a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    int *sh = reinterpret_cast<int *>(smem_raw + a.ctl_off);
    if (threadIdx.x == 0) sh[kShEntry] = -1;
    for (;;) {
        if (threadIdx.x == 0) take_item(a, sh);
        __syncthreads();
        if (sh[kShEntry] < 0) break;
        const int bars = run_item(a, sh);
        __syncthreads();  // the unit's writes are issued and its shared memory is free
        if (threadIdx.x == 0) {
            // retire the unit's mbarriers before the next unit lays out shared memory anew
            if (bars == 2) {
                uint64_t *ring = reinterpret_cast<uint64_t *>(smem_raw + fs3::bars_offset<T>());
                for (int q = 0; q < fs3::RING; q++) mbar_inval(ring + q);
            } else if (bars == 1) {
                mbar_inval(reinterpret_cast<uint64_t *>(smem_raw));  // offset 0 in every boundary layout
            }
            finish_item(a, sh);
        }
    }
}

// the first stage (with items) of step 0 of every slot that runs in this launch
template <typename T> __global__ void k_queue_seed(const __grid_constant__ PersistArgs<T> a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int n = 0;
    for (int r = 0; r < a.nslots; r++) {
        if (a.steps[r] <= 0) continue;
        int stage = 0;
        while (stage < kStages && a.units[r][stage] == 0) stage++;
        if (stage == kStages || n >= a.nq) continue;
        QueueEntry *e = a.q + n++;
        e->slot = r;
        e->step = 0;
        e->stage = stage;
        e->count = a.units[r][stage];
        e->ready = 1;
    }
    a.ctl[kQTail] = n;
}

template <typename T> cudaError_t persist_configure(size_t smem) {
    return cudaFuncSetAttribute(k_persistent<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename T> int persist_blocks(size_t smem) {
    int nb = 0, dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_persistent<T>, fs3::NT, smem) != cudaSuccess)
        return 0;
    return nb * sms;
}

template <typename T> cudaError_t launch_persistent(const PersistArgs<T> &a, int grid, size_t smem, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(a.q, 0, (size_t)a.nq * sizeof(QueueEntry), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.ctl, 0, kQWords * sizeof(int), st);
    if (e != cudaSuccess) return e;
    k_queue_seed<T><<<1, 32, 0, st>>>(a);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(fs3::NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;  // every CTA resident: a CTA may wait for the stages of others
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_persistent<T>, a);
}

int persist_threads() { return fs3::NT; }

#define INST(T)                                                                                          \
    template cudaError_t persist_configure<T>(size_t);                                                  \
    template int persist_blocks<T>(size_t);                                                             \
    template cudaError_t launch_persistent<T>(const PersistArgs<T> &, int, size_t, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace tcsem
