// Persistent batch schedule: all steps of a graph block of every slot in one launch.
//
// A slot's step is a chain of six stages -- rows_fwd, cols, rows_inv, bilinear (the
// boundary), sweep (every z-chunk) and receivers -- each made of independent items that
// one CTA processes (a row pair, a column, a tile, ...).  The launch keeps a device queue
// of the stages whose inputs are complete: a CTA takes the next item of the oldest stage
// in the queue; the CTA that finishes a stage's last item appends the slot's next stage.
// So a slot moves on as soon as its own chain allows, while the other slots' items keep
// the GPU busy, and no CTA ever waits for work it holds.  Every wait for the queue is
// bounded in time: a CTA that gives up marks the launch as aborted and the error words
// of the slots, and every CTA leaves.
#pragma once
#include "boundary.cuh"
#include "kernels.cuh"
#include "rx.cuh"

namespace tcsem {

constexpr int kStages = 6;  // rows_fwd, cols, rows_inv, bilinear, sweep, receivers

// one stage of one slot's step, in the order stages became ready (zeroed before each launch)
struct QueueEntry {
    int ready;  // 1 once the entry is filled in (release store)
    int slot, step, stage, count;  // count: the stage's units
    int claimed;  // units handed out
    int done;     // units finished
    int pad;
};
enum { kQHead = 0, kQTail = 1, kQAbort = 2, kQWords = 4 };

template <typename T> struct PersistArgs {
    const SweepSlot<T> *sw[2];  // per field-set parity of the step
    const BoundarySlot<T> *bs[2];
    const RxSlot<T> *rs[2];
    QueueEntry *q;
    int *ctl;                            // kQWords control words
    int *err;                            // the schedule's own error word
    int nq;                              // entries this launch appends in total
    int nslots;
    int steps[kMaxSlots];                // steps of each slot in this launch
    // A stage of a slot has nitems items (row pairs, columns, rows, output points, tiles,
    // receiver stencils) handed out in `units` claims of up to `per` consecutive items
    // (0 units: stage skipped).  The bilinear stage's units split its output points
    // evenly; the receiver stage's unit is one CTA's worth of stencils.
    int units[kMaxSlots][kStages];
    int per[kMaxSlots][kStages];
    int nitems[kMaxSlots][kStages];
    long long wait_ns;                   // a wait for the queue gives up after this long
    int ctl_off;                         // byte offset of the CTA's scheduling words in shared memory
};

template <typename T> cudaError_t persist_configure(size_t smem);
template <typename T> int persist_blocks(size_t smem);  // co-resident CTAs on the device
// a zeroed queue with the first stage of every slot, then the persistent launch of `grid` CTAs
template <typename T> cudaError_t launch_persistent(const PersistArgs<T> &a, int grid, size_t smem, cudaStream_t st);
int persist_threads();

}  // namespace tcsem
