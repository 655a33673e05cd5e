/*
 * tcsem.h -- C ABI of the GB300-native TCSEM_FDTD time-stepping path.
 *
 * One handle (tcsem_sim) holds one survey (model, grid, receivers, all
 * transmitters) and owns all of its device memory; handles are independent
 * (no global or __constant__ state), each works on its own CUDA stream, and a
 * handle must be used from one host thread at a time.  Every entry point
 * returns a tcsem_status; no entry point exits the process or reads stdin.
 *
 * Field arrays exchanged with the host use the reference's layout (FTDT.h:62-74,
 * prepare_free_mem.cu:63-81), x fastest:
 *   Ex[N+1][M+1][L]  Ey[N+1][M][L+1]  Ez[N][M+1][L+1]
 *   Bx[N][M][L+1]    By[N][M+1][L]    Bz[N+1][M][L]
 *   BxAir[M][L+1]    ByAir[M+1][L]    Con[N][M][L]
 * Traces are double [nr][NComp][Nt] like the Tx<k>.bout payload (main.cu:278-292).
 */
#ifndef TCSEM_H_INCLUDED
#define TCSEM_H_INCLUDED

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    TCSEM_OK = 0,
    TCSEM_ERR_IO = 1,       /* an input or output file could not be opened/written */
    TCSEM_ERR_PARSE = 2,    /* malformed input file */
    TCSEM_ERR_INVALID = 3,  /* inconsistent model/survey or bad argument */
    TCSEM_ERR_CUDA = 4,     /* CUDA runtime error or no usable GPU */
    TCSEM_ERR_NOMEM = 5,    /* device or host allocation failed */
    TCSEM_ERR_STATE = 6,    /* call not valid in the handle's current state */
    TCSEM_ERR_NUMERIC = 7   /* a non-finite value appeared in the fields */
} tcsem_status;

enum { TCSEM_FP32 = 32, TCSEM_FP64 = 64 };

typedef struct tcsem_sim tcsem_sim_t;

enum {
    TCSEM_EX = 0, TCSEM_EY = 1, TCSEM_EZ = 2, TCSEM_BX = 3, TCSEM_BY = 4, TCSEM_BZ = 5,
    TCSEM_BXAIR = 6, TCSEM_BYAIR = 7, TCSEM_CON = 8
};

typedef struct {
    int precision;        /* TCSEM_FP32 (default) or TCSEM_FP64 */
    int device;           /* CUDA device ordinal, default 0 */
    int fix_dual_bipole;  /* 1: inject the second bipole of ort=5 at its own cells (default 0 = as the reference) */
    int graph_steps;      /* steps per captured CUDA graph, 0 = default (even numbers only) */
    int zchunks;          /* z-chunks of the fused sweep, 0 = chosen from the grid and the GPU,
                             -1 = the fastest of the layouts near that choice, timed at open
                             (the last bits of the traces may then differ between runs) */
    int serial_boundary;  /* 1: boundary pipeline strictly before the whole sweep; default 0 = the
                             boundary and the top z-chunk run beside the lower chunks */
    int top_planes;       /* planes of the top z-chunk, 0 = default (one plane beside the boundary, so
                             that little of the sweep waits for it; an even split with
                             serial_boundary), -1 = an even split */
    int padded_plane;     /* continue the air field on a wider transform plane whose points beyond
                             the uniform grid taper from its edge values to zero (raised cosine,
                             the padding UpContinuation.cpp:21-49 sketches): 1 = the powers of two
                             above L1 and M1, 2 = the smallest lengths >= L1, M1 without prime
                             factors above 5; not the reference's arithmetic (default 0) */
    int persistent_batch; /* batches only: 1 = every block of graph_steps steps of all slots is one
                             persistent launch whose CTAs take boundary, sweep and receiver items
                             from a device queue of the stages whose inputs are complete, so each
                             slot moves on as soon as its own chain allows; default 0 = a captured
                             graph of one launch per kernel per step for all slots together */
} tcsem_opts;

typedef struct {
    int L, M, N;          /* cells in x, y, z */
    int L1, M1;           /* uniform continuation plane */
    int NRx, NTx, Nt, NComp, nefcmp;
    long nsteps;          /* time steps of one transmitter run */
    int precision;
    size_t device_bytes;  /* device memory held by the handle */
    int launches_per_step; /* kernels launched per time step by tcsem_advance (a batch slot: for
                              all slots together; 0 with persistent_batch, which launches three
                              kernels per block of graph_steps steps) */
    int zchunks;          /* z-chunks of the fused sweep in use */
    int top_planes;       /* planes of the top z-chunk when it runs beside the others, else 0 */
    size_t uploaded_bytes; /* host-to-device bytes the open copied (conductivity, grid, boundary and
                              step tables); the fields start as zero on the device */
} tcsem_info;

/* Opening a survey.  tcsem_open_dir reads FDTD_setup.in, Cond.bin, Receiver.in
 * and Transmitter.in from `dir` -- the reference reads them from its working
 * directory (ModelingSetup.cpp:43-209, LoadRxTxPos.cpp:43-200). */
void tcsem_default_opts(tcsem_opts *opts);
tcsem_status tcsem_open_dir(const char *dir, const tcsem_opts *opts, tcsem_sim_t **out);

/* In-memory open: the same survey from host buffers, for a host that already
 * holds the model and the survey (the reference's ModelingSetup and
 * LoadRxTxPos, ModelingSetup.cpp:34-234 and LoadRxTxPos.cpp:35-200, fill the
 * same values from the four files).  The fields of tcsem_model are the eight
 * lines of FDTD_setup.in in file order plus the conductivity of Cond.bin;
 * those of tcsem_survey are Receiver.in and Transmitter.in (transmitter t has
 * id t+1, receiver r has id r+1; angles in degrees, as in the file).  Every
 * buffer is copied during the call.  The checks and error codes are those of
 * tcsem_open_dir: TCSEM_ERR_PARSE for what would be a malformed file (an
 * orientation outside 1..5, a receiver id out of range, no receivers),
 * TCSEM_ERR_INVALID for an inconsistent grid. */
typedef struct {
    double sfa1, sfa2;               /* line 1: factors of the time step and of gamma */
    int n1;                          /* line 2: source samples (nsrc = n1/2) ... */
    double sita_t;                   /*         ... and the width of the Gaussian source pulse */
    double x0, y0, z0;               /* line 3: origin of the grid */
    double dxmin, dymin, dzmin;      /* line 4: core cell sizes */
    double arg1, arg2;               /* line 5: growth factors of the boundary strips */
    int ALx2, ALx1, Nx, ARx1, ARx2;  /* line 6: cells along x */
    int Ay2, Ay1, Ny;                /* line 7: cells along y */
    int Az2, Az1, Nz;                /* line 8: cells along z */
    const double *con;               /* Cond.bin: conductivity (S/m) [N][M][L], x fastest */
} tcsem_model;

typedef struct {
    int ort;                          /* 1 x, 2 y, 3 z, 4 azimuth/dip, 5 two bipoles (LoadRxTxPos.cpp:151-200) */
    double len, x, y, z;              /* bipole length and centre */
    double azi, dip;                  /* degrees (ort 4 and 5) */
    double len1, x1, y1, z1, azi1, dip1; /* second bipole (ort 5) */
    int nr;                           /* receivers of this transmitter ... */
    const int *rx;                    /* ... their ids, 1..NRx, in output order */
} tcsem_transmitter;

typedef struct {
    double T0, Tn;             /* Receiver.in line 1: first and last sampling time */
    int Nt, IsLog;             /* line 2: samples, log (1) or linear (0) spacing */
    int comps[6];              /* line 3: record Ex Ey Ez Bx By Bz */
    int NRx;                   /* receivers */
    const double *rx_xyz;      /* [NRx][3] positions */
    int NTx;                   /* transmitters */
    const tcsem_transmitter *tx;
} tcsem_survey;

tcsem_status tcsem_open(const tcsem_model *model, const tcsem_survey *survey, const tcsem_opts *opts,
                        tcsem_sim_t **out);
tcsem_status tcsem_close(tcsem_sim_t *sim);
const char *tcsem_last_error(const tcsem_sim_t *sim); /* message of the last failed call on `sim` */
const char *tcsem_open_error(void);                   /* message of the last failed open (per thread) */
tcsem_status tcsem_get_info(const tcsem_sim_t *sim, tcsem_info *out);

/* Whole runs: the transmitter loop body of main.cu:195-298 (with the state
 * reset per transmitter that the reference omits).  traces: [nr][NComp][Nt]. */
tcsem_status tcsem_run(tcsem_sim_t *sim, int itx, double *traces);
tcsem_status tcsem_write_bout(tcsem_sim_t *sim, int itx, const double *traces, const char *path);

/* Stepwise form of tcsem_run: begin resets the fields for transmitter itx;
 * advance runs exactly min(nsteps, steps left) more steps (whole blocks as
 * replays of one captured CUDA graph, the rest launched directly); done is set
 * once the last step has run; traces can be read at any time. */
tcsem_status tcsem_begin(tcsem_sim_t *sim, int itx);
tcsem_status tcsem_advance(tcsem_sim_t *sim, long nsteps, int *done);
tcsem_status tcsem_get_traces(tcsem_sim_t *sim, double *traces);
tcsem_status tcsem_synchronize(tcsem_sim_t *sim);

/* Checkpoint of a run in progress (no counterpart in the reference; for moving
 * or preempting long runs): save_state writes, after tcsem_begin and any number
 * of tcsem_advance calls, what the next step needs -- the current fields, their
 * Bz chunk totals, the receiver samples so far and the step -- to `path`;
 * load_state reads it into a handle opened on the same survey with the same
 * precision, z-chunk layout, padded-plane mode and dual-bipole option
 * (TCSEM_ERR_INVALID otherwise: the run would continue under other physics), after which
 * tcsem_advance continues the run: its traces equal those of the uninterrupted
 * run bit for bit. */
tcsem_status tcsem_save_state(tcsem_sim_t *sim, const char *path);
tcsem_status tcsem_load_state(tcsem_sim_t *sim, const char *path);

/* Per-stage entry points, the seam of FTDT.h:291-344.  They act on the
 * handle's current fields like the reference's functions act on DArrays:
 *   tcsem_upcontinuation   <- UpContinuation_gpu (UpContinuation_gpu.cu:166)
 *   tcsem_electric_field   <- ElectricalField    (ElectricalFiled.cu:478)
 *   tcsem_bderivate        <- Bderivate          (Bderivate.cu:269)
 *   tcsem_rx_sample        <- EFXInterp/BFXInterp (EFInterp2Rx.cu:410-470), into slot 0 or 1
 *   tcsem_fused_step       <- ElectricalField followed by Bderivate, as one fused sweep */
tcsem_status tcsem_select_tx(tcsem_sim_t *sim, int itx);
tcsem_status tcsem_upcontinuation(tcsem_sim_t *sim);
tcsem_status tcsem_electric_field(tcsem_sim_t *sim, double lambda, double dt, double wave);
tcsem_status tcsem_bderivate(tcsem_sim_t *sim, double dt);
tcsem_status tcsem_fused_step(tcsem_sim_t *sim, double lambda, double dt, double dt_b, double wave);
tcsem_status tcsem_rx_sample(tcsem_sim_t *sim, int efield, int slot, double *values /* [NComp][nr] slot image */);

/* Host <-> device field access in the reference layout (comp = TCSEM_EX ...). */
tcsem_status tcsem_get_field(tcsem_sim_t *sim, int comp, double *host);
tcsem_status tcsem_set_field(tcsem_sim_t *sim, int comp, const double *host);
tcsem_status tcsem_field_size(const tcsem_sim_t *sim, int comp, size_t *count);

/* Source waveform of SourceWave.cpp:8-58 (what the reference writes to
 * testwaveform.dat): nsrc = n1/2, arrays of 2*nsrc+1 entries (may be NULL). */
tcsem_status tcsem_get_waveform(const tcsem_sim_t *sim, int *nsrc, double *t, double *dt, double *wave);

/* Host-side schedule, for inspection: per step dt1, dt2, lambda and source
 * amplitude (main.cu:212-260); each array may be NULL; `cap` entries at most. */
tcsem_status tcsem_get_schedule(const tcsem_sim_t *sim, double *dt1, double *dt2, double *lambda, double *wave, long cap);

/* Device time (CUDA events on the handle's stream) of tcsem_advance(nsteps)
 * from the current state; the state advances like tcsem_advance. */
tcsem_status tcsem_timed_advance(tcsem_sim_t *sim, long nsteps, double *ms);

/* Timing of the captured step loop on the handle's stream: runs `nsteps`
 * steps of transmitter itx from a fresh state and reports the elapsed device
 * time (CUDA events), plus, if non-NULL, the time of the fused volume sweep
 * and of the boundary pipeline measured separately with events. */
tcsem_status tcsem_time_steps(tcsem_sim_t *sim, int itx, long nsteps, double *ms_total, double *ms_sweep,
                              double *ms_boundary);

/* Batches: many surveys of different sizes advanced together on one GPU, one
 * launch per kernel per time step for all of them (no counterpart in the
 * reference, which runs one survey per process; the batch entry points of
 * the drop-in boundary).  A batch holds up to 64 slots; each slot is one
 * transmitter run of one survey directory (the same four input files) with
 * its own fields, schedule and receivers resident on the device.
 *   tcsem_batch_create   device, precision, graph block length and z-chunks per
 *                        slot (0 = 2) from opts;
 *                        device_budget (bytes, 0 = no limit) bounds the sum of
 *                        the slots' device memory
 *   tcsem_batch_add      reads and sets up a survey; TCSEM_ERR_NOMEM (nothing
 *                        allocated) when its estimated footprint does not fit
 *                        the budget or the batch is full
 *   tcsem_batch_advance  enqueues whole blocks of graph_steps steps (at least
 *                        nsteps) for every slot still running; returns before
 *                        they finish; slots added since the last call join here
 *   tcsem_batch_poll     waits for the enqueued work, then lists (up to cap)
 *                        the slots whose runs are complete; count = all of them
 *   tcsem_batch_traces   traces [nr][NComp][Nt] of a slot (after it completed)
 *   tcsem_batch_write_bout  the slot's Tx<k>.bout (format of main.cu:280-292)
 *   tcsem_batch_remove   frees a slot
 * A batch is used from one host thread at a time. */
typedef struct tcsem_batch tcsem_batch_t;
tcsem_status tcsem_batch_create(const tcsem_opts *opts, size_t device_budget, tcsem_batch_t **out);
tcsem_status tcsem_batch_destroy(tcsem_batch_t *batch);
const char *tcsem_batch_error(const tcsem_batch_t *batch); /* last failure (batch may be NULL after a failed create) */
tcsem_status tcsem_batch_add(tcsem_batch_t *batch, const char *dir, int itx, int *slot);
tcsem_status tcsem_batch_advance(tcsem_batch_t *batch, long nsteps);
tcsem_status tcsem_batch_poll(tcsem_batch_t *batch, int *slots, int cap, int *count);
tcsem_status tcsem_batch_slot_info(tcsem_batch_t *batch, int slot, tcsem_info *info, long *steps_done);
tcsem_status tcsem_batch_traces(tcsem_batch_t *batch, int slot, double *traces);
tcsem_status tcsem_batch_write_bout(tcsem_batch_t *batch, int slot, const char *path);
tcsem_status tcsem_batch_remove(tcsem_batch_t *batch, int slot);
tcsem_status tcsem_batch_stats(tcsem_batch_t *batch, int *slots, int *running, size_t *device_bytes);

/* tcsem_upcontinuation_noalloc: the boundary step of tcsem_upcontinuation
 * (same kernels, same result) that allocates nothing when called.  It has no
 * counterpart in the reference.
 *
 * It is meant for callers that cannot allocate device memory at the moment
 * they run the boundary step -- a host whose memory pool already owns the
 * device, or a step that runs while another library holds the allocator.  The
 * four work arrays of the pipeline (x-spectra, the two filtered column sets,
 * the packed inverse rows) are carved from one static device array of
 * TCSEM_NOALLOC_SCRATCH_BYTES (16 MiB) built into the library, instead of the
 * handle's own buffers.  A survey whose continuation plane needs more scratch
 * than that (about 11.8 MB for a 736 x 736 plane over 256 rows in FP64) is
 * refused with TCSEM_ERR_INVALID and a message giving both sizes.
 *
 * The first call on each device, with that device current, looks up the
 * array's address with cudaGetSymbolAddress and keeps it; make that first call
 * before any stream capture.  The address belongs to the device's primary
 * context: after cudaDeviceReset (or anything else that destroys that context)
 * the kept address is stale, so do not call this entry point again in the same
 * process after a reset.  Nothing in the scratch has to start at zero:
 * every element a call reads is written earlier in the same call.  There is
 * one scratch per device, shared by all handles: calls that can overlap on a
 * device (different handles, threads or streams) race on it, so the caller
 * must serialise them. */
#define TCSEM_NOALLOC_SCRATCH_BYTES ((size_t)16 << 20)
tcsem_status tcsem_upcontinuation_noalloc(tcsem_sim_t *sim);

/* Self-test of the bounded waits every kernel uses on its bulk copies (no
 * counterpart in the reference): one CTA on `device` waits on an mbarrier that
 * nothing completes, gives up after `polls` polls and records that in a device
 * error word, read back into *gave_up (1 when the wait gave up).  The device
 * stays usable afterwards.  A production kernel that gives up the same way
 * makes the next synchronising call on its handle return TCSEM_ERR_CUDA. */
tcsem_status tcsem_selftest_bounded_wait(int device, int polls, int *gave_up);

/* Self-test of the bounded wait of the persistent batch schedule (persistent_batch; no
 * counterpart in the reference): its kernel runs on one CTA of `device` with a queue that
 * expects one stage and has no slot to publish it, so the CTA's wait for a ready stage gives
 * up after wait_ns nanoseconds and records that in the schedule's error word, read back into
 * *gave_up (1 when the wait gave up).  The device stays usable afterwards.  In a batch, a wait
 * that gives up the same way also marks every slot's error word, and the next tcsem_batch_poll
 * (or tcsem_batch_traces of a slot) returns TCSEM_ERR_CUDA. */
tcsem_status tcsem_selftest_queue_wait(int device, long long wait_ns, int *gave_up);

#ifdef __cplusplus
}
#endif

#endif /* TCSEM_H_INCLUDED */
