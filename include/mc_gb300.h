/*
 * mc_gb300.h -- C ABI of the GB300 (sm_103a) phonon particle-advance library.
 *
 * The library replaces the run loop of montecarlocpp's field problems,
 * `ArrayXXd FieldProblem::solve(Rng& gen, Progress* prog) const`
 * (montecarlo/problem.h:141, montecarlo/problem.cpp:370-445), with
 * hand-written CUDA kernels. Plain pointers and sizes only; all device memory
 * is owned by the library; every entry point returns an int status
 * (MC_OK = 0, negative on error, message from mc_last_error()) where the
 * reference aborts on BOOST_ASSERT_MSG. There is no CPU fallback: without a
 * CUDA device the compute entry points return MC_ERR_NO_DEVICE.
 *
 * Array layouts: matrices are row-major (M[3*r + c], columns of M are the
 * edge vectors as in the reference's Parallelepiped(o, mat, ...)); field
 * results are rows x cols in COLUMN-major order, i.e. the memory layout of
 * the reference's Eigen::ArrayXXd, so a C++ caller can wrap the buffer with
 * Eigen::Map<ArrayXXd>(out, rows, cols).
 */
#ifndef MC_GB300_H
#define MC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define MC_OK 0
#define MC_ERR_ARG (-1)          /* invalid argument (reference: assert)  */
#define MC_ERR_CUDA (-2)         /* CUDA runtime error                     */
#define MC_ERR_NO_DEVICE (-3)    /* no CUDA device: no CPU fallback        */
#define MC_ERR_UNSUPPORTED (-4)  /* geometry outside the kernels' limits   */
#define MC_ERR_IO (-5)           /* file could not be read                 */
#define MC_ERR_REPLAY (-6)       /* replay stream exhausted                */
#define MC_ERR_NONFINITE (-7)    /* non-finite phonon state                */
#define MC_ERR_BUSY (-8)         /* admission refused (serving)            */
#define MC_ERR_TIMEOUT (-9)      /* a bounded device-side wait gave up     */
#define MC_ERR_CANCELLED (-10)   /* request cancelled (serving)            */

/* Message of the last error on the calling thread. */
const char* mc_last_error(void);
/* Library version string. */
const char* mc_version(void);

/* ------------------------------------------------------------- material */
typedef struct mc_material_s* mc_material_h;

/* Material(disp, relax, T) from the parsed file contents
 * (montecarlo/material.cpp:154-234): disp is nw rows of
 * (omega, domega, (vel_p, dos_p) x np) row-major; relax is np rows of 8
 * coefficients (two terms c0 w^c1 T^c2 exp(-c3/T)). */
int mc_material_create(const double* disp, long nw, long np, const double* relax, double T,
                       mc_material_h* out);
/* Material(disp, relax, T) reading the two files
 * (montecarlo/material.cpp:158-186). */
int mc_material_load(const char* disp_path, const char* relax_path, double T, mc_material_h* out);
/* Material(disp, relax, T[t]) for n temperatures at once (no counterpart
 * in the reference, which builds one Material per run; it serves batches
 * and request streams of many temperatures): the temperature-dependent
 * tables of montecarlo/material.cpp:116-161 -- relaxation times, the
 * energy, flux and scattering pdfs, their sums and the inverse-CDF
 * thresholds -- are built on the GPU in one launch. out[t] is, bit for bit,
 * the material mc_material_create(disp, nw, np, relax, T[t]) returns: both
 * builds evaluate the same FP64 formulas in the same order. Synchronous. */
int mc_material_create_many(const double* disp, long nw, long np, const double* relax, const double* T, int n,
                            mc_material_h* out);
/* The integer inverse-CDF thresholds the kernels sample (no counterpart in
 * the reference, whose Boost discrete distributions hold their own
 * tables): scattering bins (nw) and branches (nw x np), flux bins and
 * branches; threshold = ceil(cdf * 2^32). Any pointer may be NULL. */
int mc_material_thresholds(mc_material_h m, uint64_t* swthr, uint64_t* spthr, uint64_t* fwthr, uint64_t* fpthr);
/* energySum, fluxSum, scatSum, cond (montecarlo/material.h:55,62-64). */
int mc_material_sums(mc_material_h m, double out[4]);
/* vel and tau tables, nw x np row-major (montecarlo/material.cpp:246-256). */
int mc_material_tables(mc_material_h m, double* vel, double* tau);
void mc_material_destroy(mc_material_h m);

/* --------------------------------------------------------------- domain */
typedef struct mc_domain_s* mc_domain_h;

enum { MC_SPEC = 0, MC_DIFF = 1, MC_ISOT = 2, MC_PERI = 3, MC_INTER = 4 };

/* Parallelepiped<Bac, Lef, Bot, Fro, Rig, Top>(o, mat, div, gradT, T)
 * (montecarlo/subdomain.h:145-158); faces in bdry<0..5>() order. */
typedef struct {
    double o[3];
    double M[9];
    long div[3];
    double gradT[3];
    int kind[6];
    double T[6];
} mc_pped_desc;

/* makePair(bdry1, bdry2[, transl, rot]) (montecarlo/boundary.cpp:361-369
 * for Inter, montecarlo/boundary.cpp:524-550 for Peri). */
typedef struct {
    int kind;
    int sdom1, face1;
    int sdom2, face2;
    double transl[3];
    double rot[9];
} mc_pair_desc;

/* Domain assembly (montecarlo/domain.cpp:88-102 addSdom and the
 * init() of each domain). Limits: <= 64 subdomains, <= 512 cells per axis
 * per subdomain. */
int mc_domain_create(const mc_pped_desc* ppeds, int n, const mc_pair_desc* pairs, int npairs,
                     mc_domain_h* out);

/* Subdomain shapes (montecarlo/subdomain.h:128-640). */
enum {
    MC_PARALLELEPIPED = 0,   /* 3 columns; faces Bac Lef Bot Fro Rig Top            */
    MC_TRIANGULAR_PRISM = 1, /* 3 columns; faces Bac Lef Bot Dia Top               */
    MC_TETRAHEDRON = 2,      /* 3 columns; faces Bac Lef Bot Dia                   */
    MC_PRISM = 3,            /* N columns: axis, then the N - 1 base vertices;
                                faces Bot Top Sid0 .. Sid(N-1)                     */
    MC_PYRAMID = 4           /* N columns: apex, then the N - 1 base vertices;
                                faces Bot Sid0 .. Sid(N-1)                         */
};
#define MC_MAX_SDOM_COLS 9
#define MC_MAX_SDOM_FACES 11

/* A subdomain of any shape: the constructor arguments (o, mat, div, gradT,
 * T) of Parallelepiped, TriangularPrism, Tetrahedron, Prism<N> and
 * Pyramid<N> (montecarlo/subdomain.h:145-158,224-236,303-314,386-410,
 * 524-547) and each face's kind, in bdry<I>() order. mat is column-major:
 * column c at mat[3c .. 3c + 2]. Prism and Pyramid take one division
 * count, div[0]: < 0 no field, else one column for the whole subdomain.
 * A subdomain takes one device slot, two when it has more than 6 faces or
 * an Inter face paired more than once (at most 64 slots, at most 6 faces
 * plus pair candidates beyond the first 6 faces); MC_ERR_UNSUPPORTED
 * otherwise. */
typedef struct {
    int shape;
    int ncols;
    double o[3];
    double mat[3 * MC_MAX_SDOM_COLS];
    long div[3];
    double gradT[3];
    int kind[MC_MAX_SDOM_FACES];
    double T[MC_MAX_SDOM_FACES];
} mc_sdom_desc;

/* mc_domain_create for subdomains of any shape; pairs name faces by their
 * bdry<I>() index in each subdomain. */
int mc_domain_create_shapes(const mc_sdom_desc* sdoms, int n, const mc_pair_desc* pairs, int npairs,
                            mc_domain_h* out);
/* Number of field columns (montecarlo/field.cpp:93-113). */
long mc_domain_cols(mc_domain_h d);
/* Cell volumes, one per column (CellVolF, montecarlo/problem.cpp:302-306). */
int mc_domain_cell_volumes(mc_domain_h d, double* out);
void mc_domain_destroy(mc_domain_h d);

/* -------------------------------------------------------------- problem */
/* MC_CUMTEMP / MC_CUMFLUX: CumTempProblem / CumFluxProblem
 * (montecarlo/problem.h:205-239): Temp / Flux binned by the scatter count
 * before each flight, cum_size + 1 bins of ceil((maxscat - 1) / cum_size)
 * scatters (bin 0: not yet scattered), returned as cumulative sums over
 * the bins (rows cum_size + 1, or 3 (cum_size + 1) with x, y, z per bin). */
enum { MC_TEMP = 0, MC_FLUX = 1, MC_MULTI = 2, MC_CUMTEMP = 3, MC_CUMFLUX = 4 };
enum { MC_TALLY_AUTO = -1, MC_TALLY_SHARED = 0, MC_TALLY_GLOBAL = 1 };

typedef struct {
    int problem;            /* MC_TEMP (1 row), MC_FLUX (3), MC_MULTI (4),
                               MC_CUMTEMP (cum_size + 1), MC_CUMFLUX
                               (3 (cum_size + 1))                          */
    long nemit;             /* requested phonons (montecarlo/problem.cpp:329-337 rounding) */
    long maxscat;
    long maxloop;           /* 0 -> 100 * maxscat (montecarlo/problem.cpp:339) */
    double dt;              /* step length, s                              */
    long nsteps;            /* time horizon = nsteps * dt                  */
    int precision;          /* 32: FP32 flight, 64: FP64 flight; tallies FP64 */
    uint64_t seed;          /* Philox key                                  */
    int steps_per_launch;   /* K dt-steps per advance launch (>= 1)        */
    int block_size;         /* 0 -> 256 (static schedule, FP32 flight: 768
                               consumer threads and a producer warp)       */
    int grid_blocks;        /* 0 -> resident blocks x SMs                  */
    int tally_mode;         /* MC_TALLY_*                                  */
    /* replay: per-phonon 32-bit words, offsets has nemit+1 entries (host) */
    const uint32_t* replay_words;
    const int64_t* replay_offsets;
    /* event log (host buffers, may be NULL): log_cap records of 12 doubles
     * per phonon id < log_phonons: loop index, subdomain, face hit (-1
     * scatter, -2 horizon, -3 escape), subdomain after, cell, x, y, z,
     * time, nscat, w, p */
    double* log;
    int64_t* log_counts;
    long log_cap;
    long log_phonons;
    void* stream;           /* cudaStream_t; NULL -> library stream        */
    int schedule;           /* MC_SCHED_*: static (state tiles streamed
                               through shared memory by bulk copies, one
                               phonon per thread, in place, partitioned by
                               next event within each tile), or dynamic
                               lane refill with in-place state             */
    int compact_interval;   /* dynamic schedule: compact dead slots every
                               this many launches (0: never)               */
    long cum_size;          /* MC_CUMTEMP / MC_CUMFLUX: bins after the first
                               (the reference's `size`, >= 1; maxscat >= 2) */
} mc_problem_desc;

enum { MC_SCHED_AUTO = 0, MC_SCHED_STATIC = 1, MC_SCHED_DYNAMIC = 2 };

typedef struct {
    long nemit;             /* phonons after rounding                      */
    double power;           /* montecarlo/problem.cpp:341                  */
    long rows, cols;
    double phonon_steps;    /* live phonon x dt-step pairs processed       */
    long events, scatters, escapes, horizon_stops, maxscat_stops, maxloop_stops, absorbed,
        nonfinite;
    unsigned status;        /* MC status bits (replay exhausted, nonfinite) */
    double kernel_ms;       /* device time of emission + advance launches   */
    int launches;
    double checksum[4];     /* per row: sum over every flight of its tally
                               amount before the cell split (equals the
                               raw tally summed over cells)                 */
} mc_stats;

/* Replaces FieldProblem::solve over all phonons of the problem
 * (montecarlo/problem.cpp:370-445) followed by the caller's reduction
 * (montecarlo/main.cpp:162-165): out is rows x cols column-major and holds
 * power * postProc(tally) / cellVol. Host buffers; synchronous. */
int mc_solve(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, double* out, mc_stats* st);

/* Repeated solves and their statistics: solveField(prob, nsim) followed by
 * calcStats (montecarlo/main.cpp:181-210) with Statistics' Welford update
 * (montecarlo/field.cpp:226-262). Replica i runs the problem with Philox key
 * p->seed + i (the reference seeds each run from random_device). mean and
 * sd (may be NULL) receive the cell-by-cell mean and sample standard
 * deviation (n - 1; zero for one replica), rows x cols column-major; st
 * (may be NULL) sums the replicas' counters and checksums. Replay streams
 * and logs are refused (MC_ERR_UNSUPPORTED). Host buffers; synchronous. */
int mc_solve_replicas(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, long nsim, double* mean, double* sd,
                      mc_stats* st);

/* No counterpart in the reference: a device self-check of the bounded
 * waits every asynchronous kernel here relies on. One block waits on an
 * mbarrier phase that nothing completes, with a deadline of limit_ms
 * (0 < limit_ms <= 1000); the wait must give up on its own. *status receives
 * the device status bits (8 = a wait gave up, which the solves report as
 * MC_ERR_TIMEOUT) and *waited_ms how long the wait took. The device stays
 * usable afterwards. */
int mc_check_bounded_wait(double limit_ms, unsigned* status, double* waited_ms);

/* Size of the fixed device scratch array behind mc_solve_noalloc: 32 MiB,
 * held on every device that loads this library until the process exits. */
#define MC_NOALLOC_SCRATCH_BYTES (32u << 20)

/* No counterpart in the reference: an extra entry point of this library.
 *
 * mc_solve without any device allocation. It is for callers that cannot
 * call cudaMalloc / cudaFree: a process whose device memory is already
 * owned by another allocator (a framework's caching pool, a runtime that
 * reserves most of the GPU at start-up), where a fresh cudaMalloc can fail
 * although that pool has room, and loops that cannot take the implicit
 * device-wide synchronisation of cudaFree. It calls no cudaMalloc,
 * cudaFree or other allocating routine: every device buffer of the solve
 * (tables, subdomain images, phonon state, counters, tally) is placed in
 * one file-scope device array of MC_NOALLOC_SCRATCH_BYTES. A problem that
 * needs more (48 B per phonon with FP32 flight, 80 B with FP64, plus the
 * tables and rows x cols x 8 B of tally) is rejected with MC_ERR_ARG
 * before any work is queued.
 *
 * Arguments, output and results are those of mc_solve, except: replay
 * streams and trajectory logs are rejected (MC_ERR_UNSUPPORTED); the
 * schedule is always the in-place dynamic one (p->schedule and
 * p->compact_interval are validated as mc_solve validates them, then not
 * used); a NULL p->stream means the legacy default stream; st->kernel_ms
 * is 0. Synchronous.
 *
 * The first call on a device looks up the array's device address there
 * (which can also load this library's device code on that device): make
 * that first call before any stream capture begins. All calls on a device
 * share the one array, which keeps the last call's contents; each call
 * clears what must start at zero (counters, status word, tally, checksum)
 * and overwrites the rest before reading it. Calls whose GPU work overlaps
 * (from two host threads, say) race on the array and corrupt each other's
 * results: serialise them. */
int mc_solve_noalloc(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, double* out, mc_stats* st);

/* ---------------------------------------------- device-resident session */
typedef struct mc_session_s* mc_session_h;

/* Allocate the phonon structure of arrays and tables on the device. A
 * session's buffers come from the device's default stream-ordered memory
 * pool (cudaMallocAsync on the session stream, freed with cudaFreeAsync by
 * mc_session_destroy); the library raises that pool's release threshold so
 * that freed memory stays with the process for the next session, and
 * creating or destroying a session never synchronises the device. A caller
 * that wants the memory back calls cudaMemPoolTrimTo on the default pool.
 * mc_solve uses a session. */
int mc_session_create(mc_material_h m, mc_domain_h d, const mc_problem_desc* p, mc_session_h* out);
/* Emit all phonons (reset tally, counters and time). Asynchronous. */
int mc_session_emit(mc_session_h s);
/* Launch up to `nlaunch` advance windows; *done = 1 once the horizon is
 * reached. Asynchronous on the session stream. */
int mc_session_advance(mc_session_h s, int nlaunch, int* done);
/* Synchronise; copy the post-processed field (may be NULL) and stats. */
int mc_session_result(mc_session_h s, double* out, mc_stats* st);
/* Bytes the phonon state of this session occupies on the device. */
size_t mc_session_state_bytes(mc_session_h s);
/* Snapshot and resume (no counterpart in the reference, whose solves run
 * to completion in one call): mc_session_snapshot synchronises and copies
 * everything a session needs to continue -- the live phonon state, live
 * counts, counters, status, raw field, checksums and replay cursors -- into
 * a host buffer of mc_session_snapshot_bytes(s) bytes; mc_session_restore
 * loads such a buffer into a session created with the same material,
 * domain and problem description (checked), which then continues with
 * mc_session_advance exactly as the original would have: every phonon's
 * random numbers depend only on its id and event index. Sessions that log
 * trajectories are refused (MC_ERR_UNSUPPORTED). */
size_t mc_session_snapshot_bytes(mc_session_h s);
int mc_session_snapshot(mc_session_h s, void* buf, size_t bytes);
int mc_session_restore(mc_session_h s, const void* buf, size_t bytes);
void mc_session_destroy(mc_session_h s);

/* ------------------------------------------------------------ batches */
/* Many solves -- each its own Material, Domain and problem, with uneven
 * phonon counts -- run to one time horizon in ONE persistent kernel launch
 * per window: each lane takes a phonon of any instance and works against
 * that instance's tables, geometry and field. With use_graph the launch
 * sequence is captured into a CUDA graph on the first run and replayed. */
typedef struct mc_batch_s* mc_batch_h;

typedef struct {
    double dt;              /* shared time step, s                         */
    long nsteps;            /* shared horizon = nsteps * dt                */
    int precision;          /* 32 or 64                                    */
    int steps_per_launch;   /* 0: the whole horizon in one launch          */
    int block_size;         /* 0 -> 256                                    */
    int grid_blocks;        /* 0 -> resident blocks x SMs                  */
    int use_graph;          /* capture and replay the launch sequence      */
    void* stream;           /* cudaStream_t; NULL -> library stream        */
} mc_batch_desc;

/* n instances; from probs[i] the batch uses problem, nemit, maxscat,
 * maxloop and seed (the time and launch fields come from bd). */
int mc_batch_create(int n, const mc_material_h* mats, const mc_domain_h* doms, const mc_problem_desc* probs,
                    const mc_batch_desc* bd, mc_batch_h* out);
/* Emission, every window and the field finish of all instances;
 * asynchronous on the batch stream. */
int mc_batch_run(mc_batch_h b);
/* Synchronise; instance i's field (rows x cols, column-major, as mc_solve)
 * and its stats (nemit, power, rows, cols, checksum; counters are
 * batch-wide). out may be NULL. */
int mc_batch_result(mc_batch_h b, int i, double* out, mc_stats* st);
/* Batch-wide counters of the last run (synchronises). */
int mc_batch_stats(mc_batch_h b, mc_stats* st);
size_t mc_batch_state_bytes(mc_batch_h b);
void mc_batch_destroy(mc_batch_h b);

/* ------------------------------------------------------------ serving */
/* A request loop on a library thread (no counterpart in the reference,
 * whose solves run one at a time to completion). Submitted solves are
 * admitted against an HBM budget: a solve is admitted when the phonon state
 * of its first round fits into a free range of the server's state buffer,
 * and keeps that state resident on the device for the whole round. Rounds
 * run in windows of steps_per_window dt-steps; every tick advances one
 * window of every admitted solve -- each with its own Material, Domain,
 * phonon count and Philox key -- in ONE persistent batched launch, so a
 * request that arrives while others are on the device joins them at the
 * next window and their work overlaps. A round splits its phonons into
 * `groups` batch means; a solve completes when the standard error of
 * kappa = -<q_axis> / gradT_axis is at most target_rel_se of its mean. The
 * first round has the requested phonons; each later round the estimated
 * remainder to the target (at least the requested count, at most a quarter
 * of the budget), and the error pools the rounds' batch means weighted by
 * their phonons. State slots are given out first come, first served
 * (solves between rounds before new requests). A solve's result depends
 * only on its own request and the server's dt, horizon, window, groups and
 * stopping rule: the same alone and in any mix. */
typedef struct mc_server_s* mc_server_h;

typedef struct {
    double dt;              /* time step, s                                 */
    long nsteps;            /* horizon of each round = nsteps * dt          */
    int precision;          /* 32 or 64                                     */
    size_t hbm_budget;      /* bytes of phonon state resident at once       */
    int max_active;         /* solves per tick (<= 512)                     */
    int groups;             /* batch means per round, 2..8                  */
    double target_rel_se;   /* e.g. 0.01                                    */
    int min_rounds;         /* rounds before the stopping rule applies     */
    int max_rounds;         /* give up (status MC_ERR_BUSY) after this many */
    int block_size;         /* 0 -> 256                                     */
    int steps_per_window;   /* dt-steps per tick, a divisor of nsteps; 0: the
                               largest divisor of nsteps <= nsteps / 2      */
} mc_server_desc;

typedef struct {
    mc_material_h mat;      /* kept alive by the caller until completion    */
    mc_domain_h dom;
    int problem;            /* MC_FLUX or MC_MULTI                          */
    long nemit;             /* phonons of the first round                   */
    long maxscat, maxloop;
    uint64_t seed;          /* round r uses seed + r                        */
    int axis;               /* flux / gradient axis                         */
    double volume;          /* averaging volume (0: sum of cell volumes)    */
    double gradient;        /* gradT along the axis (0: the first subdomain's) */
    int field;              /* 1: keep the mean field (returned at the end);
                               0: kappa only -- flights are not split over
                               cells, kappa comes from the per-flight sums  */
    int max_rounds;         /* this request's round limit (0: the server's) */
} mc_request;

typedef struct {
    double kappa, kappa_se; /* W / m / K                                    */
    long rounds, phonons;
    double phonon_steps;
    double t_submit, t_admit, t_done;  /* seconds on the server clock       */
    int status;             /* MC_OK; MC_ERR_BUSY if its max_rounds ran out
                               or its first round can never fit the budget;
                               MC_ERR_CANCELLED after mc_server_cancel;
                               MC_ERR_NONFINITE if its phonons went
                               non-finite                                   */
} mc_result;

typedef struct {
    long submitted, admitted, completed, queued, active, ticks;
    double busy_s, uptime_s, phonon_steps;
} mc_server_counters;

int mc_server_create(const mc_server_desc* d, mc_server_h* out);
/* Thread-safe; returns at once with a ticket. A request with invalid
 * host inputs (null handles, nemit <= 0, an axis outside 0..2, a volume or
 * gradient that is not finite, a negative max_rounds) is refused with
 * MC_ERR_ARG and gets no ticket; the requests already submitted are not
 * affected. */
int mc_server_submit(mc_server_h s, const mc_request* r, long* ticket);
/* Cancel a request: a queued one at once, a running one at the next window
 * boundary (its device state is released then); its result reports
 * MC_ERR_CANCELLED. Returns 1 if it was cancelled, 0 if it had completed
 * already, < 0 for an unknown ticket. The other requests are not affected. */
int mc_server_cancel(mc_server_h s, long ticket);
/* 1 if done (result and, if field != NULL, the mean field rows x cols are
 * written), 0 if pending, < 0 on error. */
int mc_server_poll(mc_server_h s, long ticket, mc_result* res, double* field);
/* Block up to timeout_s; same return values as mc_server_poll. */
int mc_server_wait(mc_server_h s, long ticket, double timeout_s, mc_result* res, double* field);
int mc_server_stats(mc_server_h s, mc_server_counters* st);
/* Seconds on the server clock (the t_* fields of mc_result). */
double mc_server_clock(mc_server_h s);
void mc_server_destroy(mc_server_h s);

#ifdef __cplusplus
}
#endif

#endif /* MC_GB300_H */
