/*
 * ptask_gb300.h -- C ABI of the GB300 FDTD task runtime (libptask_gb300.so).
 *
 * This is the thin layer between host code (the PTask-compatible C++ runtime in include/ptask/,
 * Python through ctypes, or any FFI) and the sm_103a kernels.  Every signature uses plain C types:
 * pointers, sizes and status codes.  No CUDA or torch type appears here; streams are passed as
 * opaque `void*` (a cudaStream_t, or NULL for the library's own stream).
 *
 * Each entry point names the reference interface it replaces (paths inside rossbach/ptask).
 *
 * Error behaviour: every function returns PTK_OK (0) or a PTK_ERR_* code and records a message
 * retrievable with ptk_last_error() (thread-local).  Nothing here exits the process; the C++ facade
 * reproduces the reference's print-and-exit policy (Runtime::HandleError, PTaskRuntime.cpp) on top.
 *
 * Field layout at the boundary is the reference's: a field with extents (d1,d2,d3) is a dense FP32
 * array indexed i + j*d1 + k*d1*d2 (ptaskUnitTest/Simple3DArray.h:33) with
 *   Hx(Nx+1,Ny,Nz) Hy(Nx,Ny+1,Nz) Hz(Nx,Ny,Nz+1) Ex(Nx,Ny+1,Nz+1) Ey(Nx+1,Ny,Nz+1) Ez(Nx+1,Ny+1,Nz)
 * (ptaskUnitTest/graphfdtd.cpp:68-86).  Field order in every array-of-six argument is
 * Hx, Hy, Hz, Ex, Ey, Ez.  Per-cell coefficient arrays (Ca, Cb, Da, Db) have extents (Nx,Ny,Nz).
 */
#ifndef PTASK_GB300_H
#define PTASK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mirror the failure classes of PTRESULT, ptask/primitive_types.h:33-77) ---- */
#define PTK_OK            0
#define PTK_ERR_INVALID   1   /* bad argument / shape */
#define PTK_ERR_CUDA      2   /* a CUDA call failed */
#define PTK_ERR_NOMEM     3   /* device or host allocation failed */
#define PTK_ERR_STATE     4   /* call not valid in the object's current state */
#define PTK_ERR_TIMEOUT   5   /* bounded wait expired */
#define PTK_ERR_BUDGET    6   /* request does not fit the HBM budget */
#define PTK_ERR_NOTFOUND  7   /* unknown kernel / ticket */

/* Location of a buffer argument. */
#define PTK_HOST    0
#define PTK_DEVICE  1

/* By-value kernel constants; same layout and meaning as FDTD_PARAMS (graphfdtd.h:6-19). */
typedef struct ptk_fdtd_params {
    int   Nx, Ny, Nz;
    float Cx, Cy, Cz;      /* 1/dx, 1/dy, 1/dz (the reference sets N/L) */
    float eps0, mu0, c0;
    float Dt;
} ptk_fdtd_params;

/* Field identifiers, also the kernel identifiers of the reference's six tasks
 * (HxComputation .. EzComputation, graphfdtd.cpp:458-597). */
enum { PTK_HX = 0, PTK_HY = 1, PTK_HZ = 2, PTK_EX = 3, PTK_EY = 4, PTK_EZ = 5 };

/* ============================== runtime / device ============================================= */

/* Last error message of the calling thread ("" when none). */
const char *ptk_last_error(void);

/* Select and initialise the CUDA device.  Replaces Runtime::Initialize (ptask/PTaskRuntime.h:182)
 * and the CUDA accelerator discovery (ptask/cuaccelerator.cpp:329).  Idempotent. */
int ptk_runtime_init(int device);

/* Release pooled memory, cached CUDA graphs and streams.  Replaces Runtime::Terminate
 * (ptask/PTaskRuntime.h:214). */
int ptk_runtime_shutdown(void);

/* Device description: name (NUL-terminated, up to `name_len` bytes), SM count, total and free HBM. */
int ptk_device_info(char *name, int name_len, int *sm_count, size_t *total_bytes, size_t *free_bytes);

/* The runtime can execute a kernel for `file`/`entry` if the entry is a registered native kernel.
 * Replaces Runtime::CanExecuteKernel (ptask/PTaskRuntime.h:264).  Returns 1 / 0. */
int ptk_can_execute_kernel(const char *file);

/* Resolve a (file, entry) pair, as passed to Runtime::GetCompiledKernel (PTaskRuntime.h:540), to a
 * registered native kernel id.  The file part (e.g. "fdtdMain.compute_10.ptx") is ignored: there is
 * no JIT, kernels are linked sm_103a code.  Returns PTK_ERR_NOTFOUND for unknown entries. */
int ptk_kernel_lookup(const char *file, const char *entry, int *kernel_id);

/* Number of inputs/outputs and by-value constant size of a registered kernel. */
int ptk_kernel_signature(int kernel_id, int *n_inputs, int *n_outputs, int *const_bytes);

/* ============================== memory, streams, events ======================================= */
/* These replace PCUBuffer (ptask/PCUBuffer.cpp:929 cuMemAlloc, :591 cuMemcpyHtoDAsync,
 * :272 cuMemcpyDtoHAsync), CUAsyncContext (ptask/CUAsyncContext.cpp:87-176) and BlockPool
 * (ptask/BlockPool.cpp:292): allocations come from a stream-ordered device pool. */

int ptk_mem_alloc(size_t bytes, void *stream, void **dptr);
int ptk_mem_free(void *dptr, void *stream);
/* Pinned host memory.  Freed buffers are kept, by exact size, for the next allocation of that size
 * (page-locking tens of megabytes takes milliseconds); at most 4 GiB stay cached for the life of
 * the process, beyond that buffers go back to the driver.  Free a buffer only after the copies
 * from or into it have completed. */
int ptk_host_alloc(size_t bytes, void **hptr);
int ptk_host_free(void *hptr);
int ptk_memcpy_h2d(void *dst, const void *src, size_t bytes, void *stream);
int ptk_memcpy_d2h(void *dst, const void *src, size_t bytes, void *stream);
int ptk_memcpy_d2d(void *dst, const void *src, size_t bytes, void *stream);
int ptk_memset(void *dst, int value, size_t bytes, void *stream);
int ptk_stream_create(void **stream);
int ptk_stream_destroy(void *stream);
int ptk_stream_sync(void *stream);
/* Wait for all work on the runtime's device (every stream).  Used around host tasks of the
 * dependent form without streams (LPFNDEPHOSTTASK), which may launch work on any stream. */
int ptk_device_sync(void);
/* Ordinal of the runtime's CUDA device (the dependent device a host task is handed). */
int ptk_device_ordinal(int *device);
int ptk_event_create(void **event);
int ptk_event_destroy(void *event);
int ptk_event_record(void *event, void *stream);
int ptk_event_sync(void *event);
int ptk_event_query(void *event);                            /* PTK_OK when complete, PTK_ERR_STATE if not */
int ptk_stream_wait_event(void *stream, void *event);
int ptk_event_elapsed_ms(void *start, void *stop, float *ms);
/* Bytes currently reserved by the runtime's device pool. */
int ptk_pool_stats(size_t *reserved_bytes, size_t *used_bytes);
/* Allocations that failed, found the pool's cached free blocks fragmented, trimmed the cache back
 * to the driver (after the queued frees ran) and succeeded or failed on the retry. */
long long ptk_pool_trim_count(void);
/* Kernel launches issued by this library since load (each CUDA-graph replay adds its node count). */
long long ptk_launch_count(void);

/* ============================== reference task kernels ======================================== */

/* Launch one of the six per-field update tasks with the reference's formal-parameter order
 * (three input fields, the FDTD_PARAMS constant, the output field; graphfdtd.cpp:398-436 and the
 * port/parameter binding of ptask/cutask.cpp:381-433).  All pointers are device pointers in the
 * reference's dense layout.  Replaces CUTask::PlatformSpecificDispatch (ptask/cutask.cpp:634-705)
 * for the kernels HxComputation .. EzComputation.  Arithmetic is FP32 with every operation
 * rounded separately, bit-identical to fdtd_Hx..EzComputation_cpu (graphfdtd.cpp:185-312):
 *   field=PTK_HX: in0=Hx in1=Ey in2=Ez     field=PTK_EX: in0=Ex in1=Hy in2=Hz
 *   field=PTK_HY: in0=Hy in1=Ex in2=Ez     field=PTK_EY: in0=Ey in1=Hx in2=Hz
 *   field=PTK_HZ: in0=Hz in1=Ex in2=Ey     field=PTK_EZ: in0=Ez in1=Hx in2=Hy */
int ptk_launch_field_update(int field, const float *in0, const float *in1, const float *in2,
                            const ptk_fdtd_params *p, float *out, void *stream);

/* Fused half-step tasks over dense reference-layout device arrays (one launch updates all three
 * components; the output arrays must not alias the inputs).  Scalar vacuum coefficients from p.
 * Equivalent to the three H tasks (graphfdtd.cpp:185-240) / three E tasks (:243-312). */
int ptk_launch_h_half_step(const float *const in[6], float *const out_h[3],
                           const ptk_fdtd_params *p, void *stream);
int ptk_launch_e_half_step(const float *const e_in[3], const float *const h_new[3],
                           float *const out_e[3], const ptk_fdtd_params *p, void *stream);

/* In-place half-step tasks of the cyclic FDTD graph with per-cell coefficients (dense reference
 * layout; Da, Db, Ca, Cb have extents (Nx,Ny,Nz), wall nodes use the nearest cell).  They replace the
 * three H tasks (graphfdtd.cpp:185-240) and the three E tasks (:243-312) of one step.
 *   H' = Da*H + Db*curl(E)           E' = Ca*E + Cb*curl(H')  (PEC walls untouched)
 * When wave/step_counter are given, wave[*step_counter] is added to Ez at interior node (si,sj,sk)
 * after its update and *step_counter (a device int) is incremented. */
int ptk_launch_h_step_coef(float *const h[3], const float *const e[3], const float *Da,
                           const float *Db, const ptk_fdtd_params *p, void *stream);
int ptk_launch_e_step_coef(float *const e[3], const float *const h[3], const float *Ca,
                           const float *Cb, const ptk_fdtd_params *p, int si, int sj, int sk,
                           const float *wave, int nwave, int *step_counter, void *stream);

/* CUDA-graph capture of a sequence of launches on `stream` (the scheduler's replay of an iteration
 * cycle; replaces per-task dispatch, ptask/task.cpp:3822-3900).  kernel_nodes is the number of
 * kernels one replay runs (for the launch counter). */
int ptk_capture_begin(void *stream);
int ptk_capture_end(void *stream, void **graph_exec);
int ptk_graph_exec_launch(void *graph_exec, void *stream, long long kernel_nodes);
int ptk_graph_exec_destroy(void *graph_exec);

/* ============================== device-resident solver ======================================== */
/* One FDTD instance whose six fields, four coefficient arrays and source waveform stay in HBM.
 * The solver replays captured CUDA graphs of the fused Yee step (H then E in one kernel).  This is
 * what the PTask scheduler runs for an iterated FDTD cycle (the MF_GENERAL_ITERATOR loop of
 * ptask/MetaPort.cpp:927-1011 applied to the task pair of graphfdtd.cpp:448-733). */

typedef struct ptk_solver ptk_solver;

/* Tile shape of the fused step kernel.  by: rows per CTA (4, 8 or 16); kc: z-planes per CTA (>=1,
 * 0 = whole depth); vec: x cells per thread (1, 2 or 4; tiles are 32*vec cells wide, 0 = choose
 * from Nx); stages: 0 = operands loaded into registers, 2..6 = operands staged into shared memory
 * by TMA tensor copies with that many z-planes in the ring.  Staged tiles are 128 cells wide with
 * by 4, 8, 10 or 11 and 64 cells wide with by 7 (four-warp CTAs, three per SM) or 23 (vec is set
 * to match); 7, 10, 11 and 23 rows, and 5 and 6 stages, exist only with the material index
 * (ptk_solver_use_material_index) except 10 and 11 rows with 3 stages.  by = kc = 0 selects the default shape. */
typedef struct ptk_tile_config {
    int by;
    int kc;
    int vec;
    int stages;
} ptk_tile_config;

int ptk_solver_create(const ptk_fdtd_params *p, ptk_solver **out);
int ptk_solver_destroy(ptk_solver *s);
/* Set the six fields (reference layout, `where` = PTK_HOST or PTK_DEVICE). */
int ptk_solver_set_fields(ptk_solver *s, const float *const f[6], int where, void *stream);
/* Set per-cell coefficients (Nx*Ny*Nz each, `where` as above). */
int ptk_solver_set_coefficients(ptk_solver *s, const float *Ca, const float *Cb, const float *Da,
                                const float *Db, int where, void *stream);
/* Uniform vacuum coefficients Ca=Da=1, Cb=fl(Dt/eps0), Db=fl(Dt/mu0): the reference's scalar update. */
int ptk_solver_set_vacuum(ptk_solver *s, void *stream);
/* Soft source at Ez node (i,j,k), 1<=i<Nx, 1<=j<Ny, 0<=k<Nz: wave[n] is added after the E update
 * of step n (n counted from the last ptk_solver_reset_clock).  nwave=0 removes the source. */
int ptk_solver_set_source(ptk_solver *s, int i, int j, int k, const float *wave, int nwave,
                          int where, void *stream);
/* Restart the step counter used to index the source waveform. */
int ptk_solver_reset_clock(ptk_solver *s, void *stream);
/* Tile shape for subsequent runs (see ptk_tile_config). */
int ptk_solver_set_tiles(ptk_solver *s, const ptk_tile_config *cfg);
/* Coefficients with few distinct (Ca, Cb, Da, Db) tuples (at most 256, the usual case: a handful of
 * materials) are also kept as a one-byte material index per node plus a table; the staged kernel
 * then reads 49 bytes per cell update instead of 64, with identical results.  On by default;
 * `enable` = 0 keeps the per-cell arrays only.  The index is rebuilt whenever coefficients are set. */
int ptk_solver_use_material_index(ptk_solver *s, int enable, void *stream);
/* Materials in the current index (0: none, the per-cell arrays are read). */
int ptk_solver_material_count(const ptk_solver *s, int *nmat);
/* The step kernel the next run uses: ring stages (0 = register kernel) and whether it reads the
 * material index.  A staged shape with no per-cell-array instantiation falls back to 4 stages. */
int ptk_solver_kernel(const ptk_solver *s, int *stages, int *material_index);
int ptk_solver_get_tiles(const ptk_solver *s, ptk_tile_config *cfg);
/* Advance `steps` time steps, asynchronously on `stream`. */
int ptk_solver_run(ptk_solver *s, int steps, void *stream);
/* Read the six fields back (reference layout). */
int ptk_solver_get_fields(ptk_solver *s, float *const f[6], int where, void *stream);
/* Device bytes held by the solver. */
int ptk_solver_bytes(const ptk_solver *s, size_t *bytes);
/* Number of kernel launches issued by the last ptk_solver_run (graph nodes included). */
int ptk_solver_last_launches(const ptk_solver *s, long long *launches);

/* One-call solve with host buffers: upload fields + coefficients + source, run, download.
 * Ca..Db may be NULL for vacuum coefficients; wave may be NULL for no source.  fields[] are
 * updated in place.  The call is synchronous.  `ms` (optional) receives the wall time of the
 * whole call measured with CUDA events on the solver stream. */
int ptk_fdtd_solve(const ptk_fdtd_params *p, float *const fields[6], const float *Ca,
                   const float *Cb, const float *Da, const float *Db, int si, int sj, int sk,
                   const float *wave, int nwave, int steps, float *ms);

/* Allocation-free solve.  No counterpart in the reference.  It is for callers that must not have a
 * library allocate GPU memory: a plugin whose host application hands out all device memory from its
 * own arena and budget (a private cudaMalloc bypasses that accounting and can fail when the arena
 * holds the rest of the GPU), and latency-critical loops that cannot take cudaMalloc / cudaFree
 * (they may synchronise the device, and their latency is unbounded).
 * fields[6] (device, reference layout) are advanced `steps` steps in place with the fused kernel;
 * Ca..Db (device, Nx*Ny*Nz each) may all be NULL for vacuum coefficients; wave (device) may be NULL.
 * stream NULL means the current device's default stream.  All scratch lives in one static device
 * array of ptk_fdtd_static_scratch_bytes() bytes (48 MiB) that every GPU loading the library holds
 * until exit: cubes up to 89^3 fit (padded node count roundup(Nx+1,32)*(Ny+1)*(Nz+1) up to 786,424);
 * larger grids are rejected with PTK_ERR_BUDGET before any device work.  No cudaMalloc, cudaFree or
 * other allocating routine is called.  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress) with that device current and keeps it: make that call before any stream
 * capture, and make no call on a device after cudaDeviceReset.  Calls share the array, which keeps
 * the previous call's contents (each call clears what it uses): calls whose GPU work overlaps race
 * and must be serialised by the caller. */
int ptk_fdtd_solve_static(const ptk_fdtd_params *p, float *const fields[6], const float *Ca,
                          const float *Cb, const float *Da, const float *Db, int si, int sj, int sk,
                          const float *wave, int nwave, int steps, void *stream);
size_t ptk_fdtd_static_scratch_bytes(void);

/* ============================== batched / served FDTD ========================================= */
/* Many device-resident FDTD instances of uneven size advanced together: every time step of every
 * active instance is one persistent launch of the fused step kernel over the concatenated tile lists,
 * chunks of steps are replayed as CUDA graphs, and requests are admitted continuously by HBM budget
 * as earlier ones finish.  No reference counterpart: the reference pipelines numBlocks copies of one
 * problem through one graph (graphfdtd.cpp:1076-1097) with one dispatch per task per copy. */

typedef struct ptk_server ptk_server;
struct ptk_problem_desc;   /* defined with the problem generator below */

typedef struct ptk_server_config {
    size_t hbm_budget_bytes;   /* device bytes the admitted instances may hold (0: 80% of free HBM) */
    int max_active;            /* instance slots (0: unlimited; 1: plain one-at-a-time dispatch) */
    int chunk_steps;           /* steps per replayed graph between admission points (0: 32) */
    int tile_rows;             /* fused-kernel tile rows 4, 8 or 16, or 7, 10, 11 or 23 with the
                                  staged kernel (7- and 23-row tiles are 64 cells wide, the others
                                  128; 0: 11 for the staged kernel, 8 for the register kernel) */
    int keep_results;          /* keep finished fields for ptk_server_fetch */
    int persistent;            /* persistent grid of resident CTAs instead of one CTA per tile */
    int stages;                /* step kernel: 0 = TMA-staged with its default ring (3 planes for 4 rows,
                                  else 4; 16 rows become 8), 2..6 = TMA-staged with that many planes where
                                  the rows have that shape, -1 = register kernel */
} ptk_server_config;

typedef struct ptk_request_info {
    long long ticket;
    int Nx, Ny, Nz, steps;
    double arrival_s, admit_s, finish_s;   /* run clock; admit/finish < 0 when not yet */
    double checksum[6];                    /* FP64 sums of the six result fields */
    int done;
} ptk_request_info;

typedef struct ptk_server_stats {
    long long submitted, completed;
    double wall_s;                 /* time spent in ptk_server_run */
    double solves_per_s;
    double p50_latency_s, p99_latency_s, mean_latency_s;   /* finish - arrival */
    double cell_updates, mcells_per_s;
    long long chunks, kernel_launches;
    int peak_active;
    size_t peak_bytes;
    /* where wall_s went: device time of the replayed chunks (CUDA events around each replay), and
     * host time spent admitting requests (allocation, problem generation, material index, tensor
     * maps), retiring them (checksums, result copies) and scheduling (work list, graph capture) */
    double chunk_device_s, admit_s, retire_s, schedule_s;
    long long graph_captures;
    long long admit_waits;         /* admissions put off because the pool had no block that fit */
} ptk_server_stats;

int ptk_server_create(const ptk_server_config *cfg, ptk_server **out);
/* Queue a request: a seeded problem (ptk_problem_desc) with zero initial fields, arriving at
 * arrival_s on the trace clock.  Rejects requests larger than the whole budget. */
int ptk_server_submit(ptk_server *s, const struct ptk_problem_desc *d, double arrival_s, long long *ticket);
/* Serve every queued request.  Arrival times are multiplied by time_scale (0: all available at
 * once); requests are admitted in arrival order as they arrive and fit the HBM budget.  A request
 * that fits the budget but finds no free device block waits for running requests to retire.
 * submit, run, request, fetch and stats_get are serialised by the server's lock: called from
 * another thread during a run, they wait for it to finish. */
int ptk_server_run(ptk_server *s, double time_scale);
int ptk_server_request(ptk_server *s, long long ticket, ptk_request_info *info);
/* Host copy of a finished request's fields (reference layout); needs keep_results. */
int ptk_server_fetch(ptk_server *s, long long ticket, float *const fields[6]);
int ptk_server_stats_get(ptk_server *s, ptk_server_stats *st);
int ptk_server_destroy(ptk_server *s);

/* ============================== self-test of the bounded waits ================================ */
/* The staged step kernel waits for its TMA copies on mbarriers for at most 1 s of global time (and
 * at most 2^22 polls) and, when a wait runs out, raises an error word, lets its copies in flight land and returns; the host
 * then reports PTK_ERR_TIMEOUT instead of hanging.  This launches one CTA that arms an mbarrier for
 * 16 bytes of transactions that nothing delivers (no copy is issued) and waits on it with the same
 * bounded wait.  Returns PTK_ERR_TIMEOUT with *error_word = 1 and *elapsed_ms = the launch's device
 * time when the wait ran out as designed; the context stays usable.  No reference counterpart. */
int ptk_selftest_wait_expiry(int *error_word, float *elapsed_ms);

/* ============================== autotuner ===================================================== */
/* Time candidate tile shapes for a grid of the given size on the current device and return the
 * fastest (cached per shape for the life of the process). */
int ptk_autotune_tiles(int Nx, int Ny, int Nz, ptk_tile_config *best, float *best_ms_per_step);
/* Tile shape without timing anything: the autotuner's choice when this process has tuned the
 * shape already, else the TMA-staged material-index kernel with 11-row tiles, a 4-plane ring and
 * the z depth that fills whole waves of resident CTAs best.  The PTask graph's loop lowering uses
 * it, so that a graph built for one request does not pay for a full autotuning pass.  Needs the
 * runtime to be initialised (the resident CTA count comes from the device). */
int ptk_default_tiles(int Nx, int Ny, int Nz, ptk_tile_config *cfg);

/* ============================== synthetic problems ============================================ */
/* Seeded problem generator used by tests and benchmarks: vacuum plus axis-aligned dielectric boxes
 * (eps_r uniform in [eps_min, eps_max], edges uniform in [box_min, box_max]), PEC walls, Courant
 * number `courant`, Gaussian soft Ez source.  Deterministic for a seed on every host. */
typedef struct ptk_problem_desc {
    int      Nx, Ny, Nz;
    int      n_boxes;
    float    eps_min, eps_max;
    int      box_min, box_max;
    float    courant;          /* Dt = courant / (c0 * sqrt(Cx^2+Cy^2+Cz^2)) */
    int      steps;            /* length of the waveform to generate */
    int      source_mode;      /* 0 none, 1 centre, 2 seeded interior position */
    uint64_t seed;
} ptk_problem_desc;

/* Fill params, the four coefficient arrays (Nx*Ny*Nz floats each, may be NULL to skip), the source
 * position and the waveform (`steps` floats, may be NULL). */
int ptk_problem_generate(const ptk_problem_desc *d, ptk_fdtd_params *p, float *Ca, float *Cb,
                         float *Da, float *Db, int *si, int *sj, int *sk, float *wave);

/* The reference's constants for an (Nx,Ny,Nz) cavity (graphfdtd.cpp:1357-1381: Lx=.05, Ly=.04,
 * Lz=.03, Courant about 0.01). */
int ptk_reference_params(int Nx, int Ny, int Nz, ptk_fdtd_params *p);

/* Seeded uniform fill in [0, scale) (stand-in for configure_raw_array, graphfdtd.cpp:106-126, whose
 * time(NULL) seed made runs unrepeatable). */
int ptk_fill_uniform(float *dst, size_t n, float scale, uint64_t seed);

#ifdef __cplusplus
}
#endif
#endif /* PTASK_GB300_H */
