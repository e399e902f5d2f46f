/*
 * mara_gb300 — C ABI of the GB300-native Godunov finite-volume update.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns an int status (MARA_OK = 0, else a mara_status code; the message of
 * the last failure on the calling host thread is mara_last_error()).
 * Buffers marked "device" are caller-owned device memory; calls are
 * stream-ordered on `stream` (a cudaStream_t, NULL = legacy default stream)
 * and return before the GPU work finishes. The library allocates no device
 * memory on its own except where a function says so.
 *
 * Mesh layout (minidisk): structure-of-arrays, component-major [3][N][N]
 * (Σ, Σvx, Σvy); axis 0 = x is the slow index, axis 1 = y is contiguous,
 * N = block_size << depth; the reference's block (level=depth, bi, bj) owns
 * rows [bi*n, bi*n+n) and columns [bj*n, bj*n+n) of that mesh (the same
 * row-major cell order as the reference's nd::shared_array, src/core_ndarray.hpp:188).
 */
#ifndef MARA_GB300_H
#define MARA_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum mara_status {
    MARA_OK = 0,
    MARA_ERR_ARGUMENT = 1,   /* invalid argument (message says which) */
    MARA_ERR_CUDA = 2,       /* a CUDA runtime call failed */
    MARA_ERR_NUMERIC = 3,    /* a zone failed (negative pressure, no convergence) */
};

enum mara_precision {
    MARA_FP64 = 0,           /* plain FP64 path: the drop-in for the reference scheme */
    MARA_MIXED = 1,          /* FP32 reconstruction/fluxes/sources, FP64 state accumulation */
};

enum mara_dt_mode {
    MARA_DT_FORMULA = 0,     /* problems/minidisk.cpp:204-206 fixed formula with start-up ramp */
    MARA_DT_CFL = 1,         /* cfl * dl / max fastest wavespeed (reduction over the mesh) */
    MARA_DT_FORMULA_HELD = 2,/* the formula at the start of each advance call, held for all its steps:
                                the reference driver's fold batches (problems/minidisk.cpp:202-213) */
};

/* Field-for-field minidisk::solver_data_t (problems/minidisk.hpp:77-93), plus
 * the PLM theta that the reference hard-codes to 2.0
 * (problems/minidisk_scheme.cpp:313-314). */
typedef struct mara_minidisk_params {
    int32_t block_size;        /* zones per block side */
    int32_t depth;             /* mesh levels: 2^depth blocks per side */
    double omega_frame;        /* frame rotation rate */
    double mach_number;
    double nu;                 /* kinematic viscosity */
    double domain_radius;      /* half-size of the domain */
    double softening_length;
    double eccentricity;
    double mass_ratio;
    double sink_radius;
    double sink_rate;
    double buffer_rate;
    double buffer_scale;
    double cfl;
    double plm_theta;
} mara_minidisk_params;

/* Device-resident simulation clock of one minidisk run. The step functions
 * read and advance it on the device, so a sequence of steps needs no host
 * round trip (and can be captured in a CUDA graph). */
typedef struct mara_minidisk_clock {
    double time;               /* simulation time at the start of the next step */
    double dt;                 /* time step of the last / current step */
    double max_wavespeed;      /* fastest wavespeed of the current state (CFL mode) */
    int64_t iteration;         /* completed steps */
    double binary[2][6];       /* per RK stage: m1, x1, y1, m2, x2, y2 in the rotating frame */
} mara_minidisk_clock;

/* ---------------------------------------------------------------- library */
const char* mara_last_error(void);
const char* mara_version(void);

/* Upload an instantiated CUDA graph (a cudaGraphExec_t, e.g. the one a host
 * captured the advance calls into) to the device on `stream`, so that its
 * first launch costs no more than later ones. No counterpart in the
 * reference, which launches no graphs. */
int mara_graph_upload(void* graph_exec, void* stream);

/* ---------------------------------------------------------------- minidisk */

/* Binary state at time t in the rotating frame, computed on the host in FP64:
 * out = {m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2}. Replaces
 * two_body::orbital_state + two_body::rotate as used at
 * problems/minidisk_scheme.cpp:329-335 (src/physics_two_body.hpp:109-157, 395-444). */
int mara_minidisk_binary(const mara_minidisk_params* sd, double time, double* out);

/* Fixed-formula time step (problems/minidisk.cpp:204-206). Host. */
int mara_minidisk_dt_formula(const mara_minidisk_params* sd, double time, double* dt);

/* Drop-in for minidisk::updated_conserved (problems/minidisk.hpp:164-170,
 * problems/minidisk_scheme.cpp:294-355): one forward-Euler update of one mesh
 * block, plain FP64. Device buffers in the reference's AoS tuple layout:
 * uc = n*n*3 conserved, pe = (n+4)*(n+4)*3 primitives with a 2-zone halo,
 * u1 = n*n*3 out; n = sd->block_size. (level, bi, bj) is the block index. */
int mara_minidisk_updated_conserved(const mara_minidisk_params* sd, const double* uc, const double* pe,
                                    double time, double dt, uint32_t level, uint64_t bi, uint64_t bj,
                                    double* u1, void* stream);

/* Drop-in for minidisk::recover_primitive_array (problems/minidisk_scheme.cpp:208-211):
 * count AoS cells (3 doubles each), device buffers. */
int mara_minidisk_recover_primitive(const double* u, int64_t count, double* p, void* stream);

/* Drop-in for minidisk::estimate_gradient (problems/minidisk_scheme.cpp:213-216):
 * AoS primitives of shape (n0, n1) -> (n0-2, n1) for axis 0, (n0, n1-2) for axis 1. */
int mara_minidisk_estimate_gradient(const double* pc, int64_t n0, int64_t n1, int32_t axis, double theta,
                                    double* out, void* stream);

/* Whole-mesh forward-Euler substep, plain FP64, SoA device buffers (the
 * reference's per-block encode_substep over every block, problems/minidisk.cpp:172-189,
 * with the periodic halo of extend, :87-120):
 *   u_out = L(u_in) at (time, dt);
 *   if u_avg != NULL: u_out = u_avg*0.5 + L(u_in)*0.5, the RK2 second stage
 *   (src/app_control.hpp:178-183, src/mesh_amr.hpp:456-467).
 * u_out may alias u_avg but not u_in. */
int mara_minidisk_substep(const mara_minidisk_params* sd, const double* u_in, const double* u_avg, double* u_out,
                          double time, double dt, void* stream);

/* Initial conserved state (problems/minidisk_scheme.cpp:87-99, 182-191) with a
 * seeded density perturbation Σ(1 + amplitude*(2U-1)), U from a counter-based
 * hash of (seed, cell index); amplitude 0 reproduces the reference exactly. */
int mara_minidisk_initial_conserved(const mara_minidisk_params* sd, uint64_t seed, double amplitude,
                                    double* u, void* stream);

/* Bytes of device workspace that mara_minidisk_advance needs for this mesh. */
int64_t mara_minidisk_workspace_bytes(const mara_minidisk_params* sd, int32_t rk_order, int32_t precision);

/* Set clock->time, reset the iteration count, and (CFL mode) reduce the
 * fastest wavespeed of u into clock->max_wavespeed. clock is device memory. */
int mara_minidisk_clock_init(const mara_minidisk_params* sd, const double* u, double time,
                             mara_minidisk_clock* clock, void* stream);

/* Advance the SoA state u (device) by `steps` steps of order rk_order (1 or 2)
 * with the time step of dt_mode, in the given precision. Time, dt and the
 * binary position live in *clock (device); the CFL reduction of the next step
 * is fused into the last stage of each step. workspace: device buffer of
 * mara_minidisk_workspace_bytes. The result is always left in u. */
int mara_minidisk_advance(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock,
                          int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                          void* workspace, void* stream);

/* Host-buffer form of mara_minidisk_advance: copies u_in
 * (host, 3*N*N doubles, SoA; pinned memory gives full bandwidth) to the
 * device, advances `steps` steps from `time`, copies the state back to u_out
 * (host) and writes the final time to *time_out. Device buffers come from
 * the caller's `workspace` of mara_minidisk_host_workspace_bytes. Synchronous
 * on `stream`. This is the reference-facing call: state in host memory, as
 * the reference's nd::shared_array holds it. With page-locked u_in and u_out
 * and mixed RK2, the kernels read u_in and write u_out over the host link
 * themselves (the same bits as the copies); u_out may alias u_in. */
int64_t mara_minidisk_host_workspace_bytes(const mara_minidisk_params* sd, int32_t rk_order, int32_t precision);
int mara_minidisk_advance_host(const mara_minidisk_params* sd, const double* u_in, double* u_out, double time,
                               int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                               double* time_out, void* workspace, void* stream);

/* One stage kernel of mara_minidisk_advance, for callers that drive the RK
 * loop themselves (the role of control::advance_runge_kutta,
 * src/app_control.hpp:169-195). dt and the binary come from clock->dt and
 * clock->binary[stage]. kind:
 *   0  FP64:    u_out = L(u_in); with u_avg: u_out = u_avg*0.5 + L(u_in)*0.5
 *   1  mixed 1: d_out = dt*L(u_in) (FP32); with d_out NULL: u_out = u_in + dt*L(u_in)
 *   2  mixed 2: u_out = u_in + (d1 + dt*L(f32(u_in) + d1))/2
 * In the mixed kinds the FP32 increment enters the FP64 sum exactly, except
 * that a zero or subnormal increment may add a value below 2^-126 in
 * magnitude (absorbed exactly wherever |u_in| >= 2^-72).
 * reduce_wavespeed != 0 also folds the fastest wavespeed of u_out into
 * clock->max_wavespeed (mixed kinds: from u_out's FP32 image, as a double;
 * mara_minidisk_advance instead re-evaluates the fastest cell in FP64).
 * u_out must not alias u_in (kind 0 may alias u_avg). */
int mara_minidisk_stage(const mara_minidisk_params* sd, int32_t kind, const double* u_in, const float* d1,
                        const double* u_avg, double* u_out, float* d_out, mara_minidisk_clock* clock,
                        int32_t stage, int32_t reduce_wavespeed, void* stream);

/* Device clock bookkeeping between stages: end_step advances time and the
 * iteration count of the step that ran (RK2: t = t*0.5 + (t+2dt)*0.5);
 * begin_step picks the next dt (dt_mode) and the binary of both stages. */
int mara_minidisk_clock_update(const mara_minidisk_params* sd, mara_minidisk_clock* clock, int32_t dt_mode,
                               int32_t rk_order, int32_t end_step, int32_t begin_step, void* stream);

/* Allocation-free form of mara_minidisk_advance (no counterpart in the
 * reference). For callers that cannot allocate device memory — a host that
 * has given all of the GPU's memory to its own pool allocator, or a plugin
 * that only receives the caller's state and clock buffers through this ABI —
 * the workspace comes from a static device array inside the library instead
 * of a caller-owned buffer. Limits and rules:
 *   - the mesh may hold at most MARA_MINIDISK_NOALLOC_MAX_CELLS cells
 *     ((block_size << depth)^2); larger meshes are rejected with
 *     MARA_ERR_ARGUMENT and a message naming the limit;
 *   - the array (36 bytes per cell of that limit plus 64, 9 MiB) is held by
 *     every GPU that loads the library until the process exits;
 *   - the first call on a device looks up the array's device address with
 *     that device current (cudaGetSymbolAddress); make that first call before
 *     any stream capture. The address is kept for the life of the process, so
 *     do not call this entry point again after cudaDeviceReset (or any other
 *     teardown of the device's primary context) in the same process;
 *   - all calls share the one array: calls whose GPU work overlaps (other
 *     streams, other threads) race and corrupt each other's results.
 *     Nothing in it needs to start at zero: every step writes its scratch
 *     before reading it.
 * No cudaMalloc/cudaFree or allocating library routine is called. u and
 * clock are caller-owned device buffers as for mara_minidisk_advance. */
#define MARA_MINIDISK_NOALLOC_MAX_CELLS (512 * 512)
int mara_minidisk_advance_noalloc(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock,
                                  int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                                  void* stream);

/* ---------------------------------------------------------------- minidisk time series */
/* Diagnostics of a minidisk run: the time series of forces, work and orbital
 * element evolution that the reference driver lists as to do
 * (problems/minidisk.cpp:69) and schedules as a side effect without writing
 * it (schedule_t::time_series, problems/minidisk.hpp:64-68). One rate vector
 * holds sums over all cells of the cell area times:
 *    0, 1   mass removal rate of sink 1, 2: Sigma sr_k, with sr_k the sink
 *           rate field (problems/minidisk_scheme.cpp:57-65)
 *    2..5   momentum removal rate of sink 1 (x, y), then of sink 2: (Sigma vx, Sigma vy) sr_k
 *    6..9   gravitational force of the gas on body 1 (x, y), then on body 2:
 *           -Sigma g_k, with g_k = two_body::gravitational_acceleration
 *           (src/physics_two_body.hpp:209-218) of body k at the cell
 *    10     mass source rate of the outer buffer: (Sigma_init - Sigma) br
 *           (buffer_rate_field, problems/minidisk_scheme.cpp:47-55)
 *    11     disk mass: Sigma
 *    12     disk angular momentum about the origin: x Sigma vy - y Sigma vx
 * and, from the force sums and the binary at the stage time,
 *    13, 14 gravitational torque on body 1, 2: x_k F_ky - y_k F_kx
 *    15     power of the gas's gravity on the binary: F_1 . v_1 + F_2 . v_2.
 * Positions, velocities and forces are in the rotating frame (the binary's
 * velocities rotated with its positions, as two_body::rotate does), so the
 * power equals the inertial-frame power. Sums 0-12 are reductions fused into
 * the mixed-precision stage kernels (FP32 per thread, FP64 across warps); the
 * FP64 path reduces the stage input in FP64 with one extra kernel per stage. */
#define MARA_DIAG_COUNT 16
typedef struct mara_minidisk_diagnostics {
    double rate[2][MARA_DIAG_COUNT];   /* the last step's stage inputs: stage 1 at t, stage 2 at t + dt (RK1: rate[0]) */
    double integral[MARA_DIAG_COUNT];  /* time integrals over completed steps with the update's RK weights:
                                          dt (rate[0] + rate[1]) / 2 (RK2), dt rate[0] (RK1); entries 11 and 12
                                          hold the values at the start of the last completed step instead */
    int64_t steps;                     /* completed steps in the integrals */
} mara_minidisk_diagnostics;

/* Zero a device mara_minidisk_diagnostics (stream-ordered). */
int mara_minidisk_diagnostics_reset(mara_minidisk_diagnostics* diag, void* stream);

/* mara_minidisk_advance that also accumulates the diagnostics of every step
 * into diag (device memory; NULL gives mara_minidisk_advance). */
int mara_minidisk_advance_diag(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock,
                               int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                               void* workspace, mara_minidisk_diagnostics* diag, void* stream);

/* The rate vector of one state at one time, in FP64: u (device, SoA), plus
 * the FP32 increment d1 when not NULL (u + d1, a mixed RK2 stage-2 input);
 * the binary at `time` from two_body::orbital_state + rotate. out: device,
 * MARA_DIAG_COUNT doubles. */
int mara_minidisk_rates(const mara_minidisk_params* sd, const double* u, const float* d1, double time,
                        double* out, void* stream);

/* two_body::recover_orbital_elements (src/physics_two_body.hpp:284-379), host
 * FP64, G = 1: state = {m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2} at time t
 * -> out = {a, M, q, e, x_cm, y_cm, vx_cm, vy_cm, pomega, tau}. An unbound
 * state (E >= 0) returns MARA_ERR_ARGUMENT, as the reference throws. */
int mara_two_body_elements(const double* state, double time, double* out);

/* Rates of change of (a, M, q, e) implied by a rate vector (entries 0-9)
 * acting on the binary state: dm_k/dt = sink mass rate k, d(m_k v_k)/dt =
 * gas force + sink momentum rate k, positions fixed; central difference of
 * mara_two_body_elements. Host FP64. out: 4 doubles. */
int mara_two_body_element_rates(const double* state, double time, const double* rates, double* out);

/* Columns per thread of the mixed-precision sweep kernels, process-wide:
 * 0 = automatic (two wherever N is even and the buffers are 16-byte aligned;
 * else one), 1 or 2 to force a form (2 still falls back to 1 where it cannot
 * run). Both forms give bit-identical results. Returns the previous setting, or -1 for a bad value (the message
 * says why). */
int mara_minidisk_sweep_columns(int32_t columns);

/* How the two-column mixed sweep stages its rows in shared memory,
 * process-wide: 0 (the default) = per-lane asynchronous copies (cp.async);
 * 1 = bulk tensor copies (TMA, one per row and field, completing on an
 * mbarrier) wherever a strip's columns lie inside the mesh and the buffers
 * allow it, per-lane copies elsewhere. Both give bit-identical results; at
 * 4096^2 the per-lane copies are the faster (0.469 against 0.526 ms per RK2
 * step). Returns the previous setting, or -1 for a bad value. */
int mara_minidisk_sweep_tma(int32_t enable);

/* Launch shape of the single-mesh mixed sweep: warps per block (1, 2 or 4;
 * 0 = 4) and how many waves of resident warps its strip segments fill
 * (0 = 2). Results do not depend on it. Returns 0, or -1 on bad arguments. */
int mara_minidisk_sweep_shape(int32_t block_warps, int32_t waves);

/* ---------------------------------------------------------------- minidisk ensemble */

/* Many independent minidisk meshes (members, each with its own parameters
 * and mesh size) advanced together: the reference runs one mesh per process
 * and folds steps on the host (problems/minidisk.cpp:202-213); here every RK
 * stage of all members is ONE persistent launch over a device work-list of
 * strip segments (MARA_MIXED), and each RK step (stages + clock update of all
 * members) is replayed from a CUDA graph captured at creation. Each member's
 * results and clock equal those of mara_minidisk_advance on that member alone
 * with the same arguments, up to FP32 rounding of a face flux at a work-list
 * cut (MARA_MIXED) and exactly (MARA_FP64). */
typedef struct mara_minidisk_ensemble mara_minidisk_ensemble;

typedef struct {
    int32_t blocks_per_sm;    /* resident 128-thread CTAs per SM of the persistent grid */
    int32_t chunks_per_warp;  /* 1: one balanced row range per warp; >1: that many per warp, claimed dynamically */
    int32_t cols_per_lane;    /* thread coarsening of the sweep: 1 or 2 columns per lane (2: even N only) */
    int32_t register_variant; /* register budget of the sweep: 0 unconstrained, 1/2 compiled for more CTAs per SM */
    double stage_ms;          /* both stages of one step of all members, as timed by the tuner (0: not timed) */
} mara_ensemble_config;

/* Host-only planner of the work-list (no GPU needed): the column strips
 * (strip_columns = 28 for the 1-column sweep, 60 for the 2-column one) of
 * every member's N x N mesh, rows laid end to end, cut into `chunks` ranges
 * of equal row count; items[4*k..] = (member, strip, row begin, row end),
 * chunk c owns items [chunk_first[c], chunk_first[c+1]). Returns the item
 * count (-1 on bad arguments); writes at most `capacity` items; either
 * output may be NULL. */
int64_t mara_minidisk_ensemble_plan(const int32_t* sizes, int32_t count, int64_t chunks, int32_t strip_columns,
                                    int32_t* items, int64_t capacity, int32_t* chunk_first);

/* Create an ensemble of `count` members. params[m] describes member m;
 * states[m] is its device SoA state (3 * N_m^2 doubles, 16-byte aligned) and
 * clocks + m its device clock; all stay caller-owned and must outlive the
 * ensemble. The ensemble allocates its own scratch (one FP64 state and, for
 * MARA_MIXED RK2, one FP32 increment per member) and captures its graphs on
 * a private stream. MARA_MIXED needs N_m >= 64. autotune: 0 = default launch
 * shape, 1 = tune on first use of this set of mesh sizes in the process (the
 * tuner synchronises the device, then only writes scratch), 2 = always tune. */
int mara_minidisk_ensemble_create(const mara_minidisk_params* params, int32_t count, double* const* states,
                                  mara_minidisk_clock* clocks, int32_t rk_order, int32_t precision,
                                  int32_t dt_mode, int32_t autotune, mara_minidisk_ensemble** out);
/* mara_minidisk_clock_init of every member at `time`, with the wavespeed
 * reduction of the ensemble's precision. */
int mara_minidisk_ensemble_clock_init(mara_minidisk_ensemble* e, double time, void* stream);
/* `steps` RK steps of every member, stream-ordered on `stream`. */
int mara_minidisk_ensemble_advance(mara_minidisk_ensemble* e, int32_t steps, void* stream);
int mara_minidisk_ensemble_get_config(const mara_minidisk_ensemble* e, mara_ensemble_config* out);
/* Replace the launch shape (recaptures the graphs; synchronises the device). */
int mara_minidisk_ensemble_set_config(mara_minidisk_ensemble* e, const mara_ensemble_config* config);
/* Time the candidate launch shapes on the members and keep the fastest. */
int mara_minidisk_ensemble_tune(mara_minidisk_ensemble* e);
/* Median CUDA-event time of each stage launch (ms[0..rk_order-1]) over
 * `reps` phase-0 launches that write only scratch (MARA_MIXED; synchronises
 * the device). */
int mara_minidisk_ensemble_stage_times(mara_minidisk_ensemble* e, int32_t reps, double* ms);
int mara_minidisk_ensemble_destroy(mara_minidisk_ensemble* e);

/* ---------------------------------------------------------------- mhd */

/* One periodic cube of ideal MHD with constrained transport, the scheme of
 * mara::advance_mhd_ct (src/scheme_mhd_v1.hpp:102-117, src/scheme_mhd_v1.cpp:265-299)
 * with local_periodic_boundary_extension. dl = 1/N. */
typedef struct mara_mhd_params {
    int32_t N;                  /* cells per side */
    double gamma_law_index;     /* the reference's scheme uses 5/3 */
    double cfl;
    double plm_theta;           /* 0 is not supported (PLM only) */
} mara_mhd_params;

/* Device clock of an MHD run (opaque, mara_mhd_clock_bytes() bytes): time,
 * the CFL dt of each RK stage, iteration, count of zones whose primitive
 * recovery failed (negative density or pressure; the reference throws). */
int64_t mara_mhd_clock_bytes(void);
int mara_mhd_clock_init(void* clock, double time, void* stream);
/* The clock's time is its first double; failures its last 8 bytes. */

/* Workspace (device) for mara_mhd_advance_ct (rk_order 1) / mara_mhd_advance (2). */
int64_t mara_mhd_workspace_bytes(const mara_mhd_params* mp, int32_t rk_order, int32_t precision);

/* Drop-in for mara::advance_mhd_ct: one CFL-limited step of the cube, time in
 * the clock advanced by dt. uc element (component q, cell c) at
 * uc[q*component_stride + c*cell_stride] (the reference's AoS tuples: 1, 5;
 * SoA: N^3, 1); uc_out is SoA [5][N^3]. bf1 [N+1][N][N], bf2 [N][N+1][N],
 * bf3 [N][N][N+1] hold B.dA/dA on the faces as the reference does. */
int mara_mhd_advance_ct(const mara_mhd_params* mp, const double* uc, int64_t component_stride, int64_t cell_stride,
                        const double* bf1, const double* bf2, const double* bf3, double* uc_out, double* bf1_out,
                        double* bf2_out, double* bf3_out, void* clock, int32_t precision, void* workspace,
                        void* stream);

/* `steps` RK2 steps of examples/mhd3d.cpp:186-215 (advance_runge_kutta over
 * advance_mhd_ct: each stage takes its own CFL dt; states and times averaged
 * with weight 1/2) in place on SoA uc [5][N^3] and the face arrays. */
int mara_mhd_advance(const mara_mhd_params* mp, double* uc, double* bf1, double* bf2, double* bf3, void* clock,
                     int32_t steps, int32_t rk_order, int32_t precision, void* workspace, void* stream);

/* Seeded Fourier-mode table (host, 11 doubles per mode: k[3], velocity phase,
 * velocity direction[3], potential phase, potential polarisation[3] / |k|),
 * integer wavevectors 0 < |k| <= 4. No counterpart in the reference. */
int mara_mhd_mode_table(uint64_t seed, int32_t modes, double* table);

/* Initial state in the discretisation of mara::construct_conserved
 * (src/scheme_mhd_v1.cpp:311-342): rho = 1, p = 1, v = v_amp * sum of velocity
 * modes, B = curl of A = a_amp * sum of potential modes taken on cell edges.
 * table is host memory; workspace (device) needs 88*modes bytes. */
int mara_mhd_initial_state(const mara_mhd_params* mp, const double* table, int32_t modes, double v_amp, double a_amp,
                           double* uc, double* bf1, double* bf2, double* bf3, void* workspace, void* stream);

/* The mixed stage as two fused launches (enable 1, the default; meshes with
 * N a multiple of 32: face solves and cell updates, then edge EMFs, face
 * updates and the next stage's primitives) or as the primitive, face and
 * update kernels (enable 0). Both give identical results. chunks > 0 fixes
 * the fused kernels' number of i-chunks (0 chooses it from the SM count).
 * Process-wide; no counterpart in the reference. */
int mara_mhd_fused_stage(int32_t enable, int32_t chunks);

/* max over cells of |div B| * dl (sum of the face differences), into *out (device double). */
int mara_mhd_max_div_b(const mara_mhd_params* mp, const double* bf1, const double* bf2, const double* bf3,
                       double* out, void* stream);

/* ---------------------------------------------------------------- srhd */

/* Conserved -> primitive recovery of n zones, replacing srhd::recover_primitive
 * (src/physics_srhd.hpp:231-285). Zone i, component k (D, S1, S2, S3, tau in;
 * rho, u1, u2, u3, p out) lives at [k*component_stride + i*zone_stride]: SoA is
 * (n, 1), the reference's AoS tuple layout is (1, 5). All buffers device.
 *   mlp_weights == NULL and refine32 == 0: the reference's method, Newton from
 *     p = 0, 50+1 iterations, |f| < 1e-12 (1e-8 on the last); bit-identical to it.
 *   mlp_weights != NULL: Newton starts from the learned guess
 *     (mara_srhd_mlp_*), optionally sharpened by refine32 FP32 Newton steps;
 *     FP64 Newton then polishes with the same stopping rule within
 *     seeded_budget iterations, else restarts from p = 0 with the full budget.
 *   mlp_weights == NULL and refine32 > 0: the same, from p = 0.
 * iterations[i] (nullable) = FP64 Newton iterations run; status[i] (nullable)
 * = 0 ok, 1 not converged, 2 non-positive pressure (the reference throws);
 * failed zones get zero primitives; *failures (nullable, device) counts them. */
int mara_srhd_recover_primitive(const double* cons, int64_t n, int64_t component_stride, int64_t zone_stride,
                                double gamma_law_index, double temperature_floor, const void* mlp_weights,
                                int32_t refine32, int32_t seeded_budget, double* prim, int32_t* iterations,
                                int32_t* status, unsigned long long* failures, void* stream);

/* The same recovery for zones in pinned HOST memory (SoA [5][n] in and out),
 * as a host program holding its zones would call srhd::recover_primitive:
 * the zones go through the GPU in `chunks` pieces on three internal streams,
 * each piece copied in, recovered and copied out in order, so that the host
 * link's transfers of some pieces overlap the recovery of others. Arguments
 * as mara_srhd_recover_primitive (no per-zone iteration or status arrays);
 * *failures (nullable, HOST) receives the count of failed zones. workspace:
 * device memory of mara_srhd_host_workspace_bytes(n, chunks) bytes. Work the
 * caller queued on `stream` before the call runs first; the call returns
 * when the primitives are in host_prim. No counterpart in the reference,
 * which recovers on the host. */
int64_t mara_srhd_host_workspace_bytes(int64_t n, int32_t chunks);
int mara_srhd_recover_primitive_host(const double* host_cons, int64_t n, double gamma_law_index,
                                     double temperature_floor, const void* mlp_weights, int32_t refine32,
                                     int32_t seeded_budget, double* host_prim, int32_t chunks, void* workspace,
                                     unsigned long long* failures, void* stream);

/* Seeded SRHD test zones (no counterpart in the reference): rho in
 * [rho_lo, rho_hi] and p in [p_lo, p_hi] log-uniform, Lorentz factor
 * log-uniform in [1, w_hi] along an isotropic direction; writes primitives and
 * srhd::conserved_density (src/physics_srhd.hpp:291-304), SoA [5][n], device. */
int mara_srhd_seeded_zones(uint64_t seed, int64_t n, double rho_lo, double rho_hi, double p_lo, double p_hi,
                           double w_hi, double gamma_law_index, double* prim, double* cons, void* stream);

/* Learned pressure guess (4-64-64-1 MLP, BF16 tensor-core inference). No
 * counterpart in the reference. The weights are one device buffer of
 * mara_srhd_mlp_weights_bytes() bytes. Training data are n zones in SoA
 * [5][n] (cons, and prim from mara_srhd_recover_primitive); workspace is
 * mara_srhd_mlp_workspace_bytes(n) bytes of device memory. */
int64_t mara_srhd_mlp_weights_bytes(void);
int32_t mara_srhd_mlp_param_count(void);
int64_t mara_srhd_mlp_workspace_bytes(int64_t n);
/* Features, targets, normalisation and Glorot initialisation of the weights. */
int mara_srhd_mlp_prepare(const double* cons, const double* prim, int64_t n, void* weights, uint64_t seed,
                          void* workspace, void* stream);
/* Mean-squared-error loss and its gradient (FP32) over all n prepared zones;
 * grad holds mara_srhd_mlp_param_count() floats, loss one float (device). */
int mara_srhd_mlp_gradient(const void* weights, const void* workspace, int64_t n, float* grad, float* loss,
                           void* stream);
/* `steps` Adam steps on mini-batches of `batch` zones taken in the order of
 * `order` (device int64[n]); loss_history (nullable, device) gets one float
 * per step. Ends by refreshing the BF16 copy used for inference. */
int mara_srhd_mlp_train(void* weights, void* workspace, int64_t n, const int64_t* order, int32_t steps,
                        int32_t batch, float lr, float* loss_history, void* stream);
/* Inference on n rows of raw features (float[n][4]): y[i] = network output. */
int mara_srhd_mlp_infer(const void* weights, const float* features, int64_t n, float* y, void* stream);

/* ---------------------------------------------------------------- srhd 2D scheme */

/* 2D Cartesian SRHD on the unit square (the relativistic shock-tube
 * benchmark). No counterpart scheme exists in the reference; it is composed
 * from the reference's srhd::recover_primitive, srhd::riemann_hlle and
 * mara::plm_gradient in the minidisk face-state pattern, with RK2 by
 * control::advance_runge_kutta and zero-gradient boundaries. State u: SoA
 * [4][N][N] (D, S1, S2, tau), device. clock: mara_srhd_tube_clock_bytes()
 * bytes of device memory (time, dt, fastest speed, iteration, failed
 * recoveries, total FP64 Newton iterations, HLLC faces whose contact speed
 * was rejected). */
int64_t mara_srhd_tube_clock_bytes(void);
int64_t mara_srhd_tube_workspace_bytes(int32_t N);
/* Two states split by the line (x - 1/2) cos(angle) + (y - 1/2) sin(angle) = 0,
 * at rest; resets the clock. */
int mara_srhd_tube_initial(int32_t N, double angle, double rho_l, double p_l, double rho_r, double p_r,
                           double gamma_law_index, double* u, void* clock, void* stream);
/* `steps` RK2 steps; dt = cfl / N / max outer wavespeed of each step's
 * initial state. guess: 0 = p = 0 (the reference's recovery, bit-identical),
 * 1 = the learned guess (mlp_weights), 2 = the previous stage's pressure;
 * refine32 FP32 Newton steps sharpen a guess before the FP64 polish.
 * riemann_solver: 0 = HLLE, 1 = HLLC (a face whose HLLC contact speed the
 * reference would reject gets the HLLE flux and is counted in the clock). */
int mara_srhd_tube_advance(int32_t N, double* u, void* clock, int32_t steps, double cfl, double plm_theta,
                           double gamma_law_index, double temperature_floor, int32_t precision, int32_t guess,
                           const void* mlp_weights, int32_t refine32, int32_t riemann_solver, void* workspace,
                           void* stream);

/* srhd::riemann_solver at fixed faces (src/physics_srhd.hpp:377-487), FP64,
 * the drop-in for its HLLE (solver 0) and HLLC (solver 1) modes: n faces,
 * left/right primitives pl, pr AoS (rho, u1, u2, u3, p) per face, axis 1..3,
 * fluxes f AoS 5 per face; status[i] (nullable) = 1 where the reference
 * throws (HLLC contact speed NaN or beyond 1e3; f holds the HLLE flux
 * there). Device buffers. */
int mara_srhd_riemann(const double* pl, const double* pr, int64_t n, int32_t axis, double gamma_law_index,
                      int32_t solver, double* f, int32_t* status, void* stream);

/* ---------------------------------------------------------------- spherical tracks (sedov2d) */
/* The moving radial-track SRHD scheme of src/scheme_sedov2d.cpp (driven by
 * problems/sedov2d.cpp), gamma 4/3, temperature floor 1e-6. Device buffers:
 *   cell_offset[track_count + 1] (int64): track j holds cells
 *     [cell_offset[j], cell_offset[j+1]) (at least 2), cells = cell_offset[track_count];
 *   theta[2 * track_count]: polar bounds (theta0, theta1) of each track;
 *   radii[cells + track_count]: face radii, track j's n_j + 1 faces from
 *     cell_offset[j] + j (the reference's radial_track_t::face_radii);
 *   u[5][cells]: SoA conserved volume integrals (D, S1, S2, S3, tau);
 *   ghost_in / ghost_out: primitives (rho, u1, u2, u3, p) beyond each
 *     track's inner / outer face, [stage][track][5] (problems/sedov2d.cpp:563-587
 *     takes them from its wind profile at the stage time);
 *   failures (nullable, int32): incremented where the reference throws
 *     (a recovery fails, an HLLC contact speed is NaN or beyond 1e3). */
int64_t mara_sedov_workspace_bytes(int32_t track_count, int64_t cells);

/* One forward-Euler advance of every track: sedov::recover_primitive,
 * radial_gradient, radial_godunov_data with the driver's inner_bc/outer_bc,
 * polar_godunov_data between neighbouring tracks, delta_conserved and
 * delta_face_positions (src/scheme_sedov2d.cpp:150-356,
 * problems/sedov2d.cpp:608-660). Optional outputs for parity checks (NULL
 * to skip): prim [5][cells], grad [5][cells], radial [6][cells + track_count]
 * (HLLC flux, contact or face speed), polar [6][2 cells + track_count] (flux,
 * area of each transverse face; interface j's faces start at
 * cell_offset[j] + cell_offset[j+1] - cell_offset[1] + j, invalid ones zero)
 * and polar_index [2][2 cells + track_count] (int32 il, ir merge counters). */
int mara_sedov_stage(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* theta,
                     const double* radii, const double* u, const double* ghost_in, const double* ghost_out, double dt,
                     int32_t use_plm, double* radii_out, double* u_out, double* prim, double* grad, double* radial,
                     double* polar, int32_t* polar_index, void* workspace, int32_t* failures, void* stream);

/* control::advance_runge_kutta (src/app_control.hpp:169-195) of that advance,
 * rk_order 1, 2 or 3, radii and u combined by weighted_sum; in place. ghost
 * arrays hold rk_order stages. */
int mara_sedov_advance(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* theta,
                       double* radii, double* u, const double* ghost_in, const double* ghost_out, double dt,
                       int32_t rk_order, int32_t use_plm, void* workspace, int32_t* failures, void* stream);

/* sedov::remesh (src/scheme_sedov2d.cpp:362-412) of every track: drop the
 * first cell while the inner face lies inside inner_radius, split the cell of
 * largest aspect dr / (r_c dtheta) above max_aspect, merge the cell of
 * smallest aspect below min_aspect with its neighbour of smaller aspect. As in
 * the reference, the recursion after a drop or a merge runs with the two
 * aspect bounds exchanged. New tracks go to separate buffers of capacity
 * cells + track_count cells: cell_offset_out[track_count + 1] (device),
 * radii_out, u_out (SoA with the new cell count as its stride); the new cell
 * count is written to *cells_out (host; the call synchronizes the stream).
 * failures counts tracks where the reference would throw. */
int64_t mara_sedov_remesh_workspace_bytes(int32_t track_count, int64_t cells);
int mara_sedov_remesh(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* theta,
                      const double* radii, const double* u, double max_aspect, double min_aspect, double inner_radius,
                      int64_t* cell_offset_out, double* radii_out, double* u_out, int64_t* cells_out, void* workspace,
                      int32_t* failures, void* stream);

/* sedov::minimum_spacing over all tracks (scheme_sedov2d.cpp:66-69, the
 * driver's dt = cfl * min spacing / c): out is one device double. */
int mara_sedov_min_spacing(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* radii,
                           double* out, void* stream);

/* ---------------------------------------------------------------- mhd: the split block API */
/* The reference's per-block CT scheme, mhd_scheme_v2 (src/scheme_mhd_v2.hpp:71-210,
 * src/scheme_mhd_v2.cpp:75-278), FP64, one call per reference function.
 * Device buffers in the reference's row-major AoS layouts: conserved
 * 5-tuples (D, S1, S2, S3, E), primitive 8-tuples (rho, v1, v2, v3, p, B1,
 * B2, B3), godunov data 8-tuples (the 5 HLLE fluxes, then E1, E2, E3), face
 * fields and edge EMFs as scalars. For a cell array of shape (n0, n1, n2) the
 * face array of axis a is one longer along a, and the edge array of axis a
 * one longer along the two other axes. The reference fixes gamma at 5/3. */

/* primitive_array (:75-81): uc (n0, n1, n2) conserved, bf1..3 the block's
 * faces; pc (n0, n1, n2) primitives. failures (device, nullable) counts cells
 * where mhd::recover_primitive throws (negative density or pressure). */
int mara_mhd_v2_primitive_array(int32_t n0, int32_t n1, int32_t n2, const double* uc, const double* bf1,
                                const double* bf2, const double* bf3, double gamma_law_index, double* pc,
                                unsigned long long* failures, void* stream);

/* godunov_fluxes (:143-163), first order: pc (m0, m1, m2) primitives (a block
 * extended by one cell on every side); bf1..3 the faces between those cells,
 * shapes (m0-1, m1, m2), (m0, m1-1, m2), (m0, m1, m2-1); gf1..3 the godunov
 * data on those faces (normal E component zero). */
int mara_mhd_v2_godunov_fluxes(int32_t m0, int32_t m1, int32_t m2, const double* pc, const double* bf1,
                               const double* bf2, const double* bf3, double gamma_law_index, double* gf1,
                               double* gf2, double* gf3, void* stream);

/* electromotive_forces (:168-192): gf1..3 of a (m0, m1, m2) cell array as
 * godunov_fluxes writes them; ee1 (m0, m1-1, m2-1), ee2 (m0-1, m1, m2-1),
 * ee3 (m0-1, m1-1, m2): each edge EMF the mean of the adjacent means of the
 * two transverse faces' E along it. */
int mara_mhd_v2_electromotive_forces(int32_t m0, int32_t m1, int32_t m2, const double* gf1, const double* gf2,
                                     const double* gf3, double* ee1, double* ee2, double* ee3, void* stream);

/* updated_conserved_density (:197-219): uc (n0, n1, n2); gf1..3 extended by
 * one zone on their transverse axes, (n0+1, n1+2, n2+2) etc.;
 * uc_out = uc - div(F) dt / dl. */
int mara_mhd_v2_updated_conserved_density(int32_t n0, int32_t n1, int32_t n2, const double* uc, const double* gf1,
                                          const double* gf2, const double* gf3, double dt, double dl,
                                          double* uc_out, void* stream);

/* curl (:224-237): the staggered curl of the block's edge values ee1
 * (n0, n1+1, n2+1), ee2 (n0+1, n1, n2+1), ee3 (n0+1, n1+1, n2), divided by
 * dl, on the block's faces cf1 (n0+1, n1, n2), cf2, cf3. */
int mara_mhd_v2_curl(int32_t n0, int32_t n1, int32_t n2, const double* ee1, const double* ee2, const double* ee3,
                     double dl, double* cf1, double* cf2, double* cf3, void* stream);

/* updated_magnetic_flux_density (:242-257): bf1..3 the block's faces; ee1..3
 * the edge EMFs of the block extended by one cell on every side (as
 * electromotive_forces gives them: (n0+2, n1+1, n2+1) etc.), of which the
 * block's own edges are used; bf_out = bf - curl(E) dt / dl. */
int mara_mhd_v2_updated_magnetic_flux_density(int32_t n0, int32_t n1, int32_t n2, const double* bf1,
                                              const double* bf2, const double* bf3, const double* ee1,
                                              const double* ee2, const double* ee3, double dt, double dl,
                                              double* bf1_out, double* bf2_out, double* bf3_out, void* stream);

/* ---------------------------------------------------------------- pointwise physics */
/* Batches of n points, device buffers, FP64, the reference's formulas and
 * order. axis is the face normal: 1..3 (unit_vector_on(axis)). */

/* mhd::recover_primitive (src/physics_mhd.hpp:290-303): u [n][5], cell
 * fields b [n][3] -> p [n][8]; status[i] (nullable) 1 where the reference
 * throws; failures (nullable, device) counts them. */
int mara_mhd_recover_primitive(const double* u, const double* b, int64_t n, double gamma_law_index, double* p,
                               int32_t* status, unsigned long long* failures, void* stream);
/* mhd::conserved_density (:305-318): p [n][8] -> u [n][5]. */
int mara_mhd_conserved_density(const double* p, int64_t n, double gamma_law_index, double* u, void* stream);
/* mhd::flux (:324-349): p [n][8] -> f [n][5]. */
int mara_mhd_flux(const double* p, int64_t n, int32_t axis, double gamma_law_index, double* f, void* stream);
/* mhd::fast_speed_squared (:216-222) along the axis: out [n]. */
int mara_mhd_fast_speed_squared(const double* p, int64_t n, int32_t axis, double gamma_law_index, double* out,
                                void* stream);
/* mhd::fastest_speed (:239-249): out [n]. */
int mara_mhd_fastest_speed(const double* p, int64_t n, double gamma_law_index, double* out, void* stream);
/* mhd::riemann_hlle (:358-390): pl, pr [n][8], the face's normal field
 * b_longitudinal [n] -> out [n][8] (HLLE flux 5, then the E-field 3). */
int mara_mhd_riemann_hlle(const double* pl, const double* pr, const double* b_longitudinal, int64_t n, int32_t axis,
                          double gamma_law_index, double* out, void* stream);

/* iso2d (src/physics_iso2d.hpp:99-173) with the local cs^2 of every point
 * (cs2 [n]); p = (Sigma, v1, v2) [n][3], axis 1 or 2. */
int mara_iso2d_flux(const double* p, const double* cs2, int64_t n, int32_t axis, double* f, void* stream);
/* out [n][2] = (vn - cs, vn + cs) */
int mara_iso2d_outer_wavespeeds(const double* p, const double* cs2, int64_t n, int32_t axis, double* out,
                                void* stream);
/* out [n] = max |outer wavespeed| over both axes */
int mara_iso2d_fastest_wavespeed(const double* p, const double* cs2, int64_t n, double* out, void* stream);
/* HLLE flux between pl and pr [n][3] -> f [n][3] */
int mara_iso2d_riemann_hlle(const double* pl, const double* pr, const double* cs2, int64_t n, int32_t axis,
                            double* f, void* stream);

/* ---------------------------------------------------------------- measurement */
/* FP64 fused multiply-add throughput of the current GPU in thread-level DFMA
 * per second (*dfma_per_second, host): a timed kernel of independent FMA
 * chains on every SM, best of three launches after a warm-up; synchronizes
 * the stream. The roofline denominator of the kernels that the FP64 pipe
 * bounds. A measurement helper with no counterpart in the reference. */
int mara_measure_fp64_rate(double* dfma_per_second, void* stream);

/* Host-link rates in GB/s (gbs[5], host): [0] copy-engine host->device,
 * [1] copy-engine device->host, [2] a kernel reading pinned host memory,
 * [3] a kernel writing it, [4] both kernels at once on halves of the buffers
 * (total bytes of both directions / time). host: pinned host memory (page-
 * locked, with a device address), device: device memory, both `bytes` long
 * and 16-byte aligned; their contents are overwritten. Best of three after a
 * warm-up round; synchronizes the stream. The bound of the host-buffer calls
 * (mara_minidisk_advance_host reads and writes the state this way). A
 * measurement helper with no counterpart in the reference. */
int mara_measure_host_link(void* host, void* device, int64_t bytes, double* gbs, void* stream);

/* Self-check of the library's integer float<->double conversions against the
 * GPU's own conversion instructions; mismatches[3] (host) receives the count
 * of wrong results of [0] float->double (all 2^32 floats), [1] the
 * increment form of float->double used by the mixed stores (all 2^32
 * floats; zeros and subnormals may give any double of their sign below
 * 2^-126), [2] double->float, rounding to nearest with ties away from zero
 * (2^32 doubles covering every sign, exponent and top-20-bit mantissa
 * pattern). All three are 0 on a correct build. Synchronizes the stream.
 * No counterpart in the reference. */
int mara_check_conversions(unsigned long long* mismatches, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MARA_GB300_H */
