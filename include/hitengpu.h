/*
 * hitengpu -- C ABI of the GB300 (sm_103a) CR3BP trajectory-propagation path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (HG_OK = 0) and is asynchronous on the given CUDA stream
 * (`stream` is a cudaStream_t passed as void*; NULL = legacy default stream).
 * All array arguments are caller-owned DEVICE memory laid out
 * structure-of-arrays, component-major: element (component c, trajectory i)
 * lives at base[c * ld + i] with ld >= N.  Component order follows the
 * reference: 6-dim states are [x, y, z, vx, vy, vz]; 42-dim states are the
 * row-major 6x6 STM Phi followed by the state (Phi[r][c] = y[6r + c],
 * state = y[36:42]).  Arithmetic is IEEE FP64 in the reference's operation
 * order (no contraction).  A handle is used by one host thread at a time;
 * separate handles may share a device.
 *
 * Allocation: hg_create allocates the handle's fixed scratch (refill
 * counters, a pinned live-count word).  The record pool of deferred event
 * refinement and the corrector's buffers are grow-only handle buffers: after
 * hg_reserve(h, N, dim, max_hits) / hg_reserve_correct(h, orbits) no
 * propagation or correction call on batches up to those sizes allocates
 * device or pinned memory (HG_COUNTER_ALLOCATIONS counts every allocation
 * made for a handle); without a reservation the first larger call grows the
 * buffer once.  Segmented and scheduled DOP853 runs take a caller workspace;
 * the connection searches take an optional caller workspace (NULL: a
 * stream-ordered allocation per call); the no-alloc DOP853 entry point never
 * allocates; the request server allocates its device and pinned arenas in
 * hg_serve_create and nothing afterwards.
 */
#ifndef HITENGPU_H
#define HITENGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (per call and per trajectory) */
#define HG_OK 0
#define HG_MAX_STEPS 1      /* adaptive step budget exhausted */
#define HG_STEP_UNDERFLOW 2 /* reserved */
#define HG_NONFINITE 3      /* state became NaN/Inf */
#define HG_NEWTON_DIVERGED 4
#define HG_EVENT_NOT_FOUND 5
#define HG_LINE_SEARCH_FAILED 6 /* per orbit: Armijo found no productive step */
#define HG_SYNC_TIMEOUT 7   /* per trajectory: a hand-off between the warps of a paired layout timed out */
#define HG_ERR_ARGS 10      /* invalid argument (call status) */
#define HG_ERR_CUDA 11      /* CUDA runtime error (call status) */
#define HG_ERR_NO_DEVICE 12
#define HG_ERR_TIMEOUT 13   /* hg_serve_wait: the request did not finish in time */

typedef struct hg_handle hg_handle;

typedef struct {
  int device;          /* CUDA device ordinal */
} hg_config;

/* Plane event g(y) = y[index] - offset.
 * index < 0 disables the event.  direction: 0 any, +1 increasing,
 * -1 decreasing (integrators/utils.py:13-68 semantics, endpoint zeros
 * count).  max_hits = 1 stops at the first crossing (the reference's
 * terminal event); max_hits > 1 records up to max_hits crossings without
 * changing the step sequence.  xtol/gtol: bisection tolerances on the
 * dense interpolant (reference defaults 1e-12). */
typedef struct {
  int index;
  double offset;
  int direction;
  int max_hits;
  double xtol;
  double gtol;
} hg_event;

/* DOP853 controls (integrators/rk.py:786-838, dynamics/base.py:441-447).
 * fwd = -1 integrates backward by negating the derivative components
 * [flip_lo, flip_hi) (dynamics/base.py:272-310). */
typedef struct {
  double rtol;
  double atol;
  double max_step;
  double min_step;
  long long max_steps; /* attempted-step budget per trajectory */
  int fwd;
  int flip_lo;
  int flip_hi;
} hg_dop853_opts;

/* Replaces: nothing (lifecycle).  Creates a handle bound to cfg->device. */
int hg_create(const hg_config* cfg, hg_handle** out);
int hg_destroy(hg_handle* h);
/* Sizes the handle's event-refinement pool so that single-pass DOP853 calls
 * (hg_propagate_dop853 and the propagations inside hg_correct_halo) on up to
 * max_N trajectories of dimension <= dim with up to max_hits crossings each
 * allocate nothing.  Synchronous; the only call besides hg_create and
 * hg_reserve_correct that allocates on purpose.
 * Replaces: nothing (the reference allocates per call). */
int hg_reserve(hg_handle* h, int max_N, int dim, int max_hits);
/* Last error message recorded on this handle ("" if none). */
const char* hg_last_error_string(hg_handle* h);
/* Library version string. */
const char* hg_version(void);

/* Fixed-step explicit RK (order 4, 6 or 8) on dim 6 or 42, N trajectories,
 * over the time nodes t_vals[0..n_nodes-1] (device array; h_n = t_{n+1} - t_n
 * as the reference computes it).  Writes the states at nodes 0, out_every,
 * 2*out_every, ... to y_out ([n_out][dim][ld_out], n_out = (n_nodes-1)/out_every + 1).
 * status[i] (nullable): HG_OK or HG_NONFINITE.
 * Replaces: integrators/rk.py:531-588 (_FixedStepRK._integrate_fixed_rk) as
 * reached from dynamics/base.py:430-434 (_propagate_dynsys, method='fixed')
 * and dynamics/rtbp.py:320-331 (_compute_stm). */
int hg_propagate_fixed(hg_handle* h, double mu, int order, int dim, int N,
                       const double* y0, long long ld_in,
                       const double* t_vals, int n_nodes, int out_every,
                       double* y_out, long long ld_out,
                       int fwd, int flip_lo, int flip_hi,
                       int* status, void* stream);

/* hg_propagate_fixed with a terminal plane event (ev required; max_hits is
 * ignored: the first crossing ends the trajectory).  Each step also
 * evaluates f(y_{n+1}); on a sign change the crossing is bisected on the
 * cubic Hermite interpolant of the step.  Rows of y_out after the crossing
 * are not written.  Outputs: hit_t [ld_out], hit_y [dim][ld_out],
 * n_hits [N] (0 or 1), status [N] (nullable).
 * Replaces: integrators/rk.py:655-718 (_integrate_fixed_rk_until_event)
 * and :286-391 (_hermite_eval_dense, _hermite_refine_in_step). */
int hg_propagate_fixed_event(hg_handle* h, double mu, int order, int dim, int N,
                             const double* y0, long long ld_in,
                             const double* t_vals, int n_nodes, int out_every,
                             double* y_out, long long ld_out,
                             int fwd, int flip_lo, int flip_hi, const hg_event* ev,
                             double* hit_t, double* hit_y, int* n_hits,
                             int* status, void* stream);

/* Adaptive DOP853 on dim 6 or 42 from t0 to tmax (per trajectory arrays
 * t0_arr/tmax_arr of length N, or NULL to use the scalars).
 * Optional plane event ev (NULL = none).  Optional dense samples at
 * linspace(t0_i, tmax_i, n_samples) into y_samples ([n_samples][dim][ld]);
 * with sample_last_only != 0 only the final sample (t = tmax_i) is
 * evaluated and written to row 0.  Outputs (all nullable): y_end [dim][ld]
 * (last accepted state), t_end [N], hit_t [max_hits][ld],
 * hit_y [max_hits][dim][ld], n_hits/n_accept/n_reject/status [N].
 * Replaces: integrators/rk.py:2375-2549 (_DOP853._integrate_dop853) and
 * :2678-2803 (_integrate_dop853_until_event with _dop853_refine_in_step
 * :2005-2102), as reached from dynamics/base.py:435-453 and
 * poincare/singlehit/backend.py:164-235. */
int hg_propagate_dop853(hg_handle* h, double mu, int dim, int N,
                        const double* y0, long long ld,
                        const double* t0_arr, const double* tmax_arr,
                        double t0, double tmax,
                        const hg_dop853_opts* opts, const hg_event* ev,
                        int n_samples, int sample_last_only, double* y_samples,
                        double* y_end, double* t_end,
                        double* hit_t, double* hit_y, int* n_hits,
                        int* n_accept, int* n_reject, int* status,
                        void* stream);

/* hg_propagate_dop853 in segments: up to max_segments launches, each
 * advancing every live trajectory by at most seg_steps attempted steps and
 * compacting the live trajectories into a dense list for the next launch
 * (lanes whose trajectory finished no longer idle in FP64 instructions).
 * All work is asynchronous with no host synchronisation, so a call can be
 * captured in a CUDA graph.  State persists in the outputs (y_end, t_end,
 * n_accept, n_reject, n_hits, status -- all required; status = -1 marks a
 * trajectory still running) and in `workspace` (caller device memory of at
 * least hg_dop853_segmented_workspace_bytes(N, dim, max_hits) bytes, with
 * max_hits the event's (0 without one); -1 for invalid arguments); it also
 * holds the steps of the event crossings, refined at the end of each call;
 * resume = 1 continues
 * a previous call's unfinished trajectories.  Results are bit-identical to
 * hg_propagate_dop853.
 * Replaces: as hg_propagate_dop853 (execution schedule only). */
long long hg_dop853_segmented_workspace_bytes(int N, int dim, int max_hits);
int hg_propagate_dop853_segmented(hg_handle* h, double mu, int dim, int N,
                                  const double* y0, long long ld,
                                  const double* t0_arr, const double* tmax_arr,
                                  double t0, double tmax,
                                  const hg_dop853_opts* opts, const hg_event* ev,
                                  int n_samples, int sample_last_only, double* y_samples,
                                  double* y_end, double* t_end,
                                  double* hit_t, double* hit_y, int* n_hits,
                                  int* n_accept, int* n_reject, int* status,
                                  int seg_steps, int max_segments, int resume,
                                  void* workspace, long long workspace_bytes,
                                  void* stream);

/* hg_propagate_dop853 run as host-scheduled segments: each segment advances
 * every live trajectory by up to HG_TUNE_SEG_STEPS attempted steps, the
 * trajectories still running are compacted into a dense list, and the host
 * reads their count back before the next segment.  For a 6-dim system the
 * layout of each segment (1, 2 or 6 lanes per trajectory) is chosen from that
 * count unless HG_TUNE_DOP853_LANES_D6 fixes it: wide layouts for the few
 * long trajectories at the end of an uneven batch cut the per-step latency
 * that bounds it.  Synchronous: returns when every trajectory has finished
 * (it synchronizes `stream` once per segment).  Same arguments and state
 * requirements as hg_propagate_dop853_segmented; results are bit-identical
 * to hg_propagate_dop853.
 * Replaces: as hg_propagate_dop853 (execution schedule only). */
int hg_propagate_dop853_scheduled(hg_handle* h, double mu, int dim, int N,
                                  const double* y0, long long ld,
                                  const double* t0_arr, const double* tmax_arr,
                                  double t0, double tmax,
                                  const hg_dop853_opts* opts, const hg_event* ev,
                                  int n_samples, int sample_last_only, double* y_samples,
                                  double* y_end, double* t_end,
                                  double* hit_t, double* hit_y, int* n_hits,
                                  int* n_accept, int* n_reject, int* status,
                                  void* workspace, long long workspace_bytes,
                                  void* stream);

/* No counterpart in the reference.  The DOP853 propagation of
 * hg_propagate_dop853, for callers that cannot call cudaMalloc (an embedding
 * runtime that owns all device memory, a loop that must not allocate after
 * start-up, a plugin that may not create a handle).  It takes no handle and
 * allocates nothing: the lane-refill counter, its only scratch, lives in a
 * file-scope __device__ array of HG_NOALLOC_SCRATCH_BYTES per device, held
 * until the process exits.  Runs on the current device.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress); make
 * it before any stream capture.  The address is looked up again when the
 * calling thread's CUDA context changes (after cudaDeviceReset), so make the
 * first call after a reset outside stream capture too.  The counter is
 * cleared at the start of each call and shared by all calls: calls that
 * overlap on the GPU race, so serialize them.  Arguments, nullable outputs
 * and results are those of hg_propagate_dop853; N > HG_NOALLOC_MAX_N (the
 * 32-bit counter's safe range) is rejected with HG_ERR_ARGS; errors are
 * reported by return code only. */
#define HG_NOALLOC_SCRATCH_BYTES 256
#define HG_NOALLOC_MAX_N (1 << 30)
int hg_propagate_dop853_noalloc(double mu, int dim, int N,
                                const double* y0, long long ld,
                                const double* t0_arr, const double* tmax_arr,
                                double t0, double tmax,
                                const hg_dop853_opts* opts, const hg_event* ev,
                                int n_samples, int sample_last_only, double* y_samples,
                                double* y_end, double* t_end,
                                double* hit_t, double* hit_y, int* n_hits,
                                int* n_accept, int* n_reject, int* status,
                                void* stream);

/* Plane crossings on sampled trajectories (the synodic Poincare map):
 * plane g = y[axis] - offset; samples [m][6][ld] (e.g. the dense output of
 * hg_propagate_dop853), times [m][times_ld] (times_ld = 0: one shared time
 * grid [m]).  direction -1/0/+1; plane_u/plane_v: the projected coordinates
 * used for de-duplication; segment_refine >= 1 sub-intervals per segment with
 * linear (cubic = 0, the reference's default path) or cubic Hermite + Newton
 * (cubic = 1) interpolation; tol_on_surface, dedup_time_tol,
 * dedup_point_tol as the reference.  Stores up to max_hits hits per
 * trajectory (hit_t [max_hits][ld], hit_y [max_hits][6][ld]); n_hits [N]
 * (stored), n_found [N] (nullable; accepted, equal to n_hits).
 * Replaces: poincare/synodic/backend.py:458-659 (_detect_with_segment_refine)
 * and :382-455 (_order_and_dedup_hits), as reached from
 * _SynodicDetectionBackend.detect_on_trajectory (:687-821). */
int hg_section_detect(int N, int m, const double* samples, long long ld,
                      const double* times, long long times_ld,
                      int axis, double offset, int direction, int plane_u, int plane_v,
                      int segment_refine, int cubic, int newton_max_iter,
                      double tol_on_surface, double dedup_time_tol, double dedup_point_tol,
                      int max_hits, double* hit_t, double* hit_y, int* n_hits, int* n_found,
                      void* stream);

/* Manifold acceptance filters on sampled trajectories: per trajectory the
 * minimum distances to the primaries and the maximum relative drift of the
 * Jacobi constant over the samples ([m][6][ld]).
 * Replaces: types/services/manifold.py:412-432 (body-radius filter) and
 * common/energy.py:26-74 (_max_rel_energy_error). */
int hg_trajectory_filters(int N, int m, const double* samples, long long ld, double mu,
                          double* min_r1, double* min_r2, double* max_rel_energy, void* stream);

/* Options of hg_correct_halo (defaults: hg_newton_opts_default; the values
 * of types/services/orbits.py:851-915 and corrector/options). */
typedef struct hg_newton_opts {
  double tol;            /* stop when the residual inf-norm < tol (1e-12) */
  int max_attempts;      /* Newton iterations (50) */
  double max_delta;      /* inf-norm cap of a step (1e-2; inf: none) */
  double alpha_reduction;/* Armijo backtracking factor (0.5) */
  double min_alpha;      /* smallest step scale tried (1e-4) */
  double armijo_c;       /* sufficient-decrease constant (0.1) */
  double cond_threshold; /* Tikhonov 1e-12 above this condition number (1e8) */
  double event_rtol, event_atol;  /* half-period crossing search (1e-12) */
  double stm_rtol, stm_atol;      /* STM propagation (1e-12) */
  int steps;             /* dense samples of the STM propagation (500; the last is used) */
} hg_newton_opts;
void hg_newton_opts_default(hg_newton_opts* o);

/* Batched single-shooting correction of halo orbits: every orbit's controls
 * (x0, vy0) are corrected so that vx and vz vanish at the first y = 0
 * crossing; all orbits still iterating share each propagation launch.  x:
 * device [6][ld] initial states, overwritten by the corrected ones;
 * half_period, residual (final inf-norm), iterations, status (HG_OK,
 * HG_NEWTON_DIVERGED, HG_EVENT_NOT_FOUND, HG_LINE_SEARCH_FAILED): device [N].
 * Synchronous on `stream`.  Its device buffers belong to the handle: after
 * hg_reserve_correct(h, M) calls with N <= M allocate nothing (otherwise the
 * first larger call grows them once).  Host arithmetic
 * follows the reference's numpy expressions; an exactly singular Jacobian
 * (which the reference hands to lstsq) ends that orbit's line search.
 * Replaces: corrector/backends/newton.py:39-143 with
 * corrector/operators.py:408-452, types/services/orbits.py:851-948,
 * corrector/backends/base.py:187-245, corrector/stepping/armijo.py:58-164
 * (orbit.correct() for halo orbits). */
int hg_correct_halo(hg_handle* h, double mu, int N, double* x, long long ld, double* half_period, int* iterations,
                    double* residual, int* status, const hg_newton_opts* opts, void* stream);
/* Sizes the handle's corrector buffers and event-refinement pool for
 * hg_correct_halo on up to max_orbits orbits.  Synchronous.
 * Replaces: nothing (the reference allocates per call). */
int hg_reserve_correct(hg_handle* h, int max_orbits);

/* hg_correct_halo run entirely on the device as one CUDA graph: the Newton
 * iterations of all N orbits and their Armijo line searches are nested
 * conditional WHILE nodes, the propagation legs run in list mode (the live
 * count read from device memory), and the Newton algebra and line-search
 * decisions are device kernels.  Asynchronous on `stream` (one graph launch
 * plus a load and a store kernel; nothing is read back).  Same arguments and
 * outputs as hg_correct_halo plus a caller workspace of at least
 * hg_correct_halo_graph_workspace_bytes(N) bytes (256-byte aligned), which
 * holds all iteration state; the call allocates nothing.  The graph is built
 * on the first call and cached on the handle (rebuilt when N, mu, the
 * options, the workspace or the lane tuning change).  Arithmetic differs from
 * hg_correct_halo in one place: the quadratic term's powers are correctly
 * rounded where the host driver calls the C library's pow (results agree to
 * the last bits of the Jacobian; iteration counts can differ by one where a
 * residual lands at the tolerance).  N <= 2^22, max_attempts <= 1000.
 * Replaces: as hg_correct_halo (execution on the device). */
long long hg_correct_halo_graph_workspace_bytes(int N);
int hg_correct_halo_graph(hg_handle* h, double mu, int N, double* x, long long ld, double* half_period,
                          int* iterations, double* residual, int* status, const hg_newton_opts* opts,
                          void* workspace, long long workspace_bytes, void* stream);

/* Native request server: continuous batching of DOP853 propagation requests
 * at the level of trajectory slots.  Every problem (mu, dim, t0, tmax,
 * options, event) with work gets a pool of device-resident trajectory slots
 * (pool_slots, halved until the server's free arenas hold the pool) on its own
 * stream; at most max_concurrent pools run at once.  A pool's thread admits
 * the waiting requests' trajectories into free slots (a request may enter
 * over several rounds), advances every live slot by seg_steps attempted
 * steps, refines the crossings saved, and returns the trajectories that
 * finished to their requests, freeing their slots: a request arriving while
 * others run enters at the next segment boundary, as slots free up.  One
 * host synchronization per segment: finished rows are gathered straight into
 * the pinned staging (mapped into the device's address space) and copied into
 * their requests while the next segment runs.
 * hg_serve_create allocates a device arena of hbm_budget_bytes and a pinned,
 * mapped host arena of staging_bytes that the pools are carved from; nothing is
 * allocated afterwards, and a request whose problem cannot get even a
 * 32-slot pool on an idle server fails (state 3, HG_ERR_ARGS).  Results equal
 * a direct hg_propagate_dop853 call on the request alone.  Requests: y0 host
 * row-major (N, dim); results host row-major: y_end (N, dim), t_end (N),
 * hit_t (N, max_hits), hit_y (N, max_hits, dim), n_hits / n_accept /
 * n_reject / status (N); null outputs are skipped.  Poll states: 0 pending,
 * 1 running (some trajectories admitted), 2 done, 3 failed.  Latency =
 * submit to completion; hg_serve_stats reports its p50 / p99 and the number
 * of segments run.
 * Replaces: nothing in the reference (its solves are synchronous calls);
 * the serving pattern of this library's Python engine behind the C ABI. */
typedef struct hg_server hg_server;
typedef struct hg_serve_config {
  int device;
  long long hbm_budget_bytes; /* device arena (default 8 GiB) */
  int max_concurrent;         /* pools (problems) in flight (default 4) */
  long long staging_bytes;    /* pinned host arena (default 1 GiB) */
  int pool_slots;             /* trajectory slots of a pool (default 32768, >= 32) */
  int seg_steps;              /* attempted steps per segment (default 16) */
} hg_serve_config;
void hg_serve_config_default(hg_serve_config* c);
int hg_serve_create(const hg_serve_config* cfg, hg_server** out);
int hg_serve_destroy(hg_server* s);
int hg_serve_submit(hg_server* s, double mu, int dim, int N, const double* y0, double t0, double tmax,
                    const hg_dop853_opts* opts, const hg_event* ev, long long* request_id);
int hg_serve_poll(hg_server* s, long long request_id, int* state);
int hg_serve_wait(hg_server* s, long long request_id, double timeout_s);
int hg_serve_fetch(hg_server* s, long long request_id, double* y_end, double* t_end, double* hit_t,
                   double* hit_y, int* n_hits, int* n_accept, int* n_reject, int* status);
int hg_serve_cancel(hg_server* s, long long request_id);
int hg_serve_stats(hg_server* s, double* p50_ms, double* p99_ms, long long* requests, long long* batches);

/* Section-point matching for connections (handle-free, asynchronous on
 * `stream`; point sets as two coordinate arrays each).
 * hg_radius_best: for each query point, the number of reference points
 * within eps (dx*dx + dy*dy <= eps^2 in FP64) and the nearest of them
 * (strict <, the lowest index wins ties; -1 if none).
 * hg_nearest_neighbor: each point's nearest other point of the same set
 * (strict <, lowest index on ties; -1 when n < 2).
 * coord_max >= every |coordinate| involved: it sizes the FP32 pre-screen,
 * whose margin provably keeps the FP64 results exact.  Each call makes an
 * FP32 copy of the scanned set (the reference set of hg_radius_best, the
 * set of hg_nearest_neighbor): into `workspace` (device, 16-byte aligned, at
 * least hg_points_workspace_bytes(n) bytes; HG_ERR_ARGS if smaller) when it
 * is given, so that the call allocates nothing, else into stream-ordered
 * scratch (cudaMallocAsync / cudaFreeAsync on `stream`; HG_ERR_CUDA if it
 * fails).
 * Replaces: connections/backends.py:31-99 (_pair_counts, _radpair2d: counts
 * and the pairs' per-query minimum used by _ConnectionsBackend.run :444-460)
 * and :174-235 (_nearest_neighbor_2d). */
long long hg_points_workspace_bytes(int n);
int hg_radius_best(int nq, const double* qx, const double* qy, int nr, const double* rx, const double* ry,
                   double eps, double coord_max, int* count, int* best_idx, double* best_d2,
                   void* workspace, long long workspace_bytes, void* stream);
int hg_nearest_neighbor(int n, const double* x, const double* y, double coord_max, int* out,
                        void* workspace, long long workspace_bytes, void* stream);

/* Segment refinement of n connection pairs (handle-free, asynchronous on
 * `stream`): pair k joins the unstable-side points pu[I[k]], pu[IU[k]] and the
 * stable-side points ps[J[k]], ps[JS[k]] (pu, ps row-major [n_set][2]; Xu, Xs
 * row-major [n_set][6] states).  Where ok[k] != 0: the closest points of the
 * two segments (the reference's scalar arithmetic and clamping), the states
 * xu = (1 - s) Xu[I] + s Xu[IU], xs = (1 - t) Xs[J] + t Xs[JS] and their
 * midpoint pt; elsewhere Xu[I], Xs[J] and pu[I].  Outputs xu, xs [n][6], pt
 * [n][2]; an index outside [0, nu) / [0, ns) gives NaN rows.
 * Replaces: connections/backends.py:237-320 (_closest_points_on_segments_2d)
 * and the per-pair interpolation of _ConnectionsBackend.run :480-520. */
int hg_connection_refine(int n, const int* I, const int* IU, const int* J, const int* JS, const unsigned char* ok,
                         int nu, const double* pu, const double* Xu, int ns, const double* ps, const double* Xs,
                         double* xu, double* xs, double* pt, void* stream);

/* Launch-shape tuning of a handle (set by hiten_gb300.autotune).
 * HG_TUNE_BLOCK_THREADS: threads per block, 32 (default), 64 or 128.
 * HG_TUNE_DOP853_LANES_D6: lanes per 6-dim DOP853 trajectory: 1 (one
 * trajectory per lane: least total work), 2 (lane pairs: 0.62x the per-step
 * latency), 6 (one component per lane: 0.40x), for batches too small to
 * fill the GPU, where the longest trajectory sets the time; 0 = automatic
 * (the default).
 * HG_TUNE_SEG_STEPS: attempted steps per segment of
 * hg_propagate_dop853_scheduled (default 16).
 * HG_TUNE_LANES_D42: lanes per 42-dim trajectory (fixed RK without an event
 * and DOP853): 7 (an STM column per lane), 14 (half a column per lane: 0.65x
 * the per-step latency), 12 (paired warps, fixed RK and single-pass DOP853
 * without an event: a state warp with the Hessian and an STM warp per five
 * trajectories, ~0.6x the per-step latency of 7 for RK8; blocks of one pair,
 * or of two pairs with HG_TUNE_BLOCK_THREADS 128; other calls then use 7),
 * 18 (three warps, fixed RK and single-pass DOP853 without an event: the
 * STM of five trajectories on two warps of half columns; other calls then
 * use 7), 0 = automatic (the default).
 * HG_TUNE_SM_CAPACITY: the layout cost models' FP64 capacity of an SM, in
 * tenths of a warp's demand (default 30: three warps run at full speed).
 * HG_TUNE_REFINE_POOL_MB: largest record pool (MB, default 8192) a single-pass
 * DOP853 call allocates to refine its event crossings after the integration;
 * larger requests (N x max_hits x (15 dim + 3) doubles) refine inline, with
 * the same results.
 * HG_TUNE_SPREAD: 1 = DOP853 launches use blocks of four warps that each
 * occupy a whole SM (one warp per SM sub-partition); 0 = HG_TUNE_BLOCK_THREADS
 * blocks (default).
 * Results are bit-identical for every setting.
 * Replaces: nothing (no reference counterpart; launch shape only). */
#define HG_TUNE_BLOCK_THREADS 1
#define HG_TUNE_DOP853_LANES_D6 2
#define HG_TUNE_SEG_STEPS 3
#define HG_TUNE_SPREAD 4
#define HG_TUNE_LANES_D42 5
#define HG_TUNE_SM_CAPACITY 6
#define HG_TUNE_REFINE_POOL_MB 7
int hg_set_tuning(hg_handle* h, int key, int value);
int hg_get_tuning(hg_handle* h, int key, int* value);

/* Counters of a handle.  HG_COUNTER_KERNEL_LAUNCHES: kernels launched
 * through the handle since hg_create (every propagation kernel, segment,
 * refinement and set-up kernel; memsets and copies are not kernels).
 * HG_COUNTER_ALLOCATIONS: device and pinned-host allocations made for the
 * handle since (and including) hg_create.
 * Replaces: nothing (instrumentation only). */
#define HG_COUNTER_KERNEL_LAUNCHES 1
#define HG_COUNTER_ALLOCATIONS 2
int hg_get_counter(hg_handle* h, int key, long long* value);

/* Host helper: out[i] = pow(x[i], e) through the C library's pow, i < n
 * (host arrays).  The reference's numpy-scalar `**` calls C pow (numpy's
 * array `**` takes other code paths that differ in the last bit); the
 * Python corrector uses this to evaluate its batched quadratic term with
 * the reference's bits.  Synchronous, no device work.
 * Replaces: the scalar `**` of types/services/orbits.py:917-948
 * (_halo_quadratic_term), evaluated per orbit in the reference. */
void hg_host_pow(long long n, const double* x, double e, double* out);

/* Self-test of the bounded inter-warp wait the paired 42-dim layouts use
 * (every hand-off wait gives up after a time limit and the kernel reports
 * HG_SYNC_TIMEOUT instead of hanging): one warp waits limit_ms on a barrier
 * nothing arrives at, then on one the other warp arrives at.  out3 (device,
 * 3 ints): [0] 1 if the first wait ran out, [1] 1 if the second completed,
 * [2] nanoseconds the first wait took.  Asynchronous on `stream`.
 * Replaces: nothing (failure-path test of the library's own waits). */
int hg_selftest_bounded_wait(hg_handle* h, int limit_ms, int* out3, void* stream);

/* Measured FP64 fused-multiply-add throughput of this device (TFLOP/s,
 * counting an FMA as 2 flops): runs a short dependent-chain-free DFMA loop
 * on all SMs and times it with CUDA events.  Synchronous. */
int hg_probe_fp64_peak(hg_handle* h, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* HITENGPU_H */
