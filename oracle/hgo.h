/*
 * CPU oracle for the CR3BP trajectory-propagation path (test infrastructure).
 *
 * This library restates, operation for operation, the reference's numba
 * kernels on the hot path so that the CUDA kernels can be checked against it:
 *
 *   dynamics/rtbp.py:30-74      _crtbp_accel      -> hgo_rhs6
 *   dynamics/rtbp.py:76-255     _jacobian_crtbp + _var_equations -> hgo_rhs42
 *   dynamics/base.py:272-310    _DirectedSystem sign flips (fwd, flip range)
 *   integrators/rk.py:154-215   rk_embedded_step_jit_kernel
 *   integrators/rk.py:531-588   _FixedStepRK._integrate_fixed_rk -> hgo_fixed_rk
 *   integrators/rk.py:1636-1708 dop853_step_jit_kernel
 *   integrators/rk.py:1790-2003 dense cache build / evaluation
 *   integrators/rk.py:2005-2102 _dop853_refine_in_step
 *   integrators/rk.py:2375-2549 _DOP853._integrate_dop853 -> hgo_dop853_dense
 *   integrators/rk.py:2678-2803 _DOP853._integrate_dop853_until_event -> hgo_dop853_event
 *   integrators/utils.py:13-296 event predicates, step-size helpers
 *
 * Arithmetic: IEEE double, no contraction (built with -ffp-contract=off, as
 * numba's fastmath=False), the same association order as the reference
 * expressions.  Powers are the one place where the reference's result
 * depends on how it is run:
 *   HGO_MODE_PYTHON  every `**` calls libm pow, as CPython does when the
 *                    reference runs without numba (reproduces the golden
 *                    fixtures bit for bit on the host that made them);
 *   HGO_MODE_NUMBA   numba's lowering: x**2 -> x*x, x**3 -> x*(x*x), and
 *                    libm pow for the fractional exponents (x**1.5, x**2.5,
 *                    step-size controller) -- the reference as shipped;
 *   HGO_MODE_DEVICE  numba's integer powers, fractional powers correctly
 *                    rounded (evaluated in quad precision, rounded once):
 *                    what the CUDA kernels compute.  It differs from NUMBA
 *                    only where libm pow misrounds (about 1e-3 of calls).
 *
 * numpy's float64 dot on the x86-64 host the fixtures come from accumulates
 * a 6-vector with sequential fused multiply-adds and a 42-vector as
 * (32-element blocked AVX-512 sum) + fused tail; hgo reproduces that order
 * for the DOP853 error norm and the initial-step heuristic.
 *
 * This code is only used by tests and the CPU-baseline leg of bench.py.
 */
#ifndef HGO_H
#define HGO_H

#ifdef __cplusplus
extern "C" {
#endif

enum { HGO_MODE_PYTHON = 0, HGO_MODE_NUMBA = 1, HGO_MODE_DEVICE = 2 };

/* Status codes (shared meaning with the CUDA library). */
enum {
  HGO_OK = 0,
  HGO_MAX_STEPS = 1,
  HGO_NONFINITE = 3,
  HGO_BAD_ARGS = 10
};

void hgo_set_mode(int mode);
int hgo_get_mode(void);
/* x**y for a fractional exponent, x**2 and x**3, under the current mode */
double hgo_fpow(double x, double y);
double hgo_ipow2(double x);
double hgo_ipow3(double x);

void hgo_rhs6(const double* y, double mu, double* dy);
void hgo_rhs42(const double* y, double mu, double* dy);

/* fixed-step RK (order 4, 6 or 8) over the nodes t_vals[0..n-1];
 * states is (n, dim) row-major; returns status. */
int hgo_fixed_rk(int order, int dim, double mu, int fwd, int flip_lo, int flip_hi,
                 const double* y0, const double* t_vals, int n, double* states);

/* DOP853 without events, dense output at t_eval[0..m-1] (t_eval ascending
 * internal time).  y_out is (m, dim).  Counters may be NULL. */
int hgo_dop853_dense(int dim, double mu, int fwd, int flip_lo, int flip_hi,
                     const double* y0, const double* t_eval, int m,
                     double rtol, double atol, double max_step, double min_step,
                     long max_steps, double* y_out, long* n_accept, long* n_reject);

/* DOP853 with a plane event g = y[ev_index] - ev_offset.  max_hits == 1
 * reproduces the reference's terminal event; max_hits > 1 records further
 * crossings without changing the step sequence.  hit_t (max_hits),
 * hit_y (max_hits, dim).  t_end / y_end: the last accepted state (for a
 * terminal hit, the end of the step containing the crossing). */
int hgo_dop853_event(int dim, double mu, int fwd, int flip_lo, int flip_hi,
                     const double* y0, double t0, double tmax,
                     double rtol, double atol, double max_step, double min_step,
                     long max_steps, int ev_index, double ev_offset, int ev_dir,
                     int max_hits, double xtol, double gtol,
                     double* hit_t, double* hit_y, int* n_hits,
                     double* t_end, double* y_end, long* n_accept, long* n_reject);

/* Fixed step with a terminal plane event, integrators/rk.py:655-718.
 * Returns 1 on a crossing (t_hit, y_hit (dim,)), 0 without, -1 on bad args. */
int hgo_fixed_rk_event(int order, int dim, double mu, int fwd, int flip_lo, int flip_hi, const double* y0,
                       const double* t_vals, int n, int ev_index, double ev_offset, int ev_dir, double xtol,
                       double gtol, double* states, double* t_hit, double* y_hit);

/* Section crossings on one sampled trajectory (plane y[axis] = offset),
 * poincare/synodic/backend.py:382-659.  times (m,), states (m, 6).  Stores
 * at most max_hits hits (hit_t (max_hits,), hit_y (max_hits, 6)) and
 * returns the number accepted. */
int hgo_section_detect(const double* times, const double* states, int m, int axis, double offset, int direction,
                       int pu, int pv, int segment_refine, int cubic, int newton_max_iter, double tol_on_surface,
                       double dedup_time_tol, double dedup_point_tol, int max_hits, double* hit_t, double* hit_y,
                       int* n_stored);

/* Batched variants over independent trajectories, threaded over `threads`
 * host threads (one trajectory per task).  Arrays are trajectory-major:
 * y0 (N, dim), states (N, n, dim) ... */
int hgo_fixed_rk_batch(int order, int dim, double mu, int fwd, int flip_lo, int flip_hi,
                       int N, const double* y0, const double* t_vals, int n,
                       int out_every, double* out, int threads);

int hgo_dop853_event_batch(int dim, double mu, int fwd, int flip_lo, int flip_hi,
                           int N, const double* y0, double t0, double tmax,
                           double rtol, double atol, double max_step, double min_step,
                           long max_steps, int ev_index, double ev_offset, int ev_dir,
                           int max_hits, double xtol, double gtol,
                           double* hit_t, double* hit_y, int* n_hits,
                           double* t_end, double* y_end, long* n_accept, long* n_reject,
                           int* status, int threads);

#ifdef __cplusplus
}
#endif

#endif /* HGO_H */
