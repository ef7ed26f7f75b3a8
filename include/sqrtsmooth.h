/*
 * sqrtsmooth: C ABI of the GB300 square-root parallel smoother.
 *
 * This is the drop-in boundary for the parallel-mode path of parsmooth
 * (EEA-sensors/sqrt-parallel-smoothers).  Each entry point replaces one
 * reference function; the citation is given beside it.  All array arguments
 * are raw device pointers of the problem's dtype (float or double) unless
 * stated otherwise, row-major, densely packed.  The library never allocates
 * device memory: scratch space is a caller-provided workspace whose size comes
 * from ss_workspace_bytes().  Every call is asynchronous on the given stream
 * and returns an ss_status.
 *
 * Batches.  B independent sequences of lengths T_i are packed back to back:
 *   observations  (sum T_i, ny), sequence i at rows [offsets[i], offsets[i+1])
 *   trajectories  (sum (T_i + 1), nx) means and (sum (T_i + 1), nx, nx)
 *                 lower Cholesky factors, sequence i at rows
 *                 [offsets[i] + i, offsets[i+1] + i + 1)
 * offsets is a device int64 array of B+1 entries with offsets[0] = 0.
 */
#ifndef SQRTSMOOTH_H_
#define SQRTSMOOTH_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* ss_stream_t; /* a cudaStream_t */

typedef enum {
  SS_OK = 0,
  SS_ERR_INVALID = 1,      /* bad argument: null pointer, size, shape (reference: TypeError/ValueError) */
  SS_ERR_UNSUPPORTED = 2,  /* model, method or dimension not built (reference: NotImplementedError) */
  SS_ERR_CUDA = 3,         /* a CUDA launch or runtime call failed */
  SS_ERR_WORKSPACE = 4     /* workspace smaller than ss_workspace_bytes() */
} ss_status;

enum { SS_F32 = 0, SS_F64 = 1 };

/* Linearisation methods: parsmooth/linearization/__init__.py:1-5 */
enum {
  SS_LIN_EXTENDED = 0,      /* parsmooth/linearization/_extended.py:9-70 */
  SS_LIN_CUBATURE = 1,      /* parsmooth/linearization/_cubature.py:10-85 */
  SS_LIN_UNSCENTED = 2,     /* parsmooth/linearization/_unscented.py:10-101 */
  SS_LIN_GAUSS_HERMITE = 3  /* parsmooth/linearization/_gh.py:13-151 */
};

/* Device model registry (the reference accepts any JAX callable in
 * FunctionalModel, parsmooth/_base.py:15-17; device code needs a known model) */
enum {
  SS_MODEL_LINEAR = 0,           /* f(x) = A x                       (tests/_lgssm.py:5-35) */
  SS_MODEL_COORDINATED_TURN = 1, /* CT transition, nx = 5            (tests/bearings/bearings_utils.py:7-44) */
  SS_MODEL_BEARINGS = 2,         /* two bearings atan2, ny = 2       (tests/bearings/bearings_utils.py:47-69) */
  SS_MODEL_RICKER = 3,           /* f(x)_i = a + x_i - exp(x_i), params[0] = a
                                    (notebooks/population_model.py:9-21, a = log 44.7) */
  SS_MODEL_POISSON_EXP = 4       /* conditional moments, ny <= nx: E[y_k|x] = Var[y_k|x] = lam exp(x_k),
                                    params[0] = lam (notebooks/population_model.py:83-118); the
                                    observation noise arguments are ignored */
};

/* Sigma-point regression form (see ss_lin.cuh): 0 = automatic (the
 * reference's downdate in FP64, the cancellation-free residual form in FP32),
 * 1 = downdate (parsmooth/linearization/_sigma_points.py:77-78), 2 = residual. */
enum { SS_SLR_AUTO = 0 };

#define SS_MAX_GH_ORDER 8

/* A FunctionalModel(function, MVNSqrt(noise_mean, noise_chol)). */
typedef struct ss_model {
  int32_t kind;            /* SS_MODEL_* */
  int32_t reserved;
  const void* matrix;      /* SS_MODEL_LINEAR: (d_out, d_in) matrix A, device */
  double params[4];        /* COORDINATED_TURN: {dt}; BEARINGS: {s1x, s1y, s2x, s2y} */
  const void* noise_mean;  /* (d_out,), device */
  const void* noise_chol;  /* (d_out, d_out) lower triangular, device */
} ss_model;

/* ss_problem.options bits.  For linear models with nx > 5, a batch of equally long
 * sequences that share one prior has one covariance recursion: the large-state path then
 * computes every factor once and only the means per sequence (up to 32 sequences).  This
 * bit forces the per-sequence computation instead. */
#define SS_OPT_PER_SEQUENCE_COVARIANCE 1
/* Covariance form: every factor argument of ss_linearize, ss_filter, ss_smooth and
 * ss_iterated is a covariance instead of a lower Cholesky factor (the models'
 * noise_chol, L0, the nominal, filtered and output trajectories, and the linearised
 * noise of ss_linearize), and the calls run the reference's covariance-form
 * ("standard") elements, operators and linearisation: parsmooth/parallel/_operators.py:7-40
 * and 80-101, parsmooth/parallel/_filtering.py:64-97 and 157-163,
 * parsmooth/parallel/_smoothing.py:60-69, parsmooth/linearization/_sigma_points.py:39-60
 * and 81-86, in the problem's precision.  Built for nx <= 5, ny <= 3 (not the
 * large-state pairs); the workspace query must see the bit. */
#define SS_OPT_COVARIANCE_FORM 2

typedef struct ss_problem {
  int32_t dtype;           /* SS_F32 or SS_F64 */
  int32_t nx, ny;
  int32_t lin_method;      /* SS_LIN_* */
  double ut_alpha, ut_beta, ut_kappa; /* unscented parameters */
  int32_t ut_kappa_default;/* nonzero: kappa = 3 + nx (parsmooth/linearization/_unscented.py:64-65) */
  int32_t gh_order;        /* Gauss-Hermite order, 1..SS_MAX_GH_ORDER */
  int32_t slr_form;        /* SS_SLR_AUTO, 1 or 2 */
  int32_t chunk;           /* steps per level-0 chunk, 0 = default */
  int32_t group;           /* summaries per group at higher scan levels, 0 = default */
  int32_t options;         /* SS_OPT_* bits, 0 = defaults */
  ss_model transition;     /* nx -> nx */
  ss_model observation;    /* nx -> ny */
  int64_t batch;           /* B >= 1 */
  int64_t total_steps;     /* sum T_i */
  int64_t max_len;         /* max T_i (upper bound is enough) */
  const int64_t* offsets;  /* device, B + 1 */
} ss_problem;

/* Library version (major * 10000 + minor * 100 + patch). */
int ss_version(void);

/* Static text of a status code. */
const char* ss_status_string(int status);

/* Nonzero if (dtype, nx, ny, lin_method, models) has compiled kernels. */
int ss_supported(const ss_problem* p);

/* Workspace bytes for any entry point below on this problem (host only). */
int ss_workspace_bytes(const ss_problem* p, size_t* bytes);

/* Linearise one model at n points x_k = N(m[k], chol[k] chol[k]^T).
 * Replaces linearization_method(model, x) of parsmooth/linearization/*.py
 * (e.g. _cubature.py:10-34), vectorised.  which = 0 transition, 1 observation.
 * Outputs F (n, d_out, nx), chol (n, d_out, d_out), b (n, d_out). */
int ss_linearize(const ss_problem* p, int32_t which, int64_t n, const void* m, const void* chol,
                 void* F, void* chol_out, void* b, ss_stream_t stream);

/* Parallel square-root filter: parsmooth/parallel/_filtering.py:13-61
 * (methods.filtering, parsmooth/methods.py:14-26, with parallel=True).
 * m0 (B or 1, nx), L0 (B or 1, nx, nx): prior_per_sequence selects B or 1.
 * nominal_m / nominal_L: the linearisation trajectory or NULL for the
 * reference's default (zero means, identity factors, _filtering.py:25-28).
 * out_m / out_L: filtered trajectory (T+1 states per sequence).
 * out_ell: NULL or (B,) double, the summed predictive log-likelihood
 * (_filtering.py:53-60). */
int ss_filter(const ss_problem* p, const void* ys, const void* m0, const void* L0,
              int32_t prior_per_sequence, const void* nominal_m, const void* nominal_L,
              void* out_m, void* out_L, double* out_ell, void* workspace, size_t workspace_bytes,
              ss_stream_t stream);

/* Parallel square-root RTS smoother: parsmooth/parallel/_smoothing.py:14-44
 * (methods.smoothing, parsmooth/methods.py:29-35, parallel=True).
 * filt_m / filt_L: a filtered trajectory; nominal: as in ss_filter. */
int ss_smooth(const ss_problem* p, const void* filt_m, const void* filt_L, const void* nominal_m,
              const void* nominal_L, void* out_m, void* out_L, void* workspace,
              size_t workspace_bytes, ss_stream_t stream);

/* Iterated smoother: parsmooth/methods.py:54-76 with parallel=True.
 * init_m / init_L: initial nominal trajectory, or NULL for the reference's
 * extra filter-smoother pass at the default nominal (:63-65).
 * n_iter: number of filter-smoother calls (criterion "i < n_iter"), or the
 * maximum number when tol > 0; with tol > 0 a sequence stops once the mean
 * squared change of its means is <= tol (_default_criterion, :50-51, uses
 * 1e-6).  out_ell: NULL or (B,) double - the log-likelihood of a final
 * filtering pass at the converged trajectory (:72-75).  out_iters: NULL or
 * (B,) int32 filter-smoother calls made per sequence.  out_flags: NULL or
 * (B,) uint32 status bits: 1 non-finite output, 2 non-finite log-likelihood,
 * 4 not converged within n_iter (tol > 0 only). */
int ss_iterated(const ss_problem* p, const void* ys, const void* m0, const void* L0,
                int32_t prior_per_sequence, const void* init_m, const void* init_L,
                int32_t n_iter, double tol, void* out_m, void* out_L, double* out_ell,
                int32_t* out_iters, uint32_t* out_flags, void* workspace, size_t workspace_bytes,
                ss_stream_t stream);

/* ss_iterated without a workspace argument, for callers that cannot allocate
 * device memory (no counterpart in the reference, which lets JAX/XLA allocate).
 * Scratch comes from a fixed array of SS_NOALLOC_SCRATCH_BYTES inside the
 * library's device image, held on every GPU that loads the library until the
 * process exits.  Problems whose ss_workspace_bytes exceed it are rejected
 * with SS_ERR_WORKSPACE.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress, with that device current); make that
 * first call before any stream capture.  The address is remembered per device
 * for the life of the process: it does not survive cudaDeviceReset or any
 * other teardown of the device's primary context, after which this entry
 * point must not be called again in the same process.  All calls share the one array, so
 * calls whose GPU work overlaps (other streams, other threads) race and must
 * be serialised by the caller; a call fully rewrites what it reads, so no
 * clearing between calls is needed.  Allocates nothing. */
#define SS_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int ss_iterated_noalloc(const ss_problem* p, const void* ys, const void* m0, const void* L0,
                        int32_t prior_per_sequence, const void* init_m, const void* init_L,
                        int32_t n_iter, double tol, void* out_m, void* out_L, double* out_ell,
                        int32_t* out_iters, uint32_t* out_flags, ss_stream_t stream);

/* Forward-mode sensitivities of the pseudo-log-likelihood.
 * The reference obtains dl/dtheta with jax.grad through its parallel filter
 * (used in notebooks/experiment_bearing_only_parameter_estimation.ipynb:91).
 * Here the filter of ss_filter (parsmooth/parallel/_filtering.py:13-61 with
 * return_loglikelihood) is run in tangent-linear arithmetic: every model
 * scalar carries up to SS_MAX_TANGENTS derivative directions d(.)/dtheta_k,
 * given by ss_tangents, and the log-likelihood of each sequence comes back
 * with its gradient (out_grad, (B, n_dir) double).  Built for
 * (nx, ny) = (5, 2) and (2, 2) with the extended, cubature and unscented
 * linearisations. */
#define SS_MAX_TANGENTS 4
typedef struct ss_tangents {
  int32_t n_dir;                      /* 1..SS_MAX_TANGENTS */
  int32_t reserved;
  double trans_params[SS_MAX_TANGENTS][4];  /* d(transition params)/dtheta_k */
  double obs_params[SS_MAX_TANGENTS][4];    /* d(observation params)/dtheta_k */
  const void* trans_matrix;           /* (n_dir, nx, nx) or NULL for zero, device */
  const void* obs_matrix;             /* (n_dir, ny, nx) or NULL */
  const void* trans_noise_mean;       /* (n_dir, nx) or NULL */
  const void* trans_noise_chol;       /* (n_dir, nx, nx) lower triangular, or NULL */
  const void* obs_noise_mean;         /* (n_dir, ny) or NULL */
  const void* obs_noise_chol;         /* (n_dir, ny, ny) lower triangular, or NULL */
} ss_tangents;

int ss_filter_grad_workspace_bytes(const ss_problem* p, size_t* bytes);
int ss_filter_grad(const ss_problem* p, const ss_tangents* tangents, const void* ys, const void* m0,
                   const void* L0, int32_t prior_per_sequence, const void* nominal_m, const void* nominal_L,
                   double* out_ell, double* out_grad, void* workspace, size_t workspace_bytes,
                   ss_stream_t stream);

/* Pathwise posterior sampler: parsmooth.sampling (parsmooth/methods.py:79-91,
 * parsmooth/_pathwise_sampler.py:13-127).  From the filtered trajectory
 * (filt_m, filt_L) and the transition linearised at the nominal (NULL: zero
 * means / identity factors; the reference's default is the smoothed trajectory,
 * which the caller passes), draws n_samples trajectories per sequence:
 * x_T = m_T + L_T e_T, x_t = E_t x_{t+1} + g_t + D_t e_t (t < T), with
 * (g_t, E_t, D_t) the square-root smoothing elements.  eps and out share the
 * trajectory layout of the states, (sum (T_i + 1), n_samples, nx); eps holds
 * standard normals (the reference draws eps[0] for the last state and eps[1 + t]
 * for step t; here eps[t] drives step t and eps[T] the last state). */
int ss_sample(const ss_problem* p, const void* filt_m, const void* filt_L, const void* nominal_m,
              const void* nominal_L, int32_t n_samples, const void* eps, void* out, void* workspace,
              size_t workspace_bytes, ss_stream_t stream);

/* Log-likelihood of the iterated smoother and its derivatives along the same
 * tangent directions: jax.grad of parsmooth.iterated_smoothing(...,
 * return_loglikelihood=True) (parsmooth/methods.py:54-76 with the fixed-point
 * VJP of parsmooth/_utils.py:113-133), as used for parameter estimation.  The
 * n_iter-call loop (after the default-nominal pass when init_m is NULL) runs in
 * tangent-linear arithmetic, so the tangent of each nominal trajectory enters
 * the next linearisation; out_ell/out_grad are those of the filtering pass at
 * the final nominal.  This is the exact derivative of the n_iter-call
 * iteration, which tends to the implicit-function derivative as it converges. */
int ss_iterated_grad_workspace_bytes(const ss_problem* p, size_t* bytes);
int ss_iterated_grad(const ss_problem* p, const ss_tangents* tangents, const void* ys, const void* m0,
                     const void* L0, int32_t prior_per_sequence, const void* init_m, const void* init_L,
                     int32_t n_iter, double* out_ell, double* out_grad, void* workspace,
                     size_t workspace_bytes, ss_stream_t stream);

/* Reverse-mode gradient of the pseudo-log-likelihood.
 * Replaces jax.grad of the reference's parallel filter log-likelihood
 * (parsmooth/parallel/_filtering.py:13-61 with return_loglikelihood, summed
 * over :149-154) at a fixed nominal trajectory: the gradient of each
 * sequence's ell with respect to every input array at once, at a cost that
 * does not grow with the number of parameters.  The filter runs forward and
 * the smoother's backward associative scan once; the gradient follows from
 * the smoothed moments of the linearised model (Fisher's identity, exact for
 * the linear-Gaussian model the filter runs), contracted per step and summed
 * in FP64.  Every output pointer is a device double array or NULL (not
 * computed):
 *   trans_matrix (B, nx, nx), obs_matrix (B, ny, nx): d ell_i / d A of linear
 *     models (left untouched for other kinds);
 *   trans_noise_mean (B, nx), obs_noise_mean (B, ny);
 *   trans_noise_chol (B, nx, nx), obs_noise_chol (B, ny, ny): lower triangles
 *     (the library reads only those entries), zero above;
 *   trans_params (B, 4), obs_params (B, 4): d ell_i / d ss_model.params
 *     (coordinated-turn dt, bearings sensor coordinates, Ricker a), chained
 *     through each step's linearisation; not with Gauss-Hermite;
 *   m0 (B, nx), L0 (B, nx, nx) (lower): the prior; with a shared prior
 *     (prior_per_sequence = 0) row i is sequence i's share, sum the rows.
 * Built for nx <= 5, ny <= 3; conditional-moments observation models
 * (SS_MODEL_POISSON_EXP) and the covariance form are not supported.  The
 * workspace also holds the call's filtered and smoothed trajectories. */
typedef struct ss_adjoints {
  double* trans_matrix;
  double* trans_noise_mean;
  double* trans_noise_chol;
  double* obs_matrix;
  double* obs_noise_mean;
  double* obs_noise_chol;
  double* trans_params;
  double* obs_params;
  double* m0;
  double* L0;
} ss_adjoints;

int ss_filter_adjoint_workspace_bytes(const ss_problem* p, size_t* bytes);
int ss_filter_adjoint(const ss_problem* p, const void* ys, const void* m0, const void* L0,
                      int32_t prior_per_sequence, const void* nominal_m, const void* nominal_L,
                      double* out_ell, const ss_adjoints* out, void* workspace, size_t workspace_bytes,
                      ss_stream_t stream);

/* Instrumentation (no counterpart in the reference, which has no tracing):
 * a counter of kernels launched by this library, and per-kernel CUDA-event
 * timing.  While profiling is enabled every launch is bracketed by two events
 * on its stream (also when the launches are captured into a CUDA graph: the
 * events are then re-recorded by every replay).  ss_profile_read waits for the
 * recorded events and writes {"kernel": [launches, total_ms], ...} as JSON;
 * ss_profile_reset destroys them (after any graph holding them is gone). */
long long ss_launch_count(void);
int ss_profile_enable(int on);
int ss_profile_read(char* buf, size_t len);
int ss_profile_reset(void);

#ifdef __cplusplus
}
#endif

#endif /* SQRTSMOOTH_H_ */
