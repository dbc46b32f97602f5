/*
 * fastreg_gb300.h -- C ABI of the GB300-native fastreg registration loop.
 *
 * Plain C: pointers, sizes and status codes only.  Every call returns an int
 * status (FR_OK = 0) and never exits the process; fr_last_error() gives the
 * message of the last failure on a handle.  Device pointers are CUDA device
 * pointers of the current device; `stream` is a cudaStream_t passed as void*
 * (NULL = the legacy default stream).
 *
 * Each entry point names the reference interface it replaces (paths are inside
 * the fastreg source tree).
 */
#ifndef FASTREG_GB300_H
#define FASTREG_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FR_ABI_VERSION 3

/* status codes */
#define FR_OK 0
#define FR_ERR_INVALID_ARG 1 /* bad pointer, size or parameter value */
#define FR_ERR_CUDA 2        /* a CUDA runtime call or kernel launch failed */
#define FR_ERR_ALLOC 3       /* device or host allocation failed */
#define FR_ERR_IO 4          /* a file could not be opened or read */
#define FR_ERR_PARSE 5       /* a params.ini line could not be parsed */
#define FR_ERR_STATE 6       /* call out of order (e.g. stats before a registration) */
#define FR_ERR_NUMERIC 7     /* the solver produced NaN/Inf */

/* solver selection (params.ini key SOLVER=) */
#define FR_SOLVER_REFERENCE 0 /* the reference's accelerated PDE flow */
#define FR_SOLVER_SOBOLEV 1   /* SSD + Gaussian-smoothed gradient + momentum */

/* fields for fr_get_field / fr_set_field */
#define FR_FIELD_PSI 0     /* psi, 3 planes of positions (voxel units) */
#define FR_FIELD_PSI_INV 1 /* psi_inv, 3 planes */
#define FR_FIELD_V 2       /* velocity, 3 planes (sobolev: momentum) */
#define FR_FIELD_RHO 3     /* density, 1 plane (reference solver only) */

#define FR_MAX_LABELS 256

/* Solver parameters: struct Params (include/params.hpp:7-26) plus the keys of the
 * sobolev solver.  Field names follow the params.ini keys. */
typedef struct fr_params {
    int volume_dims[3];    /* VOL_DIMS_X/Y/Z */
    float volume_size[3];  /* VOL_SIZE_X/Y/Z (parsed, unused by the solver, as in the reference) */
    int no_labels;         /* NO_LABELS (<= FR_MAX_LABELS) */
    int max_iter;          /* MAX_ITER */
    float max_update_norm; /* MAX_UPDATE_NORM */
    float rho_0;           /* RHO_0 */
    float tau;             /* TAU */
    float w_reg;           /* W_REG */
    float alpha;           /* ALPHA */
    float p;               /* p */
    float C;               /* C */
    int reset_iter;        /* RESET_ITER (<= 0: never) */
    int verbosity;         /* 0, 1 (--verbose), 2 (--vverbose) */
    /* additions (new params.ini keys) */
    int solver;            /* SOLVER=reference|sobolev */
    float smooth_sigma;    /* SMOOTH_SIGMA (sobolev) */
    int smooth_width;      /* SMOOTH_WIDTH, odd, <= 15 (sobolev) */
    float damping;         /* DAMPING (sobolev momentum) */
    float step;            /* STEP (sobolev step size) */
    int keep_state;        /* KEEP_STATE=1: continue from the previous call's fields,
                              as FastReg::operator() does on a reused instance */
    int autotune;          /* AUTOTUNE=1 (default): time a few tile shapes and block counts
                              per kernel on the first registration of a size class and
                              keep the fastest (results do not depend on the shapes) */
    int staging;           /* STAGING=0 (default): each kernel's staging is the default or
                              the autotuner's choice; 1: per-thread cp.async only; 2: TMA
                              tensor copies wherever a kernel has them (results do not
                              depend on it) */
} fr_params;

typedef struct fr_handle fr_handle;

/* One pair of a cohort: caller-owned device buffers, overwritten in place
 * (img_T/lab_T <- T o psi_inv, img_S/lab_S <- S o psi; fastreg.cpp:71-72). */
typedef struct fr_pair {
    int dims[3];
    float *img_T;
    int16_t *lab_T;
    float *img_S;
    int16_t *lab_S;
} fr_pair;

/* Results of the last registration of one pair. */
typedef struct fr_stats {
    int iterations;            /* iterations run */
    int converged;             /* 1 if MAX_UPDATE_NORM stopped the solver */
    float last_max_update_norm;
    int64_t last_max_update_voxel; /* linear index x + X*(y + Y*z) */
    double e_data;             /* 0.5 * sum (T - S o psi)^2, FP64 */
    double e_reg;              /* 0.5 * sum ||J_u||_F^2, FP64 */
    double energy;             /* e_data + w_reg * e_reg */
    int64_t folds;             /* #{voxels : det(I + J_u) <= 0} */
    int no_labels;
    double dice[FR_MAX_LABELS]; /* per label 2|A n B| / (|A| + |B|) (NaN if both empty) */
    double dice_all;           /* pooled over labels 1..no_labels-1 */
    int64_t dice_out_of_range; /* voxels whose label is outside [0, no_labels) */
    int64_t dice_inter[FR_MAX_LABELS];
    int64_t dice_count[FR_MAX_LABELS];
} fr_stats;

/* ---- parameters: Params + the app's Boost parse of params.ini (demo.cpp:96-149) ---- */
int fr_params_default(fr_params *p);
int fr_params_parse_ini(const char *text, fr_params *p); /* text of a params.ini */
int fr_params_load_ini(const char *path, fr_params *p);

/* ---- solver lifetime: FastReg(const Params&) (fastreg.hpp:14, fastreg.cpp:24-46)
 *      and Solver(Params&) (solver.hpp:64-66, solver.cpp:7-65) ---- */
int fr_create(const fr_params *p, fr_handle **out);
int fr_destroy(fr_handle *h);

/* ---- one registration: FastReg::operator() (fastreg.hpp:24, fastreg.cpp:58-75) ->
 *      Solver::estimate_psi (solver.hpp:68-78) -> device::estimate_psi (solver.cu:295-444).
 *      Enqueued on `stream`; outputs are ready when the stream reaches them. ---- */
int fr_register(fr_handle *h, float *img_T, int16_t *lab_T, float *img_S, int16_t *lab_S, void *stream);

/* ---- a cohort of independent pairs of uneven sizes in one set of launches per
 *      iteration (no counterpart in the reference, which runs one pair per process) ---- */
int fr_register_batch(fr_handle *h, const fr_pair *pairs, int n_pairs, void *stream);

/* ---- results: the reference prints them (solver.cu:40-47,408-424, reductor.cpp:357-360) ---- */
int fr_get_stats(fr_handle *h, int pair, fr_stats *out);
int fr_get_trace(fr_handle *h, int pair, float *norms, int64_t *voxels, int cap, int *n_out);

/* ---- fields of the last registration: FastReg::getDeformationField() (fastreg.hpp:22).
 *      d_buf holds 3*N floats for vector fields, N for rho. ---- */
int fr_get_field(fr_handle *h, int pair, int which, float *d_buf, void *stream);
int fr_set_field(fr_handle *h, int pair, int which, const float *d_buf, void *stream);

/* ---- the phases of one registration, for callers that step the solver themselves
 *      (the reference's estimate_psi loop body, solver.cu:329-433) ---- */
int fr_begin(fr_handle *h, const fr_pair *pairs, int n_pairs, void *stream); /* pack + init */
int fr_step(fr_handle *h, int iter, float t, void *stream);                 /* one iteration */
int fr_finish(fr_handle *h, void *stream);                                  /* outputs + stats */

/* ---- measurement: run `iters` iterations from the current state with CUDA events
 *      around every launch on `stream`; ms[k] = mean duration of kernel k of one
 *      iteration (reference solver: k = 0 Laplacian, 1 pass A, 2 pass B; sobolev:
 *      0 gradient, 1 smoothing + momentum, 2 pass B);
 *      n_kernels receives the count.  No counterpart in the reference. ---- */
int fr_time_kernels(fr_handle *h, int iters, float *ms, int *n_kernels, void *stream);

/* Per-pair regularisation weights (W_REG) for the cohorts registered from now on: w_reg[p]
 * for pair p of the next fr_register_batch / fr_begin, which must have n pairs; NULL or
 * n <= 0 goes back to params.w_reg for every pair.  (The reference has one W_REG per
 * FastReg; this lets one batched launch register pairs with their own weights, e.g. each
 * tuned by fr_sobolev_loss_grad.) */
int fr_set_pair_w_reg(fr_handle *h, const float *w_reg, int n);

/* Tile shape of kernel k (0..2: the active solver's kernels in launch order -- reference:
 * Laplacian, pass A, pass B; sobolev: gradient, smoothing, update) after the last
 * fr_register / fr_begin: slices per tile and blocks per SM (-1: one block per tile),
 * the defaults or the autotuner's choice (AUTOTUNE). */
int fr_tile_shape(const fr_handle *h, int k, int *depth, int *blocks_per_sm);

/* How kernel k (as in fr_tile_shape) stages its stencil operands after the last
 * fr_register / fr_begin: *tma = 1 for tensor copies (TMA, cp.async.bulk.tensor), 0 for
 * per-thread 16-byte cp.async; the default or the autotuner's choice.  No counterpart in
 * the reference. */
int fr_tile_staging(const fr_handle *h, int k, int *tma);

/* ---- standalone kernels of the hot path ---- */
/* apply (vector_fields.cu:81-107): out = img o pos (trilinear), out_lab = lab at the floor
 * corner; pos is 3 planes of N positions; d_lab/d_out_lab may be NULL. */
int fr_warp(const float *d_pos, const float *d_img, const int16_t *d_lab, const int dims[3], float *d_out,
            int16_t *d_out_lab, void *stream);

/* The reference's DeformationField::get_inverse / estimate_inverse
 * (src/fastreg/vector_fields.cpp:96-103, src/fastreg/cuda/vector_fields.cu:109-136),
 * which its registration never calls: `sweeps` passes (48 in the reference) of
 *   psi_inv(x) <- -(psi o psi_inv(x))     (unchecked trilinear sample, every voxel)
 * with d_psi_inv (3 planes of N floats, device) updated in place.  Same results as the
 * reference's 48 launches, in one launch. */
int fr_estimate_inverse(const float *d_psi, float *d_psi_inv, const int dims[3], int sweeps, void *stream);

/* The reference's interpolate_gradient (src/fastreg/cuda/vector_fields.cu:194-225): a
 * 3-component field (3 planes of N) sampled at the positions d_pos (3 planes) into d_out. */
int fr_interpolate_field(const float *d_field, const float *d_pos, const int dims[3], float *d_out, void *stream);

/* ---- the differentiated sobolev registration (no counterpart in the reference) ----
 * J(v0, lambda) = 0.5 * sum (S(phi_K) - T)^2 + 0.1 * sum |m_K|^2 after `iters` sobolev
 * iterations (damping, step, smooth_sigma, smooth_width as the SOLVER=sobolev keys) from
 * phi_0 = identity and momentum m_0 = d_v0 (3 planes of N), with the displacement
 * regulariser weighted by lambda (W_REG).  Writes J to *loss and, when d_grad_v0 is not
 * NULL, dJ/dv0 (3 planes, device) and dJ/dlambda to *grad_lambda, by hand-written
 * adjoint kernels with the forward states checkpointed every `checkpoint_every`
 * iterations.  d_T, d_S: target and source (N floats each).  Synchronises `stream`.
 * Its device workspace (checkpoints and adjoint fields, about 3 N floats x (2 (iters /
 * checkpoint_every + 1) + 2 checkpoint_every + 8)) is kept per device after the call and
 * reused by later calls of the same or a smaller size; a call made while another host
 * thread's call holds it allocates a private one. */
int fr_sobolev_loss_grad(const float *d_T, const float *d_S, const int dims[3], const float *d_v0, float lambda,
                         int iters, int checkpoint_every, float damping, float step, float smooth_sigma,
                         int smooth_width, double *loss, float *d_grad_v0, double *grad_lambda, void *stream);

/* adjoint of the warp W = img(pos) (trilinear, floor clamped to dim-2): d_pos_bar = wbar *
 * d img/d pos (3 planes; 0 along an axis where pos was clamped), d_img_bar = scatter-add of
 * the trilinear weights times wbar (N floats, zeroed first).  Either output may be NULL. */
int fr_warp_adjoint(const float *d_pos, const float *d_img, const float *d_wbar, const int dims[3], float *d_pos_bar,
                    float *d_img_bar, void *stream);

/* ---- statistics without device allocation ----
 * No counterpart in the reference.  For callers that cannot call cudaMalloc when they
 * need the statistics of a registration (a process whose device memory belongs to
 * another framework's pool, a real-time pipeline that forbids allocation after
 * start-up): the same e_data / e_reg / energy / folds / Dice that fr_get_stats reports,
 * computed from buffers the caller holds -- the original target d_T and its labels
 * d_labT, the warped source d_warped_S / d_warped_labS (S o psi) and psi (3 planes of
 * N positions) -- and written to the host struct *out (other fields zeroed).
 * Its scratch is one file-scope __device__ array of FR_NOALLOC_SCRATCH_BYTES; the
 * function allocates nothing and calls no allocating routine.  The first call on a
 * device is its set-up: it looks up that array's device address, and under CUDA's lazy
 * module loading (the default) that lookup is what loads the array's module onto the
 * device, which may allocate device memory once.  So make the first call on each device
 * at start-up, while allocation is still allowed; from the second call on nothing is
 * allocated, and the array stays on the device until the process exits.  The address is
 * kept per device for the life of the process: do not use this function on a device
 * after cudaDeviceReset.  Calls share the array: calls that overlap on the GPU race and
 * must be serialised by the caller.  Limits: dims >= 2, N <= FR_NOALLOC_MAX_VOXELS,
 * no_labels <= FR_MAX_LABELS; larger inputs return FR_ERR_INVALID_ARG with a message
 * in fr_last_error(NULL).  The call copies its results to the host and synchronises
 * `stream`, so it cannot be called while `stream` is being captured into a graph. */
#define FR_NOALLOC_SCRATCH_BYTES 28712
#define FR_NOALLOC_MAX_VOXELS 2147483647LL
int fr_stats_noalloc(const float *d_T, const int16_t *d_labT, const float *d_warped_S, const int16_t *d_warped_labS,
                     const float *d_psi, const int dims[3], int no_labels, float w_reg, fr_stats *out, void *stream);

/* Self-test of the TMA-staged kernels' failure path (no counterpart in the reference): one
 * block waits, with the kernels' bounded wait, on an mbarrier armed for bytes that no copy
 * delivers, gives up after the limit (about 2^31 clock cycles, a second), and sets the
 * device error word as a staged kernel would.  Returns FR_OK when the wait gave up as
 * designed (*seconds: the call's wall time), FR_ERR_STATE otherwise; the GPU stays usable
 * either way.  Synchronises `stream`. */
int fr_selftest_wait_limit(double *seconds, void *stream);

const char *fr_last_error(const fr_handle *h);
const char *fr_status_string(int status);
int fr_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FASTREG_GB300_H */
