/* caustica_gb300 -- C ABI of the GB300 (sm_103a) k-space CW solver and the
 * Pennes / CEM43 thermal step.
 *
 * Every entry point returns 0 on success or a CG_ERR_* code; the message of
 * the last failure on the calling thread is cg_last_error(). No C++
 * exception crosses this boundary. Pointers named "host or device" may be
 * either (the library copies with unified addressing); all others are
 * host. One CUDA stream per handle; a handle is not thread-safe.
 *
 * Reference interfaces named below are files of ebx0/caustica
 * (paths relative to src/caustica/).
 */
#ifndef CAUSTICA_GB300_H
#define CAUSTICA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CG_ABI_VERSION 10000

/* ------------------------------------------------------------------ misc */

/* Message of the last failed call on this thread ("" if none). */
const char* cg_last_error(void);
/* CG_ABI_VERSION of the loaded library. */
int cg_version(void);
/* Make `device` current for this host thread; handles created afterwards
 * live on it (one process per GPU). */
int cg_set_device(int device);

/* ---------------------------------------------------- k-space CW solver */

typedef struct cg_solver cg_solver;

/* Geometry and run policy of one solve (or of B solves over one medium).
 * The padded grid is nx x ny x nz (z fastest); a 1-D grid of n cells is
 * 1 x 1 x n and a 2-D grid a x b is 1 x a x b. The fields mirror what
 * run_cw_kspace_pstd derives before its time loop (solvers/kspace/engine.py:
 * 234 spp/dt, 251-254 k-space tables with c_ref = c_max, 256-263 sponge,
 * 293-296 convergence region, 299-301 record region). */
typedef struct cg_solver_config {
  int nx, ny, nz;     /* padded grid (2/3/5-smooth, each <= 2048)           */
  int batch;          /* right-hand sides sharing the medium (>= 1)         */
  int nonlinear;      /* 1: Westervelt term (engine.py:473-475)              */
  int spp;            /* steps per period (engine.py:86-113)                 */
  int max_periods;    /* capacity of the per-period peak log                 */
  int n_harmonics;    /* 1..8                                                */
  int harmonics[8];   /* harmonic numbers, first is 1                        */
  int pml[3];         /* sponge width per axis, cells (core/pml.py:203-207)  */
  double pml_edge;    /* sponge edge factor (core/pml.py:25-50)              */
  double dx, dt;      /* spacing [m], time step [s]                          */
  double c_ref;       /* kappa reference speed = c_max (engine.py:252)       */
  int rec_lo[3], rec_hi[3];   /* record box, half-open                       */
  int conv_lo[3], conv_hi[3]; /* convergence box, half-open                  */
} cg_solver_config;

/* Allocate a solver and build its k-space, twiddle and sponge tables in FP64
 * on the device. Replaces the set-up of run_cw_kspace_pstd
 * (solvers/kspace/engine.py:225-266, operators.py:60-157). */
int cg_solver_create(const cg_solver_config* cfg, cg_solver** out);
int cg_solver_destroy(cg_solver* s);

/* Medium as a uint8 label volume (nx*ny*nz, host or device) plus a table of
 * n_labels rows (dt/rho, rho c^2 dt, exp(-alpha c dt), 2 beta dt) -- the
 * per-voxel maps of engine.py:239-249, stored once per distinct material. */
int cg_solver_set_medium_labels(cg_solver* s, const uint8_t* labels, int n_labels, const float* table);
/* Medium as four dense float32 maps (host or device), engine.py:239-249.
 * beta2_dt may be NULL for a linear solve. */
int cg_solver_set_medium_dense(cg_solver* s, const float* dt_over_rho, const float* rhoc2_dt,
                               const float* absorb, const float* beta2_dt);

/* Source voxels (n_src x 3 int32 x,y,z, unique) and per-member amplitudes
 * amp_cos/amp_sin [batch][n_src] = (2 c dt/dx) cos/sin(phase)
 * (engine.py:268-278, sources.py:26-96). */
int cg_solver_set_source(cg_solver* s, int n_src, const int32_t* xyz, const float* amp_cos,
                         const float* amp_sin);
/* Per-step drive (n_steps x 4 float: amp*ramp(n dt), sin(w n dt),
 * cos(w n dt), 0), host or device (engine.py:478-482, sources.py:98-102). */
int cg_solver_set_drive(cg_solver* s, int n_steps, const float* drive);

/* Zero p, u, the spectra, the period-peak log and the step counter. */
int cg_solver_reset(cg_solver* s);
/* Advance n_steps steps (the step of engine.py:458-482), recording the
 * harmonic bins and p_max when record != 0 (engine.py:538-549). Async. */
int cg_solver_run(cg_solver* s, int n_steps, int record);
/* Advance n_periods whole periods through a captured CUDA graph. Async. */
int cg_solver_run_periods(cg_solver* s, int n_periods, int record);
/* Zero the record accumulators (engine.py:536-537). */
int cg_solver_begin_record(cg_solver* s);
/* Per-period max |p| over the convergence box (engine.py:490-495) for
 * periods [first, first+count), as float [batch][count]. Synchronises. */
int cg_solver_read_peaks(cg_solver* s, int first, int count, float* out);
/* Phasors of every harmonic, FP64-normalised by 2/n_record_steps
 * (engine.py:551-552), as complex64 [batch][n_harmonics][record box], and
 * p_max [batch][record box]; either may be NULL. Host or device. */
int cg_solver_finalize(cg_solver* s, int n_record_steps, float* phasors, float* pmax);
/* Checkpoint state (engine.py:359-371): p [batch][cells], u [3][batch][cells]. */
int cg_solver_get_state(cg_solver* s, float* p, float* u);
int cg_solver_set_state(cg_solver* s, const float* p, const float* u, long long step);
int cg_solver_synchronize(cg_solver* s);
/* *idle = 1 when every call queued on the solver's stream has finished;
 * never blocks (lets one host thread drive many solvers). */
int cg_solver_query(cg_solver* s, int* idle);
/* Device time [ms] of n_steps steps, CUDA events on the solver's stream;
 * graph != 0 runs whole periods through the captured graph. Synchronises. */
int cg_solver_timed_run(cg_solver* s, int n_steps, int record, int graph, float* ms);
/* Per-launch device time [ms] summed over n_steps steps, 8 entries in step
 * order (y fwd, x grad, y inv grad, z u, y fwd div, x div, y inv, z p). */
int cg_solver_profile(cg_solver* s, int n_steps, int record, float* ms8);
/* ncell, nspec, nrec, smem y/x/z, batch, launches per step. */
int cg_solver_info(const cg_solver* s, long long* out8);

/* ------------------------------------------------- batched 3-D R2C/C2R */

typedef struct cg_fft3d cg_fft3d;

/* Batched 3-D real FFT with the solver's own passes; replaces
 * backend.fft.rfftn / irfftn (engine.py:459-469, core/backend.py:153-172).
 * Spectrum layout is [batch][x][kz][y] (kz < nz/2+1), complex64;
 * inverse is unnormalised. Inputs/outputs host or device. */
int cg_fft3d_create(int nx, int ny, int nz, int batch, cg_fft3d** out);
int cg_fft3d_destroy(cg_fft3d* f);
int cg_fft3d_forward(cg_fft3d* f, const float* in, float* out_spec);
int cg_fft3d_inverse(cg_fft3d* f, const float* in_spec, float* out);

/* The forward transform above for callers that may not allocate device
 * memory: code running inside another framework's memory pool, serving
 * loops that must avoid cudaMalloc's implicit synchronisation, plug-ins
 * whose host application owns the CUDA heap. No counterpart in the
 * reference (it has no device code). in_dev [batch][x][y][z] float32 and
 * out_dev [batch][x][kz][y] complex64 are the caller's device buffers;
 * work is queued on `stream` (a cudaStream_t, NULL = legacy default) and
 * the call returns without synchronising. The only scratch, three per-axis
 * twiddle tables, lives in a fixed 48 KB device array that every GPU which
 * loads the library keeps until the process exits; every axis must be
 * <= 2048 (larger shapes are refused with CG_ERR_INVALID). The first call on
 * a device resolves that array's address there, so make it before any
 * stream capture. Calls share the array and rewrite it in full: calls whose
 * work overlaps on the GPU (different streams, no ordering) race. No
 * cudaMalloc, cudaFree or allocating library call is made. */
int cg_fft3d_forward_noalloc(int nx, int ny, int nz, int batch, const float* in_dev, float* out_dev,
                             void* stream);

/* -------------------------------------------------------- Pennes / CEM43 */

typedef struct cg_pennes cg_pennes;

/* Explicit conservative 7-point Pennes step with in-loop trapezoidal CEM43
 * dose (thermal/pennes.py:451-689, thermal/dose.py:74-89). The grid is
 * nx x ny x nz (a 2-D grid is 1 x a x b). */
typedef struct cg_pennes_config {
  int nx, ny, nz;
  int dirichlet;            /* 0 insulated, 1 walls held at theta_wall      */
  int dose;                 /* accumulate CEM43                              */
  float theta_wall;         /* boundary temperature minus t_ref              */
  float t_ref;              /* state offset (pennes.py:524-531)              */
  float half_dt_min;        /* float32(0.5 dt_sub / 60) (pennes.py:596)      */
  int n_labels;             /* 0: dense coefficient maps                     */
} cg_pennes_config;

int cg_pennes_create(const cg_pennes_config* cfg, cg_pennes** out);
int cg_pennes_destroy(cg_pennes* h);
/* Coefficients (host or device): faces kf_x [(nx-1)*ny*nz], kf_y
 * [nx*(ny-1)*nz], kf_z [nx*ny*(nz-1)] (pennes.py:404-412), walls lo/hi per
 * axis packed as 6 planes (pennes.py:414-426, may be NULL when insulated),
 * perf = w_b rho_b C_b [cells], coeff = dt_sub/(rho C) [cells], q [cells]
 * (may be NULL), perf_offset [cells] (may be NULL). */
int cg_pennes_set_coefficients(cg_pennes* h, const float* kf_x, const float* kf_y, const float* kf_z,
                               const float* walls, const float* perf, const float* coeff, const float* q,
                               const float* perf_offset);
/* Coefficients as a uint8 material label volume [cells] plus n_labels rows
 * (k, dt_sub/(rho C), w_b rho_b C_b, perfusion offset); the kernel forms the
 * harmonic-mean faces ((2 k_i) k_j / (k_i + k_j)) inv_dx2 and the Dirichlet
 * walls (2 k) inv_dx2 in float32 in the reference's order (pennes.py:404-447).
 * wall_axes: bit a set when axis a carries walls. q [cells] may be NULL.
 * Replaces cg_pennes_set_coefficients. */
int cg_pennes_set_labels(cg_pennes* h, const uint8_t* labels, int n_labels, const float* table, float inv_dx2,
                         int has_perf_offset, int wall_axes, const float* q);
/* State (host or device): theta = T - t_ref, theta_max, dose, and the
 * dose-rate carry; dose/dose_comp may be NULL when dose is off. */
int cg_pennes_set_state(cg_pennes* h, const float* theta, const float* theta_max, const float* dose);
/* n_sub sub-steps (pennes.py:608-649). Async. */
int cg_pennes_run(cg_pennes* h, int n_sub);
/* Bit 0 set when theta is finite everywhere, bit 1 when the dose is
 * (pennes.py:756-781). */
int cg_pennes_check_finite(cg_pennes* h, int* finite);
int cg_pennes_get_state(cg_pennes* h, float* theta, float* theta_max, float* dose);

#ifdef __cplusplus
}
#endif

#endif /* CAUSTICA_GB300_H */
