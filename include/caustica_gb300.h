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

#include <stddef.h>
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
/* Autotuner: on a fresh handle (medium, source and drive set) time each
 * launch configuration the grid admits -- cluster-fused or three-pass
 * transverse chain, persistent or one-tile-per-CTA z-passes, cp.async or
 * tensor-map staging of the persistent z-tiles (CG_ZTMA=0/1 pins it; see
 * cg_solver_set_zstaging), and slab counts (cg_solver_set_slabs) when
 * CG_TUNE_SLABS=1 -- over
 * n_steps steps of the handle itself, keep the fastest and reset the
 * handle's state. The choice is remembered per (grid, batch, physics,
 * medium storage) for the process; a batch of several members reuses the
 * one-member choice of its grid when the process has one. out4 = {fused,
 * persistent z, configurations
 * timed, 1 when taken from the process cache}. No counterpart in the
 * reference (it has one code path). */
int cg_solver_autotune(cg_solver* s, int n_steps, int* out4);

/* Run the plane-local passes slab by slab: 1 <= slabs <= 8; 1 is the plain
 * eight-launch step. With k > 1 slabs a step is x grad, then for each of k
 * runs of x-planes [y inv grad, z u, y fwd div], x div, then for each run
 * [y inv, z p, y fwd]: a run's spectra and fields stay in L2 between its
 * three passes. Results are bit-identical in every mode. Needs the
 * size-specialised passes on all three axes and an even ny. Synchronises.
 * No counterpart in the reference (it has one code path). */
int cg_solver_set_slabs(cg_solver* s, int slabs);
/* How the persistent z-passes stage a tile's half spectra in shared
 * memory: 0 = 16-byte cp.async by every thread into padded rows; 1 = two
 * tensor-map (TMA) box copies per tile, issued by one thread, completed on
 * an mbarrier and read through the 128-byte swizzle (needs nz / 2 + 1 <=
 * 256, an even ny and the plain step; tma = 1 also selects the persistent
 * z-passes). Results are bit-identical either way. A staging wait that gives
 * up (bounded) makes the next finalize, peak read or timed run return
 * CG_ERR_TIMEOUT. No counterpart in the reference. */
int cg_solver_set_zstaging(cg_solver* s, int tma);
int cg_solver_get_zstaging(const cg_solver* s, int* tma);
/* out4 = {cluster-fused transverse chain, persistent z-passes, slabs,
 * kernel launches per step} of the handle's current launch configuration. */
int cg_solver_get_config(const cg_solver* s, int* out4);

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
 * loads the library keeps until the process exits; that array bounds every
 * axis at 2048. The transform's shared-memory tiles bound them further: on a
 * device with 227 KB per block (GB300) ny <= 540, nx <= 576 and nz <= 810.
 * Larger shapes are refused with CG_ERR_INVALID before anything is queued.
 * The first call on a device resolves that array's address there, so make
 * it before any stream capture; the address is kept for the process, so
 * cudaDeviceReset while the library is loaded is not supported. Calls share
 * the array and rewrite it in full: calls whose work overlaps on the GPU
 * (different streams, no ordering) race. No cudaMalloc, cudaFree or
 * allocating library call is made. */
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
/* State from temperatures T [cells] (host or device): theta = T - t_ref and
 * theta_max = theta, formed on the device in float32 with round to nearest
 * (the host's float32 subtraction bit for bit); dose NULL = zero. *finite = 1
 * when every theta is finite (pennes.py:531-536). */
int cg_pennes_set_temperature(cg_pennes* h, const float* T, const float* dose, int* finite);
/* n_sub sub-steps (pennes.py:608-649). Async. */
int cg_pennes_run(cg_pennes* h, int n_sub);
/* Device time [ms] of n_sub sub-steps, CUDA events on the handle's stream.
 * Synchronises. */
int cg_pennes_timed_run(cg_pennes* h, int n_sub, float* ms);
/* Bit 0 set when theta is finite everywhere, bit 1 when the dose is
 * (pennes.py:756-781). */
int cg_pennes_check_finite(cg_pennes* h, int* finite);
int cg_pennes_get_state(cg_pennes* h, float* theta, float* theta_max, float* dose);
/* T = theta + t_ref, T_max = theta_max + t_ref (float32 on the device) and the
 * dose; any output may be NULL. */
int cg_pennes_get_temperature(cg_pennes* h, float* T, float* T_max, float* dose);

/* ------------------------------------------ post-processing on the device */

/* Focal metrics of one record region (report/metrics.py:192-313): the
 * fundamental's amplitude maximum over an interior box (first in C order,
 * as argmax_interior, metrics.py:123-127), the -6 dB crossings of the
 * profiles through it (extent_6db, metrics.py:140-152), the interior voxel
 * count at or above half the peak (the -6 dB volume, metrics.py:228), and
 * the values the reference reads at the peak. Amplitudes are the correctly
 * rounded float32 |P|. */
typedef struct cg_focus_input {
  const float* p1;    /* device complex64 [nx][ny][nz]: harmonic 1 over the record region */
  const float* p2;    /* device complex64 harmonic 2, or NULL */
  const float* pmax;  /* device float32 time-domain max |p|, or NULL */
  int shape[3];       /* record region extents */
  int lo[3], hi[3];   /* interior box, record frame, half-open (interior_slices, metrics.py:96-120) */
  int probe[3];       /* record-frame voxel whose |P1| is returned (the requested focus); any < 0: none */
  int offset[3];      /* record origin minus the apex voxel: coordinate of index i is (i + offset) dx */
  double dx;          /* voxel size [m] */
} cg_focus_input;

typedef struct cg_focus_report {
  long long peak;          /* record-frame linear index of the interior |P1| maximum */
  float p_peak;            /* |P1| there */
  float p_max_at_peak;     /* p_max there (NaN without p_max) */
  long long n_above_half;  /* interior voxels with |P1| >= 0.5 p_peak */
  float p_probe;           /* |P1| at the probe voxel (NaN without one) */
  int has_a2;              /* 1 when harmonic 2 was given */
  float a2_at_peak;        /* |P2| at the |P1| peak */
  float a2_peak;           /* interior |P2| maximum */
  long long a2_peak_index; /* its record-frame linear index (-1 without P2) */
  int truncated[3];        /* x, y, z: the profile never falls below half the peak on one side */
  double left[3], right[3];/* x, y, z -6 dB crossings [m] from the apex (NaN when truncated) */
} cg_focus_report;

/* On caller device buffers; queued on `stream` (a cudaStream_t) and
 * synchronised before return. Allocates its few-KB scratch stream-ordered. */
int cg_focus_metrics(const cg_focus_input* in, cg_focus_report* out, void* stream);
/* On member `member`'s phasors of the last cg_solver_finalize (the solver
 * fills p1, p2, pmax and shape itself; no host copy of the field). */
int cg_solver_focus_metrics(cg_solver* s, int member, const cg_focus_input* in, cg_focus_report* out);

/* Volumetric heating Q [W/m^3] from recorded phasors
 * (HeatingSource.from_phasors, sensors.py:193-295):
 *   Q = sum over terms t of (alpha_t |P_t|^2) / (rho c)
 * in float64 in the given term order, rounded to float32, times `scale`
 * in float32. The heating grid gets Q over the record region and 0 elsewhere.
 * Label mode (n_labels > 0): coef[l][t] = alpha_t of material l and
 * coef[l][n_terms] = 1 / (rho c) of l, float64, host memory; dense mode:
 * float32 device maps with alpha_t = alpha * alpha_factor[t]. */
typedef struct cg_heating_spec {
  int n_terms;
  int harmonics[8];          /* harmonic of each term (cg_solver_heating_q) */
  const float* phasor[8];    /* device complex64 phasor of each term over the record region */
  int shape[3];              /* record region extents */
  int n_labels;              /* 0: dense mode */
  const double* coef;        /* label mode: [n_labels][n_terms + 1], host */
  const uint8_t* labels;     /* label mode: device label map */
  const float* alpha;        /* dense mode: device maps */
  const float* rho;
  const float* c;
  double alpha_factor[8];    /* dense mode: per-term multiplier of alpha (n^y) */
  int map_shape[3];          /* extents of the label / dense maps */
  int map_origin[3];         /* map voxel of record voxel (0, 0, 0) */
  int q_shape[3];            /* heating grid */
  int q_origin[3];           /* heating-grid voxel of record voxel (0, 0, 0) */
  float scale;
} cg_heating_spec;

/* Q into the caller's device buffer q_dev [q_shape]; queued on `stream`,
 * synchronised before return. term_sums (host, n_terms, or NULL) receives
 * each term's float64 sum over the record region (its mean times the voxel
 * count: the reference's mean_q_by_harmonic_w_m3, sensors.py:272). */
int cg_heating_q(const cg_heating_spec* spec, float* q_dev, double* term_sums, void* stream);
/* The same from member `member`'s phasors of the last cg_solver_finalize:
 * the solver fills phasor[] from harmonics[] and shape; in label mode with
 * labels == NULL it uses its own label map (padded frame, map_origin = the
 * record box start). The field stays on the device: q_dev can go straight
 * to cg_pennes_set_coefficients / cg_pennes_set_labels as their q. */
int cg_solver_heating_q(cg_solver* s, int member, const cg_heating_spec* spec, float* q_dev,
                        double* term_sums);

/* Dynamic float16 quantisation of stored result fields: the output
 * contract of the caustica-result/1 store (try_float16, io/quantize.py:45-67,
 * called per field by _quantized_dataset, io/store.py:69-89). Per field
 * (n float32 values, `stride` floats apart: 1 for p_max, 2 for the real or
 * imaginary part of a complex64 phasor): peak = max |x|; a zero peak stores
 * the plain float16 cast with scale 1; otherwise q = half_rn(x / peak) and
 * err = max |float(q) * peak - x| / peak, all float32 operations as NumPy
 * performs them, and the field keeps float16 with scale = peak when
 * err <= max_norm_err, else its float32 values with scale 1 (a NaN peak
 * always falls back, like the reference's NaN error). Outputs, per field f
 * at the offset of its first value in the concatenation of all fields:
 * f16_out gets the float16 bits of float16 fields, f32_out the values of
 * float32 fields (may be NULL when none falls back; the call then fails if
 * one does); info[4 f + 0..3] = scale, norm_err, 1 for float16 / 0 for
 * float32, and the peak. Outputs may be host or device memory; the fields
 * must be device memory. Synchronises before return. */
#define CG_QUANT_MAX_FIELDS 32
typedef struct cg_qfield {
  const float* data;
  long long n;
  long long stride;
} cg_qfield;

int cg_quantize_f16(const cg_qfield* fields, int n_fields, double max_norm_err, uint16_t* f16_out,
                    float* f32_out, float* info, void* stream);
/* The same on member `member`'s result of the last cg_solver_finalize, in
 * the order the store writes its datasets: for each recorded harmonic in
 * ascending order p_real_h{n} then p_imag_h{n}, then p_max; each field has
 * the record region's voxel count (io/store.py:146-151). Finalize may be
 * called with NULL outputs first, so the float32 result never crosses to
 * the host. */
int cg_solver_quantize(cg_solver* s, int member, double max_norm_err, uint16_t* f16_out, float* f32_out,
                       float* info);

/* Device-resident label volumes (a medium whose uint8 label map a caller
 * keeps on the device and passes by pointer, as the Python fronts do for
 * DLPack / __cuda_array_interface__ tensors): counts256[l] = voxels holding
 * label l (the host picks the time step from the materials present,
 * solvers/kspace/engine.py:86-113), and the labels at n flat voxel indices
 * (the source scale 2 c dt / dx uses the local sound speed,
 * engine.py:268-278). Both synchronise. */
int cg_label_counts(const uint8_t* labels_dev, long long n, unsigned long long* counts256);
int cg_gather_u8(const uint8_t* src_dev, const long long* idx, int n, uint8_t* out_host);
/* cudaStreamSynchronize on a caller's stream (a producer stream named by
 * __cuda_array_interface__ before its data is read on the library's own
 * streams); NULL is the legacy default stream. */
int cg_stream_synchronize(void* stream);

/* Plain device buffers for callers without a CUDA runtime of their own. */
int cg_buffer_alloc(size_t bytes, void** out);
int cg_buffer_free(void* p);
/* cudaMemcpy with the kind inferred from the pointers (host or device). */
int cg_buffer_copy(void* dst, const void* src, size_t bytes);

#ifdef __cplusplus
}
#endif

#endif /* CAUSTICA_GB300_H */
