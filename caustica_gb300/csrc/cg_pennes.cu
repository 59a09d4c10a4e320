// Pennes bioheat sub-step with CEM43 dose for GB300 (sm_103a).
//
// Reference: thermal/pennes.py:608-649 (loop body), :404-426 (faces and
// walls), thermal/dose.py:74-89 (rate). Per sub-step, for every cell:
//   work  = sum_axes [ kf_hi (th_up - th) - kf_lo (th - th_dn) ]   (faces that exist)
//         + walls (Dirichlet) + q - perf th - perf_offset
//   th'   = th + work * coeff            coeff = dt_sub / (rho C)
//   thmax = max(thmax, th')
//   dose += (R^(43 - T') + R^(43 - T)) * half_dt_min       (Kahan-compensated)
// The accumulation follows the reference's order (axis by axis: the face
// above, then the face below; walls; q; perfusion) with explicit
// round-to-nearest operations, so the temperature equals the reference's
// float32 NumPy result.
#include <stdlib.h>
#include <string.h>

#include "cg_common.cuh"
#include "caustica_gb300.h"

struct PennesDev {
  int nx, ny, nz;
  const float* kfx;  // [(nx-1)][ny][nz]
  const float* kfy;  // [nx][(ny-1)][nz]
  const float* kfz;  // [nx][ny][(nz-1)]
  const float* walls;  // 6 planes: x lo, x hi [ny*nz], y lo, y hi [nx*nz], z lo, z hi [nx*ny]
  const float* perf;
  const float* coeff;
  const float* q;
  const float* poff;
  int dirichlet, dose;
  float theta_wall, t_ref, half_dt_min;
  // label mode: per-material (k, dt_sub/(rho C), w_b rho_b C_b, perfusion offset)
  const uint8_t* labels;
  const float4* ltab;
  float inv_dx2;
  int has_poff;
  int wall_axes;  // label mode: bit a set when axis a has Dirichlet walls
};

// Harmonic-mean face conductance over dx^2 with the reference's float32
// operation order: ((2 lo) hi / (lo + hi)) inv_dx2 (pennes.py:404-412).
__device__ __forceinline__ float face_k(float lo, float hi, float inv_dx2) {
  return __fmul_rn(__fdiv_rn(__fmul_rn(__fmul_rn(2.0f, lo), hi), __fadd_rn(lo, hi)), inv_dx2);
}

__device__ __forceinline__ float cem43_rate_dev(float T) {
  // R^(43 - T) with R = 0.5 above 43 C, 0.25 at or below (dose.py:74-89):
  // 0.5^e = 2^-e, 0.25^e = 2^-2e.
  float e = __fsub_rn(43.0f, T);
  return (T > 43.0f) ? exp2f(-e) : exp2f(-2.0f * e);
}

__global__ void k_pennes_step(PennesDev P, const float* __restrict__ th, float* __restrict__ thn, float* thmax,
                              float* dose, float* dcomp) {
  __shared__ float4 tab[256];
  if (P.labels)
    for (int i = threadIdx.x; i < 256; i += blockDim.x) tab[i] = P.ltab[i];
  __syncthreads();
  const long long ncell = (long long)P.nx * P.ny * P.nz;
  const long long sx = (long long)P.ny * P.nz, sy = P.nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ncell;
       i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i % P.nz);
    const long long r = i / P.nz;
    const int y = (int)(r % P.ny);
    const int x = (int)(r / P.ny);
    const float t0 = th[i];
    const bool lab = P.labels != nullptr;
    const float4 me = lab ? tab[P.labels[i]] : make_float4(0.f, 0.f, 0.f, 0.f);
    float w = 0.0f;
    // axis x: face above (x, x+1) then face below (x-1, x)
    if (x + 1 < P.nx) {
      const float kf = lab ? face_k(me.x, tab[P.labels[i + sx]].x, P.inv_dx2)
                           : P.kfx[((long long)x * P.ny + y) * P.nz + z];
      w = __fadd_rn(w, __fmul_rn(__fsub_rn(th[i + sx], t0), kf));
    }
    if (x > 0) {
      const float kf = lab ? face_k(tab[P.labels[i - sx]].x, me.x, P.inv_dx2)
                           : P.kfx[((long long)(x - 1) * P.ny + y) * P.nz + z];
      w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, th[i - sx]), kf));
    }
    if (y + 1 < P.ny) {
      const float kf = lab ? face_k(me.x, tab[P.labels[i + sy]].x, P.inv_dx2)
                           : P.kfy[((long long)x * (P.ny - 1) + y) * P.nz + z];
      w = __fadd_rn(w, __fmul_rn(__fsub_rn(th[i + sy], t0), kf));
    }
    if (y > 0) {
      const float kf = lab ? face_k(tab[P.labels[i - sy]].x, me.x, P.inv_dx2)
                           : P.kfy[((long long)x * (P.ny - 1) + (y - 1)) * P.nz + z];
      w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, th[i - sy]), kf));
    }
    if (z + 1 < P.nz) {
      const float kf = lab ? face_k(me.x, tab[P.labels[i + 1]].x, P.inv_dx2)
                           : P.kfz[((long long)x * P.ny + y) * (P.nz - 1) + z];
      w = __fadd_rn(w, __fmul_rn(__fsub_rn(th[i + 1], t0), kf));
    }
    if (z > 0) {
      const float kf = lab ? face_k(tab[P.labels[i - 1]].x, me.x, P.inv_dx2)
                           : P.kfz[((long long)x * P.ny + y) * (P.nz - 1) + (z - 1)];
      w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, th[i - 1]), kf));
    }
    if (P.dirichlet) {
      const long long pyz = (long long)P.ny * P.nz, pxz = (long long)P.nx * P.nz, pxy = (long long)P.nx * P.ny;
      const float* W = P.walls;
      const float dwall = __fsub_rn(P.theta_wall, t0);
      // 2 k_edge / dx^2 (pennes.py:414-426); label mode: walls only on the grid's own axes
      const float wk = lab ? __fmul_rn(__fmul_rn(2.0f, me.x), P.inv_dx2) : 0.f;
      const bool wx = !lab || (P.wall_axes & 1), wy = !lab || (P.wall_axes & 2), wz = !lab || (P.wall_axes & 4);
      if (wx && x == 0) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[(long long)y * P.nz + z], dwall));
      if (wx && x == P.nx - 1) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[pyz + (long long)y * P.nz + z], dwall));
      if (!lab) W += 2 * pyz;
      if (wy && y == 0) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[(long long)x * P.nz + z], dwall));
      if (wy && y == P.ny - 1) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[pxz + (long long)x * P.nz + z], dwall));
      if (!lab) W += 2 * pxz;
      if (wz && z == 0) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[(long long)x * P.ny + y], dwall));
      if (wz && z == P.nz - 1) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[pxy + (long long)x * P.ny + y], dwall));
    }
    if (P.q) w = __fadd_rn(w, P.q[i]);
    if (lab) {
      if (me.z != 0.0f || P.has_poff) {
        w = __fsub_rn(w, __fmul_rn(me.z, t0));
        if (P.has_poff) w = __fsub_rn(w, me.w);
      }
      w = __fmul_rn(w, me.y);
    } else {
      if (P.perf) {
        w = __fsub_rn(w, __fmul_rn(P.perf[i], t0));
        if (P.poff) w = __fsub_rn(w, P.poff[i]);
      }
      w = __fmul_rn(w, P.coeff[i]);
    }
    const float t1 = __fadd_rn(t0, w);
    thn[i] = t1;
    const float tm = thmax[i];
    thmax[i] = (t1 > tm || t1 != t1) ? t1 : tm;
    if (P.dose) {
      const float r_new = cem43_rate_dev(__fadd_rn(t1, P.t_ref));
      const float r_old = cem43_rate_dev(__fadd_rn(t0, P.t_ref));
      const float inc = __fmul_rn(__fadd_rn(r_new, r_old), P.half_dt_min);
      // Kahan: true dose = s - c
      const float s = dose[i], c = dcomp[i];
      const float yk = __fsub_rn(inc, c);
      const float tk = __fadd_rn(s, yk);
      dcomp[i] = __fsub_rn(__fsub_rn(tk, s), yk);
      dose[i] = tk;
    }
  }
}

// flag bit 0 cleared: a non-finite temperature; bit 1 cleared: a non-finite dose
__global__ void k_pennes_finite(const float* th, const float* dose, long long n, int* flag) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (!isfinite(th[i])) atomicAnd(flag, ~1);
    if (dose && !isfinite(dose[i])) atomicAnd(flag, ~2);
  }
}

struct cg_pennes {
  cg_pennes_config cfg;
  long long ncell;
  float* th[2] = {nullptr, nullptr};
  int cur = 0;
  float* thmax = nullptr;
  float* dose = nullptr;
  float* dcomp = nullptr;
  float *kfx = nullptr, *kfy = nullptr, *kfz = nullptr, *walls = nullptr;
  float *perf = nullptr, *coeff = nullptr, *q = nullptr, *poff = nullptr;
  int* flag = nullptr;
  uint8_t* labels = nullptr;
  float4* ltab = nullptr;
  float inv_dx2 = 0.f;
  int lab_poff = 0, wall_axes = 7;
  int has_coef = 0, has_state = 0;
  cudaStream_t stream = nullptr;
};

static void pennes_free(cg_pennes* h) {
  if (!h) return;
  void* ptrs[] = {h->th[0], h->th[1], h->thmax, h->dose, h->dcomp, h->kfx, h->kfy, h->kfz,
                  h->walls, h->perf, h->coeff, h->q, h->poff, h->flag, h->labels, h->ltab};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

static int palloc(float** p, long long n) {
  if (n < 1) n = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(float) * (size_t)n);
  if (e != cudaSuccess) {
    cg_set_error("cudaMalloc of %lld floats failed: %s", n, cudaGetErrorString(e));
    *p = nullptr;
    return CG_ERR_OOM;
  }
  return CG_OK;
}

extern "C" int cg_pennes_create(const cg_pennes_config* cfg, cg_pennes** out) {
  CG_REQUIRE(cfg && out, "null argument");
  *out = nullptr;
  CG_REQUIRE(cfg->nx >= 1 && cfg->ny >= 1 && cfg->nz >= 1, "invalid thermal grid %dx%dx%d", cfg->nx, cfg->ny, cfg->nz);
  cg_pennes* h = new cg_pennes();
  h->cfg = *cfg;
  const long long nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
  h->ncell = nx * ny * nz;
  int rc = CG_OK;
  if ((rc = palloc(&h->th[0], h->ncell)) || (rc = palloc(&h->th[1], h->ncell)) || (rc = palloc(&h->thmax, h->ncell)) ||
      (rc = palloc(&h->dose, h->ncell)) || (rc = palloc(&h->dcomp, h->ncell)) ||
      (rc = palloc(&h->kfx, (nx - 1) * ny * nz)) || (rc = palloc(&h->kfy, nx * (ny - 1) * nz)) ||
      (rc = palloc(&h->kfz, nx * ny * (nz - 1))) || (rc = palloc(&h->walls, 2 * (ny * nz + nx * nz + nx * ny))) ||
      (rc = palloc(&h->perf, h->ncell)) || (rc = palloc(&h->coeff, h->ncell)) || (rc = palloc(&h->q, h->ncell)) ||
      (rc = palloc(&h->poff, h->ncell))) {
    pennes_free(h);
    return rc;
  }
  cudaError_t e = cudaMalloc((void**)&h->flag, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cg_set_error("pennes set-up: %s", cudaGetErrorString(e));
    pennes_free(h);
    return CG_ERR_CUDA;
  }
  *out = h;
  return CG_OK;
}

extern "C" int cg_pennes_destroy(cg_pennes* h) {
  if (h) {
    cudaStreamSynchronize(h->stream);
    pennes_free(h);
  }
  return CG_OK;
}

static int copy_opt(float* dst, const float* src, long long n, int* present, cudaStream_t st) {
  *present = src != nullptr;
  if (!src || n <= 0) return CG_OK;
  CG_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(float) * (size_t)n, cudaMemcpyDefault, st));
  return CG_OK;
}

extern "C" int cg_pennes_set_coefficients(cg_pennes* h, const float* kf_x, const float* kf_y, const float* kf_z,
                                          const float* walls, const float* perf, const float* coeff,
                                          const float* q, const float* perf_offset) {
  CG_REQUIRE(h && coeff, "null argument");
  const long long nx = h->cfg.nx, ny = h->cfg.ny, nz = h->cfg.nz;
  CG_REQUIRE(nx == 1 || kf_x, "kf_x is required when nx > 1");
  CG_REQUIRE(ny == 1 || kf_y, "kf_y is required when ny > 1");
  CG_REQUIRE(nz == 1 || kf_z, "kf_z is required when nz > 1");
  CG_REQUIRE(!h->cfg.dirichlet || walls, "a Dirichlet solve needs the wall planes");
  int pr = 0, has_walls = 0, has_perf = 0, has_q = 0, has_poff = 0;
  int rc;
  if ((rc = copy_opt(h->kfx, kf_x, (nx - 1) * ny * nz, &pr, h->stream)) ||
      (rc = copy_opt(h->kfy, kf_y, nx * (ny - 1) * nz, &pr, h->stream)) ||
      (rc = copy_opt(h->kfz, kf_z, nx * ny * (nz - 1), &pr, h->stream)) ||
      (rc = copy_opt(h->walls, walls, 2 * (ny * nz + nx * nz + nx * ny), &has_walls, h->stream)) ||
      (rc = copy_opt(h->perf, perf, h->ncell, &has_perf, h->stream)) ||
      (rc = copy_opt(h->coeff, coeff, h->ncell, &pr, h->stream)) ||
      (rc = copy_opt(h->q, q, h->ncell, &has_q, h->stream)) ||
      (rc = copy_opt(h->poff, perf_offset, h->ncell, &has_poff, h->stream)))
    return rc;
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->has_coef = 1 | (has_perf << 1) | (has_q << 2) | (has_poff << 3);
  return CG_OK;
}

extern "C" int cg_pennes_set_labels(cg_pennes* h, const uint8_t* labels, int n_labels, const float* table,
                                     float inv_dx2, int has_perf_offset, int wall_axes, const float* q) {
  CG_REQUIRE(h && labels && table, "null argument");
  CG_REQUIRE(n_labels >= 1 && n_labels <= 256, "n_labels must be 1..256, got %d", n_labels);
  if (!h->labels) {
    CG_CUDA_TRY(cudaMalloc((void**)&h->labels, (size_t)h->ncell));
    CG_CUDA_TRY(cudaMalloc((void**)&h->ltab, 256 * sizeof(float4)));
  }
  float4 tab[256];
  memset(tab, 0, sizeof(tab));
  for (int i = 0; i < n_labels; ++i) tab[i] = make_float4(table[4 * i], table[4 * i + 1], table[4 * i + 2], table[4 * i + 3]);
  CG_CUDA_TRY(cudaMemcpyAsync(h->labels, labels, (size_t)h->ncell, cudaMemcpyDefault, h->stream));
  CG_CUDA_TRY(cudaMemcpyAsync(h->ltab, tab, sizeof(tab), cudaMemcpyHostToDevice, h->stream));
  if (q) CG_CUDA_TRY(cudaMemcpyAsync(h->q, q, sizeof(float) * (size_t)h->ncell, cudaMemcpyDefault, h->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->inv_dx2 = inv_dx2;
  h->lab_poff = has_perf_offset;
  h->wall_axes = wall_axes;
  h->has_coef = 1 | (q ? 4 : 0);
  return CG_OK;
}

extern "C" int cg_pennes_set_state(cg_pennes* h, const float* theta, const float* theta_max, const float* dose) {
  CG_REQUIRE(h && theta && theta_max, "null argument");
  const size_t n = (size_t)h->ncell;
  h->cur = 0;
  CG_CUDA_TRY(cudaMemcpyAsync(h->th[0], theta, 4 * n, cudaMemcpyDefault, h->stream));
  CG_CUDA_TRY(cudaMemcpyAsync(h->thmax, theta_max, 4 * n, cudaMemcpyDefault, h->stream));
  if (dose) CG_CUDA_TRY(cudaMemcpyAsync(h->dose, dose, 4 * n, cudaMemcpyDefault, h->stream));
  else CG_CUDA_TRY(cudaMemsetAsync(h->dose, 0, 4 * n, h->stream));
  CG_CUDA_TRY(cudaMemsetAsync(h->dcomp, 0, 4 * n, h->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->has_state = 1;
  return CG_OK;
}

static PennesDev make_dev(const cg_pennes* h) {
  PennesDev P;
  P.nx = h->cfg.nx; P.ny = h->cfg.ny; P.nz = h->cfg.nz;
  P.kfx = h->kfx; P.kfy = h->kfy; P.kfz = h->kfz; P.walls = h->walls;
  P.perf = (h->has_coef & 2) ? h->perf : nullptr;
  P.coeff = h->coeff;
  P.q = (h->has_coef & 4) ? h->q : nullptr;
  P.poff = (h->has_coef & 8) ? h->poff : nullptr;
  P.dirichlet = h->cfg.dirichlet;
  P.dose = h->cfg.dose;
  P.theta_wall = h->cfg.theta_wall;
  P.t_ref = h->cfg.t_ref;
  P.half_dt_min = h->cfg.half_dt_min;
  P.labels = h->labels;
  P.ltab = h->ltab;
  P.inv_dx2 = h->inv_dx2;
  P.has_poff = h->lab_poff;
  P.wall_axes = h->wall_axes;
  return P;
}

extern "C" int cg_pennes_run(cg_pennes* h, int n_sub) {
  CG_REQUIRE(h, "null handle");
  CG_REQUIRE(h->has_coef && h->has_state, "set coefficients and state before running");
  CG_REQUIRE(n_sub >= 0, "n_sub must be >= 0");
  const PennesDev P = make_dev(h);
  const int threads = 256;
  long long blocks = (h->ncell + threads - 1) / threads;
  if (blocks > 152 * 64) blocks = 152 * 64;
  for (int i = 0; i < n_sub; ++i) {
    k_pennes_step<<<(unsigned)blocks, threads, 0, h->stream>>>(P, h->th[h->cur], h->th[1 - h->cur], h->thmax, h->dose,
                                                               h->dcomp);
    h->cur = 1 - h->cur;
  }
  CG_CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

extern "C" int cg_pennes_check_finite(cg_pennes* h, int* finite) {
  CG_REQUIRE(h && finite, "null argument");
  const int one = 3;
  CG_CUDA_TRY(cudaMemcpyAsync(h->flag, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  k_pennes_finite<<<1024, 256, 0, h->stream>>>(h->th[h->cur], h->cfg.dose ? h->dose : nullptr, h->ncell, h->flag);
  CG_CUDA_TRY(cudaGetLastError());
  int v = 0;
  CG_CUDA_TRY(cudaMemcpyAsync(&v, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  *finite = v;
  return CG_OK;
}

extern "C" int cg_pennes_get_state(cg_pennes* h, float* theta, float* theta_max, float* dose) {
  CG_REQUIRE(h, "null handle");
  const size_t n = (size_t)h->ncell;
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (theta) CG_CUDA_TRY(cudaMemcpy(theta, h->th[h->cur], 4 * n, cudaMemcpyDefault));
  if (theta_max) CG_CUDA_TRY(cudaMemcpy(theta_max, h->thmax, 4 * n, cudaMemcpyDefault));
  if (dose) CG_CUDA_TRY(cudaMemcpy(dose, h->dose, 4 * n, cudaMemcpyDefault));
  return CG_OK;
}
