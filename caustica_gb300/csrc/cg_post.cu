// Device post-processing of recorded phasors for GB300 (sm_103a): focal
// metrics and the acoustic -> thermal heating source.
//
// Focal metrics follow report/metrics.py:96-313 (interior argmax, -6 dB
// extents through the peak, -6 dB volume); the heating source follows
// sensors.py:259-273 (Q = sum_n alpha_n |P_n|^2 / (rho c) in float64,
// returned as float32).
//
// |P| is the correctly rounded float32 of sqrt(re^2 + im^2): the squares of
// two floats are exact in float64, so one float64 add, one float64 square
// root and one rounding give it. A float32 estimate (relative error below
// 2^-22 while the amplitude exceeds 1e-12) settles every comparison whose
// operands are further apart than a 2^-20 band; inside the band the exact
// value decides, so argmax and counts equal those of the exact amplitudes
// while the float64 unit (slow on GB300) runs only for the few voxels near a
// decision.
//
// The reductions are one pass each and HBM-bound: argmax reads P1 (and P2)
// over the interior once, the count reads P1 once more (its threshold is
// half the maximum, known only after the first pass).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cg_solver.cuh"
#include "caustica_gb300.h"

namespace {

constexpr int kPostThreads = 256;
constexpr float kBandLo = 1.0f - 1.0f / 1048576.0f;  // 1 - 2^-20
constexpr float kBandHi = 1.0f + 1.0f / 1048576.0f;
// Below this amplitude the squares approach float32 underflow and the
// estimate's error is no longer relative: the exact value decides.
constexpr float kTiny = 1e-12f;

__device__ __forceinline__ float amp_exact(float2 v) {
  const double re = (double)v.x, im = (double)v.y;
  return __double2float_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im))));
}

__device__ __forceinline__ float amp_estimate(float2 v) { return sqrtf(fmaf(v.x, v.x, v.y * v.y)); }

// Order key: larger amplitude first, then the smaller index (NumPy's argmax
// returns the first maximum in C order). Amplitudes are >= 0, so their bit
// patterns order like the values.
__device__ __forceinline__ unsigned long long amp_key(float a, unsigned int idx) {
  return ((unsigned long long)__float_as_uint(a) << 32) | (unsigned long long)(0xFFFFFFFFu - idx);
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

struct Box {
  int ny, nz;        // record region strides (x-major, z fastest)
  int lo[3];         // interior start
  unsigned int ey, ez;  // interior extents along y and z
  unsigned long long count;  // interior voxels
};

__device__ __forceinline__ unsigned int box_index(const Box& b, unsigned long long t) {
  const unsigned int tt = (unsigned int)t;
  const unsigned int z = tt % b.ez;
  const unsigned int r = tt / b.ez;
  const unsigned int y = r % b.ey;
  const unsigned int x = r / b.ey;
  return ((unsigned int)(b.lo[0] + x) * (unsigned int)b.ny + (unsigned int)(b.lo[1] + y)) * (unsigned int)b.nz +
         (unsigned int)(b.lo[2] + z);
}

struct FocusScratch {
  unsigned long long key1, key2, count;
  float p_max_at_peak, a2_at_peak, p_probe, pad;
  // followed by the three profiles through the peak: nx + ny + nz floats
};

// Running argmax of one field: the exact amplitude is formed only where the
// estimate is not clearly below the current best.
struct ArgMax {
  float best = -1.0f;
  unsigned long long key = 0ull;
  __device__ __forceinline__ void push(float2 v, unsigned int idx) {
    const float e = amp_estimate(v);
    if (!(e < best * kBandLo) || best < kTiny) {
      const float a = amp_exact(v);
      const unsigned long long k = amp_key(a, idx);
      if (k > key) {
        key = k;
        best = a;
      }
    }
  }
};

__device__ void block_max_commit(unsigned long long k, unsigned long long* dst, unsigned long long* sh) {
  k = warp_max_u64(k);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = k;
  __syncthreads();
  if (w == 0) {
    unsigned long long v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0ull;
    v = warp_max_u64(v);
    if (lane == 0 && v) atomicMax(dst, v);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kPostThreads) k_focus_argmax(const float2* __restrict__ p1,
                                                                const float2* __restrict__ p2, Box b,
                                                                FocusScratch* out) {
  __shared__ unsigned long long sh[kPostThreads / 32];
  ArgMax m1, m2;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < b.count; t += stride) {
    const unsigned int i = box_index(b, t);
    m1.push(p1[i], i);
    if (p2) m2.push(p2[i], i);
  }
  block_max_commit(m1.key, &out->key1, sh);
  if (p2) block_max_commit(m2.key, &out->key2, sh);
}

// Interior voxels with |P1| >= half the peak; the first nx + ny + nz threads
// also gather the profiles through the peak and the values at the peak.
__global__ void __launch_bounds__(kPostThreads) k_focus_count(const float2* __restrict__ p1,
                                                               const float2* __restrict__ p2,
                                                               const float* __restrict__ pmax, Box b, int nx,
                                                               long long probe, FocusScratch* out) {
  const unsigned long long key = out->key1;
  const unsigned int pk = 0xFFFFFFFFu - (unsigned int)(key & 0xFFFFFFFFull);
  const float thr = 0.5f * __uint_as_float((unsigned int)(key >> 32));
  const unsigned long long gid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const int ny = b.ny, nz = b.nz;
  const unsigned int px = pk / (unsigned int)(ny * nz), py = (pk / (unsigned int)nz) % (unsigned int)ny,
                     pz = pk % (unsigned int)nz;
  float* prof = reinterpret_cast<float*>(out + 1);
  if (gid < (unsigned long long)(nx + ny + nz)) {
    const int g = (int)gid;
    unsigned int i;
    if (g < nx)
      i = ((unsigned int)g * ny + py) * nz + pz;
    else if (g < nx + ny)
      i = (px * ny + (unsigned int)(g - nx)) * nz + pz;
    else
      i = (px * ny + py) * nz + (unsigned int)(g - nx - ny);
    prof[g] = amp_exact(p1[i]);
  }
  if (gid == 0) {
    out->p_max_at_peak = pmax ? pmax[pk] : __int_as_float(0x7FC00000);
    out->a2_at_peak = p2 ? amp_exact(p2[pk]) : __int_as_float(0x7FC00000);
    out->p_probe = probe >= 0 ? amp_exact(p1[probe]) : __int_as_float(0x7FC00000);
  }
  unsigned int n = 0;
  const float hi = thr * kBandHi, lo = thr * kBandLo;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long t = gid; t < b.count; t += stride) {
    const float2 v = p1[box_index(b, t)];
    const float e = amp_estimate(v);
    if (thr < kTiny)
      n += amp_exact(v) >= thr ? 1u : 0u;
    else if (e >= hi)
      ++n;
    else if (!(e < lo))
      n += amp_exact(v) >= thr ? 1u : 0u;
  }
  n = __reduce_add_sync(0xFFFFFFFFu, n);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(&out->count, (unsigned long long)n);
}

int post_grid(unsigned long long work) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned long long want = (work + kPostThreads - 1) / kPostThreads;
  const unsigned long long cap = (unsigned long long)sms * 8;
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// First coordinate where the profile drops below `level` walking from `i0`
// in direction `dir`, interpolated linearly (metrics.py:126-137). The
// interpolation weight is formed in float32 as the reference's NumPy
// float32 scalars do; the coordinate arithmetic is float64.
bool crossing(const float* prof, int n, int i0, int dir, float level, int off, double dx, double* at) {
  for (int k = i0; k + dir >= 0 && k + dir < n; k += dir) {
    const float a = prof[k], b = prof[k + dir];
    if (b < level && level <= a) {
      const float t = (a - level) / (a - b);
      const double ca = (double)(k + off) * dx, cb = (double)(k + dir + off) * dx;
      const double d = cb - ca;
      const double td = (double)t * d;
      *at = ca + td;
      return true;
    }
  }
  return false;
}

int focus_run(const cg_focus_input* in, cg_focus_report* out, void* scratch, cudaStream_t st) {
  const int nx = in->shape[0], ny = in->shape[1], nz = in->shape[2];
  Box b;
  b.ny = ny;
  b.nz = nz;
  unsigned long long cnt = 1;
  for (int a = 0; a < 3; ++a) {
    b.lo[a] = in->lo[a];
    cnt *= (unsigned long long)(in->hi[a] - in->lo[a]);
  }
  b.ey = (unsigned int)(in->hi[1] - in->lo[1]);
  b.ez = (unsigned int)(in->hi[2] - in->lo[2]);
  b.count = cnt;
  long long probe = -1;
  if (in->probe[0] >= 0 && in->probe[1] >= 0 && in->probe[2] >= 0 && in->probe[0] < nx && in->probe[1] < ny &&
      in->probe[2] < nz)
    probe = ((long long)in->probe[0] * ny + in->probe[1]) * nz + in->probe[2];
  FocusScratch* sc = static_cast<FocusScratch*>(scratch);
  const float2* p1 = reinterpret_cast<const float2*>(in->p1);
  const float2* p2 = reinterpret_cast<const float2*>(in->p2);
  const int nprof = nx + ny + nz;
  CG_CUDA_TRY(cudaMemsetAsync(sc, 0, sizeof(FocusScratch), st));
  k_focus_argmax<<<post_grid(cnt), kPostThreads, 0, st>>>(p1, p2, b, sc);
  CG_CUDA_TRY(cudaGetLastError());
  const unsigned long long w2 = cnt > (unsigned long long)nprof ? cnt : (unsigned long long)nprof;
  k_focus_count<<<post_grid(w2), kPostThreads, 0, st>>>(p1, p2, in->pmax, b, nx, probe, sc);
  CG_CUDA_TRY(cudaGetLastError());
  const size_t bytes = sizeof(FocusScratch) + sizeof(float) * (size_t)nprof;
  char* host = static_cast<char*>(malloc(bytes));
  if (!host) {
    cg_set_error("out of host memory");
    return CG_ERR_OOM;
  }
  cudaError_t e = cudaMemcpyAsync(host, sc, bytes, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    free(host);
    cg_set_error("focus metrics: %s", cudaGetErrorString(e));
    return CG_ERR_CUDA;
  }
  FocusScratch r;
  memcpy(&r, host, sizeof(r));
  const float* prof = reinterpret_cast<const float*>(host + sizeof(FocusScratch));
  memset(out, 0, sizeof(*out));
  const unsigned int pk = 0xFFFFFFFFu - (unsigned int)(r.key1 & 0xFFFFFFFFull);
  uint32_t bits = (uint32_t)(r.key1 >> 32);
  memcpy(&out->p_peak, &bits, 4);
  out->peak = pk;
  out->n_above_half = (long long)r.count;
  out->p_max_at_peak = r.p_max_at_peak;
  out->p_probe = r.p_probe;
  out->has_a2 = in->p2 != nullptr;
  out->a2_at_peak = r.a2_at_peak;
  if (in->p2) {
    out->a2_peak_index = 0xFFFFFFFFu - (unsigned int)(r.key2 & 0xFFFFFFFFull);
    bits = (uint32_t)(r.key2 >> 32);
    memcpy(&out->a2_peak, &bits, 4);
  } else {
    out->a2_peak_index = -1;
    out->a2_peak = NAN;
  }
  const int pidx[3] = {(int)(pk / (unsigned int)(ny * nz)), (int)((pk / (unsigned int)nz) % (unsigned int)ny),
                       (int)(pk % (unsigned int)nz)};
  const float* lines[3] = {prof, prof + nx, prof + nx + ny};
  for (int a = 0; a < 3; ++a) {
    const float level = 0.5f * lines[a][pidx[a]];
    double right = 0.0, left = 0.0;
    const bool okr = crossing(lines[a], in->shape[a], pidx[a], +1, level, in->offset[a], in->dx, &right);
    const bool okl = crossing(lines[a], in->shape[a], pidx[a], -1, level, in->offset[a], in->dx, &left);
    out->truncated[a] = !(okr && okl);
    out->left[a] = out->truncated[a] ? NAN : left;
    out->right[a] = out->truncated[a] ? NAN : right;
  }
  free(host);
  return CG_OK;
}

int focus_check(const cg_focus_input* in) {
  CG_REQUIRE(in->p1, "no fundamental phasor");
  CG_REQUIRE(in->dx > 0.0, "dx must be > 0");
  long long n = 1;
  for (int a = 0; a < 3; ++a) {
    CG_REQUIRE(in->shape[a] >= 1, "record region axis %d is empty", a);
    CG_REQUIRE(0 <= in->lo[a] && in->lo[a] < in->hi[a] && in->hi[a] <= in->shape[a],
               "axis %d: the interior [%d, %d) is empty or outside the record region of %d", a, in->lo[a],
               in->hi[a], in->shape[a]);
    n *= in->shape[a];
  }
  CG_REQUIRE(n < 0xFFFFFFFFll, "record region of %lld voxels exceeds 2^32 - 1", n);
  return CG_OK;
}

// ------------------------------------------------------------ heating --

constexpr int kHeatMaxLabels = 256;

struct HeatArgs {
  const float2* ph[CG_MAX_H];
  int nt;
  int rx, ry, rz;           // record region
  int qx, qy, qz;           // heating grid
  int qo[3];                // heating-grid voxel of record voxel 0
  const uint8_t* labels;    // label mode
  int my, mz;               // map strides (x-major, z fastest)
  int mo[3];                // map voxel of record voxel 0
  const double* coef;       // [n_labels][nt + 1] (device)
  int n_labels;
  const float *alpha, *rho, *c;  // dense mode, in the map frame
  double factor[CG_MAX_H];
  float scale;
};

__device__ __forceinline__ double warp_sum_f64(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// One thread per heating-grid voxel (grid-stride); the float64 sum of each
// term over the record region goes to sums[t] when sums is given.
__global__ void __launch_bounds__(kPostThreads) k_heating_q(HeatArgs A, float* __restrict__ q, double* sums) {
  extern __shared__ double tab[];
  __shared__ double part[kPostThreads / 32][CG_MAX_H];
  const int row = A.nt + 1;
  if (A.labels)
    for (int i = threadIdx.x; i < A.n_labels * row; i += blockDim.x) tab[i] = A.coef[i];
  __syncthreads();
  double tsum[CG_MAX_H];
#pragma unroll
  for (int h = 0; h < CG_MAX_H; ++h) tsum[h] = 0.0;
  const long long total = (long long)A.qx * A.qy * A.qz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i % A.qz);
    const long long r = i / A.qz;
    const int y = (int)(r % A.qy);
    const int x = (int)(r / A.qy);
    const int ax = x - A.qo[0], ay = y - A.qo[1], az = z - A.qo[2];
    float out = 0.0f;
    if (ax >= 0 && ax < A.rx && ay >= 0 && ay < A.ry && az >= 0 && az < A.rz) {
      const long long ri = ((long long)ax * A.ry + ay) * A.rz + az;
      const long long mi = ((long long)(ax + A.mo[0]) * A.my + (ay + A.mo[1])) * A.mz + (az + A.mo[2]);
      double irc;
      const double* an = nullptr;
      if (A.labels) {
        an = tab + (int)A.labels[mi] * row;
        irc = an[A.nt];
      } else {
        irc = __ddiv_rn(1.0, __dmul_rn((double)A.rho[mi], (double)A.c[mi]));
      }
      double acc = 0.0;
#pragma unroll
      for (int h = 0; h < CG_MAX_H; ++h) {
        if (h < A.nt) {
          const double a = (double)amp_exact(A.ph[h][ri]);
          const double p2 = __dmul_rn(a, a);
          const double alpha_n = an ? an[h] : __dmul_rn((double)A.alpha[mi], A.factor[h]);
          const double term = __dmul_rn(__dmul_rn(alpha_n, p2), irc);
          acc = __dadd_rn(acc, term);
          tsum[h] += term;
        }
      }
      out = __fmul_rn(__double2float_rn(acc), A.scale);
    }
    q[i] = out;
  }
  if (!sums) return;  // uniform over the grid
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int h = 0; h < CG_MAX_H; ++h) {
    const double v = warp_sum_f64(tsum[h]);
    if (lane == 0) part[w][h] = v;
  }
  __syncthreads();
  if (threadIdx.x < A.nt) {
    double v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) v += part[k][threadIdx.x];
    atomicAdd(&sums[threadIdx.x], v);
  }
}

int heating_run(const cg_heating_spec* sp, float* q_dev, double* coef_dev, double* sums_dev, cudaStream_t st) {
  HeatArgs A;
  memset(&A, 0, sizeof(A));
  A.nt = sp->n_terms;
  for (int h = 0; h < A.nt; ++h) {
    A.ph[h] = reinterpret_cast<const float2*>(sp->phasor[h]);
    A.factor[h] = sp->alpha_factor[h];
  }
  A.rx = sp->shape[0];
  A.ry = sp->shape[1];
  A.rz = sp->shape[2];
  A.qx = sp->q_shape[0];
  A.qy = sp->q_shape[1];
  A.qz = sp->q_shape[2];
  A.my = sp->map_shape[1];
  A.mz = sp->map_shape[2];
  for (int a = 0; a < 3; ++a) {
    A.qo[a] = sp->q_origin[a];
    A.mo[a] = sp->map_origin[a];
  }
  A.labels = sp->n_labels > 0 ? sp->labels : nullptr;
  A.n_labels = sp->n_labels;
  A.coef = coef_dev;
  A.alpha = sp->alpha;
  A.rho = sp->rho;
  A.c = sp->c;
  A.scale = sp->scale;
  const size_t smem = A.labels ? sizeof(double) * (size_t)A.n_labels * (A.nt + 1) : 0;
  const long long total = (long long)A.qx * A.qy * A.qz;
  if (sums_dev) CG_CUDA_TRY(cudaMemsetAsync(sums_dev, 0, sizeof(double) * A.nt, st));
  k_heating_q<<<post_grid((unsigned long long)total), kPostThreads, smem, st>>>(A, q_dev, sums_dev);
  CG_CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

int heating_check(const cg_heating_spec* sp) {
  CG_REQUIRE(sp->n_terms >= 1 && sp->n_terms <= CG_MAX_H, "n_terms must be 1..%d, got %d", CG_MAX_H,
             sp->n_terms);
  for (int h = 0; h < sp->n_terms; ++h) CG_REQUIRE(sp->phasor[h], "phasor of term %d is null", h);
  for (int a = 0; a < 3; ++a) {
    CG_REQUIRE(sp->shape[a] >= 1 && sp->q_shape[a] >= 1 && sp->map_shape[a] >= 1, "empty extent on axis %d", a);
    CG_REQUIRE(sp->q_origin[a] >= 0 && sp->q_origin[a] + sp->shape[a] <= sp->q_shape[a],
               "axis %d: the record region does not fit the heating grid", a);
    CG_REQUIRE(sp->map_origin[a] >= 0 && sp->map_origin[a] + sp->shape[a] <= sp->map_shape[a],
               "axis %d: the record region does not fit the medium map", a);
  }
  if (sp->n_labels > 0) {
    CG_REQUIRE(sp->n_labels <= kHeatMaxLabels, "n_labels must be <= %d", kHeatMaxLabels);
    CG_REQUIRE(sp->labels && sp->coef, "label mode needs labels and coef");
  } else {
    CG_REQUIRE(sp->alpha && sp->rho && sp->c, "dense mode needs alpha, rho and c maps");
  }
  return CG_OK;
}

}  // namespace

// ---------------------------------------------------------------- C ABI --

extern "C" int cg_focus_metrics(const cg_focus_input* in, cg_focus_report* out, void* stream) {
  CG_REQUIRE(in && out, "null argument");
  int rc = focus_check(in);
  if (rc != CG_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  const size_t bytes = sizeof(FocusScratch) + sizeof(float) * (size_t)(in->shape[0] + in->shape[1] + in->shape[2]);
  CG_CUDA_TRY(cudaMallocAsync(&scratch, bytes, st));
  rc = focus_run(in, out, scratch, st);
  cudaFreeAsync(scratch, st);
  return rc;
}

static int solver_phasor(cg_solver* s, int member, int harmonic, const float** out) {
  for (int h = 0; h < s->nh; ++h)
    if (s->harm[h] == harmonic) {
      *out = reinterpret_cast<const float*>(s->ph + ((size_t)member * s->nh + h) * s->nrec);
      return CG_OK;
    }
  *out = nullptr;
  return CG_ERR_INVALID;
}

static void record_shape(const cg_solver* s, int shape[3]) {
  for (int a = 0; a < 3; ++a) shape[a] = s->rec_hi[a] - s->rec_lo[a];
}

extern "C" int cg_solver_focus_metrics(cg_solver* s, int member, const cg_focus_input* in, cg_focus_report* out) {
  CG_REQUIRE(s && in && out, "null argument");
  CG_REQUIRE(s->ph_valid, "no finalized record window (call cg_solver_finalize first)");
  CG_REQUIRE(member >= 0 && member < s->B, "member %d out of range [0, %d)", member, s->B);
  cg_focus_input q = *in;
  if (solver_phasor(s, member, 1, &q.p1) != CG_OK) {
    cg_set_error("the fundamental (harmonic 1) was not recorded");
    return CG_ERR_INVALID;
  }
  solver_phasor(s, member, 2, &q.p2);
  q.pmax = s->pmax + (size_t)member * s->nrec;
  record_shape(s, q.shape);
  int rc = focus_check(&q);
  if (rc != CG_OK) return rc;
  const size_t bytes = sizeof(FocusScratch) + sizeof(float) * (size_t)(q.shape[0] + q.shape[1] + q.shape[2]);
  rc = cg_solver_post_scratch(s, bytes);
  if (rc != CG_OK) return rc;
  return focus_run(&q, out, s->post, s->stream);
}

// Device scratch of a heating call: coefficient table, then the term sums.
static size_t heating_scratch_bytes(const cg_heating_spec* sp) {
  const size_t ncoef = sp->n_labels > 0 ? (size_t)sp->n_labels * (sp->n_terms + 1) : 0;
  return sizeof(double) * (ncoef + CG_MAX_H);
}

static int heating_exec(const cg_heating_spec* sp, float* q_dev, double* term_sums, double* scratch,
                        cudaStream_t st) {
  double* coef = nullptr;
  double* sums = scratch;
  if (sp->n_labels > 0) {
    const size_t n = (size_t)sp->n_labels * (sp->n_terms + 1);
    coef = scratch;
    sums = scratch + n;
    CG_CUDA_TRY(cudaMemcpyAsync(coef, sp->coef, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  }
  int rc = heating_run(sp, q_dev, coef, term_sums ? sums : nullptr, st);
  if (rc != CG_OK) return rc;
  if (term_sums)
    CG_CUDA_TRY(cudaMemcpyAsync(term_sums, sums, sizeof(double) * sp->n_terms, cudaMemcpyDeviceToHost, st));
  CG_CUDA_TRY(cudaStreamSynchronize(st));
  return CG_OK;
}

extern "C" int cg_heating_q(const cg_heating_spec* spec, float* q_dev, double* term_sums, void* stream) {
  CG_REQUIRE(spec && q_dev, "null argument");
  int rc = heating_check(spec);
  if (rc != CG_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* scratch = nullptr;
  CG_CUDA_TRY(cudaMallocAsync((void**)&scratch, heating_scratch_bytes(spec), st));
  rc = heating_exec(spec, q_dev, term_sums, scratch, st);
  cudaFreeAsync(scratch, st);
  return rc;
}

extern "C" int cg_solver_heating_q(cg_solver* s, int member, const cg_heating_spec* spec, float* q_dev,
                                   double* term_sums) {
  CG_REQUIRE(s && spec && q_dev, "null argument");
  CG_REQUIRE(s->ph_valid, "no finalized record window (call cg_solver_finalize first)");
  CG_REQUIRE(member >= 0 && member < s->B, "member %d out of range [0, %d)", member, s->B);
  cg_heating_spec h = *spec;
  CG_REQUIRE(h.n_terms >= 1 && h.n_terms <= CG_MAX_H, "n_terms must be 1..%d", CG_MAX_H);
  for (int t = 0; t < h.n_terms; ++t)
    if (solver_phasor(s, member, spec->harmonics[t], &h.phasor[t]) != CG_OK) {
      cg_set_error("harmonic %d was not recorded", spec->harmonics[t]);
      return CG_ERR_INVALID;
    }
  record_shape(s, h.shape);
  if (h.n_labels > 0 && !h.labels) {
    CG_REQUIRE(s->labels, "label mode needs the solver's label map (set with cg_solver_set_medium_labels)");
    h.labels = s->labels;
    h.map_shape[0] = s->d.nx;
    h.map_shape[1] = s->d.ny;
    h.map_shape[2] = s->d.nz;
    for (int a = 0; a < 3; ++a) h.map_origin[a] = s->rec_lo[a];
  }
  int rc = heating_check(&h);
  if (rc != CG_OK) return rc;
  rc = cg_solver_post_scratch(s, heating_scratch_bytes(&h));
  if (rc != CG_OK) return rc;
  return heating_exec(&h, q_dev, term_sums, static_cast<double*>(s->post), s->stream);
}

// ----------------------------------------------------- device buffers --

extern "C" int cg_buffer_alloc(size_t bytes, void** out) {
  CG_REQUIRE(out, "null argument");
  *out = nullptr;
  cudaError_t e = cudaMalloc(out, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cg_set_error("cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    *out = nullptr;
    return CG_ERR_OOM;
  }
  return CG_OK;
}

extern "C" int cg_buffer_free(void* p) {
  if (p) CG_CUDA_TRY(cudaFree(p));
  return CG_OK;
}

extern "C" int cg_buffer_copy(void* dst, const void* src, size_t bytes) {
  CG_REQUIRE(dst && src, "null argument");
  CG_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
  return CG_OK;
}

// ----------------------------------------- device-resident label volumes --
// Callers that keep a medium's label map on the device (a framework tensor
// passed by pointer) still need two small facts on the host: which labels
// occur (the time step follows the fastest material present) and the labels
// of the source voxels (the injection scale uses the local sound speed).

__global__ void k_label_counts(const uint8_t* __restrict__ lab, long long n, unsigned long long* counts) {
  __shared__ unsigned int h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0u;
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    atomicAdd(&h[lab[i]], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&counts[i], (unsigned long long)h[i]);
}

__global__ void k_gather_u8(const uint8_t* __restrict__ src, const long long* __restrict__ idx, int n,
                            uint8_t* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = src[idx[i]];
}

extern "C" int cg_label_counts(const uint8_t* labels_dev, long long n, unsigned long long* counts256) {
  CG_REQUIRE(labels_dev && counts256, "null argument");
  CG_REQUIRE(n >= 0, "negative length");
  cudaPointerAttributes at;
  CG_CUDA_TRY(cudaPointerGetAttributes(&at, labels_dev));
  CG_REQUIRE(at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged,
             "the label volume must be device memory");
  unsigned long long* d = nullptr;
  CG_CUDA_TRY(cudaMalloc(&d, 256 * sizeof(unsigned long long)));
  cudaError_t e = cudaMemset(d, 0, 256 * sizeof(unsigned long long));
  if (e == cudaSuccess && n > 0) {
    const long long blocks = (n + 255) / 256;
    k_label_counts<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256>>>(labels_dev, n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(counts256, d, 256 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  CG_CUDA_TRY(e);
  return CG_OK;
}

extern "C" int cg_gather_u8(const uint8_t* src_dev, const long long* idx, int n, uint8_t* out_host) {
  CG_REQUIRE(src_dev && (n == 0 || (idx && out_host)), "null argument");
  CG_REQUIRE(n >= 0, "negative count");
  if (n == 0) return CG_OK;
  long long* di = nullptr;
  uint8_t* dout = nullptr;
  CG_CUDA_TRY(cudaMalloc(&di, sizeof(long long) * n));
  cudaError_t e = cudaMalloc(&dout, n);
  if (e == cudaSuccess) e = cudaMemcpy(di, idx, sizeof(long long) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_gather_u8<<<(n + 255) / 256, 256>>>(src_dev, di, n, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out_host, dout, n, cudaMemcpyDeviceToHost);
  cudaFree(di);
  if (dout) cudaFree(dout);
  CG_CUDA_TRY(e);
  return CG_OK;
}

extern "C" int cg_stream_synchronize(void* stream) {
  CG_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return CG_OK;
}
