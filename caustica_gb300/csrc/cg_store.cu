// Dynamic float16 quantisation of stored result fields for GB300 (sm_103a):
// the output contract of the caustica-result/1 store (io/quantize.py:45-67,
// applied per field by io/store.py:69-89).
//
// Per field x (float32, n values at a fixed stride):
//   peak = max |x|                                    (k_q_absmax)
//   q    = half_rn(x / peak), err = max |float(q) peak - x|   (k_q_half)
// with x / peak, float(q) * peak and the difference each one correctly
// rounded float32 operation, as NumPy evaluates them for a float32 array
// and a Python-float peak; the float32 -> float16 conversion rounds to
// nearest even like NumPy's astype. The host then keeps the float16 copy
// when err / peak (a float32 division) is at most the caller's bound, stores
// the plain cast with scale 1 when the peak is 0, and falls back to the
// float32 values otherwise (also for a NaN peak, where the reference's error
// is NaN). Both reductions are maxima of non-negative floats, taken as
// unsigned integers of their bits, so their result does not depend on the
// order of the blocks; a NaN outranks every finite value and infinity.
//
// One read of each field per pass and a 2-byte write per value: HBM-bound.
// A stored config-2 result (three harmonics and p_max over 192x192x256)
// leaves the device as 132 MB of float16 instead of 264 MB of float32.
#include <cuda_fp16.h>
#include <math.h>
#include <string.h>

#include "cg_solver.cuh"
#include "caustica_gb300.h"

namespace {

constexpr int kQThreads = 256;
constexpr int kQMaxFields = CG_QUANT_MAX_FIELDS;

struct QField {
  const float* x;
  long long n, stride, off;  // off: first value of the field in the dense output
};

struct QArgs {
  QField f[kQMaxFields];
};

__device__ __forceinline__ void block_max_to(unsigned m, unsigned* dst) {
  __shared__ unsigned part[kQThreads / 32];
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned v = threadIdx.x < kQThreads / 32 ? part[threadIdx.x] : 0u;
    v = __reduce_max_sync(0xffffffffu, v);
    if (threadIdx.x == 0 && v) atomicMax(dst, v);
  }
}

__global__ void __launch_bounds__(kQThreads) k_q_absmax(QArgs a, unsigned* __restrict__ peak_bits) {
  const QField f = a.f[blockIdx.y];
  unsigned m = 0;
  for (long long i = (long long)blockIdx.x * kQThreads + threadIdx.x; i < f.n; i += (long long)gridDim.x * kQThreads)
    m = max(m, __float_as_uint(fabsf(f.x[i * f.stride])));
  block_max_to(m, peak_bits + blockIdx.y);
}

__global__ void __launch_bounds__(kQThreads) k_q_half(QArgs a, const unsigned* __restrict__ peak_bits,
                                                      __half* __restrict__ q, unsigned* __restrict__ err_bits) {
  const QField f = a.f[blockIdx.y];
  const float peak = __uint_as_float(peak_bits[blockIdx.y]);
  const bool scaled = peak > 0.f;  // a zero peak stores the plain cast; a NaN peak falls back on the host
  unsigned m = 0;
  for (long long i = (long long)blockIdx.x * kQThreads + threadIdx.x; i < f.n; i += (long long)gridDim.x * kQThreads) {
    const float x = f.x[i * f.stride];
    __half h;
    if (scaled) {
      h = __float2half_rn(__fdiv_rn(x, peak));
      const float r = __fmul_rn(__half2float(h), peak);
      m = max(m, __float_as_uint(fabsf(__fsub_rn(r, x))));
    } else {
      h = __float2half_rn(x);
    }
    q[f.off + i] = h;
  }
  block_max_to(m, err_bits + blockIdx.y);
}

// The float32 values of one field, dense (a field that keeps float32).
__global__ void __launch_bounds__(kQThreads) k_q_gather(QField f, float* __restrict__ out) {
  for (long long i = (long long)blockIdx.x * kQThreads + threadIdx.x; i < f.n; i += (long long)gridDim.x * kQThreads)
    out[i] = f.x[i * f.stride];
}

int q_blocks(long long n) {
  // about eight values per thread, at most eight CTAs per SM per field
  const long long b = (n + 8LL * kQThreads - 1) / (8LL * kQThreads);
  return (int)(b < 1 ? 1 : (b > 8 * 152 ? 8 * 152 : b));
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// scratch: peak bits | err bits | float16 values of every field | one dense float32 field
size_t q_scratch_bytes(const QField* f, int nf) {
  long long total = 0, mx = 0;
  for (int i = 0; i < nf; ++i) {
    total += f[i].n;
    mx = f[i].n > mx ? f[i].n : mx;
  }
  return align256(sizeof(unsigned) * 2 * (size_t)nf) + align256(sizeof(__half) * (size_t)total) +
         sizeof(float) * (size_t)mx;
}

int q_check(const QField* f, int nf) {
  CG_REQUIRE(nf >= 1 && nf <= kQMaxFields, "n_fields must be 1..%d", kQMaxFields);
  for (int i = 0; i < nf; ++i) {
    CG_REQUIRE(f[i].n >= 0 && f[i].stride >= 1, "field %d: n must be >= 0 and stride >= 1", i);
    CG_REQUIRE(f[i].n == 0 || f[i].x, "field %d: null data", i);
    if (f[i].n == 0) continue;
    cudaPointerAttributes at;
    CG_CUDA_TRY(cudaPointerGetAttributes(&at, f[i].x));
    CG_REQUIRE(at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged,
               "field %d: data must be device memory", i);
  }
  return CG_OK;
}

int q_run(const QField* fin, int nf, double max_norm_err, uint16_t* f16_out, float* f32_out, float* info,
          void* scratch, cudaStream_t st) {
  QArgs a;
  memset(&a, 0, sizeof(a));
  long long off = 0, mx = 0;
  for (int i = 0; i < nf; ++i) {
    a.f[i] = fin[i];
    a.f[i].off = off;
    off += fin[i].n;
    mx = fin[i].n > mx ? fin[i].n : mx;
  }
  unsigned* bits = static_cast<unsigned*>(scratch);
  char* base = static_cast<char*>(scratch);
  __half* q = reinterpret_cast<__half*>(base + align256(sizeof(unsigned) * 2 * (size_t)nf));
  float* dense = reinterpret_cast<float*>(reinterpret_cast<char*>(q) + align256(sizeof(__half) * (size_t)off));
  CG_CUDA_TRY(cudaMemsetAsync(bits, 0, sizeof(unsigned) * 2 * (size_t)nf, st));
  if (mx > 0) {
    const dim3 grid(q_blocks(mx), nf);
    k_q_absmax<<<grid, kQThreads, 0, st>>>(a, bits);
    k_q_half<<<grid, kQThreads, 0, st>>>(a, bits, q, bits + nf);
    CG_CUDA_TRY(cudaGetLastError());
  }
  unsigned hb[2 * kQMaxFields];
  CG_CUDA_TRY(cudaMemcpyAsync(hb, bits, sizeof(unsigned) * 2 * (size_t)nf, cudaMemcpyDeviceToHost, st));
  CG_CUDA_TRY(cudaStreamSynchronize(st));
  for (int i = 0; i < nf; ++i) {
    const QField& f = a.f[i];
    float peak, maxerr;
    memcpy(&peak, &hb[i], sizeof(float));
    memcpy(&maxerr, &hb[nf + i], sizeof(float));
    float scale = 1.f, norm_err = 0.f;
    bool half = true;
    if (f.n > 0 && peak != 0.f) {
      if (peak != peak) {
        half = false;  // NaN peak: the reference's error is NaN, which fails the bound
      } else {
        volatile float e = maxerr / peak;  // float32, as NumPy divides a float32 by a Python float
        if ((double)e <= max_norm_err) {
          scale = peak;
          norm_err = e;
        } else {
          half = false;
        }
      }
    }
    info[4 * i + 0] = half ? scale : 1.f;
    info[4 * i + 1] = half ? norm_err : 0.f;
    info[4 * i + 2] = half ? 1.f : 0.f;
    info[4 * i + 3] = peak;
    if (f.n == 0) continue;
    if (half) {
      if (f16_out)
        CG_CUDA_TRY(cudaMemcpyAsync(f16_out + f.off, q + f.off, sizeof(__half) * (size_t)f.n, cudaMemcpyDefault, st));
    } else {
      CG_REQUIRE(f32_out, "field %d keeps float32 but f32_out is NULL", i);
      k_q_gather<<<q_blocks(f.n), kQThreads, 0, st>>>(f, dense);
      CG_CUDA_TRY(cudaGetLastError());
      CG_CUDA_TRY(cudaMemcpyAsync(f32_out + f.off, dense, sizeof(float) * (size_t)f.n, cudaMemcpyDefault, st));
    }
  }
  CG_CUDA_TRY(cudaStreamSynchronize(st));
  return CG_OK;
}

}  // namespace

extern "C" int cg_quantize_f16(const cg_qfield* fields, int n_fields, double max_norm_err, uint16_t* f16_out,
                               float* f32_out, float* info, void* stream) {
  CG_REQUIRE(fields && info, "null argument");
  CG_REQUIRE(n_fields >= 1 && n_fields <= kQMaxFields, "n_fields must be 1..%d", kQMaxFields);
  QField f[kQMaxFields];
  for (int i = 0; i < n_fields; ++i) f[i] = QField{fields[i].data, fields[i].n, fields[i].stride, 0};
  int rc = q_check(f, n_fields);
  if (rc != CG_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  CG_CUDA_TRY(cudaMallocAsync(&scratch, q_scratch_bytes(f, n_fields), st));
  rc = q_run(f, n_fields, max_norm_err, f16_out, f32_out, info, scratch, st);
  cudaFreeAsync(scratch, st);
  return rc;
}

extern "C" int cg_solver_quantize(cg_solver* s, int member, double max_norm_err, uint16_t* f16_out, float* f32_out,
                                  float* info) {
  CG_REQUIRE(s && info, "null argument");
  CG_REQUIRE(s->ph_valid, "no finalized record window (call cg_solver_finalize first)");
  CG_REQUIRE(member >= 0 && member < s->B, "member %d out of range [0, %d)", member, s->B);
  // harmonics ascending, each as its real then its imaginary part, then p_max
  int order[CG_MAX_H];
  for (int h = 0; h < s->nh; ++h) order[h] = h;
  for (int i = 1; i < s->nh; ++i)
    for (int j = i; j > 0 && s->harm[order[j - 1]] > s->harm[order[j]]; --j) {
      const int t = order[j];
      order[j] = order[j - 1];
      order[j - 1] = t;
    }
  QField f[kQMaxFields];
  int nf = 0;
  for (int i = 0; i < s->nh; ++i) {
    const float* ph = reinterpret_cast<const float*>(s->ph + ((size_t)member * s->nh + order[i]) * s->nrec);
    f[nf++] = QField{ph, s->nrec, 2, 0};
    f[nf++] = QField{ph + 1, s->nrec, 2, 0};
  }
  f[nf++] = QField{s->pmax + (size_t)member * s->nrec, s->nrec, 1, 0};
  int rc = cg_solver_post_scratch(s, q_scratch_bytes(f, nf));
  if (rc != CG_OK) return rc;
  return q_run(f, nf, max_norm_err, f16_out, f32_out, info, s->post, s->stream);
}
