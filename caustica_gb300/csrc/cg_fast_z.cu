// Dispatch of the size-specialised z-passes to the per-length launchers
// (cg_fast_z.cuh, instantiated by the cg_fast_z_*.cu units).
#include <cudaTypedefs.h>  // PFN_cuTensorMapEncodeTiled_v12000
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "cg_kspace.cuh"

template <int N>
void zp_run_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
              int batch, cudaStream_t st, const ZTma* ztma);
template <int N>
void zp_run_p(const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src, const RecordDev& rec,
              const long long* ctl, int n_local, int record, float* p, float2* S0, int batch, cudaStream_t st,
              const ZTma* ztma);
template <int N>
void zp_run_fwd(const Dims& d, const Tables& t, const MediumDev& m, float* p, float2* S0, int batch,
                cudaStream_t st);
template <int N>
int zp_prepare();
template <int N>
void zt_run_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
              int batch, cudaStream_t st);
template <int N>
void zt_run_p(int mode, const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src, const RecordDev& rec,
              const long long* ctl, int n_local, int record, float* p, float2* S0, int batch, cudaStream_t st);
template <int N>
int zt_prepare();

bool fast_zpass_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
                  int batch, cudaStream_t st, bool persistent) {
  if ((persistent || !fast_has(d.nz)) && d.ny % 2 == 0) {
    switch (d.nz) {
#define CASE(n)                                          \
  case n:                                                \
    zp_run_u<n>(d, t, m, u, S0, S1, S2, batch, st, nullptr);     \
    return true;
      CG_FAST_ZSIZES(CASE)
#undef CASE
      default:
        return false;
    }
  }
  switch (d.nz) {
#define CASE(n)                                          \
  case n:                                                \
    zt_run_u<n>(d, t, m, u, S0, S1, S2, batch, st);     \
    return true;
    CG_FAST_SIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

bool fast_zpass_p(int mode, const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src,
                  const RecordDev& rec, const long long* ctl, int n_local, int record, float* p, float2* S0,
                  int batch, cudaStream_t st, bool persistent) {
  if (mode == 1 && (persistent || !fast_has(d.nz)) && d.ny % 2 == 0) {
    switch (d.nz) {
#define CASE(n)                                                                   \
  case n:                                                                         \
    zp_run_p<n>(d, t, m, src, rec, ctl, n_local, record, p, S0, batch, st, nullptr);      \
    return true;
      CG_FAST_ZSIZES(CASE)
#undef CASE
      default:
        return false;
    }
  }
  switch (d.nz) {
#define CASE(n)                                                                         \
  case n:                                                                               \
    zt_run_p<n>(mode, d, t, m, src, rec, ctl, n_local, record, p, S0, batch, st);      \
    return true;
    CG_FAST_SIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

bool fast_zpass_fwd_step(const Dims& d, const Tables& t, const MediumDev& m, float* p, float2* S0, int batch,
                         cudaStream_t st, bool persistent) {
  // the kernel family the step's p-pass runs on this grid (fast_zpass_p, mode 1)
  if ((persistent || !fast_has(d.nz)) && d.ny % 2 == 0) {
    switch (d.nz) {
#define CASE(n)                                      \
  case n:                                            \
    zp_run_fwd<n>(d, t, m, p, S0, batch, st);        \
    return true;
      CG_FAST_ZSIZES(CASE)
#undef CASE
      default:
        return false;
    }
  }
  SourceDev src;
  memset(&src, 0, sizeof(src));
  RecordDev rec;
  memset(&rec, 0, sizeof(rec));
  rec.spp = 1;
  return fast_zpass_p(0, d, t, m, src, rec, nullptr, 0, 0, p, S0, batch, st, false);
}

// ------------------------------------------------ tensor-map staging --
int ztma_supported(const Dims& d) {
  if (d.ny % 2 != 0 || d.nz / 2 + 1 > 256) return 0;
  switch (d.nz) {
#define CASE(k) case k:
    CG_FAST_ZSIZES(CASE)
#undef CASE
    return 1;
    default:
      return 0;
  }
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library links the static CUDA runtime only); looked up once, thread-safe
// (handles are created from several host threads in a serving process)
static PFN_cuTensorMapEncodeTiled_v12000 tensormap_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    return nullptr;
  }();
  return fn;
}

int ztma_encode(ZTma* z, const Dims& d, int batch, float2* S1, float2* S0, float2* S2) {
  CG_REQUIRE(ztma_supported(d), "tensor-map staging needs an even ny and nz / 2 + 1 <= 256");
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensormap_encoder();
  if (!enc) {
    cg_set_error("cuTensorMapEncodeTiled is not available from the driver");
    return CG_ERR_CUDA;
  }
  const int nh = d.nz / 2 + 1;
  // [member x][kz][2 ny floats]; a box is 32 floats (16 complex y, 8
  // pencils: 128 bytes, the swizzle span) by all nh k rows of one x plane
  const cuuint64_t dims[3] = {(cuuint64_t)2 * d.ny, (cuuint64_t)nh, (cuuint64_t)d.nx * (cuuint64_t)batch};
  const cuuint64_t strides[2] = {(cuuint64_t)8 * d.ny, (cuuint64_t)8 * d.ny * nh};  // bytes, multiples of 16
  const cuuint32_t box[3] = {32, (cuuint32_t)nh, 1};
  const cuuint32_t unit[3] = {1, 1, 1};
  float2* const bufs[3] = {S1, S0, S2};
  for (int i = 0; i < 3; ++i) {
    CG_REQUIRE(((uintptr_t)bufs[i] & 15) == 0, "spectrum %d is not 16-byte aligned", i);
    const CUresult r = enc(&z->map[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, bufs[i], dims, strides, box, unit,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      cg_set_error("cuTensorMapEncodeTiled refused spectrum %d (CUresult %d)", i, (int)r);
      return CG_ERR_CUDA;
    }
  }
  return CG_OK;
}

bool fast_zpass_u_tma(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1,
                      float2* S2, int batch, cudaStream_t st, const ZTma& z) {
  if (!ztma_supported(d)) return false;
  switch (d.nz) {
#define CASE(n)                                          \
  case n:                                                \
    zp_run_u<n>(d, t, m, u, S0, S1, S2, batch, st, &z);    \
    return true;
    CG_FAST_ZSIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

bool fast_zpass_p_tma(const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src, const RecordDev& rec,
                      const long long* ctl, int n_local, int record, float* p, float2* S0, int batch,
                      cudaStream_t st, const ZTma& z) {
  if (!ztma_supported(d)) return false;
  switch (d.nz) {
#define CASE(n)                                                                  \
  case n:                                                                        \
    zp_run_p<n>(d, t, m, src, rec, ctl, n_local, record, p, S0, batch, st, &z);    \
    return true;
    CG_FAST_ZSIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

int fast_prepare_z() {
#define SET(n) \
  if (zt_prepare<n>()) return -1;
  CG_FAST_SIZES(SET)
#undef SET
#define SETP(n) \
  if (zp_prepare<n>()) return -1;
  CG_FAST_ZSIZES(SETP)
#undef SETP
  return 0;
}

int fast_prepare_yx();

bool fast_has(int n) {
  switch (n) {
#define CASE(k) case k:
    CG_FAST_SIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}

int fast_prepare() { return (fast_prepare_yx() == 0 && fast_prepare_z() == 0) ? 0 : -1; }
