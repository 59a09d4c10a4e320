// Dispatch of the size-specialised z-passes to the per-length launchers
// (cg_fast_z.cuh, instantiated by the cg_fast_z_*.cu units).
#include <cuda_runtime.h>
#include <string.h>

#include "cg_kspace.cuh"

template <int N>
void zp_run_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
              int batch, cudaStream_t st);
template <int N>
void zp_run_p(const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src, const RecordDev& rec,
              const long long* ctl, int n_local, int record, float* p, float2* S0, int batch, cudaStream_t st);
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
    zp_run_u<n>(d, t, m, u, S0, S1, S2, batch, st);     \
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
    zp_run_p<n>(d, t, m, src, rec, ctl, n_local, record, p, S0, batch, st);      \
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
