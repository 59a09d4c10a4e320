// Dispatch of the size-specialised y- and x-passes to the per-length
// launchers (cg_fast_yx.cuh, instantiated by the cg_fast_yx_*.cu units).
#include <cuda_runtime.h>

#include "cg_kspace.cuh"

template <int N>
bool yx_launch_y(int mode, const Dims& d, const Tables& t, float2* S0, float2* S1, float2* S2, int batch,
                 cudaStream_t st);
template <int N>
bool yx_launch_x(int mode, const Dims& d, const Tables& t, float kcoef, float invN, float2* S0, float2* S1,
                 float2* S2, int batch, cudaStream_t st);
template <int N>
int yx_prepare();

bool fast_ypass(int mode, const Dims& d, const Tables& t, float2* S0, float2* S1, float2* S2, int batch,
                cudaStream_t st) {
  switch (d.ny) {
#define CASE(n) \
  case n:       \
    return yx_launch_y<n>(mode, d, t, S0, S1, S2, batch, st);
    CG_FAST_XYSIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

bool fast_xpass(int mode, const Dims& d, const Tables& t, float kcoef, float invN, float2* S0, float2* S1,
                float2* S2, int batch, cudaStream_t st) {
  switch (d.nx) {
#define CASE(n) \
  case n:       \
    return yx_launch_x<n>(mode, d, t, kcoef, invN, S0, S1, S2, batch, st);
    CG_FAST_XYSIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

int fast_prepare_yx() {
#define SET(n) \
  if (yx_prepare<n>()) return -1;
  CG_FAST_XYSIZES(SET)
#undef SET
  return 0;
}

bool fast_xy_has(int n) {
  switch (n) {
#define CASE(k) case k:
    CG_FAST_XYSIZES(CASE)
#undef CASE
    return true;
    default:
      return false;
  }
}
