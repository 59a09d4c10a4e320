// Common device/host helpers for the caustica GB300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#define CG_OK 0
#define CG_ERR_INVALID 1
#define CG_ERR_OOM 2
#define CG_ERR_CUDA 3
#define CG_ERR_NONFINITE 4
#define CG_ERR_TIMEOUT 5
#define CG_ERR_STATE 6

// Last error message, one per host thread.
void cg_set_error(const char* fmt, ...);

#define CG_CUDA_TRY(expr)                                                              \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess) {                                                           \
      cg_set_error("%s:%d: %s -> %s", __FILE__, __LINE__, #expr, cudaGetErrorString(_e)); \
      return CG_ERR_CUDA;                                                              \
    }                                                                                  \
  } while (0)

#define CG_REQUIRE(cond, ...)      \
  do {                             \
    if (!(cond)) {                 \
      cg_set_error(__VA_ARGS__);   \
      return CG_ERR_INVALID;       \
    }                              \
  } while (0)

// ---------------------------------------------------------------- complex --
__host__ __device__ __forceinline__ float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 c_mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }
// i * a
__host__ __device__ __forceinline__ float2 c_muli(float2 a) { return make_float2(-a.y, a.x); }
// -i * a
__host__ __device__ __forceinline__ float2 c_mulmi(float2 a) { return make_float2(a.y, -a.x); }

// Largest pencil length any axis may have (radix plan in a fixed array).
#define CG_MAX_N 2048
#define CG_MAX_STAGES 16

// Radix plan for one axis. Stockham autosort, stages applied in order.
struct AxisPlan {
  int n;
  int nstages;
  int radix[CG_MAX_STAGES];
};

// Build a plan of radices {8,4,2,3,5}; returns 0 on success.
static inline int cg_make_plan(int n, AxisPlan* pl) {
  pl->n = n;
  pl->nstages = 0;
  if (n < 1 || n > CG_MAX_N) return -1;
  int m = n;
  while (m % 8 == 0) { pl->radix[pl->nstages++] = 8; m /= 8; }
  while (m % 4 == 0) { pl->radix[pl->nstages++] = 4; m /= 4; }
  while (m % 2 == 0) { pl->radix[pl->nstages++] = 2; m /= 2; }
  while (m % 3 == 0) { pl->radix[pl->nstages++] = 3; m /= 3; }
  while (m % 5 == 0) { pl->radix[pl->nstages++] = 5; m /= 5; }
  return m == 1 ? 0 : -1;
}
