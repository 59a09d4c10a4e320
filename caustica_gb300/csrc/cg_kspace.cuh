// Device-side structures shared by the k-space passes (generic and
// size-specialised translation units).
#pragma once

#include <cuda.h>  // CUtensorMap (types only: the encoder is reached through the runtime)

#include "cg_common.cuh"

// ------------------------------------------------------------ structures --
#define CG_TILE 16   // pencils per tile
#define CG_ZROWS 32  // real rows per z tile (two per complex pencil)
#define CG_MAX_H 8
#define CG_THREADS 256
#define CG_MAX_SLABS 8  // x-slabs of the slab-mode step

enum YMode { Y_FWD = 0, Y_INV = 1, Y_INV_GRAD = 2, Y_FWD_DIV = 3 };
enum XMode { X_GRAD = 0, X_DIV = 1, X_FWD = 2, X_INV = 3 };

struct Dims {
  int nx, ny, nz, nzh;
  long long ncell;  // nx*ny*nz
  long long nspec;  // nx*nzh*ny
};

struct Tables {
  const float2* twx;
  const float2* twy;
  const float2* twz;
  const float* kx;  // derivative wavenumbers, Nyquist zeroed
  const float* ky;
  const float* kz;
  const float* kx2;  // true k^2
  const float* ky2;
  const float* kz2;
  const float* sx;  // sponge profiles
  const float* sy;
  const float* sz;
};

struct MediumDev {
  const uint8_t* labels;  // null when dense
  const float4* ltab;     // per label (dt/rho, rho c^2 dt, absorb, 2 beta dt)
  const float* dtr;
  const float* rc2;
  const float* ab;
  const float* b2;  // null when linear
  int nonlinear;
};

struct SourceDev {
  const int* row_ptr;  // CSR over rows x*ny + y (size nx*ny + 1)
  const int* zidx;     // z of each source voxel
  const float* ac;     // [B][S] scale * cos(phase)
  const float* as;     // [B][S] scale * sin(phase)
  int S;
  const float4* drive;  // per step: (amp*env, sin wt, cos wt, 0)
  int n_drive;
};

struct RecordDev {
  int lo[3], hi[3];  // record box (padded coords, inside the active grid)
  long long nrec;
  float* bins;  // [B][spp][nrec]
  float* comp;  // [B][spp][nrec]  Kahan compensation
  float* pmax;  // [B][nrec]
  int clo[3], chi[3];  // convergence box
  unsigned int* peaks;  // [B][max_periods] float bits of the per-period max |p|
  int max_periods;
  int spp;
};

// -------------------------------------------------------------- helpers --
__device__ __forceinline__ float sinc_a2(float a2) {
  // sin(a)/a = sum_n (-1)^n a^(2n) / (2n+1)!, truncated after a^14; for
  // a <= 2 the first omitted term is below 2e-10.
  if (a2 > 4.0f) {
    float a = sqrtf(a2);
    return sinf(a) / a;
  }
  float r = -7.6471637318198164759e-13f;
  r = fmaf(r, a2, 1.6059043836821614599e-10f);
  r = fmaf(r, a2, -2.5052108385441718775e-08f);
  r = fmaf(r, a2, 2.7557319223985890653e-06f);
  r = fmaf(r, a2, -1.9841269841269841270e-04f);
  r = fmaf(r, a2, 8.3333333333333333333e-03f);
  r = fmaf(r, a2, -1.6666666666666666667e-01f);
  r = fmaf(r, a2, 1.0f);
  return r;
}

__device__ __forceinline__ void load_tw(float2* dst, const float2* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// coefficients of one cell: (dt/rho, rho c^2 dt, absorb, 2 beta dt)
__device__ __forceinline__ float4 cell_coef(const MediumDev& m, long long i) {
  if (m.labels) return m.ltab[m.labels[i]];
  float4 r;
  r.x = m.dtr[i];
  r.y = m.rc2[i];
  r.z = m.ab[i];
  r.w = m.b2 ? m.b2[i] : 0.0f;
  return r;
}


// ---------------------------------------------- size-specialised passes --
// Launch the size-specialised kernel for this axis length when one exists
// (returns false otherwise; the caller then uses the generic kernel).
bool fast_has(int n);
bool fast_xy_has(int n);  // n in CG_FAST_XYSIZES
int fast_prepare();  // lift the dynamic shared-memory limits (once per device)
// fused transverse passes (cg_fused_xy.cu): 1 when they apply to the grid
int fused_xy_supported(const Dims& d);
bool fused_xy(bool grad, const Dims& d, const Tables& t, float kcoef, float invN, float2* S0, float2* S1,
              float2* S2, int batch, cudaStream_t st);
bool fast_ypass(int mode, const Dims& d, const Tables& t, float2* S0, float2* S1, float2* S2, int batch,
                cudaStream_t st);
bool fast_xpass(int mode, const Dims& d, const Tables& t, float kcoef, float invN, float2* S0, float2* S1,
                float2* S2, int batch, cudaStream_t st);
// persistent = false keeps the one-tile-per-CTA z kernels (autotuner choice)
bool fast_zpass_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
                  int batch, cudaStream_t st, bool persistent = true);
bool fast_zpass_p(int mode, const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src,
                  const RecordDev& rec, const long long* ctl, int n_local, int record, float* p, float2* S0,
                  int batch, cudaStream_t st, bool persistent = true);

// Tensor-map (TMA) staging of the persistent z-tiles: one descriptor per
// spectrum in the u-pass's component order (S1, S0, S2; the p-pass reads
// map[1] = S0), each a [member x][kz][2 ny floats] grid of 32-float x kz
// boxes, and a device flag that a staging wait sets if it gives up. Kernels
// take the whole struct by value as a __grid_constant__ parameter, so every
// launch carries its own copy of the descriptors.
struct ZTma {
  CUtensorMap map[3];
  int* err;
};
// 1 when the persistent z-passes of this grid can stage by tensor map: ny
// even, nz one of their lengths with nz / 2 + 1 <= 256 (a box dimension)
int ztma_supported(const Dims& d);
// Encode the three descriptors for `batch` members into *z (host memory);
// CG_OK, or an error (set) when the driver refuses them.
int ztma_encode(ZTma* z, const Dims& d, int batch, float2* S1, float2* S0, float2* S2);
// u- and p-passes staged by tensor map (persistent kernels; z: the encoded
// descriptors, host memory). False when the grid has no such kernel.
bool fast_zpass_u_tma(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1,
                      float2* S2, int batch, cudaStream_t st, const ZTma& z);
bool fast_zpass_p_tma(const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src, const RecordDev& rec,
                      const long long* ctl, int n_local, int record, float* p, float2* S0, int batch,
                      cudaStream_t st, const ZTma& z);

// The forward z-transform of p into S0 with the kernel family the step's
// p-pass runs on this grid (bitwise the spectrum a step leaves); false when
// no size-specialised kernel covers nz.
bool fast_zpass_fwd_step(const Dims& d, const Tables& t, const MediumDev& m, float* p, float2* S0, int batch,
                         cudaStream_t st, bool persistent);

// Axis lengths with a size-specialised kernel.
#define CG_FAST_SIZES(X) X(8) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(160) X(192) X(256)
// lengths of the x/y passes and of the persistent z-passes (ny even): the
// above, 320 and 400 (20 threads per pencil), 512 and 640 (32 threads per
// pencil)
#define CG_FAST_ZSIZES(X) CG_FAST_SIZES(X) X(320) X(400) X(512) X(640)
#define CG_FAST_XYSIZES(X) CG_FAST_ZSIZES(X)
