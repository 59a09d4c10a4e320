// k-space pseudospectral CW solver step for GB300 (sm_103a).
//
// Scheme (reference: solvers/kspace/engine.py:458-482, operators.py:60-157):
//   u_i <- (u_i - dt/rho * IFFT{ i k_i kappa FFT{p} }) * absorb * sponge
//   p   <- (p - (rho c^2 dt + 2 beta dt p) * IFFT{ kappa sum_i i k_i FFT{u_i} }) * absorb * sponge
//   p[src] += amp ramp(t) (2 c dt/dx) sin(omega t - phase)
// with kappa = sinc(c_ref |k| dt / 2) and i k_i zero at the Nyquist bin of
// even axes.
//
// Layouts (per batch member):
//   real fields  p, u_x, u_y, u_z : [x][y][z]          (z fastest)
//   spectra      S0, S1, S2       : [x][kz][y] float2  (y fastest; kz < nz/2+1)
// Axis passes:
//   z-pass  rows (x, 32 consecutive y) -> real<->half-spectrum along z, two
//           real rows per complex transform, fused with the pointwise update
//   y-pass  contiguous rows (x, kz) of length ny
//   x-pass  column tiles of 16 consecutive (kz, y), stride nzh*ny, fused with
//           kappa and the i k_x factors
// One step = 8 launches:
//   Yf(S0) -> Xgrad(S0 -> S1 = IFFTx(i kx Q), S2 = IFFTx(Q)) ->
//   Yinv_grad(S1 -> Ax, S2 -> Az, i ky S2 -> Ay) -> Zu(u update, R2C u) ->
//   Yf_div(-> S1 = FFTy Vx, S0 = i ky FFTy Vy + FFTy Wz) -> Xdiv(-> S0) ->
//   Yinv(S0) -> Zp(p update, source, peak, record, R2C p -> S0)
// The 1/N of the inverse transforms is folded into kappa.
#include <math.h>

#include <map>
#include <mutex>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include "cg_common.cuh"
#include "cg_fft.cuh"

using cgfft::tile_fft;

// ---------------------------------------------------------------- errors --
static thread_local char g_err[1024] = "";

void cg_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

extern "C" const char* cg_last_error(void) { return g_err; }
extern "C" int cg_version(void) { return 10000; }

extern "C" int cg_set_device(int device) {
  CG_CUDA_TRY(cudaSetDevice(device));
  return CG_OK;
}

#include "cg_kspace.cuh"

// ============================================================ y-pass ====
// Rows (x, kz) of length ny, contiguous. A tile holds 16 rows as pencils:
// element (row c, index n) at buf[n * 17 + c].
#define YLD 17

__device__ __forceinline__ void y_load(float2* dst, const float2* __restrict__ src, long long row0, int nrows,
                                       int N, const float* mul_k) {
  // mul_k: optional per-index factor i*k[n]
  for (int idx = threadIdx.x; idx < CG_TILE * N; idx += blockDim.x) {
    int c = idx / N;
    int n = idx - c * N;
    float2 v = make_float2(0.f, 0.f);
    if (c < nrows) v = src[(row0 + c) * N + n];
    if (mul_k) v = c_muli(c_scale(v, mul_k[n]));
    dst[n * YLD + c] = v;
  }
}

__device__ __forceinline__ void y_store(float2* __restrict__ dst, const float2* src, long long row0, int nrows,
                                        int N) {
  for (int idx = threadIdx.x; idx < CG_TILE * N; idx += blockDim.x) {
    int c = idx / N;
    int n = idx - c * N;
    if (c < nrows) dst[(row0 + c) * N + n] = src[n * YLD + c];
  }
}


// S0 forward/inverse in place; GRAD: S1 -> inv -> S1, i ky S2 -> inv -> S0,
// S2 -> inv -> S2; DIV: S1 -> fwd -> S1, i ky fwd(S0) + fwd(S2) -> S0.
__global__ void __launch_bounds__(CG_THREADS) k_ypass(int mode, Dims d, AxisPlan pl, Tables t, float2* S0,
                                                      float2* S1, float2* S2) {
  extern __shared__ float2 sm[];
  const int N = d.ny;
  float2* tw = sm;
  float2* A = sm + N;
  float2* B = A + N * YLD;
  float2* H = B + N * YLD;
  load_tw(tw, t.twy, N);
  const long long nrows_all = (long long)d.nx * d.nzh;
  const long long row0 = (long long)blockIdx.x * CG_TILE;
  const int nrows = (int)min((long long)CG_TILE, nrows_all - row0);
  const long long off = (long long)blockIdx.y * d.nspec;
  S0 += off;
  S1 += off;
  S2 += off;
  const int c = threadIdx.x % CG_TILE, g = threadIdx.x / CG_TILE, G = blockDim.x / CG_TILE;

  if (mode == Y_FWD || mode == Y_INV) {
    y_load(A, S0, row0, nrows, N, nullptr);
    __syncthreads();
    float2* r = (mode == Y_FWD) ? tile_fft<false>(A, B, YLD, tw, pl, c, g, G) : tile_fft<true>(A, B, YLD, tw, pl, c, g, G);
    y_store(S0, r, row0, nrows, N);
    return;
  }
  if (mode == Y_INV_GRAD) {
    y_load(A, S1, row0, nrows, N, nullptr);
    __syncthreads();
    float2* r = tile_fft<true>(A, B, YLD, tw, pl, c, g, G);
    y_store(S1, r, row0, nrows, N);
    __syncthreads();
    y_load(A, S2, row0, nrows, N, t.ky);
    __syncthreads();
    r = tile_fft<true>(A, B, YLD, tw, pl, c, g, G);
    y_store(S0, r, row0, nrows, N);
    __syncthreads();
    y_load(A, S2, row0, nrows, N, nullptr);
    __syncthreads();
    r = tile_fft<true>(A, B, YLD, tw, pl, c, g, G);
    y_store(S2, r, row0, nrows, N);
    return;
  }
  // Y_FWD_DIV
  y_load(A, S1, row0, nrows, N, nullptr);
  __syncthreads();
  float2* r = tile_fft<false>(A, B, YLD, tw, pl, c, g, G);
  y_store(S1, r, row0, nrows, N);
  __syncthreads();
  y_load(A, S0, row0, nrows, N, nullptr);
  __syncthreads();
  r = tile_fft<false>(A, B, YLD, tw, pl, c, g, G);
  // H = i ky * r
  for (int n = g; n < N; n += G) H[n * YLD + c] = c_muli(c_scale(r[n * YLD + c], t.ky[n]));
  __syncthreads();
  y_load(A, S2, row0, nrows, N, nullptr);
  __syncthreads();
  r = tile_fft<false>(A, B, YLD, tw, pl, c, g, G);
  for (int n = g; n < N; n += G) r[n * YLD + c] = c_add(r[n * YLD + c], H[n * YLD + c]);
  __syncthreads();
  y_store(S0, r, row0, nrows, N);
}

// ============================================================ x-pass ====
// Columns (kz, y) flattened, col = kz*ny + y; element (x, col) at x*ncol + col.
#define XLD CG_TILE

__device__ __forceinline__ void x_load(float2* dst, const float2* __restrict__ src, long long col0, int ncols,
                                       long long ncol, int N) {
  for (int idx = threadIdx.x; idx < CG_TILE * N; idx += blockDim.x) {
    int n = idx / CG_TILE;
    int c = idx - n * CG_TILE;
    float2 v = make_float2(0.f, 0.f);
    if (c < ncols) v = src[(long long)n * ncol + col0 + c];
    dst[n * XLD + c] = v;
  }
}

__device__ __forceinline__ void x_store(float2* __restrict__ dst, const float2* src, long long col0, int ncols,
                                        long long ncol, int N) {
  for (int idx = threadIdx.x; idx < CG_TILE * N; idx += blockDim.x) {
    int n = idx / CG_TILE;
    int c = idx - n * CG_TILE;
    if (c < ncols) dst[(long long)n * ncol + col0 + c] = src[n * XLD + c];
  }
}


// GRAD: S0 -> Q = kappa/N FFTx(S0); S1 = IFFTx(i kx Q), S2 = IFFTx(Q)
// DIV : S0 = IFFTx(kappa/N (FFTx(S0) + i kx FFTx(S1)))
__global__ void __launch_bounds__(CG_THREADS) k_xpass(int mode, Dims d, AxisPlan pl, Tables t, float kcoef,
                                                      float invN, float2* S0, float2* S1, float2* S2) {
  extern __shared__ float2 sm[];
  const int N = d.nx;
  float2* tw = sm;
  float2* b0 = sm + N;
  float2* b1 = b0 + N * XLD;
  float2* b2 = b1 + N * XLD;
  load_tw(tw, t.twx, N);
  const long long ncol = (long long)d.nzh * d.ny;
  const long long col0 = (long long)blockIdx.x * CG_TILE;
  const int ncols = (int)min((long long)CG_TILE, ncol - col0);
  const long long off = (long long)blockIdx.y * d.nspec;
  S0 += off;
  S1 += off;
  S2 += off;
  const int c = threadIdx.x % CG_TILE, g = threadIdx.x / CG_TILE, G = blockDim.x / CG_TILE;
  // k^2 of this thread's column without the x part
  float kyz2 = 0.f;
  {
    long long col = col0 + min(c, ncols - 1);
    int kz = (int)(col / d.ny);
    int ky = (int)(col - (long long)kz * d.ny);
    kyz2 = t.ky2[ky] + t.kz2[kz];
  }
  if (mode == X_FWD || mode == X_INV) {
    x_load(b0, S0, col0, ncols, ncol, N);
    __syncthreads();
    float2* r = (mode == X_FWD) ? tile_fft<false>(b0, b1, XLD, tw, pl, c, g, G) : tile_fft<true>(b0, b1, XLD, tw, pl, c, g, G);
    x_store(S0, r, col0, ncols, ncol, N);
    return;
  }
  if (mode == X_GRAD) {
    x_load(b0, S0, col0, ncols, ncol, N);
    __syncthreads();
    float2* q = tile_fft<false>(b0, b1, XLD, tw, pl, c, g, G);
    for (int n = g; n < N; n += G) {
      float kap = sinc_a2(kcoef * (t.kx2[n] + kyz2)) * invN;
      float2 v = c_scale(q[n * XLD + c], kap);
      q[n * XLD + c] = v;
      b2[n * XLD + c] = c_muli(c_scale(v, t.kx[n]));
    }
    __syncthreads();
    float2* free_buf = (q == b0) ? b1 : b0;
    float2* r = tile_fft<true>(q, free_buf, XLD, tw, pl, c, g, G);
    x_store(S2, r, col0, ncols, ncol, N);
    __syncthreads();
    float2* other = (r == b0) ? b1 : b0;  // any buffer but b2
    r = tile_fft<true>(b2, other, XLD, tw, pl, c, g, G);
    x_store(S1, r, col0, ncols, ncol, N);
    return;
  }
  // X_DIV
  x_load(b0, S1, col0, ncols, ncol, N);
  __syncthreads();
  float2* xv = tile_fft<false>(b0, b1, XLD, tw, pl, c, g, G);
  // move the result into b2 so b0/b1 are free
  for (int n = g; n < N; n += G) b2[n * XLD + c] = xv[n * XLD + c];
  __syncthreads();
  x_load(b0, S0, col0, ncols, ncol, N);
  __syncthreads();
  float2* tv = tile_fft<false>(b0, b1, XLD, tw, pl, c, g, G);
  for (int n = g; n < N; n += G) {
    float kap = sinc_a2(kcoef * (t.kx2[n] + kyz2)) * invN;
    float2 s = c_add(tv[n * XLD + c], c_muli(c_scale(b2[n * XLD + c], t.kx[n])));
    tv[n * XLD + c] = c_scale(s, kap);
  }
  __syncthreads();
  float2* free_buf = (tv == b0) ? b1 : b0;
  float2* r = tile_fft<true>(tv, free_buf, XLD, tw, pl, c, g, G);
  x_store(S0, r, col0, ncols, ncol, N);
}

// ============================================================ z-pass ====
// Tile = (x, 32 consecutive y). Real rows y0+2c and y0+2c+1 form complex
// pencil c: z_n = f_{2c}[n] + i f_{2c+1}[n]. Element (n, c) at buf[n*ZLD + c].
#define ZLD 17
#define STLD 33

// Load half spectra (x, kz, y0..y0+31) into stg[kz*STLD + t], optionally
// times i*kz[kz]; then build the full complex pencils Z(k, c) in `out`.
__device__ void z_build_inverse(float2* out, float2* stg, const float2* __restrict__ S, const Dims& d, int x, int y0,
                                int nyv, const float* mul_k) {
  const int nz = d.nz, nzh = d.nzh;
  const float2* base = S + ((long long)x * nzh) * d.ny + y0;
  for (int idx = threadIdx.x; idx < nzh * CG_ZROWS; idx += blockDim.x) {
    int k = idx / CG_ZROWS;
    int tt = idx - k * CG_ZROWS;
    float2 v = make_float2(0.f, 0.f);
    if (tt < nyv) v = base[(long long)k * d.ny + tt];
    if (mul_k) v = c_muli(c_scale(v, mul_k[k]));
    // a complex-to-real transform reads only the real part of the
    // self-paired bins (DC, and Nyquist on an even axis)
    if (k == 0 || (2 * k == nz)) v.y = 0.f;
    stg[k * STLD + tt] = v;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < nz * CG_TILE; idx += blockDim.x) {
    int k = idx / CG_TILE;
    int c = idx - k * CG_TILE;
    int kk = (k < nzh) ? k : nz - k;
    float2 a = stg[kk * STLD + 2 * c];
    float2 b = stg[kk * STLD + 2 * c + 1];
    if (k >= nzh) {
      a = c_conj(a);
      b = c_conj(b);
    }
    out[k * ZLD + c] = make_float2(a.x - b.y, a.y + b.x);  // a + i b
  }
  __syncthreads();
}

// After a forward transform of packed real rows in `z`, write the two half
// spectra per pencil to S (x, kz, y0 + t), optionally times i*kz[kz].
__device__ void z_store_forward(float2* __restrict__ S, const float2* z, const Dims& d, int x, int y0, int nyv,
                                const float* mul_k) {
  const int nz = d.nz, nzh = d.nzh;
  float2* base = S + ((long long)x * nzh) * d.ny + y0;
  for (int idx = threadIdx.x; idx < nzh * CG_ZROWS; idx += blockDim.x) {
    int k = idx / CG_ZROWS;
    int tt = idx - k * CG_ZROWS;
    if (tt >= nyv) continue;
    int c = tt >> 1;
    float2 zk = z[k * ZLD + c];
    float2 zm = c_conj(z[((nz - k) % nz) * ZLD + c]);
    float2 v;
    if ((tt & 1) == 0) {
      v = c_scale(c_add(zk, zm), 0.5f);
    } else {
      v = c_scale(c_mulmi(c_sub(zk, zm)), 0.5f);  // (zk - zm) / (2i)
    }
    if (mul_k) v = c_muli(c_scale(v, mul_k[k]));
    base[(long long)k * d.ny + tt] = v;
  }
}

__device__ __forceinline__ float z_get(const float2* z, int n, int tt) {
  float2 v = z[n * ZLD + (tt >> 1)];
  return (tt & 1) ? v.y : v.x;
}
__device__ __forceinline__ void z_set(float2* z, int n, int tt, float val) {
  float* f = reinterpret_cast<float*>(&z[n * ZLD + (tt >> 1)]);
  f[tt & 1] = val;
}

// Velocity update for all three components. S1 = Ax, S0 = Ay, S2 = Az on
// entry; on exit S1 = FFTz(u_x), S0 = FFTz(u_y), S2 = i kz FFTz(u_z).
__global__ void __launch_bounds__(CG_THREADS) k_zpass_u(Dims d, AxisPlan pl, Tables t, MediumDev m, float* u,
                                                        float2* S0, float2* S1, float2* S2) {
  extern __shared__ float2 sm[];
  const int nz = d.nz;
  float2* tw = sm;
  float2* A = sm + nz;
  float2* B = A + nz * ZLD;  // also the half-spectrum staging area
  load_tw(tw, t.twz, nz);
  const int ytiles = (d.ny + CG_ZROWS - 1) / CG_ZROWS;
  const int x = blockIdx.x / ytiles;
  const int y0 = (blockIdx.x - x * ytiles) * CG_ZROWS;
  const int nyv = min(CG_ZROWS, d.ny - y0);
  const int b = blockIdx.y;
  const long long off = (long long)b * d.nspec;
  const int c = threadIdx.x % CG_TILE, g = threadIdx.x / CG_TILE, G = blockDim.x / CG_TILE;
  const float sxv = t.sx[x];
  __syncthreads();
  for (int comp = 0; comp < 3; ++comp) {
    float2* S = (comp == 0 ? S1 : (comp == 1 ? S0 : S2)) + off;
    const float* mk = (comp == 2) ? t.kz : nullptr;
    float* uc = u + ((long long)comp * gridDim.y + b) * d.ncell;
    z_build_inverse(A, B, S, d, x, y0, nyv, mk);
    float2* z = tile_fft<true>(A, B, ZLD, tw, pl, c, g, G);
    // u <- (u - dt/rho * g) * absorb * sponge   (engine.py:462-464)
    for (int idx = threadIdx.x; idx < nyv * nz; idx += blockDim.x) {
      int tt = idx / nz;
      int zz = idx - tt * nz;
      int y = y0 + tt;
      long long cell = ((long long)x * d.ny + y) * nz + zz;
      float4 cf = cell_coef(m, cell);
      float sp = (sxv * t.sy[y]) * t.sz[zz];
      float gv = z_get(z, zz, tt);
      float un = uc[cell] - cf.x * gv;
      un = un * cf.z;
      un = un * sp;
      uc[cell] = un;
      z_set(z, zz, tt, un);
    }
    // rows beyond the grid edge carry zeros
    for (int idx = threadIdx.x; idx < (CG_ZROWS - nyv) * nz; idx += blockDim.x) {
      int tt = nyv + idx / nz;
      int zz = idx % nz;
      z_set(z, zz, tt, 0.f);
    }
    __syncthreads();
    float2* other = (z == A) ? B : A;
    float2* f = tile_fft<false>(z, other, ZLD, tw, pl, c, g, G);
    z_store_forward(S, f, d, x, y0, nyv, mk);
    __syncthreads();
  }
}

// Pressure update + source + convergence peak + record, then R2C of the new
// p into S0. mode 0: only the forward transform of the current p (state
// load); mode 1: full update.
__global__ void __launch_bounds__(CG_THREADS) k_zpass_p(int mode, Dims d, AxisPlan pl, Tables t, MediumDev m,
                                                        SourceDev src, RecordDev rec, const long long* ctl,
                                                        int n_local, int record, float* p, float2* S0) {
  extern __shared__ float2 sm[];
  __shared__ unsigned int s_peak;
  const int nz = d.nz;
  float2* tw = sm;
  float2* A = sm + nz;
  float2* B = A + nz * ZLD;
  load_tw(tw, t.twz, nz);
  const int ytiles = (d.ny + CG_ZROWS - 1) / CG_ZROWS;
  const int x = blockIdx.x / ytiles;
  const int y0 = (blockIdx.x - x * ytiles) * CG_ZROWS;
  const int nyv = min(CG_ZROWS, d.ny - y0);
  const int b = blockIdx.y;
  float2* S = S0 + (long long)b * d.nspec;
  float* pb = p + (long long)b * d.ncell;
  const int c = threadIdx.x % CG_TILE, g = threadIdx.x / CG_TILE, G = blockDim.x / CG_TILE;
  if (threadIdx.x == 0) s_peak = 0u;
  __syncthreads();
  float2* z;
  if (mode == 2) {
    // inverse only: half spectra -> real rows (unnormalised), no update
    z_build_inverse(A, B, S, d, x, y0, nyv, nullptr);
    z = tile_fft<true>(A, B, ZLD, tw, pl, c, g, G);
    for (int idx = threadIdx.x; idx < nyv * nz; idx += blockDim.x) {
      int tt = idx / nz;
      int zz = idx - tt * nz;
      pb[((long long)x * d.ny + y0 + tt) * nz + zz] = z_get(z, zz, tt);
    }
    return;
  }
  if (mode == 0) {
    z = A;
    for (int idx = threadIdx.x; idx < CG_ZROWS * nz; idx += blockDim.x) {
      int tt = idx / nz;
      int zz = idx - tt * nz;
      float v = 0.f;
      if (tt < nyv) v = pb[((long long)x * d.ny + y0 + tt) * nz + zz];
      z_set(z, zz, tt, v);
    }
    __syncthreads();
  } else {
    const long long n = ctl[0] + n_local;
    z_build_inverse(A, B, S, d, x, y0, nyv, nullptr);
    z = tile_fft<true>(A, B, ZLD, tw, pl, c, g, G);
    const float sxv = t.sx[x];
    // p <- (p - (rho c^2 dt [+ 2 beta dt p]) * div u) * absorb * sponge   (engine.py:470-477)
    for (int idx = threadIdx.x; idx < nyv * nz; idx += blockDim.x) {
      int tt = idx / nz;
      int zz = idx - tt * nz;
      int y = y0 + tt;
      long long cell = ((long long)x * d.ny + y) * nz + zz;
      float4 cf = cell_coef(m, cell);
      float sp = (sxv * t.sy[y]) * t.sz[zz];
      float dv = z_get(z, zz, tt);
      float po = pb[cell];
      float pn;
      if (m.nonlinear) pn = po - (cf.y + cf.w * po) * dv;
      else pn = po - cf.y * dv;
      pn = pn * cf.z;
      pn = pn * sp;
      z_set(z, zz, tt, pn);
    }
    for (int idx = threadIdx.x; idx < (CG_ZROWS - nyv) * nz; idx += blockDim.x) {
      int tt = nyv + idx / nz;
      int zz = idx % nz;
      z_set(z, zz, tt, 0.f);
    }
    __syncthreads();
    // source injection (engine.py:478-482): rows x*ny + y0 .. +nyv
    if (src.S > 0 && n < src.n_drive) {
      const float4 dr = src.drive[n];
      const int r0 = x * d.ny + y0;
      const int e0 = src.row_ptr[r0], e1 = src.row_ptr[r0 + nyv];
      for (int e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        // row of entry e: binary search in row_ptr[r0 .. r0+nyv]
        int lo = 0, hi = nyv;  // find tt with row_ptr[r0+tt] <= e < row_ptr[r0+tt+1]
        while (hi - lo > 1) {
          int mid = (lo + hi) >> 1;
          if (src.row_ptr[r0 + mid] <= e) lo = mid;
          else hi = mid;
        }
        const int zz = src.zidx[e];
        const float acv = src.ac[(long long)b * src.S + e];
        const float asv = src.as[(long long)b * src.S + e];
        const float add = dr.x * (dr.y * acv - dr.z * asv);
        float* f = reinterpret_cast<float*>(&z[zz * ZLD + (lo >> 1)]);
        f[lo & 1] += add;
      }
      __syncthreads();
    }
    // write p, convergence peak, record window
    unsigned int lpeak = 0u;
    const int m_bin = (int)(n % rec.spp);
    const long long Ry = rec.hi[1] - rec.lo[1], Rz = rec.hi[2] - rec.lo[2];
    const bool x_conv = (x >= rec.clo[0] && x < rec.chi[0]);
    const bool x_rec = record && (x >= rec.lo[0] && x < rec.hi[0]);
    float* bins = rec.bins + ((long long)b * rec.spp + m_bin) * rec.nrec;
    float* comp = rec.comp + ((long long)b * rec.spp + m_bin) * rec.nrec;
    float* pmax = rec.pmax + (long long)b * rec.nrec;
    for (int idx = threadIdx.x; idx < nyv * nz; idx += blockDim.x) {
      int tt = idx / nz;
      int zz = idx - tt * nz;
      int y = y0 + tt;
      long long cell = ((long long)x * d.ny + y) * nz + zz;
      float pn = z_get(z, zz, tt);
      pb[cell] = pn;
      float apn = fabsf(pn);
      if (x_conv && y >= rec.clo[1] && y < rec.chi[1] && zz >= rec.clo[2] && zz < rec.chi[2])
        lpeak = max(lpeak, __float_as_uint(apn));
      if (x_rec && y >= rec.lo[1] && y < rec.hi[1] && zz >= rec.lo[2] && zz < rec.hi[2]) {
        long long ri = ((long long)(x - rec.lo[0]) * Ry + (y - rec.lo[1])) * Rz + (zz - rec.lo[2]);
        // Kahan: sum s, compensation cmp (true sum = s - cmp)
        float s = bins[ri];
        float cm = comp[ri];
        float yk = pn - cm;
        float tk = s + yk;
        cm = (tk - s) - yk;
        bins[ri] = tk;
        comp[ri] = cm;
        float pm = pmax[ri];
        // NaN-propagating max like numpy.maximum
        pmax[ri] = (apn > pm || apn != apn) ? apn : pm;
      }
    }
    // block max -> atomic max on the period slot
    lpeak = __reduce_max_sync(0xffffffffu, lpeak);
    if ((threadIdx.x & 31) == 0) atomicMax(&s_peak, lpeak);
    __syncthreads();
    if (threadIdx.x == 0 && s_peak != 0u) {
      long long per = n / rec.spp;
      if (per < rec.max_periods) atomicMax(&rec.peaks[(long long)b * rec.max_periods + per], s_peak);
    }
  }
  float2* other = (z == A) ? B : A;
  float2* f = tile_fft<false>(z, other, ZLD, tw, pl, c, g, G);
  z_store_forward(S, f, d, x, y0, nyv, nullptr);
}

// Final phasors in FP64: P_h = 2/K sum_m (s_m - c_m) exp(+2 pi i h m / spp)
// (engine.py:538-552: buffers[h] += p exp(+i h w t); *= 2/rec_steps).
// The nh x spp unit phasors are formed once per block in shared memory (FP64
// sincospi is slow on GB300); every bin is read once and feeds all
// harmonics, each summed over m in increasing order.
__global__ void k_finalize(RecordDev rec, int B, int nh, const int* harm, int K, float2* out) {
  extern __shared__ double2 uph[];  // [nh][spp] (cos, sin)
  for (int i = threadIdx.x; i < nh * rec.spp; i += blockDim.x) {
    const int h = i / rec.spp, mm = i - h * rec.spp;
    double sn, cs;
    sincospi(2.0 * (double)((harm[h] * (long long)mm) % rec.spp) / rec.spp, &sn, &cs);
    uph[i] = make_double2(cs, sn);
  }
  __syncthreads();
  const long long total = (long long)B * rec.nrec;
  const double sc = 2.0 / K;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / rec.nrec;
    const long long r = i - b * rec.nrec;
    double re[CG_MAX_H], im[CG_MAX_H];
#pragma unroll
    for (int h = 0; h < CG_MAX_H; ++h) re[h] = im[h] = 0.0;
    for (int mm = 0; mm < rec.spp; ++mm) {
      const long long o = (b * rec.spp + mm) * rec.nrec + r;
      const double v = (double)rec.bins[o] - (double)rec.comp[o];
#pragma unroll
      for (int h = 0; h < CG_MAX_H; ++h)
        if (h < nh) {
          const double2 u = uph[h * rec.spp + mm];
          re[h] += v * u.x;
          im[h] += v * u.y;
        }
    }
#pragma unroll
    for (int h = 0; h < CG_MAX_H; ++h)
      if (h < nh) out[(b * nh + h) * rec.nrec + r] = make_float2((float)(re[h] * sc), (float)(im[h] * sc));
  }
}

// ------------------------------------------------------------ set-up ----
__global__ void k_twiddles(float2* tw, int n) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)m / (double)n, &s, &c);
    tw[m] = make_float2((float)c, (float)(-s));
  }
}

// k = 2 pi fftfreq(n, dx) (rfft layout when rfft != 0); kd zeroes the
// Nyquist bin of an even axis (operators.py:60-73, 90-142).
__global__ void k_wavenumbers(float* kd, float* k2, int n, int nk, double dx, int rfft) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nk; i += gridDim.x * blockDim.x) {
    double f = (rfft || i <= (n - 1) / 2) ? (double)i : (double)(i - n);
    double k = 2.0 * 3.14159265358979323846 * f / ((double)n * dx);
    k2[i] = (float)(k * k);
    kd[i] = (n % 2 == 0 && 2 * i == n) ? 0.0f : (float)k;
  }
}

// s(r) = exp(-edge ((w - r)/w)^2) on w cells at both ends (core/pml.py:210-230)
__global__ void k_sponge(float* s, int n, int width, double edge) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = 1.0;
    if (width > 0) {
      int r = -1;
      if (i < width) r = i;
      else if (i >= n - width) r = n - 1 - i;
      if (r >= 0) {
        double q = (double)(width - r) / (double)width;
        v = exp(-edge * q * q);
      }
    }
    s[i] = (float)v;
  }
}

__global__ void k_advance(long long* ctl, long long by) { ctl[0] += by; }
__global__ void k_set_ctl(long long* ctl, long long v) { ctl[0] = v; }

// =============================================================== host ====
#include "cg_solver.cuh"
#include "caustica_gb300.h"

static Tables make_tables(const cg_solver* s) {
  Tables t;
  t.twx = s->twx; t.twy = s->twy; t.twz = s->twz;
  t.kx = s->kx; t.ky = s->ky; t.kz = s->kz;
  t.kx2 = s->kx2; t.ky2 = s->ky2; t.kz2 = s->kz2;
  t.sx = s->sx; t.sy = s->sy; t.sz = s->sz;
  return t;
}

static MediumDev make_medium(const cg_solver* s) {
  MediumDev m;
  m.labels = s->labels;
  m.ltab = s->ltab;
  m.dtr = s->dtr; m.rc2 = s->rc2; m.ab = s->ab; m.b2 = s->b2;
  m.nonlinear = s->nonlinear;
  return m;
}

static RecordDev make_record(const cg_solver* s) {
  RecordDev r;
  for (int i = 0; i < 3; ++i) {
    r.lo[i] = s->rec_lo[i]; r.hi[i] = s->rec_hi[i];
    r.clo[i] = s->conv_lo[i]; r.chi[i] = s->conv_hi[i];
  }
  r.nrec = s->nrec;
  r.bins = s->bins; r.comp = s->comp; r.pmax = s->pmax;
  r.peaks = s->peaks;
  r.max_periods = s->max_periods;
  r.spp = s->spp;
  return r;
}

static SourceDev make_source(const cg_solver* s) {
  SourceDev q;
  q.row_ptr = s->src_ptr;
  q.zidx = s->src_z;
  q.ac = s->src_ac;
  q.as = s->src_as;
  q.S = s->n_src;
  q.drive = s->drive;
  q.n_drive = s->n_drive;
  return q;
}

// Cached period graphs hold kernel parameters (pointers, sizes) by value:
// any call that changes them must drop the graphs first.
static void invalidate_graphs(cg_solver* s) {
  for (int i = 0; i < 2; ++i)
    if (s->graph[i]) {
      cudaStreamSynchronize(s->stream);
      cudaGraphExecDestroy(s->graph[i]);
      s->graph[i] = nullptr;
    }
}

// The tensor-map staging flag: CG_ERR_TIMEOUT when a z-pass gave up waiting
// for a staged tile since the handle was created (its results are not to be
// trusted). Synchronises the handle's stream; free when the staging is off.
static int ztma_check(cg_solver* s) {
  if (!s->ztma_err) return CG_OK;
  int v = 0;
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  CG_CUDA_TRY(cudaMemcpy(&v, s->ztma_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) {
    cg_set_error("a z-pass gave up waiting for a tensor-map copy of its tile");
    return CG_ERR_TIMEOUT;
  }
  return CG_OK;
}

template <typename T>
static int dev_alloc(T** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    cg_set_error("cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    *p = nullptr;
    return CG_ERR_OOM;
  }
  return CG_OK;
}

#define CG_TRY(expr)          \
  do {                        \
    int _r = (expr);          \
    if (_r != CG_OK) return _r; \
  } while (0)

static void solver_free(cg_solver* s) {
  if (!s) return;
  for (int i = 0; i < 2; ++i)
    if (s->graph[i]) cudaGraphExecDestroy(s->graph[i]);
  void* ptrs[] = {s->p, s->u, s->S0, s->S1, s->S2, s->twx, s->twy, s->twz, s->kx, s->ky, s->kz, s->kx2, s->ky2,
                  s->kz2, s->sx, s->sy, s->sz, s->labels, s->ltab, s->dtr, s->rc2, s->ab, s->b2, s->src_ptr,
                  s->src_z, s->src_ac, s->src_as, s->drive, s->bins, s->comp, s->pmax, s->peaks, s->harm_dev,
                  s->ctl, s->ph, s->post, s->ztma_err};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

// Allow a kernel the device's opt-in shared memory minus its static usage.
static cudaError_t allow_max_smem(const void* func) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, func);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  return e;
}

static size_t smem_limit() {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  return (size_t)optin - 64;  // room for the kernels' static shared variables
}

static size_t smem_ypass(int ny) { return sizeof(float2) * ((size_t)ny + 3 * (size_t)ny * YLD); }
static size_t smem_xpass(int nx) { return sizeof(float2) * ((size_t)nx + 3 * (size_t)nx * XLD); }
static size_t smem_zpass(int nz) {
  size_t a = (size_t)nz * ZLD;
  size_t st = (size_t)(nz / 2 + 1) * STLD;
  return sizeof(float2) * ((size_t)nz + a + (a > st ? a : st));
}

extern "C" int cg_solver_create(const cg_solver_config* cfg, cg_solver** out) {
  CG_REQUIRE(cfg && out, "null argument");
  *out = nullptr;
  CG_REQUIRE(cfg->nx >= 1 && cfg->ny >= 1 && cfg->nz >= 2, "grid %dx%dx%d: every axis needs >= 1 cell and nz >= 2",
             cfg->nx, cfg->ny, cfg->nz);
  CG_REQUIRE(cfg->batch >= 1 && cfg->batch <= 65535, "batch %d out of range", cfg->batch);
  CG_REQUIRE(cfg->spp >= 2, "spp must be >= 2");
  CG_REQUIRE((long long)cfg->spp * (cfg->n_harmonics > 0 ? cfg->n_harmonics : 1) <= 8192,
             "spp x n_harmonics must be <= 8192 (the finalize unit-phasor table), got %d x %d", cfg->spp,
             cfg->n_harmonics);
  CG_REQUIRE(cfg->n_harmonics >= 1 && cfg->n_harmonics <= CG_MAX_H, "n_harmonics must be 1..%d", CG_MAX_H);
  CG_REQUIRE(cfg->max_periods >= 1, "max_periods must be >= 1");
  cg_solver* s = new cg_solver();
  s->d.nx = cfg->nx;
  s->d.ny = cfg->ny;
  s->d.nz = cfg->nz;
  s->d.nzh = cfg->nz / 2 + 1;
  s->d.ncell = (long long)cfg->nx * cfg->ny * cfg->nz;
  s->d.nspec = (long long)cfg->nx * s->d.nzh * cfg->ny;
  s->B = cfg->batch;
  if (cg_make_plan(cfg->nx, &s->px) || cg_make_plan(cfg->ny, &s->py) || cg_make_plan(cfg->nz, &s->pz)) {
    cg_set_error("grid %dx%dx%d: every axis must be 2/3/5-smooth and <= %d", cfg->nx, cfg->ny, cfg->nz, CG_MAX_N);
    delete s;
    return CG_ERR_INVALID;
  }
  s->spp = cfg->spp;
  s->max_periods = cfg->max_periods;
  s->nh = cfg->n_harmonics;
  for (int i = 0; i < s->nh; ++i) s->harm[i] = cfg->harmonics[i];
  const double half = 0.5 * cfg->c_ref * cfg->dt;
  s->kcoef = half * half;
  s->invN = (float)(1.0 / (double)s->d.ncell);
  s->nonlinear = cfg->nonlinear;
  long long nrec = 1;
  for (int i = 0; i < 3; ++i) {
    int n = i == 0 ? cfg->nx : (i == 1 ? cfg->ny : cfg->nz);
    if (!(cfg->rec_lo[i] >= 0 && cfg->rec_hi[i] <= n && cfg->rec_lo[i] < cfg->rec_hi[i])) {
      cg_set_error("record box axis %d [%d, %d) invalid for extent %d", i, cfg->rec_lo[i], cfg->rec_hi[i], n);
      delete s;
      return CG_ERR_INVALID;
    }
    s->rec_lo[i] = cfg->rec_lo[i];
    s->rec_hi[i] = cfg->rec_hi[i];
    s->conv_lo[i] = cfg->conv_lo[i];
    s->conv_hi[i] = cfg->conv_hi[i];
    nrec *= (cfg->rec_hi[i] - cfg->rec_lo[i]);
  }
  s->nrec = nrec;
  s->smem_y = smem_ypass(cfg->ny);
  s->smem_x = smem_xpass(cfg->nx);
  s->smem_z = smem_zpass(cfg->nz);
  // the runtime-plan passes must fit wherever an axis has no size-specialised
  // kernel (the runtime-plan z-pass also loads states and runs short z-rows)
  const size_t smem_max = smem_limit();
  if ((!fast_xy_has(cfg->ny) && s->smem_y > smem_max) || (!fast_xy_has(cfg->nx) && s->smem_x > smem_max) ||
      s->smem_z > smem_max) {
    cg_set_error("grid %dx%dx%d needs more than 227 KB of shared memory per tile", cfg->nx, cfg->ny, cfg->nz);
    delete s;
    return CG_ERR_INVALID;
  }
  int rc = CG_OK;
#define ALLOC(ptr, n)                          \
  if ((rc = dev_alloc(&(ptr), (n))) != CG_OK) { \
    solver_free(s);                            \
    return rc;                                 \
  }
  const long long B = s->B;
  ALLOC(s->p, B * s->d.ncell);
  ALLOC(s->u, 3 * B * s->d.ncell);
  ALLOC(s->S0, B * s->d.nspec);
  ALLOC(s->S1, B * s->d.nspec);
  ALLOC(s->S2, B * s->d.nspec);
  ALLOC(s->twx, cfg->nx);
  ALLOC(s->twy, cfg->ny);
  ALLOC(s->twz, cfg->nz);
  ALLOC(s->kx, cfg->nx);
  ALLOC(s->ky, cfg->ny);
  ALLOC(s->kz, s->d.nzh);
  ALLOC(s->kx2, cfg->nx);
  ALLOC(s->ky2, cfg->ny);
  ALLOC(s->kz2, s->d.nzh);
  ALLOC(s->sx, cfg->nx);
  ALLOC(s->sy, cfg->ny);
  ALLOC(s->sz, cfg->nz);
  ALLOC(s->pmax, B * s->nrec);
  ALLOC(s->peaks, B * s->max_periods);
  ALLOC(s->harm_dev, CG_MAX_H);
  ALLOC(s->ctl, 2);
  ALLOC(s->src_ptr, (long long)cfg->nx * cfg->ny + 1);
#undef ALLOC
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cg_set_error("cudaStreamCreate: %s", cudaGetErrorString(e));
    solver_free(s);
    return CG_ERR_CUDA;
  }
  // tensor-map descriptors of the three spectra for the persistent
  // z-passes (launches pass them by value) and the staging flag on the
  // device; a grid the driver refuses them for keeps the cp.async staging
  if (ztma_supported(s->d)) {
    int* flag = nullptr;
    if (ztma_encode(&s->ztma_host, s->d, s->B, s->S1, s->S0, s->S2) == CG_OK &&
        cudaMalloc(&flag, sizeof(int)) == cudaSuccess) {
      if (cudaMemset(flag, 0, sizeof(int)) == cudaSuccess) {
        s->ztma_host.err = flag;
        s->ztma_err = flag;
        s->ztma_ok = 1;
        s->ztma = 1;  // the default where it exists (measured faster on config 2); the tuner times both
      } else {
        cudaFree(flag);
      }
    }
    cudaGetLastError();
    if (!s->ztma_ok) cg_set_error("%s", "");  // a refused descriptor is not an error of the create call
  }
  cudaStream_t st = s->stream;
  k_twiddles<<<(cfg->nx + 255) / 256, 256, 0, st>>>(s->twx, cfg->nx);
  k_twiddles<<<(cfg->ny + 255) / 256, 256, 0, st>>>(s->twy, cfg->ny);
  k_twiddles<<<(cfg->nz + 255) / 256, 256, 0, st>>>(s->twz, cfg->nz);
  k_wavenumbers<<<(cfg->nx + 255) / 256, 256, 0, st>>>(s->kx, s->kx2, cfg->nx, cfg->nx, cfg->dx, 0);
  k_wavenumbers<<<(cfg->ny + 255) / 256, 256, 0, st>>>(s->ky, s->ky2, cfg->ny, cfg->ny, cfg->dx, 0);
  k_wavenumbers<<<(s->d.nzh + 255) / 256, 256, 0, st>>>(s->kz, s->kz2, cfg->nz, s->d.nzh, cfg->dx, 1);
  k_sponge<<<(cfg->nx + 255) / 256, 256, 0, st>>>(s->sx, cfg->nx, cfg->pml[0], cfg->pml_edge);
  k_sponge<<<(cfg->ny + 255) / 256, 256, 0, st>>>(s->sy, cfg->ny, cfg->pml[1], cfg->pml_edge);
  k_sponge<<<(cfg->nz + 255) / 256, 256, 0, st>>>(s->sz, cfg->nz, cfg->pml[2], cfg->pml_edge);
  int hbuf[CG_MAX_H] = {0};
  for (int i = 0; i < s->nh; ++i) hbuf[i] = s->harm[i];
  e = cudaMemcpyAsync(s->harm_dev, hbuf, sizeof(hbuf), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->src_ptr, 0, sizeof(int) * ((size_t)cfg->nx * cfg->ny + 1), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_ypass);
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_xpass);
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_zpass_u);
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_zpass_p);
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_finalize);
  if (e == cudaSuccess && fast_prepare() != 0) e = cudaErrorInvalidValue;
  if (e != cudaSuccess) {
    cg_set_error("solver set-up: %s", cudaGetErrorString(e));
    solver_free(s);
    return CG_ERR_CUDA;
  }
  {
    // CG_FUSED_XY=1 selects the cluster-fused transverse passes where they
    // apply; measured slower than the three-pass chain on a 192^2 x 256 grid
    // (one CTA per SM, cluster placement leaves SMs idle), so opt-in
    const char* env = getenv("CG_FUSED_XY");
    s->fused_xy = (env && env[0] == '1') ? fused_xy_supported(s->d) : 0;
  }
  rc = cg_solver_reset(s);
  if (rc != CG_OK) {
    solver_free(s);
    return rc;
  }
  *out = s;
  return CG_OK;
}

extern "C" int cg_solver_destroy(cg_solver* s) {
  if (s) {
    cudaStreamSynchronize(s->stream);
    solver_free(s);
  }
  return CG_OK;
}

extern "C" int cg_solver_set_medium_labels(cg_solver* s, const uint8_t* labels, int n_labels, const float* table) {
  CG_REQUIRE(s && labels && table, "null argument");
  invalidate_graphs(s);
  CG_REQUIRE(n_labels >= 1 && n_labels <= 256, "n_labels must be 1..256, got %d", n_labels);
  if (!s->labels && dev_alloc(&s->labels, (size_t)s->d.ncell) != CG_OK) return CG_ERR_OOM;
  if (!s->ltab && dev_alloc(&s->ltab, 256) != CG_OK) return CG_ERR_OOM;
  CG_CUDA_TRY(cudaMemcpyAsync(s->labels, labels, (size_t)s->d.ncell, cudaMemcpyDefault, s->stream));
  float4 tab[256];
  memset(tab, 0, sizeof(tab));
  for (int i = 0; i < n_labels; ++i) tab[i] = make_float4(table[4 * i], table[4 * i + 1], table[4 * i + 2], table[4 * i + 3]);
  CG_CUDA_TRY(cudaMemcpyAsync(s->ltab, tab, sizeof(tab), cudaMemcpyHostToDevice, s->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->has_medium = 1;
  return CG_OK;
}

extern "C" int cg_solver_set_medium_dense(cg_solver* s, const float* dt_over_rho, const float* rhoc2_dt,
                                          const float* absorb, const float* beta2_dt) {
  CG_REQUIRE(s && dt_over_rho && rhoc2_dt && absorb, "null argument");
  invalidate_graphs(s);
  CG_REQUIRE(!s->nonlinear || beta2_dt, "a nonlinear solver needs the 2 beta dt map");
  const size_t n = (size_t)s->d.ncell;
  if (!s->dtr && dev_alloc(&s->dtr, n) != CG_OK) return CG_ERR_OOM;
  if (!s->rc2 && dev_alloc(&s->rc2, n) != CG_OK) return CG_ERR_OOM;
  if (!s->ab && dev_alloc(&s->ab, n) != CG_OK) return CG_ERR_OOM;
  CG_CUDA_TRY(cudaMemcpyAsync(s->dtr, dt_over_rho, n * 4, cudaMemcpyDefault, s->stream));
  CG_CUDA_TRY(cudaMemcpyAsync(s->rc2, rhoc2_dt, n * 4, cudaMemcpyDefault, s->stream));
  CG_CUDA_TRY(cudaMemcpyAsync(s->ab, absorb, n * 4, cudaMemcpyDefault, s->stream));
  if (beta2_dt) {
    if (!s->b2 && dev_alloc(&s->b2, n) != CG_OK) return CG_ERR_OOM;
    CG_CUDA_TRY(cudaMemcpyAsync(s->b2, beta2_dt, n * 4, cudaMemcpyDefault, s->stream));
  }
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (s->labels) {
    cudaFree(s->labels);
    s->labels = nullptr;
  }
  s->has_medium = 1;
  return CG_OK;
}

extern "C" int cg_solver_set_source(cg_solver* s, int n_src, const int32_t* xyz, const float* amp_cos,
                                    const float* amp_sin) {
  CG_REQUIRE(s, "null solver");
  invalidate_graphs(s);
  CG_REQUIRE(n_src >= 0, "n_src must be >= 0");
  const int nx = s->d.nx, ny = s->d.ny, nz = s->d.nz;
  const long long nrows = (long long)nx * ny;
  // sort entries by row (x, y), stable; keep z and the per-member amplitudes
  int* order = (int*)malloc(sizeof(int) * (n_src > 0 ? n_src : 1));
  int* count = (int*)calloc((size_t)nrows + 1, sizeof(int));
  int* zs = (int*)malloc(sizeof(int) * (n_src > 0 ? n_src : 1));
  float* ac = (float*)malloc(sizeof(float) * (size_t)s->B * (n_src > 0 ? n_src : 1));
  float* as = (float*)malloc(sizeof(float) * (size_t)s->B * (n_src > 0 ? n_src : 1));
  if (!order || !count || !zs || !ac || !as) {
    free(order); free(count); free(zs); free(ac); free(as);
    cg_set_error("host allocation failed");
    return CG_ERR_OOM;
  }
  for (int i = 0; i < n_src; ++i) {
    int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) {
      free(order); free(count); free(zs); free(ac); free(as);
      cg_set_error("source voxel %d (%d, %d, %d) is outside the %dx%dx%d grid", i, x, y, z, nx, ny, nz);
      return CG_ERR_INVALID;
    }
    count[(long long)x * ny + y + 1]++;
  }
  for (long long r = 0; r < nrows; ++r) count[r + 1] += count[r];
  int* fill = (int*)malloc(sizeof(int) * (size_t)nrows);
  memcpy(fill, count, sizeof(int) * (size_t)nrows);
  for (int i = 0; i < n_src; ++i) {
    long long r = (long long)xyz[3 * i] * ny + xyz[3 * i + 1];
    order[fill[r]++] = i;
  }
  free(fill);
  for (int e = 0; e < n_src; ++e) {
    int i = order[e];
    zs[e] = xyz[3 * i + 2];
    for (int b = 0; b < s->B; ++b) {
      ac[(size_t)b * n_src + e] = amp_cos[(size_t)b * n_src + i];
      as[(size_t)b * n_src + e] = amp_sin[(size_t)b * n_src + i];
    }
  }
  // duplicates would race in the scatter (the reference refuses them too, sources.py:67-73)
  for (long long r = 0; r < nrows; ++r)
    for (int e = count[r] + 1; e < count[r + 1]; ++e)
      for (int f = count[r]; f < e; ++f)
        if (zs[e] == zs[f]) {
          free(order); free(count); free(zs); free(ac); free(as);
          cg_set_error("source contains duplicate voxel indices");
          return CG_ERR_INVALID;
        }
  int rc = CG_OK;
  if (s->src_z) { cudaFree(s->src_z); s->src_z = nullptr; }
  if (s->src_ac) { cudaFree(s->src_ac); s->src_ac = nullptr; }
  if (s->src_as) { cudaFree(s->src_as); s->src_as = nullptr; }
  if ((rc = dev_alloc(&s->src_z, (size_t)n_src)) == CG_OK && (rc = dev_alloc(&s->src_ac, (size_t)s->B * n_src)) == CG_OK &&
      (rc = dev_alloc(&s->src_as, (size_t)s->B * n_src)) == CG_OK) {
    cudaError_t e = cudaMemcpyAsync(s->src_ptr, count, sizeof(int) * ((size_t)nrows + 1), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess && n_src > 0) {
      e = cudaMemcpyAsync(s->src_z, zs, sizeof(int) * n_src, cudaMemcpyHostToDevice, s->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(s->src_ac, ac, sizeof(float) * s->B * n_src, cudaMemcpyHostToDevice, s->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(s->src_as, as, sizeof(float) * s->B * n_src, cudaMemcpyHostToDevice, s->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
      cg_set_error("set_source: %s", cudaGetErrorString(e));
      rc = CG_ERR_CUDA;
    }
  }
  free(order); free(count); free(zs); free(ac); free(as);
  if (rc == CG_OK) s->n_src = n_src;
  return rc;
}

extern "C" int cg_solver_set_drive(cg_solver* s, int n_steps, const float* drive) {
  CG_REQUIRE(s && drive, "null argument");
  invalidate_graphs(s);
  CG_REQUIRE(n_steps >= 1, "n_steps must be >= 1");
  if (s->drive) { cudaFree(s->drive); s->drive = nullptr; }
  int rc = dev_alloc(&s->drive, (size_t)n_steps);
  if (rc != CG_OK) return rc;
  CG_CUDA_TRY(cudaMemcpyAsync(s->drive, drive, sizeof(float4) * (size_t)n_steps, cudaMemcpyDefault, s->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->n_drive = n_steps;
  return CG_OK;
}

extern "C" int cg_solver_reset(cg_solver* s) {
  CG_REQUIRE(s, "null solver");
  const long long B = s->B;
  cudaStream_t st = s->stream;
  CG_CUDA_TRY(cudaMemsetAsync(s->p, 0, sizeof(float) * B * s->d.ncell, st));
  CG_CUDA_TRY(cudaMemsetAsync(s->u, 0, sizeof(float) * 3 * B * s->d.ncell, st));
  CG_CUDA_TRY(cudaMemsetAsync(s->S0, 0, sizeof(float2) * B * s->d.nspec, st));
  CG_CUDA_TRY(cudaMemsetAsync(s->peaks, 0, sizeof(unsigned int) * B * s->max_periods, st));
  CG_CUDA_TRY(cudaMemsetAsync(s->ctl, 0, sizeof(long long) * 2, st));
  CG_CUDA_TRY(cudaStreamSynchronize(st));
  s->ph_valid = 0;
  return CG_OK;
}

// Per-launch event log of one step: an event before each launch and one
// after the last, each launch tagged with its slot of the step (0 y fwd,
// 1 x grad, 2 y inv grad, 3 z u, 4 y fwd div, 5 x div, 6 y inv, 7 z p).
struct EvLog {
  static constexpr int kMax = 2 + 6 * CG_MAX_SLABS + 1;
  cudaEvent_t ev[kMax];
  int slot[kMax];
  int n = 0;
  void mark(int sl, cudaStream_t st) {
    slot[n] = sl;
    cudaEventRecord(ev[n++], st);
  }
};

// The x-planes [x0, x0 + n) of the solver's grid as a grid of their own for
// the plane-local (y and z) passes: offset field, spectrum, medium, source
// and sponge pointers, record and convergence boxes shifted by x0. Member
// strides (ncell, nspec) stay those of the whole grid.
struct Slab {
  Dims d;
  Tables t;
  MediumDev m;
  SourceDev src;
  RecordDev rec;
  float *p, *u;
  float2 *S0, *S1, *S2;
};

static Slab make_slab(const cg_solver* s, int x0, int n) {
  Slab sl;
  const long long cell0 = (long long)x0 * s->d.ny * s->d.nz;
  const long long spec0 = (long long)x0 * s->d.nzh * s->d.ny;
  sl.d = s->d;
  sl.d.nx = n;
  sl.t = make_tables(s);
  sl.t.sx = s->sx + x0;
  sl.m = make_medium(s);
  if (sl.m.labels) sl.m.labels += cell0;
  if (sl.m.dtr) {
    sl.m.dtr += cell0;
    sl.m.rc2 += cell0;
    sl.m.ab += cell0;
    if (sl.m.b2) sl.m.b2 += cell0;
  }
  sl.src = make_source(s);
  if (sl.src.row_ptr) sl.src.row_ptr += (long long)x0 * s->d.ny;
  sl.rec = make_record(s);
  sl.rec.lo[0] -= x0;
  sl.rec.hi[0] -= x0;
  sl.rec.clo[0] -= x0;
  sl.rec.chi[0] -= x0;
  sl.p = s->p + cell0;
  sl.u = s->u + cell0;
  sl.S0 = s->S0 + spec0;
  sl.S1 = s->S1 + spec0;
  sl.S2 = s->S2 + spec0;
  return sl;
}

// Slab mode needs the size-specialised y-pass and the persistent z-passes.
static bool slabs_supported(const Dims& d) {
  return d.nx >= 2 && d.ny % 2 == 0 && fast_xy_has(d.ny) && fast_xy_has(d.nx) && fast_xy_has(d.nz);
}

// One step in slab mode: x grad, then per slab [y inv grad, z u, y fwd div],
// x div, then per slab [y inv, z p, y fwd]. The pressure spectrum leaves the
// step y- and z-transformed, which is what the next step's x grad reads.
static int launch_step_slabs(cg_solver* s, int n_local, int record, EvLog* log) {
  const Dims d = s->d;
  const Tables t = make_tables(s);
  const int B = s->B;
  const int K = s->slabs;
  cudaStream_t st = s->stream;
  bool ok = true;
  auto mark = [&](int sl) {
    if (log) log->mark(sl, st);
  };
  auto x0_of = [&](int k) { return (int)((long long)d.nx * k / K); };
  mark(1);
  ok = ok && fast_xpass(X_GRAD, d, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2, B, st);
  for (int k = 0; k < K && ok; ++k) {
    const int x0 = x0_of(k), n = x0_of(k + 1) - x0;
    const Slab sl = make_slab(s, x0, n);
    mark(2);
    ok = ok && fast_ypass(Y_INV_GRAD, sl.d, sl.t, sl.S0, sl.S1, sl.S2, B, st);
    mark(3);
    ok = ok && fast_zpass_u(sl.d, sl.t, sl.m, sl.u, sl.S0, sl.S1, sl.S2, B, st, true);
    mark(4);
    ok = ok && fast_ypass(Y_FWD_DIV, sl.d, sl.t, sl.S0, sl.S1, sl.S2, B, st);
  }
  mark(5);
  ok = ok && fast_xpass(X_DIV, d, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2, B, st);
  for (int k = 0; k < K && ok; ++k) {
    const int x0 = x0_of(k), n = x0_of(k + 1) - x0;
    const Slab sl = make_slab(s, x0, n);
    mark(6);
    ok = ok && fast_ypass(Y_INV, sl.d, sl.t, sl.S0, sl.S1, sl.S2, B, st);
    mark(7);
    ok = ok && fast_zpass_p(1, sl.d, sl.t, sl.m, sl.src, sl.rec, s->ctl, n_local, record, sl.p, sl.S0, B, st, true);
    mark(0);
    ok = ok && fast_ypass(Y_FWD, sl.d, sl.t, sl.S0, sl.S1, sl.S2, B, st);
  }
  if (log) cudaEventRecord(log->ev[log->n], st);
  if (!ok) {
    cg_set_error("slab step: a size-specialised pass is missing for grid %dx%dx%d", d.nx, d.ny, d.nz);
    return CG_ERR_INVALID;
  }
  return CG_OK;
}

// One step = 8 launches (or 2 + 6 per slab in slab mode). With `log` an
// event is recorded before each launch and after the last, for per-kernel
// timing.
static int launch_step(cg_solver* s, int n_local, int record, EvLog* log = nullptr) {
  if (s->slabs > 1) return launch_step_slabs(s, n_local, record, log);
  const Dims d = s->d;
  const Tables t = make_tables(s);
  const MediumDev m = make_medium(s);
  const int B = s->B;
  cudaStream_t st = s->stream;
  const dim3 gy((unsigned)((d.nx * (long long)d.nzh + CG_TILE - 1) / CG_TILE), B);
  const dim3 gx((unsigned)(((long long)d.nzh * d.ny + CG_TILE - 1) / CG_TILE), B);
  const dim3 gz((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), B);
  auto mark = [&](int sl) {
    if (log) log->mark(sl, st);
  };
  const bool fx = s->fused_xy != 0;
  if (fx) {
    mark(0);
    if (!fused_xy(true, d, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2, B, st)) {
      cg_set_error("fused transverse pass launch failed: %s", cudaGetErrorString(cudaGetLastError()));
      return CG_ERR_CUDA;
    }
  } else {
    mark(0);
    if (!fast_ypass(Y_FWD, d, t, s->S0, s->S1, s->S2, B, st))
      k_ypass<<<gy, CG_THREADS, s->smem_y, st>>>(Y_FWD, d, s->py, t, s->S0, s->S1, s->S2);
    mark(1);
    if (!fast_xpass(X_GRAD, d, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2, B, st))
      k_xpass<<<gx, CG_THREADS, s->smem_x, st>>>(X_GRAD, d, s->px, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2);
    mark(2);
    if (!fast_ypass(Y_INV_GRAD, d, t, s->S0, s->S1, s->S2, B, st))
      k_ypass<<<gy, CG_THREADS, s->smem_y, st>>>(Y_INV_GRAD, d, s->py, t, s->S0, s->S1, s->S2);
  }
  mark(3);
  const bool zt = s->ztma && s->zpers && s->ztma_ok;
  if (!(zt && fast_zpass_u_tma(d, t, m, s->u, s->S0, s->S1, s->S2, B, st, s->ztma_host)) &&
      !fast_zpass_u(d, t, m, s->u, s->S0, s->S1, s->S2, B, st, s->zpers != 0))
    k_zpass_u<<<gz, CG_THREADS, s->smem_z, st>>>(d, s->pz, t, m, s->u, s->S0, s->S1, s->S2);
  if (fx) {
    mark(4);
    if (!fused_xy(false, d, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2, B, st)) {
      cg_set_error("fused transverse pass launch failed: %s", cudaGetErrorString(cudaGetLastError()));
      return CG_ERR_CUDA;
    }
  } else {
    mark(4);
    if (!fast_ypass(Y_FWD_DIV, d, t, s->S0, s->S1, s->S2, B, st))
      k_ypass<<<gy, CG_THREADS, s->smem_y, st>>>(Y_FWD_DIV, d, s->py, t, s->S0, s->S1, s->S2);
    mark(5);
    if (!fast_xpass(X_DIV, d, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2, B, st))
      k_xpass<<<gx, CG_THREADS, s->smem_x, st>>>(X_DIV, d, s->px, t, (float)s->kcoef, s->invN, s->S0, s->S1, s->S2);
    mark(6);
    if (!fast_ypass(Y_INV, d, t, s->S0, s->S1, s->S2, B, st))
      k_ypass<<<gy, CG_THREADS, s->smem_y, st>>>(Y_INV, d, s->py, t, s->S0, s->S1, s->S2);
  }
  mark(7);
  if (!(zt && fast_zpass_p_tma(d, t, m, make_source(s), make_record(s), s->ctl, n_local, record, s->p, s->S0, B,
                               st, s->ztma_host)) &&
      !fast_zpass_p(1, d, t, m, make_source(s), make_record(s), s->ctl, n_local, record, s->p, s->S0, B, st,
                    s->zpers != 0))
    k_zpass_p<<<gz, CG_THREADS, s->smem_z, st>>>(1, d, s->pz, t, m, make_source(s), make_record(s), s->ctl, n_local,
                                                 record, s->p, s->S0);
  if (log) cudaEventRecord(log->ev[log->n], st);
  return CG_OK;
}

// The pressure spectrum a step starts from, from the pressure field: its
// z-transform (every mode), then its y-transform in slab mode.
static int spectrum_from_pressure(cg_solver* s) {
  const dim3 gz((unsigned)(s->d.nx * ((s->d.ny + CG_ZROWS - 1) / CG_ZROWS)), s->B);
  if (!fast_zpass_fwd_step(s->d, make_tables(s), make_medium(s), s->p, s->S0, s->B, s->stream, s->zpers != 0))
    k_zpass_p<<<gz, CG_THREADS, s->smem_z, s->stream>>>(0, s->d, s->pz, make_tables(s), make_medium(s),
                                                         make_source(s), make_record(s), s->ctl, 0, 0, s->p, s->S0);
  if (s->slabs > 1 && !fast_ypass(Y_FWD, s->d, make_tables(s), s->S0, s->S1, s->S2, s->B, s->stream)) {
    cg_set_error("slab mode without a size-specialised y-pass");
    return CG_ERR_INVALID;
  }
  CG_CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

extern "C" int cg_solver_run(cg_solver* s, int n_steps, int record) {
  CG_REQUIRE(s, "null solver");
  CG_REQUIRE(!record || s->bins, "recording needs cg_solver_begin_record first");
  CG_REQUIRE(s->has_medium, "set a medium before running");
  CG_REQUIRE(n_steps >= 0, "n_steps must be >= 0");
  for (int i = 0; i < n_steps; ++i) launch_step(s, i, record);
  k_advance<<<1, 1, 0, s->stream>>>(s->ctl, n_steps);
  CG_CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

extern "C" int cg_solver_run_periods(cg_solver* s, int n_periods, int record) {
  CG_REQUIRE(s, "null solver");
  CG_REQUIRE(!record || s->bins, "recording needs cg_solver_begin_record first");
  CG_REQUIRE(s->has_medium, "set a medium before running");
  CG_REQUIRE(n_periods >= 0, "n_periods must be >= 0");
  const int gi = record ? 1 : 0;
  if (!s->graph[gi]) {
    cudaGraph_t g;
    CG_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < s->spp; ++i) launch_step(s, i, record);
    k_advance<<<1, 1, 0, s->stream>>>(s->ctl, s->spp);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (e != cudaSuccess) {
      cg_set_error("graph capture: %s", cudaGetErrorString(e));
      return CG_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&s->graph[gi], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      cg_set_error("graph instantiate: %s", cudaGetErrorString(e));
      s->graph[gi] = nullptr;
      return CG_ERR_CUDA;
    }
  }
  for (int i = 0; i < n_periods; ++i) CG_CUDA_TRY(cudaGraphLaunch(s->graph[gi], s->stream));
  return CG_OK;
}

extern "C" int cg_solver_begin_record(cg_solver* s) {
  CG_REQUIRE(s, "null solver");
  const size_t nb = (size_t)s->B * s->spp * s->nrec;
  // the phase-bin accumulators exist only from the first record window on
  if (!s->bins) {
    invalidate_graphs(s);
    int rc = dev_alloc(&s->bins, nb);
    if (rc == CG_OK) rc = dev_alloc(&s->comp, nb);
    if (rc != CG_OK) return rc;
  }
  CG_CUDA_TRY(cudaMemsetAsync(s->bins, 0, sizeof(float) * nb, s->stream));
  CG_CUDA_TRY(cudaMemsetAsync(s->comp, 0, sizeof(float) * nb, s->stream));
  CG_CUDA_TRY(cudaMemsetAsync(s->pmax, 0, sizeof(float) * (size_t)s->B * s->nrec, s->stream));
  s->ph_valid = 0;
  return CG_OK;
}

extern "C" int cg_solver_read_peaks(cg_solver* s, int first, int count, float* out) {
  CG_REQUIRE(s && out, "null argument");
  CG_REQUIRE(first >= 0 && count >= 0 && first + count <= s->max_periods, "period range out of bounds");
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (s->ztma) {
    const int rc = ztma_check(s);
    if (rc != CG_OK) return rc;
  }
  for (int b = 0; b < s->B; ++b)
    CG_CUDA_TRY(cudaMemcpy(out + (size_t)b * count, s->peaks + (size_t)b * s->max_periods + first,
                           sizeof(float) * count, cudaMemcpyDefault));
  return CG_OK;
}

extern "C" int cg_solver_finalize(cg_solver* s, int n_record_steps, float* phasors, float* pmax) {
  CG_REQUIRE(s, "null solver");
  CG_REQUIRE(s->bins, "no record window has run (call cg_solver_begin_record first)");
  CG_REQUIRE(n_record_steps >= 1, "n_record_steps must be >= 1");
  if (!s->ph) {
    int rc = dev_alloc(&s->ph, (size_t)s->B * s->nh * s->nrec);
    if (rc != CG_OK) return rc;
  }
  k_finalize<<<1024, 256, sizeof(double2) * (size_t)s->nh * s->spp, s->stream>>>(make_record(s), s->B, s->nh,
                                                                                  s->harm_dev, n_record_steps, s->ph);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && phasors)
    e = cudaMemcpyAsync(phasors, s->ph, sizeof(float2) * (size_t)s->B * s->nh * s->nrec, cudaMemcpyDefault,
                        s->stream);
  if (e == cudaSuccess && pmax)
    e = cudaMemcpyAsync(pmax, s->pmax, sizeof(float) * (size_t)s->B * s->nrec, cudaMemcpyDefault, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    cg_set_error("finalize: %s", cudaGetErrorString(e));
    return CG_ERR_CUDA;
  }
  s->ph_valid = 1;
  return s->ztma ? ztma_check(s) : CG_OK;
}

int cg_solver_post_scratch(cg_solver* s, size_t bytes) {
  if (s->post_bytes >= bytes) return CG_OK;
  if (s->post) cudaFree(s->post);
  s->post = nullptr;
  s->post_bytes = 0;
  int rc = dev_alloc((char**)&s->post, bytes);
  if (rc == CG_OK) s->post_bytes = bytes;
  return rc;
}

extern "C" int cg_solver_get_state(cg_solver* s, float* p, float* u) {
  CG_REQUIRE(s, "null solver");
  const size_t n = (size_t)s->B * s->d.ncell;
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (p) CG_CUDA_TRY(cudaMemcpy(p, s->p, sizeof(float) * n, cudaMemcpyDefault));
  if (u) CG_CUDA_TRY(cudaMemcpy(u, s->u, sizeof(float) * 3 * n, cudaMemcpyDefault));
  return CG_OK;
}

extern "C" int cg_solver_set_state(cg_solver* s, const float* p, const float* u, long long step) {
  CG_REQUIRE(s && p && u, "null argument");
  CG_REQUIRE(step >= 0, "step must be >= 0");
  const size_t n = (size_t)s->B * s->d.ncell;
  CG_CUDA_TRY(cudaMemcpyAsync(s->p, p, sizeof(float) * n, cudaMemcpyDefault, s->stream));
  CG_CUDA_TRY(cudaMemcpyAsync(s->u, u, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
  k_set_ctl<<<1, 1, 0, s->stream>>>(s->ctl, step);
  const int rc = spectrum_from_pressure(s);
  if (rc != CG_OK) return rc;
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return CG_OK;
}

extern "C" int cg_solver_synchronize(cg_solver* s) {
  CG_REQUIRE(s, "null solver");
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  CG_CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

extern "C" int cg_solver_query(cg_solver* s, int* idle) {
  CG_REQUIRE(s && idle, "null argument");
  cudaError_t e = cudaStreamQuery(s->stream);
  if (e == cudaErrorNotReady) {
    *idle = 0;
    return CG_OK;
  }
  CG_CUDA_TRY(e);
  *idle = 1;
  return CG_OK;
}

extern "C" int cg_solver_info(const cg_solver* s, long long* out /* 8 */) {
  CG_REQUIRE(s && out, "null argument");
  out[0] = s->d.ncell;
  out[1] = s->d.nspec;
  out[2] = s->nrec;
  out[3] = (long long)s->smem_y;
  out[4] = (long long)s->smem_x;
  out[5] = (long long)s->smem_z;
  out[6] = s->B;
  out[7] = s->slabs > 1 ? 2 + 6 * s->slabs : (s->fused_xy ? 4 : 8);  // kernel launches per step
  return CG_OK;
}


// Device time of n_steps steps measured with CUDA events on the solver's
// stream (graph = 1: whole periods through the captured graph; n_steps must
// then be a multiple of spp).
extern "C" int cg_solver_timed_run(cg_solver* s, int n_steps, int record, int graph, float* ms) {
  CG_REQUIRE(s && ms, "null argument");
  CG_REQUIRE(!graph || n_steps % s->spp == 0, "graph timing needs whole periods (n_steps %% spp == 0)");
  cudaEvent_t a, b;
  CG_CUDA_TRY(cudaEventCreate(&a));
  CG_CUDA_TRY(cudaEventCreate(&b));
  CG_CUDA_TRY(cudaEventRecord(a, s->stream));
  int rc = graph ? cg_solver_run_periods(s, n_steps / s->spp, record) : cg_solver_run(s, n_steps, record);
  CG_CUDA_TRY(cudaEventRecord(b, s->stream));
  CG_CUDA_TRY(cudaEventSynchronize(b));
  CG_CUDA_TRY(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc == CG_OK && s->ztma) rc = ztma_check(s);
  return rc;
}

// ------------------------------------------------------------ autotuner --
// Per (grid, batch, physics, medium storage): time every launch configuration
// the grid admits -- fused or three-pass transverse chain, persistent or
// one-tile-per-CTA z-passes -- over a few steps of the handle itself, keep
// the fastest, and remember it for the process. The handle must be fresh
// (the trial steps run on its state, which is reset afterwards).
namespace {
struct TuneKey {
  int nx, ny, nz, B, nonlinear, labels;
  bool operator<(const TuneKey& o) const {
    const int a[6] = {nx, ny, nz, B, nonlinear, labels}, b[6] = {o.nx, o.ny, o.nz, o.B, o.nonlinear, o.labels};
    for (int i = 0; i < 6; ++i)
      if (a[i] != b[i]) return a[i] < b[i];
    return false;
  }
};
struct TuneChoice {
  int fused, zpers, slabs, ztma;
};
std::map<TuneKey, TuneChoice> g_tuned;
std::mutex g_tune_mu;
}  // namespace

// Slab counts the tuner tries: each slab's working set (three spectra,
// three velocity fields and the labels of its x-planes) between about 20 and
// 90 MB, so that it stays in L2 between the slab's three passes, capped at
// CG_MAX_SLABS and at one x-plane per slab.
static int slab_candidates(const cg_solver* s, int* out) {
  if (!slabs_supported(s->d)) return 0;
  const double plane = (double)s->B * ((double)s->d.nzh * s->d.ny * 8.0 * 3.0 + (double)s->d.ny * s->d.nz * 13.0);
  const double total = plane * s->d.nx;
  int n = 0;
  for (int k = 2; k <= CG_MAX_SLABS && k <= s->d.nx; ++k) {
    const double ws = total / k;
    if (ws <= 90e6 && ws >= 20e6) out[n++] = k;
  }
  return n;
}

extern "C" int cg_solver_autotune(cg_solver* s, int n_steps, int* out4) {
  CG_REQUIRE(s && out4, "null argument");
  CG_REQUIRE(s->has_medium, "set a medium before tuning");
  CG_REQUIRE(n_steps >= 1, "n_steps must be >= 1");
  const TuneKey key{s->d.nx, s->d.ny, s->d.nz, s->B, s->nonlinear, s->labels != nullptr};
  // CG_FUSED_XY=0 / =1 pin the transverse chain and CG_SLABS=k the slab
  // count (comparison runs): no cache then
  const char* fenv = getenv("CG_FUSED_XY");
  const char* senv = getenv("CG_SLABS");
  const bool slab_pinned = senv && senv[0] >= '0' && senv[0] <= '9';
  const bool pinned = (fenv && (fenv[0] == '0' || fenv[0] == '1')) || slab_pinned;
  if (!pinned) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    // a batch runs the same kernels with one grid dimension per member: it
    // takes the choice made for one member on this grid when there is one
    if (it == g_tuned.end() && key.B > 1) it = g_tuned.find(TuneKey{key.nx, key.ny, key.nz, 1, key.nonlinear,
                                                                    key.labels});
    if (it != g_tuned.end()) {
      invalidate_graphs(s);
      s->fused_xy = it->second.fused;
      s->zpers = it->second.zpers;
      s->slabs = it->second.slabs;
      s->ztma = (it->second.ztma && s->ztma_ok) ? 1 : 0;
      out4[0] = s->fused_xy;
      out4[1] = s->zpers;
      out4[2] = 0;
      out4[3] = 1;
      return cg_solver_reset(s);
    }
  }
  const bool fx_ok = !(fenv && fenv[0] == '0') && !slab_pinned && fused_xy_supported(s->d);
  const int fx_lo = (fx_ok && fenv && fenv[0] == '1') ? 1 : 0;
  // the per-tile z-passes exist for the lengths of CG_FAST_SIZES only
  const bool zp_choice = (s->d.ny % 2 == 0) && fast_has(s->d.nz) && !slab_pinned;
  invalidate_graphs(s);
  cudaEvent_t a, b;
  CG_CUDA_TRY(cudaEventCreate(&a));
  CG_CUDA_TRY(cudaEventCreate(&b));
  // Candidates are timed in interleaved rounds and each keeps its fastest
  // round, so work that other streams put on the GPU meanwhile (a serving
  // process tunes while other solves run) cannot hand the choice to a
  // slower configuration.
  constexpr int kRounds = 3;
  constexpr int kMaxCand = 8 + CG_MAX_SLABS;
  TuneChoice cand[kMaxCand];
  float cand_ms[kMaxCand];
  int nc = 0;
  // CG_ZTMA=0 / =1 keep the persistent z-tiles on cp.async / on tensor-map
  // staging (where the grid allows it); unset, both are timed
  const char* tenv_z = getenv("CG_ZTMA");
  const int zt_lo = (s->ztma_ok && tenv_z && tenv_z[0] == '1') ? 1 : 0;
  const int zt_hi = (s->ztma_ok && !(tenv_z && tenv_z[0] == '0')) ? 1 : 0;
  if (slab_pinned) {
    const int k = atoi(senv);
    cand[nc++] = {0, 1, (k > 1 && slabs_supported(s->d)) ? (k > CG_MAX_SLABS ? CG_MAX_SLABS : k) : 1, 0};
  } else {
    for (int fx = fx_lo; fx <= (fx_ok ? 1 : 0); ++fx)
      for (int zp = 1; zp >= (zp_choice ? 0 : 1); --zp)
        for (int zt = (zp ? zt_lo : 0); zt <= (zp ? zt_hi : 0); ++zt) cand[nc++] = {fx, zp, 1, zt};
    // slab counts join the candidates only on request (CG_TUNE_SLABS=1): on
    // GB300 they measured slower than the plain step on every grid tried
    const char* tenv = getenv("CG_TUNE_SLABS");
    if (!(fenv && fenv[0] == '1') && tenv && tenv[0] == '1') {
      int ks[CG_MAX_SLABS];
      const int nk = slab_candidates(s, ks);
      for (int i = 0; i < nk; ++i) cand[nc++] = {0, 1, ks[i], 0};
    }
  }
  for (int c = 0; c < nc; ++c) cand_ms[c] = 1e30f;
  for (int r = 0; r < kRounds; ++r)
    for (int c = 0; c < nc; ++c) {
      s->fused_xy = cand[c].fused;
      s->zpers = cand[c].zpers;
      s->slabs = cand[c].slabs;
      s->ztma = cand[c].ztma;
      int rc = CG_OK;
      for (int k = 0; k < (r == 0 ? 2 : 1) && rc == CG_OK; ++k) rc = launch_step(s, k % s->spp, 0);
      CG_CUDA_TRY(cudaEventRecord(a, s->stream));
      for (int k = 0; k < n_steps && rc == CG_OK; ++k) rc = launch_step(s, (k + 2) % s->spp, 0);
      CG_CUDA_TRY(cudaEventRecord(b, s->stream));
      CG_CUDA_TRY(cudaEventSynchronize(b));
      if (rc != CG_OK) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return rc;
      }
      float ms = 0.f;
      CG_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
      if (ms < cand_ms[c]) cand_ms[c] = ms;
    }
  float best_ms = 1e30f;
  TuneChoice best = cand[0];
  for (int c = 0; c < nc; ++c)
    if (cand_ms[c] < best_ms) {
      best_ms = cand_ms[c];
      best = cand[c];
    }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  s->fused_xy = best.fused;
  s->zpers = best.zpers;
  s->slabs = best.slabs;
  s->ztma = best.ztma;
  int rc = ztma_check(s);
  if (rc != CG_OK) return rc;
  rc = cg_solver_reset(s);
  if (rc != CG_OK) return rc;
  if (!pinned) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[key] = best;
  }
  out4[0] = best.fused;
  out4[1] = best.zpers;
  out4[2] = nc;
  out4[3] = 0;
  return CG_OK;
}

extern "C" int cg_solver_set_slabs(cg_solver* s, int slabs) {
  CG_REQUIRE(s, "null solver");
  CG_REQUIRE(slabs >= 1 && slabs <= CG_MAX_SLABS, "slabs must lie in [1, %d], got %d", CG_MAX_SLABS, slabs);
  CG_REQUIRE(slabs == 1 || slabs <= s->d.nx, "%d slabs on %d x-planes", slabs, s->d.nx);
  CG_REQUIRE(slabs == 1 || slabs_supported(s->d),
             "slab mode needs size-specialised passes on every axis and an even ny (grid %dx%dx%d)", s->d.nx,
             s->d.ny, s->d.nz);
  if (slabs == s->slabs) return CG_OK;
  invalidate_graphs(s);
  s->fused_xy = 0;
  s->zpers = 1;
  s->slabs = slabs;
  // the step-start spectrum of the new mode, from the current pressure
  const int rc = spectrum_from_pressure(s);
  if (rc != CG_OK) return rc;
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return CG_OK;
}

extern "C" int cg_solver_set_zstaging(cg_solver* s, int tma) {
  CG_REQUIRE(s, "null solver");
  CG_REQUIRE(tma == 0 || tma == 1, "tma must be 0 or 1, got %d", tma);
  CG_REQUIRE(!tma || s->ztma_ok,
             "tensor-map staging needs persistent z-passes with nz / 2 + 1 <= 256 and an even ny (grid %dx%dx%d)",
             s->d.nx, s->d.ny, s->d.nz);
  CG_REQUIRE(!tma || s->slabs == 1, "tensor-map staging runs the plain step only (slabs = %d)", s->slabs);
  if (tma == s->ztma && (!tma || s->zpers)) return CG_OK;
  invalidate_graphs(s);
  if (tma) s->zpers = 1;
  s->ztma = tma;
  return CG_OK;
}

extern "C" int cg_solver_get_zstaging(const cg_solver* s, int* tma) {
  CG_REQUIRE(s && tma, "null argument");
  *tma = (s->ztma && s->zpers && s->slabs == 1) ? 1 : 0;
  return CG_OK;
}

extern "C" int cg_solver_get_config(const cg_solver* s, int* out4) {
  CG_REQUIRE(s && out4, "null argument");
  out4[0] = s->fused_xy;
  out4[1] = s->zpers;
  out4[2] = s->slabs;
  out4[3] = s->slabs > 1 ? 2 + 6 * s->slabs : (s->fused_xy ? 4 : 8);
  return CG_OK;
}

// Per-kernel device time summed over n_steps steps (ms8[i] = launch i of
// the step, in step order), events recorded between launches.
extern "C" int cg_solver_profile(cg_solver* s, int n_steps, int record, float* ms8) {
  CG_REQUIRE(s && ms8, "null argument");
  CG_REQUIRE(!record || s->bins, "recording needs cg_solver_begin_record first");
  EvLog log;
  for (int i = 0; i < EvLog::kMax; ++i) CG_CUDA_TRY(cudaEventCreate(&log.ev[i]));
  for (int i = 0; i < 8; ++i) ms8[i] = 0.f;
  int rc = CG_OK;
  for (int k = 0; k < n_steps && rc == CG_OK; ++k) {
    log.n = 0;
    rc = launch_step(s, k % s->spp, record, &log);
    if (rc != CG_OK) break;
    CG_CUDA_TRY(cudaEventSynchronize(log.ev[log.n]));
    for (int i = 0; i < log.n; ++i) {
      float t = 0.f;
      CG_CUDA_TRY(cudaEventElapsedTime(&t, log.ev[i], log.ev[i + 1]));
      ms8[log.slot[i]] += t;
    }
  }
  k_advance<<<1, 1, 0, s->stream>>>(s->ctl, n_steps);
  for (int i = 0; i < EvLog::kMax; ++i) cudaEventDestroy(log.ev[i]);
  CG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return rc;
}

// ------------------------------------------------ standalone 3-D FFT ----
// The solver's own axis passes as a batched 3-D R2C/C2R transform.
// Forward: real [b][x][y][z] -> spectrum [b][x][kz][y] (kz < nz/2+1);
// inverse: the reverse, unnormalised (a round trip multiplies by nx*ny*nz).
struct cg_fft3d {
  Dims d;
  int B;
  AxisPlan px, py, pz;
  float2 *twx = nullptr, *twy = nullptr, *twz = nullptr;
  float* zeros = nullptr;  // k tables / sponge stand-ins, never read by the plain passes
  float* real = nullptr;   // staging for host inputs
  float2* spec = nullptr;
  cudaStream_t stream = nullptr;
  size_t smem_y, smem_x, smem_z;
};

static void fft_free(cg_fft3d* f) {
  if (!f) return;
  void* ptrs[] = {f->twx, f->twy, f->twz, f->zeros, f->real, f->spec};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (f->stream) cudaStreamDestroy(f->stream);
  delete f;
}

extern "C" int cg_fft3d_create(int nx, int ny, int nz, int batch, cg_fft3d** out) {
  CG_REQUIRE(out, "null argument");
  *out = nullptr;
  CG_REQUIRE(nx >= 1 && ny >= 1 && nz >= 2 && batch >= 1 && batch <= 65535, "invalid FFT shape %dx%dx%d batch %d",
             nx, ny, nz, batch);
  cg_fft3d* f = new cg_fft3d();
  f->d.nx = nx; f->d.ny = ny; f->d.nz = nz; f->d.nzh = nz / 2 + 1;
  f->d.ncell = (long long)nx * ny * nz;
  f->d.nspec = (long long)nx * f->d.nzh * ny;
  f->B = batch;
  if (cg_make_plan(nx, &f->px) || cg_make_plan(ny, &f->py) || cg_make_plan(nz, &f->pz)) {
    cg_set_error("FFT shape %dx%dx%d: every axis must be 2/3/5-smooth and <= %d", nx, ny, nz, CG_MAX_N);
    delete f;
    return CG_ERR_INVALID;
  }
  f->smem_y = smem_ypass(ny);
  f->smem_x = smem_xpass(nx);
  f->smem_z = smem_zpass(nz);
  const size_t smem_max = smem_limit();
  if ((!fast_xy_has(ny) && f->smem_y > smem_max) || (!fast_xy_has(nx) && f->smem_x > smem_max) ||
      f->smem_z > smem_max) {
    cg_set_error("FFT shape %dx%dx%d needs more than 227 KB of shared memory per tile", nx, ny, nz);
    delete f;
    return CG_ERR_INVALID;
  }
  int rc;
  int mx = nx > ny ? nx : ny;
  mx = mx > nz ? mx : nz;
  if ((rc = dev_alloc(&f->twx, nx)) || (rc = dev_alloc(&f->twy, ny)) || (rc = dev_alloc(&f->twz, nz)) ||
      (rc = dev_alloc(&f->zeros, (size_t)mx + 1)) || (rc = dev_alloc(&f->real, (size_t)batch * f->d.ncell)) ||
      (rc = dev_alloc(&f->spec, (size_t)batch * f->d.nspec))) {
    fft_free(f);
    return rc;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    k_twiddles<<<(nx + 255) / 256, 256, 0, f->stream>>>(f->twx, nx);
    k_twiddles<<<(ny + 255) / 256, 256, 0, f->stream>>>(f->twy, ny);
    k_twiddles<<<(nz + 255) / 256, 256, 0, f->stream>>>(f->twz, nz);
    e = cudaMemsetAsync(f->zeros, 0, sizeof(float) * ((size_t)mx + 1), f->stream);
  }
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_ypass);
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_xpass);
  if (e == cudaSuccess) e = allow_max_smem((const void*)k_zpass_p);
  if (e == cudaSuccess && fast_prepare() != 0) e = cudaErrorInvalidValue;
  if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
  if (e != cudaSuccess) {
    cg_set_error("fft set-up: %s", cudaGetErrorString(e));
    fft_free(f);
    return CG_ERR_CUDA;
  }
  *out = f;
  return CG_OK;
}

extern "C" int cg_fft3d_destroy(cg_fft3d* f) {
  if (f) {
    cudaStreamSynchronize(f->stream);
    fft_free(f);
  }
  return CG_OK;
}

static Tables fft_tables(const cg_fft3d* f) {
  Tables t;
  t.twx = f->twx; t.twy = f->twy; t.twz = f->twz;
  t.kx = t.ky = t.kz = t.kx2 = t.ky2 = t.kz2 = t.sx = t.sy = t.sz = f->zeros;
  return t;
}

extern "C" int cg_fft3d_forward(cg_fft3d* f, const float* in, float* out_spec) {
  CG_REQUIRE(f && in && out_spec, "null argument");
  const Dims d = f->d;
  const Tables t = fft_tables(f);
  MediumDev m;
  memset(&m, 0, sizeof(m));
  SourceDev sd;
  memset(&sd, 0, sizeof(sd));
  RecordDev rd;
  memset(&rd, 0, sizeof(rd));
  rd.spp = 1;
  CG_CUDA_TRY(cudaMemcpyAsync(f->real, in, sizeof(float) * f->B * d.ncell, cudaMemcpyDefault, f->stream));
  const dim3 gy((unsigned)((d.nx * (long long)d.nzh + CG_TILE - 1) / CG_TILE), f->B);
  const dim3 gx((unsigned)(((long long)d.nzh * d.ny + CG_TILE - 1) / CG_TILE), f->B);
  const dim3 gz((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), f->B);
  if (!fast_zpass_p(0, d, t, m, sd, rd, nullptr, 0, 0, f->real, f->spec, f->B, f->stream))
    k_zpass_p<<<gz, CG_THREADS, f->smem_z, f->stream>>>(0, d, f->pz, t, m, sd, rd, nullptr, 0, 0, f->real, f->spec);
  if (!fast_ypass(Y_FWD, d, t, f->spec, nullptr, nullptr, f->B, f->stream))
    k_ypass<<<gy, CG_THREADS, f->smem_y, f->stream>>>(Y_FWD, d, f->py, t, f->spec, nullptr, nullptr);
  if (!fast_xpass(X_FWD, d, t, 0.f, 1.f, f->spec, nullptr, nullptr, f->B, f->stream))
    k_xpass<<<gx, CG_THREADS, f->smem_x, f->stream>>>(X_FWD, d, f->px, t, 0.f, 1.f, f->spec, nullptr, nullptr);
  CG_CUDA_TRY(cudaGetLastError());
  CG_CUDA_TRY(cudaMemcpyAsync(out_spec, f->spec, sizeof(float2) * f->B * d.nspec, cudaMemcpyDefault, f->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(f->stream));
  return CG_OK;
}

extern "C" int cg_fft3d_inverse(cg_fft3d* f, const float* in_spec, float* out) {
  CG_REQUIRE(f && in_spec && out, "null argument");
  const Dims d = f->d;
  const Tables t = fft_tables(f);
  MediumDev m;
  memset(&m, 0, sizeof(m));
  SourceDev sd;
  memset(&sd, 0, sizeof(sd));
  RecordDev rd;
  memset(&rd, 0, sizeof(rd));
  rd.spp = 1;
  CG_CUDA_TRY(cudaMemcpyAsync(f->spec, in_spec, sizeof(float2) * f->B * d.nspec, cudaMemcpyDefault, f->stream));
  const dim3 gy((unsigned)((d.nx * (long long)d.nzh + CG_TILE - 1) / CG_TILE), f->B);
  const dim3 gx((unsigned)(((long long)d.nzh * d.ny + CG_TILE - 1) / CG_TILE), f->B);
  const dim3 gz((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), f->B);
  if (!fast_xpass(X_INV, d, t, 0.f, 1.f, f->spec, nullptr, nullptr, f->B, f->stream))
    k_xpass<<<gx, CG_THREADS, f->smem_x, f->stream>>>(X_INV, d, f->px, t, 0.f, 1.f, f->spec, nullptr, nullptr);
  if (!fast_ypass(Y_INV, d, t, f->spec, nullptr, nullptr, f->B, f->stream))
    k_ypass<<<gy, CG_THREADS, f->smem_y, f->stream>>>(Y_INV, d, f->py, t, f->spec, nullptr, nullptr);
  if (!fast_zpass_p(2, d, t, m, sd, rd, nullptr, 0, 0, f->real, f->spec, f->B, f->stream))
    k_zpass_p<<<gz, CG_THREADS, f->smem_z, f->stream>>>(2, d, f->pz, t, m, sd, rd, nullptr, 0, 0, f->real, f->spec);
  CG_CUDA_TRY(cudaGetLastError());
  CG_CUDA_TRY(cudaMemcpyAsync(out, f->real, sizeof(float) * f->B * d.ncell, cudaMemcpyDefault, f->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(f->stream));
  return CG_OK;
}

// ------------------------------------- 3-D forward FFT without allocation --
// For callers that may not allocate device memory themselves: code that runs
// inside another framework's memory pool (every byte accounted for by that
// pool), serving loops that must not pay cudaMalloc's implicit device-wide
// synchronisation, and plug-ins whose host application owns the CUDA heap.
// The transform's only scratch -- the three per-axis twiddle tables -- lives
// in this fixed array, reserved on every device that loads the library until
// the process exits. Inputs and outputs are the caller's device buffers.
#define CG_NOALLOC_AXIS_MAX CG_MAX_N  // longest axis the array can hold tables for
static __device__ __align__(256) float2 g_noalloc_twiddles[3 * CG_NOALLOC_AXIS_MAX];

#include <mutex>

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[128];  // per-device address of g_noalloc_twiddles

// Once per device, with that device current: resolve the array's device
// address (the host-side symbol is only a stand-in) and lift the kernels'
// dynamic shared-memory limit. Neither allocates. Both results are kept for
// the life of the process, so destroying a device's primary context while
// the library is loaded (cudaDeviceReset) is not supported: the next call
// would launch against the old context's address.
static int noalloc_setup(int dev, float2** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    CG_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_twiddles));
    CG_CUDA_TRY(allow_max_smem((const void*)k_ypass));
    CG_CUDA_TRY(allow_max_smem((const void*)k_xpass));
    CG_CUDA_TRY(allow_max_smem((const void*)k_zpass_p));
    g_noalloc_ptr[dev] = p;
  }
  *out = (float2*)g_noalloc_ptr[dev];
  return CG_OK;
}

extern "C" int cg_fft3d_forward_noalloc(int nx, int ny, int nz, int batch, const float* in_dev, float* out_dev,
                                        void* stream) {
  CG_REQUIRE(in_dev && out_dev, "null argument");
  CG_REQUIRE(batch >= 1 && batch <= 65535, "batch %d out of range", batch);
  CG_REQUIRE(nx >= 1 && ny >= 1 && nz >= 2, "invalid FFT shape %dx%dx%d", nx, ny, nz);
  CG_REQUIRE(nx <= CG_NOALLOC_AXIS_MAX && ny <= CG_NOALLOC_AXIS_MAX && nz <= CG_NOALLOC_AXIS_MAX,
             "FFT shape %dx%dx%d exceeds the fixed scratch of the no-allocation entry point (every axis <= %d)",
             nx, ny, nz, CG_NOALLOC_AXIS_MAX);
  Dims d;
  d.nx = nx; d.ny = ny; d.nz = nz; d.nzh = nz / 2 + 1;
  d.ncell = (long long)nx * ny * nz;
  d.nspec = (long long)nx * d.nzh * ny;
  AxisPlan px, py, pz;
  if (cg_make_plan(nx, &px) || cg_make_plan(ny, &py) || cg_make_plan(nz, &pz)) {
    cg_set_error("FFT shape %dx%dx%d: every axis must be 2/3/5-smooth", nx, ny, nz);
    return CG_ERR_INVALID;
  }
  // this entry point always launches the runtime-plan passes below, so all
  // three of their tiles must fit (on a 227 KB device: ny <= 540, nx <= 576,
  // nz <= 810), whether or not a size-specialised pass exists for an axis;
  // the check runs before anything is queued, so a refused call writes nothing
  const size_t sy = smem_ypass(ny), sx = smem_xpass(nx), sz = smem_zpass(nz), lim = smem_limit();
  CG_REQUIRE(sy <= lim && sx <= lim && sz <= lim,
             "FFT shape %dx%dx%d needs more shared memory per tile than the device offers "
             "(y tile %zu, x tile %zu, z tile %zu bytes; limit %zu)", nx, ny, nz, sy, sx, sz, lim);
  int dev = 0;
  CG_CUDA_TRY(cudaGetDevice(&dev));
  CG_REQUIRE(dev >= 0 && dev < 128, "device ordinal %d out of range", dev);
  float2* tw = nullptr;
  int rc = noalloc_setup(dev, &tw);
  if (rc != CG_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // the tables are rewritten by every call: nothing carries over between calls
  k_twiddles<<<(nx + 255) / 256, 256, 0, st>>>(tw, nx);
  k_twiddles<<<(ny + 255) / 256, 256, 0, st>>>(tw + CG_NOALLOC_AXIS_MAX, ny);
  k_twiddles<<<(nz + 255) / 256, 256, 0, st>>>(tw + 2 * CG_NOALLOC_AXIS_MAX, nz);
  Tables t;
  t.twx = tw;
  t.twy = tw + CG_NOALLOC_AXIS_MAX;
  t.twz = tw + 2 * CG_NOALLOC_AXIS_MAX;
  // k and sponge tables are never read by the plain transform passes
  t.kx = t.ky = t.kz = t.kx2 = t.ky2 = t.kz2 = t.sx = t.sy = t.sz = (const float*)tw;
  MediumDev m;
  memset(&m, 0, sizeof(m));
  SourceDev sd;
  memset(&sd, 0, sizeof(sd));
  RecordDev rd;
  memset(&rd, 0, sizeof(rd));
  rd.spp = 1;
  float2* spec = (float2*)out_dev;
  const dim3 gy((unsigned)((d.nx * (long long)d.nzh + CG_TILE - 1) / CG_TILE), batch);
  const dim3 gx((unsigned)(((long long)d.nzh * d.ny + CG_TILE - 1) / CG_TILE), batch);
  const dim3 gz((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), batch);
  k_zpass_p<<<gz, CG_THREADS, sz, st>>>(0, d, pz, t, m, sd, rd, nullptr, 0, 0, (float*)in_dev, spec);
  k_ypass<<<gy, CG_THREADS, sy, st>>>(Y_FWD, d, py, t, spec, nullptr, nullptr);
  k_xpass<<<gx, CG_THREADS, sx, st>>>(X_FWD, d, px, t, 0.f, 1.f, spec, nullptr, nullptr);
  CG_CUDA_TRY(cudaGetLastError());
  return CG_OK;
}
