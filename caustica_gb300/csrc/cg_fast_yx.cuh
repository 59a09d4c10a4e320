// Size-specialised y- and x-passes (axis length N known at compile time):
// kernels and per-length launchers. The launchers are instantiated by the
// cg_fast_yx_*.cu units (a few lengths each, so they compile in parallel)
// and dispatched by cg_fast_yx.cu.
//
// y-pass: rows (x, kz) of length ny, YP rows per CTA; thread (p, s) =
// (threadIdx / TPP, threadIdx % TPP) owns row p (TPP = threads per pencil:
// 16, or 20 / 32 for the 320/400 and 512/640 splits). x-pass: CG_XP
// consecutive (kz, y) columns per CTA; thread (c, s) = (threadIdx % CG_XP,
// threadIdx / CG_XP) owns column c. Pencil data moves global -> registers -> one exchange per
// transform -> registers -> global (cg_fast.cuh).
#pragma once

#include "cg_fast.cuh"
#include "cg_kspace.cuh"

// resident CTAs per SM the register allocation targets (y: 4-row CTAs,
// ~102 registers per thread, no spills; x: 16-column CTAs, ~85 registers;
// both measured best on a 192^2 x 256 grid)
#ifndef CG_FAST_MINB_Y
#define CG_FAST_MINB_Y 10
#endif
#ifndef CG_FAST_MINB_X
#define CG_FAST_MINB_X 3
#endif
// the same for the x-pass modes other than X_DIV (the divergence pass parks
// a spectrum tile and needs the larger register budget)
#ifndef CG_FAST_MINB_XG
#define CG_FAST_MINB_XG CG_FAST_MINB_X
#endif
// and for those modes on the 320-point x axis (20-thread pencils: two CTAs
// per SM measured 1408 -> 1365 us per 320^3 step; the 400-point axis keeps
// one, two measured 2464 -> 2675 us per 400^3 step)
#ifndef CG_FAST_MINB_X20
#define CG_FAST_MINB_X20 2
#endif
// rows per y-CTA and columns per x-CTA (16 threads each)
#ifndef CG_YP20
#define CG_YP20 4  // rows per y-CTA on 20-thread pencils
#endif
#ifndef CG_YP
#define CG_YP 4
#endif
#ifndef CG_XP
#define CG_XP 16
#endif

using cgf::ColEx;
using cgf::PSplit;
using cgf::RowEx;
using cgf::fft2;
using cgf::static_for;

// Threads and resident CTAs per SM of the y- and x-pass CTAs for length N
// (20-thread pencils get the register budget that avoids spills).
template <int N>
struct YT {
  static constexpr int TPP = PSplit<N>::TPP, YP = TPP == 20 ? CG_YP20 : CG_YP, THREADS = TPP * YP;
  static constexpr int MINB = TPP == 16 ? CG_FAST_MINB_Y : 4;
};
template <int N>
struct XT {
  static constexpr int TPP = PSplit<N>::TPP, THREADS = TPP * CG_XP;
  static constexpr int MINB = TPP == 16 ? CG_FAST_MINB_X : 1;
  // 320-point axis: CG_FAST_MINB_X20 CTAs per SM except for X_DIV (its
  // parked tile needs the registers of one)
  static constexpr int minb(int mode) {
    return TPP == 16 ? (mode != X_DIV ? CG_FAST_MINB_XG : MINB) : (N == 320 && mode != X_DIV ? CG_FAST_MINB_X20 : MINB);
  }
};

// One instantiation per mode keeps each kernel's code small enough for the
// instruction cache (the x-pass gradient loops over one copy of its inverse
// transform; the y-pass modes stay straight-line, where the compiler hoists
// the next input's loads above the current transform).
template <int N, int MODE>
__global__ void __launch_bounds__(YT<N>::THREADS, YT<N>::MINB) kf_ypass(Dims d, Tables t, float2* __restrict__ S0,
                                                                        float2* __restrict__ S1,
                                                                        float2* __restrict__ S2) {
  constexpr int A = PSplit<N>::A, B = PSplit<N>::B, TPP = PSplit<N>::TPP;
  using Ex = RowEx<A, B, (32 % TPP == 0)>;  // pencil-local exchange: warp barriers
  extern __shared__ float2 sm[];
  cgf::pdl_trigger();
  float2* tw = sm;  // (A, B) order
  cgf::fill_twt<A, B>(tw, t.twy);
  cgf::pdl_wait();
  const int s = threadIdx.x % TPP, p = threadIdx.x / TPP;
  const Ex ex{sm + N + p * Ex::SLAB};
  const long long nrows = (long long)d.nx * d.nzh;
  const long long row = (long long)blockIdx.x * YT<N>::YP + p;
  const bool valid = row < nrows;
  const long long off = (long long)blockIdx.y * d.nspec + row * N;
  __syncthreads();
  float2 v[A], w[B];
  auto load = [&](const float2* __restrict__ src) {
    static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      v[a] = (valid && s < B) ? src[off + s + B * a] : make_float2(0.f, 0.f);
    });
  };
  auto store = [&](float2* __restrict__ dst) {
    if (valid && s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      dst[off + s + A * b] = w[b];
    });
  };
  if constexpr (MODE == Y_FWD || MODE == Y_INV) {
    load(S0);
    fft2<A, B, MODE == Y_INV>(v, w, s, tw, ex);
    store(S0);
  } else if constexpr (MODE == Y_INV_GRAD) {
    // S1 <- IFFT(S1); S0 <- IFFT(i ky S2); S2 <- IFFT(S2)
    load(S1);
    fft2<A, B, true>(v, w, s, tw, ex);
    store(S1);
    load(S2);
    float2 g[A];
    static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      const float k = (s < B) ? t.ky[s + B * a] : 0.f;
      g[a] = c_muli(c_scale(v[a], k));
    });
    fft2<A, B, true>(g, w, s, tw, ex);
    store(S0);
    fft2<A, B, true>(v, w, s, tw, ex);
    store(S2);
  } else {
    // Y_FWD_DIV: S1 <- FFT(S1); S0 <- i ky FFT(S0) + FFT(S2)
    load(S1);
    fft2<A, B, false>(v, w, s, tw, ex);
    store(S1);
    load(S0);
    fft2<A, B, false>(v, w, s, tw, ex);
    float2 h[B];
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const float k = (s < A) ? t.ky[s + A * b] : 0.f;
      h[b] = c_muli(c_scale(w[b], k));
    });
    load(S2);
    fft2<A, B, false>(v, w, s, tw, ex);
    static_for<0, B>([&](auto bi) { w[decltype(bi)::value] = c_add(w[decltype(bi)::value], h[decltype(bi)::value]); });
    store(S0);
  }
}

template <int N, int MODE>
__global__ void __launch_bounds__(XT<N>::THREADS, XT<N>::minb(MODE)) kf_xpass(Dims d, Tables t, float kcoef, float invN,
                                                                        float2* __restrict__ S0,
                                                                        float2* __restrict__ S1,
                                                                        float2* __restrict__ S2) {
  constexpr int A = PSplit<N>::A, B = PSplit<N>::B;
  extern __shared__ float2 sm[];
  cgf::pdl_trigger();
  float2* tw = sm;       // (A, B) order
  float2* twi = sm + N;  // (B, A) order
  cgf::fill_twt<A, B>(tw, t.twx);
  cgf::fill_twt<B, A>(twi, t.twx);
  float* kxs = reinterpret_cast<float*>(sm + 2 * N + 2 * N * CG_XP);  // k_x | k_x^2
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    kxs[i] = t.kx[i];
    kxs[N + i] = t.kx2[i];
  }
  cgf::pdl_wait();
  const int c = threadIdx.x % CG_XP, s = threadIdx.x / CG_XP;
  const ColEx<A, B, CG_XP> exf{sm + 2 * N + c};
  const ColEx<B, A, CG_XP> exi{sm + 2 * N + c};
  const long long ncol = (long long)d.nzh * d.ny;
  const long long col = (long long)blockIdx.x * CG_XP + c;
  const bool valid = col < ncol;
  const long long base = (long long)blockIdx.y * d.nspec + col;
  float kyz2 = 0.f;
  {
    const long long cc = valid ? col : ncol - 1;
    const int kz = (int)(cc / d.ny);
    const int ky = (int)(cc - (long long)kz * d.ny);
    kyz2 = t.ky2[ky] + t.kz2[kz];
  }
  __syncthreads();
  float2 v[A], w[B], z[A];
  auto load = [&](const float2* __restrict__ src) {
    static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      v[a] = (valid && s < B) ? src[base + (long long)(s + B * a) * ncol] : make_float2(0.f, 0.f);
    });
  };
  // after an inverse (B, A) transform thread s < B owns z[a] = element s + B a
  auto store_z = [&](float2* __restrict__ dst) {
    if (valid && s < B) static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      dst[base + (long long)(s + B * a) * ncol] = z[a];
    });
  };
  auto kappa = [&](int k) { return sinc_a2(kcoef * (kxs[N + k] + kyz2)) * invN; };
  if constexpr (MODE == X_FWD || MODE == X_INV) {
    load(S0);
    fft2<A, B, MODE == X_INV>(v, w, s, tw, exf);
    if (valid && s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      S0[base + (long long)(s + A * b) * ncol] = w[b];
    });
  } else if constexpr (MODE == X_GRAD) {
    // S2 <- IFFT(q); S1 <- IFFT(i kx q), q = kappa/N FFT(S0); q waits in shared
    // memory during the first inverse transform instead of in registers
    float2* qs = sm + 2 * N + N * CG_XP;
    load(S0);
    fft2<A, B, false>(v, w, s, tw, exf);
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int k = (s < A) ? s + A * b : 0;
      w[b] = c_scale(w[b], kappa(k));
      if (s < A) qs[(s + A * b) * CG_XP + c] = w[b];
    });
    fft2<B, A, true>(w, z, s, twi, exi);
    store_z(S2);
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int k = (s < A) ? s + A * b : 0;
      w[b] = (s < A) ? c_muli(c_scale(qs[(s + A * b) * CG_XP + c], kxs[k])) : make_float2(0.f, 0.f);
    });
    fft2<B, A, true>(w, z, s, twi, exi);
    store_z(S1);
  } else {
    // X_DIV: S0 <- IFFT(kappa/N (FFT(S0) + i kx FFT(S1))); FFT(S1) waits in shared memory
    float2* hs = sm + 2 * N + N * CG_XP;
    load(S1);
    fft2<A, B, false>(v, w, s, tw, exf);
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      hs[(s + A * b) * CG_XP + c] = w[b];
    });
    load(S0);
    fft2<A, B, false>(v, w, s, tw, exf);
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int k = (s < A) ? s + A * b : 0;
      const float2 h = (s < A) ? hs[(s + A * b) * CG_XP + c] : make_float2(0.f, 0.f);
      w[b] = c_scale(c_add(w[b], c_muli(c_scale(h, kxs[k]))), kappa(k));
    });
    fft2<B, A, true>(w, z, s, twi, exi);
    store_z(S0);
  }
}

// twiddles | exchange | (x: a parked spectrum tile, k_x, k_x^2)
template <int N>
static size_t smem_y() {
  return sizeof(float2) * (N + YT<N>::YP * RowEx<PSplit<N>::A, PSplit<N>::B>::SLAB);
}
template <int N>
static size_t smem_x() {
  return sizeof(float2) * (2 * N + 2 * (size_t)N * CG_XP) + 2 * sizeof(float) * N;  // + parked tile, k_x, k_x^2
}

// ------------------------------------------------ per-length launchers --
template <int N>
bool yx_launch_y(int mode, const Dims& d, const Tables& t, float2* S0, float2* S1, float2* S2, int batch,
                 cudaStream_t st) {
  const dim3 grid((unsigned)((d.nx * (long long)d.nzh + YT<N>::YP - 1) / YT<N>::YP), batch);
  const dim3 block(YT<N>::THREADS);
  switch (mode) {
    case Y_FWD: cgf::launch(kf_ypass<N, Y_FWD>, grid, block, smem_y<N>(), st, d, t, S0, S1, S2); break;
    case Y_INV: cgf::launch(kf_ypass<N, Y_INV>, grid, block, smem_y<N>(), st, d, t, S0, S1, S2); break;
    case Y_INV_GRAD: cgf::launch(kf_ypass<N, Y_INV_GRAD>, grid, block, smem_y<N>(), st, d, t, S0, S1, S2); break;
    default: cgf::launch(kf_ypass<N, Y_FWD_DIV>, grid, block, smem_y<N>(), st, d, t, S0, S1, S2); break;
  }
  return true;
}

template <int N>
bool yx_launch_x(int mode, const Dims& d, const Tables& t, float kcoef, float invN, float2* S0, float2* S1,
                 float2* S2, int batch, cudaStream_t st) {
  const dim3 grid((unsigned)(((long long)d.nzh * d.ny + CG_XP - 1) / CG_XP), batch);
  const dim3 block(XT<N>::THREADS);
  switch (mode) {
    case X_GRAD: cgf::launch(kf_xpass<N, X_GRAD>, grid, block, smem_x<N>(), st, d, t, kcoef, invN, S0, S1, S2); break;
    case X_DIV: cgf::launch(kf_xpass<N, X_DIV>, grid, block, smem_x<N>(), st, d, t, kcoef, invN, S0, S1, S2); break;
    case X_FWD: cgf::launch(kf_xpass<N, X_FWD>, grid, block, smem_x<N>(), st, d, t, kcoef, invN, S0, S1, S2); break;
    default: cgf::launch(kf_xpass<N, X_INV>, grid, block, smem_x<N>(), st, d, t, kcoef, invN, S0, S1, S2); break;
  }
  return true;
}

template <int N, int M>
static int allow_yx() {
  const int sy = (int)smem_y<N>(), sx = (int)smem_x<N>();
  if (cudaFuncSetAttribute(kf_ypass<N, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, sy) != cudaSuccess) return -1;
  if (cudaFuncSetAttribute(kf_xpass<N, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, sx) != cudaSuccess) return -1;
  return 0;
}

// Y_* and X_* modes are both 0..3
template <int N>
int yx_prepare() {
  return (allow_yx<N, 0>() || allow_yx<N, 1>() || allow_yx<N, 2>() || allow_yx<N, 3>()) ? -1 : 0;
}

#define CG_YX_INSTANTIATE(n)                                                                                   \
  template bool yx_launch_y<n>(int, const Dims&, const Tables&, float2*, float2*, float2*, int, cudaStream_t); \
  template bool yx_launch_x<n>(int, const Dims&, const Tables&, float, float, float2*, float2*, float2*, int,   \
                               cudaStream_t);                                                                  \
  template int yx_prepare<n>();
