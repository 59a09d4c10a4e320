// Size-specialised z-passes (nz = N known at compile time): kernels and
// per-length launchers. The launchers are instantiated by the cg_fast_z_*.cu
// units (a few lengths each, so they compile in parallel) and dispatched by
// cg_fast_z.cu.
//
// Tile = (batch member, x, 32 consecutive y). Real rows y0+2p and y0+2p+1
// form complex pencil p (p = threadIdx / TPP, TPP = threads per pencil: 16,
// or 20 / 32 for the 320/400 and 512/640 splits); s = threadIdx % TPP runs
// along the pencil. The inverse (complex-to-real) transform is an (A, B) fft2, the
// forward one a (B, A) fft2, so the values produced by the inverse arrive in
// exactly the registers the forward transform reads; the pointwise update
// runs in between, on cells (x, y, s + A b) with coalesced row accesses.
// Half spectra are staged through shared memory in both directions (the
// spectral layout has y fastest, the real layout z fastest).
#pragma once

#include <string.h>

#include "cg_fast.cuh"
#include "cg_kspace.cuh"

// resident CTAs per SM the register allocation targets
#ifndef CG_FAST_MINB_Z
#define CG_FAST_MINB_Z 2
#endif
#define CG_FAST_MINB CG_FAST_MINB_Z

using cgf::RowEx;
using cgf::Split;
using cgf::fft2;
using cgf::static_for;

template <int N>
using ZSplit = cgf::PSplit<N>;

template <int N>
struct ZShape {
  static constexpr int A = Split<N>::A, B = Split<N>::B, NH = N / 2 + 1;
  static constexpr int EX_I = RowEx<A, B>::SLAB, EX_F = RowEx<B, A>::SLAB;
  static constexpr int EX = EX_I > EX_F ? EX_I : EX_F;
  static constexpr int STG = (NH * 34 > N * 17) ? NH * 34 : N * 17;  // float2 units
  // twiddles (two orders) | staging (aliased by xb) | exchange | material table | labels
  static constexpr size_t OFF_STG = 2 * N, OFF_EX = OFF_STG + STG, OFF_TAB = OFF_EX + (size_t)CG_TILE * EX;
  static constexpr size_t smem = sizeof(float2) * OFF_TAB + 256 * sizeof(float4) + (size_t)CG_ZROWS * N;
};

// Stage the half spectra of the tile: stg4[k * 17 + p] = (A_k, B_k) of pencil p,
// times i*mk[k] when mk is given; Im of the self-paired bins dropped.
template <int N>
__device__ __forceinline__ void z_stage(float4* stg4, const float2* __restrict__ S, const Dims& d, int x, int y0,
                                        const float* mk) {
  constexpr int NH = N / 2 + 1;
  constexpr int ITER = (NH * CG_TILE + CG_THREADS - 1) / CG_THREADS;
  const float2* base = S + (long long)x * NH * d.ny + y0;
  const bool even_ny = (d.ny & 1) == 0;
  float4 f[ITER];
  // every load of the tile is issued before the first shared-memory store
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = threadIdx.x + it * CG_THREADS;
    const int k = idx >> 4, pp = idx & 15;
    const int ya = y0 + 2 * pp;
    const float2* q = base + (long long)k * d.ny + 2 * pp;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (idx < NH * CG_TILE) {
      if (even_ny && ya + 1 < d.ny) {
        r = __ldg(reinterpret_cast<const float4*>(q));
      } else {
        if (ya < d.ny) {
          const float2 a = q[0];
          r.x = a.x;
          r.y = a.y;
        }
        if (ya + 1 < d.ny) {
          const float2 b = q[1];
          r.z = b.x;
          r.w = b.y;
        }
      }
    }
    f[it] = r;
  }
#pragma unroll
  for (int it = 0; it < ITER; ++it) {
    const int idx = threadIdx.x + it * CG_THREADS;
    if (idx >= NH * CG_TILE) break;
    const int k = idx >> 4, pp = idx & 15;
    float2 a = make_float2(f[it].x, f[it].y), b = make_float2(f[it].z, f[it].w);
    if (mk) {
      const float kk = mk[k];
      a = c_muli(c_scale(a, kk));
      b = c_muli(c_scale(b, kk));
    }
    if (k == 0 || 2 * k == N) {
      a.y = 0.f;
      b.y = 0.f;
    }
    stg4[k * 17 + pp] = make_float4(a.x, a.y, b.x, b.y);
  }
}

// The tile's material labels (32 rows x N bytes) and the material table in
// shared memory; returns false when the medium is dense (no labels).
template <int N>
__device__ __forceinline__ bool z_stage_labels(uint8_t* lab_s, float4* tab_s, const MediumDev& m, const Dims& d,
                                               int x, int y0) {
  if (!m.labels) return false;
  const int nyv = min(CG_ZROWS, d.ny - y0);
  const uint8_t* src = m.labels + ((long long)x * d.ny + y0) * N;
  const int nbytes = nyv * N;
  if ((N % 16) == 0) {
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(lab_s);
    for (int i = threadIdx.x; i < nbytes / 16; i += blockDim.x) d4[i] = __ldg(s4 + i);
  } else {
    for (int i = threadIdx.x; i < nbytes; i += blockDim.x) lab_s[i] = src[i];
  }
  for (int i = threadIdx.x; i < 256; i += blockDim.x) tab_s[i] = m.ltab[i];
  return true;
}

// Phase-1 inputs of the inverse transform for thread (p, s): Z_n = A_n + i B_n
// with the Hermitian extension above N/2, n = s + B a.
template <int N>
__device__ __forceinline__ void z_inputs(float2 (&v)[Split<N>::A], const float4* stg4, int p, int s) {
  constexpr int A = Split<N>::A, B = Split<N>::B;
  static_for<0, A>([&](auto ai) {
    constexpr int a = decltype(ai)::value;
    const int n = s + B * a;
    float2 z = make_float2(0.f, 0.f);
    if (s < B) {
      const bool hi = 2 * n > N;
      const float4 f = stg4[(hi ? N - n : n) * 17 + p];
      z = hi ? make_float2(f.x + f.w, f.z - f.y)   // conj(A) + i conj(B)
             : make_float2(f.x - f.w, f.y + f.z);  // A + i B
    }
    v[a] = z;
  });
}

// After the forward transform thread (p, s < B) owns X[s + B a]; put them in
// xb[k * 17 + p], then split each pencil into its two half spectra and store
// them to S (x, k, y0 + 2p + {0, 1}), times i*mk[k] when given.
template <int N>
__device__ __forceinline__ void z_split_store(float2* xb, const float2 (&X)[ZSplit<N>::A], float2* __restrict__ S,
                                              const Dims& d, int x, int y0, int p, int s, const float* mk) {
  constexpr int A = ZSplit<N>::A, B = ZSplit<N>::B, NH = N / 2 + 1;
  // every pencil of the tile is done with the buffer (its exchange slab or
  // the staged spectrum) before any column lands in it
  __syncthreads();
  if (s < B) static_for<0, A>([&](auto ai) {
    constexpr int a = decltype(ai)::value;
    xb[(s + B * a) * 17 + p] = X[a];
  });
  __syncthreads();
  float2* base = S + (long long)x * NH * d.ny + y0;
  const bool even_ny = (d.ny & 1) == 0;
  for (int idx = threadIdx.x; idx < NH * CG_TILE; idx += blockDim.x) {
    const int k = idx >> 4, pp = idx & 15;
    const int ya = y0 + 2 * pp;
    if (ya >= d.ny) continue;
    const float2 zk = xb[k * 17 + pp];
    const float2 zm = c_conj(xb[((N - k) % N) * 17 + pp]);
    float2 a = c_scale(c_add(zk, zm), 0.5f);
    float2 b = c_scale(c_mulmi(c_sub(zk, zm)), 0.5f);
    if (mk) {
      a = c_muli(c_scale(a, mk[k]));
      b = c_muli(c_scale(b, mk[k]));
    }
    float2* q = base + (long long)k * d.ny + 2 * pp;
    if (even_ny && ya + 1 < d.ny) {
      *reinterpret_cast<float4*>(q) = make_float4(a.x, a.y, b.x, b.y);
    } else {
      q[0] = a;
      if (ya + 1 < d.ny) q[1] = b;
    }
  }
  __syncthreads();
}

template <int N>
__global__ void __launch_bounds__(CG_THREADS, CG_FAST_MINB) kf_zpass_u(Dims d, Tables t, MediumDev m, float* __restrict__ u,
                                                           float2* __restrict__ S0, float2* __restrict__ S1,
                                                           float2* __restrict__ S2) {
  using Z = ZShape<N>;
  constexpr int A = Z::A, B = Z::B;
  extern __shared__ float2 sm[];
  cgf::pdl_trigger();
  float2* tw = sm;        // (A, B) order: inverse transforms
  float2* twf = sm + N;   // (B, A) order: forward transforms
  float4* stg4 = reinterpret_cast<float4*>(sm + Z::OFF_STG);
  float2* xb = sm + Z::OFF_STG;
  cgf::fill_twt<A, B>(tw, t.twz);
  cgf::fill_twt<B, A>(twf, t.twz);
  cgf::pdl_wait();
  const int s = threadIdx.x & 15, p = threadIdx.x >> 4;
  const RowEx<A, B, true> exi{sm + Z::OFF_EX + p * Z::EX};  // 16 threads per pencil: warp-local
  const RowEx<B, A, true> exf{sm + Z::OFF_EX + p * Z::EX};
  const int ytiles = (d.ny + CG_ZROWS - 1) / CG_ZROWS;
  const int x = blockIdx.x / ytiles;
  const int y0 = (blockIdx.x - x * ytiles) * CG_ZROWS;
  const int ya = y0 + 2 * p, yb = ya + 1;
  const bool va = ya < d.ny, vb = yb < d.ny;
  const int b_idx = blockIdx.y;
  const long long off = (long long)b_idx * d.nspec;
  const float spx = t.sx[x];
  const float spa = va ? spx * t.sy[ya] : 0.f, spb = vb ? spx * t.sy[yb] : 0.f;
  const long long rowa = ((long long)x * d.ny + ya) * N, rowb = rowa + N;
  // shared tables: tw | stg (aliased by xb) | exchange | material table | labels
  float4* tab_s = reinterpret_cast<float4*>(sm + Z::OFF_TAB);
  uint8_t* lab_s = reinterpret_cast<uint8_t*>(tab_s + 256);
  const bool lab = z_stage_labels<N>(lab_s, tab_s, m, d, x, y0);
  const uint8_t* la = lab_s + (2 * p) * N;
  const uint8_t* lb = la + N;
#pragma unroll 1
  for (int comp = 0; comp < 3; ++comp) {
    float2* S = (comp == 0 ? S1 : (comp == 1 ? S0 : S2)) + off;
    const float* mk = (comp == 2) ? t.kz : nullptr;
    float* uc = u + ((long long)comp * gridDim.y + b_idx) * d.ncell;
    z_stage<N>(stg4, S, d, x, y0, mk);
    // the velocities of this thread's cells load while the inverse transform runs
    float ua[B], ub[B];
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      ua[b] = (s < A && va) ? __ldg(uc + rowa + n) : 0.f;
      ub[b] = (s < A && vb) ? __ldg(uc + rowb + n) : 0.f;
    });
    __syncthreads();
    float2 v[A], w[B];
    z_inputs<N>(v, stg4, p, s);
    fft2<A, B, true>(v, w, s, tw, exi);
    // u <- (u - dt/rho g) * absorb * sponge   (engine.py:462-464)
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      const float sz = t.sz[n];
      float2 r = make_float2(0.f, 0.f);
      if (va) {
        const float4 cf = lab ? tab_s[la[n]] : cell_coef(m, rowa + n);
        float un = ua[b] - cf.x * w[b].x;
        un = un * cf.z;
        un = un * (spa * sz);
        uc[rowa + n] = un;
        r.x = un;
      }
      if (vb) {
        const float4 cf = lab ? tab_s[lb[n]] : cell_coef(m, rowb + n);
        float un = ub[b] - cf.x * w[b].y;
        un = un * cf.z;
        un = un * (spb * sz);
        uc[rowb + n] = un;
        r.y = un;
      }
      w[b] = r;
    });
    float2 X[A];
    fft2<B, A, false>(w, X, s, twf, exf);
    z_split_store<N>(xb, X, S, d, x, y0, p, s, mk);
  }
}

// MODE 0: forward transform of p only; 2: inverse only into p; 1: full update
template <int N, int MODE>
__global__ void __launch_bounds__(CG_THREADS, CG_FAST_MINB) kf_zpass_p(Dims d, Tables t, MediumDev m, SourceDev src,
                                                           RecordDev rec, const long long* ctl, int n_local,
                                                           int record, float* __restrict__ p_all,
                                                           float2* __restrict__ S0) {
  using Z = ZShape<N>;
  constexpr int A = Z::A, B = Z::B;
  extern __shared__ float2 sm[];
  __shared__ unsigned int s_peak;
  float2* tw = sm;        // (A, B) order: inverse transforms
  float2* twf = sm + N;   // (B, A) order: forward transforms
  float4* stg4 = reinterpret_cast<float4*>(sm + Z::OFF_STG);
  float2* xb = sm + Z::OFF_STG;
  cgf::pdl_trigger();
  cgf::fill_twt<A, B>(tw, t.twz);
  cgf::fill_twt<B, A>(twf, t.twz);
  cgf::pdl_wait();
  if (threadIdx.x == 0) s_peak = 0u;
  const int s = threadIdx.x & 15, p = threadIdx.x >> 4;
  const RowEx<A, B, true> exi{sm + Z::OFF_EX + p * Z::EX};  // 16 threads per pencil: warp-local
  const RowEx<B, A, true> exf{sm + Z::OFF_EX + p * Z::EX};
  const int ytiles = (d.ny + CG_ZROWS - 1) / CG_ZROWS;
  const int x = blockIdx.x / ytiles;
  const int y0 = (blockIdx.x - x * ytiles) * CG_ZROWS;
  const int ya = y0 + 2 * p, yb = ya + 1;
  const bool va = ya < d.ny, vb = yb < d.ny;
  const int b_idx = blockIdx.y;
  float2* S = S0 + (long long)b_idx * d.nspec;
  float* pb = p_all + (long long)b_idx * d.ncell;
  const long long rowa = ((long long)x * d.ny + ya) * N, rowb = rowa + N;
  __syncthreads();
  float2 w[B];
  if constexpr (MODE == 0) {
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      w[b] = make_float2(va ? pb[rowa + n] : 0.f, vb ? pb[rowb + n] : 0.f);
    });
  } else {
    float4* tab_s = reinterpret_cast<float4*>(sm + Z::OFF_TAB);
    uint8_t* lab_s = reinterpret_cast<uint8_t*>(tab_s + 256);
    const bool lab = (MODE == 1) && z_stage_labels<N>(lab_s, tab_s, m, d, x, y0);
    const uint8_t* la = lab_s + (2 * p) * N;
    const uint8_t* lb = la + N;
    z_stage<N>(stg4, S, d, x, y0, nullptr);
    // this thread's pressures load while the inverse transform runs
    float pa[B], pbv[B];
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      pa[b] = (MODE == 1 && s < A && va) ? __ldg(pb + rowa + n) : 0.f;
      pbv[b] = (MODE == 1 && s < A && vb) ? __ldg(pb + rowb + n) : 0.f;
    });
    __syncthreads();
    float2 v[A];
    z_inputs<N>(v, stg4, p, s);
    fft2<A, B, true>(v, w, s, tw, exi);
    if constexpr (MODE == 2) {
      if (s < A) static_for<0, B>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        const int n = s + A * b;
        if (va) pb[rowa + n] = w[b].x;
        if (vb) pb[rowb + n] = w[b].y;
      });
      return;
    }
    const long long n_step = ctl[0] + n_local;
    const float spx = t.sx[x];
    const float spa = va ? spx * t.sy[ya] : 0.f, spb = vb ? spx * t.sy[yb] : 0.f;
    // p <- (p - (rho c^2 dt [+ 2 beta dt p]) div u) * absorb * sponge   (engine.py:470-477)
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      const float sz = t.sz[n];
      float2 r = make_float2(0.f, 0.f);
      if (va) {
        const float4 cf = lab ? tab_s[la[n]] : cell_coef(m, rowa + n);
        const float po = pa[b];
        float pn = m.nonlinear ? po - (cf.y + cf.w * po) * w[b].x : po - cf.y * w[b].x;
        pn = pn * cf.z;
        r.x = pn * (spa * sz);
      }
      if (vb) {
        const float4 cf = lab ? tab_s[lb[n]] : cell_coef(m, rowb + n);
        const float po = pbv[b];
        float pn = m.nonlinear ? po - (cf.y + cf.w * po) * w[b].y : po - cf.y * w[b].y;
        pn = pn * cf.z;
        r.y = pn * (spb * sz);
      }
      w[b] = r;
    });
    // source (engine.py:478-482): entries of rows ya, yb owned by this thread
    if (src.S > 0 && n_step < src.n_drive && s < A && va) {
      const float4 dr = src.drive[n_step];
      const int ra = x * d.ny + ya;
      const int e0 = src.row_ptr[ra], e1 = src.row_ptr[ra + 1], e2 = vb ? src.row_ptr[ra + 2] : e1;
      for (int e = e0; e < e2; ++e) {
        const int zz = src.zidx[e];
        if (zz % A != s) continue;
        const int k2 = zz / A;
        const float acv = src.ac[(long long)b_idx * src.S + e];
        const float asv = src.as[(long long)b_idx * src.S + e];
        const float add = dr.x * (dr.y * acv - dr.z * asv);
        const bool on_b = e >= e1;
        static_for<0, B>([&](auto bi) {
          constexpr int b = decltype(bi)::value;
          if (k2 == b) {
            if (on_b) w[b].y += add;
            else w[b].x += add;
          }
        });
      }
    }
    // write p, convergence peak, record window
    unsigned int lpeak = 0u;
    const int m_bin = (int)(n_step % rec.spp);
    const long long Ry = rec.hi[1] - rec.lo[1], Rz = rec.hi[2] - rec.lo[2];
    const bool x_conv = x >= rec.clo[0] && x < rec.chi[0];
    const bool x_rec = record && x >= rec.lo[0] && x < rec.hi[0];
    float* bins = rec.bins + ((long long)b_idx * rec.spp + m_bin) * rec.nrec;
    float* comp = rec.comp + ((long long)b_idx * rec.spp + m_bin) * rec.nrec;
    float* pmax = rec.pmax + (long long)b_idx * rec.nrec;
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      for (int r = 0; r < 2; ++r) {
        const int y = r ? yb : ya;
        if (r ? !vb : !va) continue;
        const float pn = r ? w[b].y : w[b].x;
        pb[(r ? rowb : rowa) + n] = pn;
        const float apn = fabsf(pn);
        if (x_conv && y >= rec.clo[1] && y < rec.chi[1] && n >= rec.clo[2] && n < rec.chi[2])
          lpeak = max(lpeak, __float_as_uint(apn));
        if (x_rec && y >= rec.lo[1] && y < rec.hi[1] && n >= rec.lo[2] && n < rec.hi[2]) {
          const long long ri = ((long long)(x - rec.lo[0]) * Ry + (y - rec.lo[1])) * Rz + (n - rec.lo[2]);
          const float sv = bins[ri], cm0 = comp[ri];
          const float yk = pn - cm0;
          const float tk = sv + yk;
          comp[ri] = (tk - sv) - yk;
          bins[ri] = tk;
          const float pm = pmax[ri];
          pmax[ri] = (apn > pm || apn != apn) ? apn : pm;
        }
      }
    });
    lpeak = __reduce_max_sync(0xffffffffu, lpeak);
    if ((threadIdx.x & 31) == 0) atomicMax(&s_peak, lpeak);
    __syncthreads();
    if (threadIdx.x == 0 && s_peak != 0u) {
      const long long per = n_step / rec.spp;
      if (per < rec.max_periods) atomicMax(&rec.peaks[(long long)b_idx * rec.max_periods + per], s_peak);
    }
  }
  if constexpr (MODE != 2) {
    float2 X[A];
    fft2<B, A, false>(w, X, s, twf, exf);
    z_split_store<N>(xb, X, S, d, x, y0, p, s, nullptr);
  }
}

// ---------------------------------------------------------------------------
// Persistent, pipelined z-passes (ny a multiple of the tile height). Each CTA
// walks a contiguous run of tiles -- for the u-pass all three velocity
// components of a tile in turn, so the tile's labels load once -- and the half
// spectrum of the next (tile, component) streams into shared memory -- by two
// tensor-map box copies on an mbarrier (TMA instantiations) or by 16-byte
// cp.async from every thread -- while the current one is transformed. An
// item's staging buffer is
// then reused as its exchange and split-store buffer, so the two buffers cost
// what the single-item kernel's staging plus exchange cost and two CTAs still
// fit on an SM.
template <int N>
struct ZPShape {
  static constexpr int A = ZSplit<N>::A, B = ZSplit<N>::B, NH = N / 2 + 1;
  static constexpr int TPP = ZSplit<N>::TPP;             // threads per pencil
  static constexpr int THREADS = CG_TILE * TPP;
  static constexpr bool WARP = (32 % TPP) == 0;  // a pencil's threads in one warp
  static constexpr int MINB = TPP == 16 ? CG_FAST_MINB : 1;  // resident CTAs per SM
  // the field values of a thread load before its inverse transform unless
  // the transform's A values per thread leave no registers for them
  static constexpr bool EARLY = A <= 20;
  static constexpr int EX_I = RowEx<A, B>::SLAB, EX_F = RowEx<B, A>::SLAB;
  static constexpr int EX = EX_I > EX_F ? EX_I : EX_F;
  static constexpr int B_STG = NH * 34, B_EX = CG_TILE * EX, B_XB = N * 17;  // float2 units
  // tensor-map staging: two 128-byte-wide boxes (8 pencils each) of NH k
  // rows, each on a 1024-byte boundary (the 128-byte swizzle repeats every 8
  // rows), plus 1024 bytes to align the first one inside the item buffer
  static constexpr bool TMA_OK = NH <= 256;
  static constexpr int BOXB = (NH * 128 + 1023) / 1024 * 1024;
  static constexpr int B_TMA = TMA_OK ? (2 * BOXB + 1024) / 8 : 0;
  static constexpr int B_MAX0 = B_STG > B_EX ? (B_STG > B_XB ? B_STG : B_XB) : (B_EX > B_XB ? B_EX : B_XB);
  static constexpr int B_MAX = B_MAX0 > B_TMA ? B_MAX0 : B_TMA;
  static constexpr int BUF = (B_MAX + 1) / 2 * 2;  // even: float4-aligned
  // without the k_z and sponge tables: they stay in shared memory when
  // everything fits the 227 KB a CTA may hold, else they are read through L1
  static constexpr size_t CORE = sizeof(float2) * (2 * N + 2 * (size_t)BUF + 2 * 256) + 2 * (size_t)CG_ZROWS * N;
  static constexpr size_t LIMIT = 232448 - 64;  // the kernels' static shared variables
  static constexpr int KZ0 = (NH + 3) / 4 * 2, SZ0 = (N + 3) / 4 * 2;  // float2 units, even
  static constexpr bool TBL = CORE + sizeof(float2) * (KZ0 + SZ0) <= LIMIT;
  static constexpr int KZF = TBL ? KZ0 : 0;  // k_z table (floats), float2 units
  static constexpr int SZF = TBL ? SZ0 : 0;  // z sponge profile (floats), float2 units
  // twiddles (two orders) | k_z | z sponge | two item buffers | material table | two label tiles
  static constexpr size_t OFF_KZ = 2 * N, OFF_SZ = OFF_KZ + KZF, OFF_BUF = OFF_SZ + SZF;
  // per material: float4 (k-space p coefficients) in the p-pass, float2
  // (dt/rho, absorb) in the u-pass, in the same place
  static constexpr size_t OFF_TAB = OFF_BUF + 2 * (size_t)BUF;
  static constexpr size_t OFF_LAB = OFF_TAB + 2 * 256;
  // then the two staging mbarriers (bytes from the start)
  static constexpr size_t OFF_BAR = sizeof(float2) * OFF_LAB + 2 * (size_t)CG_ZROWS * N;
  static constexpr size_t smem = OFF_BAR + 2 * sizeof(unsigned long long);
  static_assert(smem <= LIMIT, "persistent z-pass tile does not fit shared memory");
};

// The half spectrum of tile (x, y0) of S into stg4[k * 17 + p], asynchronously
// (ny even; a ragged last tile stages only its rows below ny).
template <int N>
__device__ __forceinline__ void z_prefetch(float4* stg4, const float2* __restrict__ S, const Dims& d, int x, int y0) {
  constexpr int NH = N / 2 + 1;
  const float2* base = S + (long long)x * NH * d.ny + y0;
  const int npp = min(CG_TILE, (d.ny - y0) >> 1);
  for (int idx = threadIdx.x; idx < NH * CG_TILE; idx += blockDim.x) {
    const int k = idx >> 4, pp = idx & 15;
    if (pp < npp) cgf::cp_async16(stg4 + k * 17 + pp, base + (long long)k * d.ny + 2 * pp);
  }
}

// The tile's labels (CG_ZROWS rows of N bytes, contiguous), asynchronously.
template <int N>
__device__ __forceinline__ void z_prefetch_labels(uint8_t* lab_s, const uint8_t* __restrict__ labels, const Dims& d,
                                                  int x, int y0) {
  const uint8_t* src = labels + ((long long)x * d.ny + y0) * N;
  const int n16 = min(CG_ZROWS, d.ny - y0) * N / 16;
  for (int i = threadIdx.x; i < n16; i += blockDim.x) cgf::cp_async16(lab_s + 16 * i, src + 16 * i);
}

// z_inputs on a staged tile: times i*mk[k] when mk is given, Im of the
// self-paired bins dropped, then the Hermitian extension. `row(k)` is the
// staged float4 (A_k, B_k) of this thread's pencil.
template <int N, class Row>
__device__ __forceinline__ void z_inputs_from(float2 (&v)[ZSplit<N>::A], int s, const float* mk, Row row) {
  constexpr int A = ZSplit<N>::A, B = ZSplit<N>::B;
  static_for<0, A>([&](auto ai) {
    constexpr int a = decltype(ai)::value;
    const int n = s + B * a;
    float2 z = make_float2(0.f, 0.f);
    if (s < B) {
      const bool hi = 2 * n > N;
      const int k = hi ? N - n : n;
      const float4 f = row(k);
      float2 fa = make_float2(f.x, f.y), fb = make_float2(f.z, f.w);
      if (mk) {
        const float kk = mk[k];
        fa = c_muli(c_scale(fa, kk));
        fb = c_muli(c_scale(fb, kk));
      }
      if (k == 0 || 2 * k == N) {
        fa.y = 0.f;
        fb.y = 0.f;
      }
      z = hi ? make_float2(fa.x + fb.y, fb.x - fa.y)   // conj(A) + i conj(B)
             : make_float2(fa.x - fb.y, fa.y + fb.x);  // A + i B
    }
    v[a] = z;
  });
}

// ... from the padded cp.async staging, stg4[k * 17 + p]
template <int N>
__device__ __forceinline__ void z_inputs_raw(float2 (&v)[ZSplit<N>::A], const float4* stg4, int p, int s,
                                             const float* mk) {
  z_inputs_from<N>(v, s, mk, [&](int k) { return stg4[k * 17 + p]; });
}

template <int N, bool UPASS>
__device__ __forceinline__ void zp_tables(float2* sm, const Tables& t, const MediumDev& m) {
  using Z = ZPShape<N>;
  cgf::fill_twt<Z::A, Z::B>(sm, t.twz);
  cgf::fill_twt<Z::B, Z::A>(sm + N, t.twz);
  if (Z::TBL) {
    float* kz_s = reinterpret_cast<float*>(sm + Z::OFF_KZ);
    for (int i = threadIdx.x; i < Z::NH; i += blockDim.x) kz_s[i] = t.kz[i];
    float* sz_s = reinterpret_cast<float*>(sm + Z::OFF_SZ);
    for (int i = threadIdx.x; i < N; i += blockDim.x) sz_s[i] = t.sz[i];
  }
  if (m.labels)
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
      const float4 c = m.ltab[i];
      if (UPASS)
        sm[Z::OFF_TAB + i] = make_float2(c.x, c.z);
      else
        reinterpret_cast<float4*>(sm + Z::OFF_TAB)[i] = c;
    }
}

// Tensor-map staging of item buffer j: its first 1024-byte boundary.
template <int N>
__device__ __forceinline__ char* zt_stage(float2* sm, int j) {
  char* b = reinterpret_cast<char*>(sm + ZPShape<N>::OFF_BUF + (size_t)j * ZPShape<N>::BUF);
  const unsigned a = cgf::smem_addr(b);
  return b + (((a + 1023u) & ~1023u) - a);
}

// The half spectrum of tile (member b, x, y0) into item buffer j by two box
// copies (pencils 0-7, 8-15), counted on bar; issued by one thread.
template <int N>
__device__ __forceinline__ void zt_issue(float2* sm, int j, unsigned long long* bar, const CUtensorMap* map,
                                         const Dims& d, long long b, int x, int y0) {
  using Z = ZPShape<N>;
  char* dst = zt_stage<N>(sm, j);
  const int c2 = (int)(b * d.nx + x);
  cgf::mbar_expect_tx(bar, 2u * Z::NH * 128u);
  cgf::tma_load_3d(dst, map, bar, 2 * y0, 0, c2);
  cgf::tma_load_3d(dst + Z::BOXB, map, bar, 2 * y0 + 32, 0, c2);
}

// z_inputs from the tensor-map staging: pencil p's 16 bytes of row k sit in
// box p / 8 at chunk (p % 8) XOR (k % 8) of the row's 128 bytes.
template <int N>
__device__ __forceinline__ void z_inputs_tma(float2 (&v)[ZSplit<N>::A], const char* stg, int p, int s,
                                             const float* mk) {
  const char* box = stg + (p >> 3) * ZPShape<N>::BOXB;
  const int c = p & 7;
  z_inputs_from<N>(v, s, mk,
                   [&](int k) { return *reinterpret_cast<const float4*>(box + k * 128 + ((c ^ (k & 7)) << 4)); });
}

// Waits for item buffer j's staging (tensor-map path); a wait that gives up
// raises the flag and the kernel carries on with whatever arrived.
__device__ __forceinline__ void zt_wait(unsigned long long* bars, unsigned& phase, int j, int* err) {
  if (!cgf::mbar_wait(bars + j, (phase >> j) & 1u)) atomicExch(err, 1);
  phase ^= 1u << j;
}

// TMA: the tile's half spectra arrive by tensor-map box copies on an
// mbarrier (ztma: the descriptors, by value) instead of per-thread cp.async;
// the labels keep cp.async. Other instantiations ignore ztma.
template <int N, bool TMA = false>
__global__ void __launch_bounds__(ZPShape<N>::THREADS, ZPShape<N>::MINB) kfp_zpass_u(Dims d, Tables t, MediumDev m,
                                                                       float* __restrict__ u, float2* __restrict__ S0,
                                                                       float2* __restrict__ S1, float2* __restrict__ S2,
                                                                       int n_members, int tiles_per_cta,
                                                                       const __grid_constant__ ZTma ztma) {
  using Z = ZPShape<N>;
  constexpr int A = Z::A, B = Z::B;
  extern __shared__ float2 sm[];
  const int ytiles = (d.ny + CG_ZROWS - 1) / CG_ZROWS;  // ny even; the last tile may be ragged
  const long long per_member = (long long)d.nx * ytiles;
  const long long total = per_member * n_members;
  const long long t0 = (long long)blockIdx.x * tiles_per_cta;
  const long long t1 = min(total, t0 + tiles_per_cta);
  cgf::pdl_trigger();
  if (t0 >= t1) return;  // the whole CTA, before any barrier
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(sm) + Z::OFF_BAR);
  unsigned phase = 0u;  // bit j: parity of item buffer j's next staging phase
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      cgf::mbar_init(bars, 1);
      cgf::mbar_init(bars + 1, 1);
      cgf::mbar_init_fence();
    }
    __syncthreads();
  }
  zp_tables<N, true>(sm, t, m);
  cgf::pdl_wait();
  const float* kz_s = Z::TBL ? reinterpret_cast<const float*>(sm + Z::OFF_KZ) : t.kz;
  const float* sz_s = Z::TBL ? reinterpret_cast<const float*>(sm + Z::OFF_SZ) : t.sz;
  const float2* tab2_s = sm + Z::OFF_TAB;
  uint8_t* lab0 = reinterpret_cast<uint8_t*>(sm + Z::OFF_LAB);
  const bool lab = m.labels != nullptr;
  const int s = threadIdx.x % Z::TPP, p = threadIdx.x / Z::TPP;
  auto spec = [&](int comp, long long b) { return (comp == 0 ? S1 : (comp == 1 ? S0 : S2)) + b * d.nspec; };
  // tiles run member-fastest: the members of one (x, y0) follow each other,
  // so the tile's labels load once for all of them (label slot per group)
  auto label_slot = [&](long long tile) { return (int)((tile / n_members - t0 / n_members) & 1); };
  auto prefetch = [&](long long tile, int comp, int j) {
    const long long b = tile % n_members, r = tile / n_members;
    const int x = (int)(r / ytiles), y0 = (int)(r - (long long)x * ytiles) * CG_ZROWS;
    if constexpr (TMA) {
      if (threadIdx.x == 0) zt_issue<N>(sm, j, bars + j, &ztma.map[comp], d, b, x, y0);  // map order = comp order
    } else {
      z_prefetch<N>(reinterpret_cast<float4*>(sm + Z::OFF_BUF + (size_t)j * Z::BUF), spec(comp, b), d, x, y0);
    }
    if (comp == 0 && lab && (tile == t0 || b == 0))
      z_prefetch_labels<N>(lab0 + label_slot(tile) * CG_ZROWS * N, m.labels, d, x, y0);
    cgf::cp_async_commit();
  };
  prefetch(t0, 0, 0);
  int j = 0;
  for (long long tile = t0; tile < t1; ++tile) {
    const long long b_idx = tile % n_members, r = tile / n_members;
    const int x = (int)(r / ytiles), y0 = (int)(r - (long long)x * ytiles) * CG_ZROWS;
    const int ya = y0 + 2 * p, yb = ya + 1;
    const bool va = ya < d.ny;  // this pencil's rows exist (ny even: yb too)
    const float spx = t.sx[x];
    const float spa = va ? spx * t.sy[ya] : 0.f, spb = va ? spx * t.sy[yb] : 0.f;
    const long long rowa = ((long long)x * d.ny + ya) * N, rowb = rowa + N;
    const uint8_t* la = lab0 + label_slot(tile) * CG_ZROWS * N + (2 * p) * N;
    const uint8_t* lb = la + N;
#pragma unroll 1
    for (int comp = 0; comp < 3; ++comp, j ^= 1) {
      float* uc = u + ((long long)comp * n_members + b_idx) * d.ncell;
      // this thread's velocities load while the staged spectrum is transformed
      // (after it where A-value registers would not leave room for them)
      float ua[B], ub[B];
      auto load_u = [&]() {
        static_for<0, B>([&](auto bi) {
          constexpr int b = decltype(bi)::value;
          const int n = s + A * b;
          ua[b] = (s < A && va) ? __ldg(uc + rowa + n) : 0.f;
          ub[b] = (s < A && va) ? __ldg(uc + rowb + n) : 0.f;
        });
      };
      if (Z::EARLY) load_u();
      // (tensor-map path) this thread's generic accesses to the buffer the
      // next copy fills are ordered before that copy
      if constexpr (TMA) cgf::fence_proxy_async();
      cgf::cp_async_wait0();
      __syncthreads();
      {
        long long nt = tile;
        int nc = comp + 1;
        if (nc == 3) {
          nc = 0;
          ++nt;
        }
        if (nt < t1) prefetch(nt, nc, j ^ 1);
      }
      float2* bufj = sm + Z::OFF_BUF + (size_t)j * Z::BUF;
      float2 v[A], w[B];
      if constexpr (TMA) {
        zt_wait(bars, phase, j, ztma.err);
        z_inputs_tma<N>(v, zt_stage<N>(sm, j), p, s, comp == 2 ? kz_s : nullptr);
      } else {
        z_inputs_raw<N>(v, reinterpret_cast<const float4*>(bufj), p, s, comp == 2 ? kz_s : nullptr);
      }
      __syncthreads();  // the staging is read: the buffer becomes the exchange
      const RowEx<A, B, Z::WARP> exi{bufj + p * Z::EX};
      const RowEx<B, A, Z::WARP> exf{bufj + p * Z::EX};
      fft2<A, B, true>(v, w, s, sm, exi);
      if (!Z::EARLY) load_u();
      // u <- (u - dt/rho g) * absorb * sponge   (engine.py:462-464)
      if (s < A) static_for<0, B>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        const int n = s + A * b;
        const float sz = sz_s[n];
        // (dt/rho, absorb) of the two cells
        const float2 ca = lab ? tab2_s[la[n]] : (va ? make_float2(m.dtr[rowa + n], m.ab[rowa + n]) : make_float2(0.f, 0.f));
        const float2 cb = lab ? tab2_s[lb[n]] : (va ? make_float2(m.dtr[rowb + n], m.ab[rowb + n]) : make_float2(0.f, 0.f));
        float una = ua[b] - ca.x * w[b].x;
        una = una * ca.y;
        una = una * (spa * sz);
        float unb = ub[b] - cb.x * w[b].y;
        unb = unb * cb.y;
        unb = unb * (spb * sz);
        if (va) {
          uc[rowa + n] = una;
          uc[rowb + n] = unb;
        }
        w[b] = make_float2(una, unb);
      });
      float2 X[A];
      fft2<B, A, false>(w, X, s, sm + N, exf);
      z_split_store<N>(bufj, X, spec(comp, b_idx), d, x, y0, p, s, comp == 2 ? kz_s : nullptr);
    }
  }
}

// REC: the step records into the phase bins (an instantiation without the
// record path keeps the non-recording steps' instruction stream short).
// FWD: only the closing forward transform, of the pressure as it is -- the
// spectrum a step leaves behind, rebuilt from a restored pressure field by
// the very code the step runs, so a restored run continues bit for bit.
// TMA: the half spectra arrive by tensor-map box copies (as in the u-pass).
template <int N, bool REC, bool FWD = false, bool TMA = false>
__global__ void __launch_bounds__(ZPShape<N>::THREADS, ZPShape<N>::MINB) kfp_zpass_p(Dims d, Tables t, MediumDev m,
                                                                       SourceDev src, RecordDev rec,
                                                                       const long long* ctl, int n_local, int record,
                                                                       float* __restrict__ p_all,
                                                                       float2* __restrict__ S0, int n_members,
                                                                       int tiles_per_cta,
                                                                       const __grid_constant__ ZTma ztma) {
  using Z = ZPShape<N>;
  constexpr int A = Z::A, B = Z::B;
  static_assert(!(FWD && TMA), "the forward-only pass stages no spectrum");
  extern __shared__ float2 sm[];
  const int ytiles = (d.ny + CG_ZROWS - 1) / CG_ZROWS;  // ny even; the last tile may be ragged
  const long long per_member = (long long)d.nx * ytiles;
  const long long total = per_member * n_members;
  const long long t0 = (long long)blockIdx.x * tiles_per_cta;
  const long long t1 = min(total, t0 + tiles_per_cta);
  cgf::pdl_trigger();
  if (t0 >= t1) return;  // the whole CTA, before any barrier
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(sm) + Z::OFF_BAR);
  unsigned phase = 0u;  // bit j: parity of item buffer j's next staging phase
  if constexpr (TMA) {
    if (threadIdx.x == 0) {
      cgf::mbar_init(bars, 1);
      cgf::mbar_init(bars + 1, 1);
      cgf::mbar_init_fence();
    }
    __syncthreads();
  }
  zp_tables<N, false>(sm, t, m);
  cgf::pdl_wait();
  const float* sz_s = Z::TBL ? reinterpret_cast<const float*>(sm + Z::OFF_SZ) : t.sz;
  const float4* tab_s = reinterpret_cast<const float4*>(sm + Z::OFF_TAB);
  uint8_t* lab0 = reinterpret_cast<uint8_t*>(sm + Z::OFF_LAB);
  const bool lab = m.labels != nullptr;
  const int s = threadIdx.x % Z::TPP, p = threadIdx.x / Z::TPP;
  // tiles run member-fastest: the members of one (x, y0) follow each other,
  // so the tile's labels load once for all of them (label slot per group)
  auto label_slot = [&](long long tile) { return (int)((tile / n_members - t0 / n_members) & 1); };
  auto prefetch = [&](long long tile, int j) {
    const long long b = tile % n_members, r = tile / n_members;
    const int x = (int)(r / ytiles), y0 = (int)(r - (long long)x * ytiles) * CG_ZROWS;
    if constexpr (TMA) {
      if (threadIdx.x == 0) zt_issue<N>(sm, j, bars + j, &ztma.map[1], d, b, x, y0);  // map[1]: S0
    } else {
      z_prefetch<N>(reinterpret_cast<float4*>(sm + Z::OFF_BUF + (size_t)j * Z::BUF), S0 + b * d.nspec, d, x, y0);
    }
    if (lab && (tile == t0 || b == 0)) z_prefetch_labels<N>(lab0 + label_slot(tile) * CG_ZROWS * N, m.labels, d, x, y0);
    cgf::cp_async_commit();
  };
  if constexpr (FWD) {
    int jf = 0;
    for (long long tile = t0; tile < t1; ++tile, jf ^= 1) {
      const long long b_idx = tile % n_members, r = tile / n_members;
      const int x = (int)(r / ytiles), y0 = (int)(r - (long long)x * ytiles) * CG_ZROWS;
      const int ya = y0 + 2 * p;
      const bool va = ya < d.ny;  // ny even: row ya + 1 too
      const float* pb = p_all + b_idx * d.ncell;
      const long long rowa = ((long long)x * d.ny + ya) * N, rowb = rowa + N;
      float2 w[B];
      if (s < A) static_for<0, B>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        const int n = s + A * b;
        w[b] = make_float2(va ? __ldg(pb + rowa + n) : 0.f, va ? __ldg(pb + rowb + n) : 0.f);
      });
      float2* bufj = sm + Z::OFF_BUF + (size_t)jf * Z::BUF;
      const RowEx<B, A, Z::WARP> exf{bufj + p * Z::EX};
      float2 X[A];
      fft2<B, A, false>(w, X, s, sm + N, exf);
      z_split_store<N>(bufj, X, S0 + b_idx * d.nspec, d, x, y0, p, s, nullptr);
    }
    return;
  }
  prefetch(t0, 0);
  const long long n_step = ctl[0] + n_local;
  const int m_bin = (int)(n_step % rec.spp);
  const long long per_log = n_step / rec.spp;
  unsigned int wpeak = 0u;
  long long wmember = -1;
  const long long Ry = rec.hi[1] - rec.lo[1], Rz = rec.hi[2] - rec.lo[2];
  const bool drive_on = src.S > 0 && n_step < src.n_drive;
  const float4 dr = drive_on ? src.drive[n_step] : make_float4(0.f, 0.f, 0.f, 0.f);
  static_assert(B <= 32, "one mask bit per cell of a thread");
  unsigned int zconv = 0u, zrec = 0u;  // bit b: this thread's cell z = s + A b is in the box
  if (s < A) static_for<0, B>([&](auto bi) {
    constexpr int b = decltype(bi)::value;
    const int n = s + A * b;
    if (n >= rec.clo[2] && n < rec.chi[2]) zconv |= 1u << b;
    if (n >= rec.lo[2] && n < rec.hi[2]) zrec |= 1u << b;
  });
  int j = 0;
  for (long long tile = t0; tile < t1; ++tile, j ^= 1) {
    const long long b_idx = tile % n_members, r = tile / n_members;
    const int x = (int)(r / ytiles), y0 = (int)(r - (long long)x * ytiles) * CG_ZROWS;
    const int ya = y0 + 2 * p, yb = ya + 1;
    const bool va = ya < d.ny;  // this pencil's rows exist (ny even: yb too)
    float* pb = p_all + b_idx * d.ncell;
    float2* S = S0 + b_idx * d.nspec;
    const long long rowa = ((long long)x * d.ny + ya) * N, rowb = rowa + N;
    // this thread's pressures load while the staged spectrum is transformed
    // (after it where A-value registers would not leave room for them)
    float pa[B], pbv[B];
    auto load_p = [&]() {
      static_for<0, B>([&](auto bi) {
        constexpr int b = decltype(bi)::value;
        const int n = s + A * b;
        pa[b] = (s < A && va) ? __ldg(pb + rowa + n) : 0.f;
        pbv[b] = (s < A && va) ? __ldg(pb + rowb + n) : 0.f;
      });
    };
    if (Z::EARLY) load_p();
    if constexpr (TMA) cgf::fence_proxy_async();  // see the u-pass
    cgf::cp_async_wait0();
    __syncthreads();
    if (tile + 1 < t1) prefetch(tile + 1, j ^ 1);
    float2* bufj = sm + Z::OFF_BUF + (size_t)j * Z::BUF;
    const uint8_t* la = lab0 + label_slot(tile) * CG_ZROWS * N + (2 * p) * N;
    const uint8_t* lb = la + N;
    float2 v[A], w[B];
    if constexpr (TMA) {
      zt_wait(bars, phase, j, ztma.err);
      z_inputs_tma<N>(v, zt_stage<N>(sm, j), p, s, nullptr);
    } else {
      z_inputs_raw<N>(v, reinterpret_cast<const float4*>(bufj), p, s, nullptr);
    }
    __syncthreads();  // the staging is read: the buffer becomes the exchange
    const RowEx<A, B, Z::WARP> exi{bufj + p * Z::EX};
    const RowEx<B, A, Z::WARP> exf{bufj + p * Z::EX};
    fft2<A, B, true>(v, w, s, sm, exi);
    if (!Z::EARLY) load_p();
    const float spx = t.sx[x];
    const float spa = va ? spx * t.sy[ya] : 0.f, spb = va ? spx * t.sy[yb] : 0.f;
    // p <- (p - (rho c^2 dt [+ 2 beta dt p]) div u) * absorb * sponge   (engine.py:470-477)
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      const float sz = sz_s[n];
      const float4 ca = lab ? tab_s[la[n]] : (va ? cell_coef(m, rowa + n) : make_float4(0.f, 0.f, 0.f, 0.f));
      const float4 cb = lab ? tab_s[lb[n]] : (va ? cell_coef(m, rowb + n) : make_float4(0.f, 0.f, 0.f, 0.f));
      const float poa = pa[b], pob = pbv[b];
      float pna = m.nonlinear ? poa - (ca.y + ca.w * poa) * w[b].x : poa - ca.y * w[b].x;
      float pnb = m.nonlinear ? pob - (cb.y + cb.w * pob) * w[b].y : pob - cb.y * w[b].y;
      pna = pna * ca.z;
      pnb = pnb * cb.z;
      w[b] = make_float2(pna * (spa * sz), pnb * (spb * sz));
    });
    // source (engine.py:478-482): entries of rows ya, yb owned by this thread
    if (drive_on && s < A && va) {
      const int ra = x * d.ny + ya;
      const int e0 = src.row_ptr[ra], e1 = src.row_ptr[ra + 1], e2 = src.row_ptr[ra + 2];
      for (int e = e0; e < e2; ++e) {
        const int zz = src.zidx[e];
        if (zz % A != s) continue;
        const int k2 = zz / A;
        const float acv = src.ac[b_idx * src.S + e];
        const float asv = src.as[b_idx * src.S + e];
        const float add = dr.x * (dr.y * acv - dr.z * asv);
        const bool on_b = e >= e1;
        static_for<0, B>([&](auto bi) {
          constexpr int b = decltype(bi)::value;
          if (k2 == b) {
            if (on_b) w[b].y += add;
            else w[b].x += add;
          }
        });
      }
    }
    // write p, convergence peak, record window (z-range membership of this
    // thread's cells is a per-kernel bit mask, the y/x membership per tile)
    unsigned int lpeak = 0u;
    const bool x_conv = va && x >= rec.clo[0] && x < rec.chi[0];
    const bool x_rec = REC && va && record && x >= rec.lo[0] && x < rec.hi[0];
    const bool conv_a = x_conv && ya >= rec.clo[1] && ya < rec.chi[1];
    const bool conv_b = x_conv && yb >= rec.clo[1] && yb < rec.chi[1];
    const bool rec_a = x_rec && ya >= rec.lo[1] && ya < rec.hi[1];
    const bool rec_b = x_rec && yb >= rec.lo[1] && yb < rec.hi[1];
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      const float pna = w[b].x, pnb = w[b].y;
      if (va) {
        pb[rowa + n] = pna;
        pb[rowb + n] = pnb;
      }
      if ((zconv >> b) & 1u) {
        if (conv_a) lpeak = max(lpeak, __float_as_uint(fabsf(pna)));
        if (conv_b) lpeak = max(lpeak, __float_as_uint(fabsf(pnb)));
      }
    });
    if constexpr (REC) {
      // phase bin m (Kahan-compensated sum) and running max |p| of this
      // thread's recorded cells, RC cells per row at a time: every load of a
      // chunk is issued before its first store, so the chunk costs one round
      // trip to memory instead of one per cell
      if (s < A && (rec_a || rec_b)) {
        float* __restrict__ bins = rec.bins + (b_idx * rec.spp + m_bin) * rec.nrec;
        float* __restrict__ comp = rec.comp + (b_idx * rec.spp + m_bin) * rec.nrec;
        float* __restrict__ pmax = rec.pmax + b_idx * rec.nrec;
        const long long ra = ((long long)(x - rec.lo[0]) * Ry + (ya - rec.lo[1])) * Rz - rec.lo[2];
        const long long rb = ra + Rz;  // row yb = ya + 1
        constexpr int RC = 4;
        static_assert(B % RC == 0, "record chunks split the thread's cells evenly");
        static_for<0, B / RC>([&](auto ci) {
          constexpr int c0 = decltype(ci)::value * RC;
          float sv[2 * RC], cm[2 * RC], pm[2 * RC];
          static_for<0, RC>([&](auto ji) {
            constexpr int j = decltype(ji)::value, b = c0 + j;
            const int n = s + A * b;
            const bool in = (zrec >> b) & 1u;
            sv[j] = (in && rec_a) ? bins[ra + n] : 0.f;
            cm[j] = (in && rec_a) ? comp[ra + n] : 0.f;
            pm[j] = (in && rec_a) ? pmax[ra + n] : 0.f;
            sv[RC + j] = (in && rec_b) ? bins[rb + n] : 0.f;
            cm[RC + j] = (in && rec_b) ? comp[rb + n] : 0.f;
            pm[RC + j] = (in && rec_b) ? pmax[rb + n] : 0.f;
          });
          static_for<0, RC>([&](auto ji) {
            constexpr int j = decltype(ji)::value, b = c0 + j;
            const int n = s + A * b;
            if (!((zrec >> b) & 1u)) return;
            for (int r = 0; r < 2; ++r) {
              if (r ? !rec_b : !rec_a) continue;
              const long long ri = (r ? rb : ra) + n;
              const float pn = r ? w[b].y : w[b].x, apn = fabsf(pn);
              const int k = r * RC + j;
              const float yk = pn - cm[k];
              const float tk = sv[k] + yk;
              comp[ri] = (tk - sv[k]) - yk;
              bins[ri] = tk;
              pmax[ri] = (apn > pm[k] || apn != apn) ? apn : pm[k];
            }
          });
        });
      }
    }
    // convergence peak: a running max per warp over its tiles, written to
    // the period log (an integer max over the float bits) when the batch
    // member changes and at the end -- no barrier per tile
    lpeak = __reduce_max_sync(0xffffffffu, lpeak);
    if (b_idx != wmember) {
      if ((threadIdx.x & 31) == 0 && wpeak && per_log < rec.max_periods)
        atomicMax(&rec.peaks[wmember * rec.max_periods + per_log], wpeak);
      wpeak = 0u;
      wmember = b_idx;
    }
    wpeak = max(wpeak, lpeak);
    float2 X[A];
    fft2<B, A, false>(w, X, s, sm + N, exf);
    z_split_store<N>(bufj, X, S, d, x, y0, p, s, nullptr);
  }
  if ((threadIdx.x & 31) == 0 && wpeak && wmember >= 0 && per_log < rec.max_periods)
    atomicMax(&rec.peaks[wmember * rec.max_periods + per_log], wpeak);
}

// ------------------------------------------------ per-length launchers --
// persistent z-passes (any N of CG_FAST_ZSIZES, ny even); ztma (encoded
// descriptors, host memory) selects the tensor-map staging where the length
// allows it
static const ZTma kNoZTma = {};
template <int N>
void zp_run_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
              int batch, cudaStream_t st, const ZTma* ztma) {
  int g = 0, per = 0;
  cgf::persistent_grid((long long)d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS) * batch, ZPShape<N>::MINB, &g, &per);
  if constexpr (ZPShape<N>::TMA_OK) {
    if (ztma) {
      cgf::launch(kfp_zpass_u<N, true>, dim3(g), dim3(ZPShape<N>::THREADS), ZPShape<N>::smem, st, d, t, m, u, S0, S1,
                  S2, batch, per, *ztma);
      return;
    }
  }
  cgf::launch(kfp_zpass_u<N>, dim3(g), dim3(ZPShape<N>::THREADS), ZPShape<N>::smem, st, d, t, m, u, S0, S1, S2,
              batch, per, kNoZTma);
}

template <int N>
void zp_run_p(const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src, const RecordDev& rec,
              const long long* ctl, int n_local, int record, float* p, float2* S0, int batch, cudaStream_t st,
              const ZTma* ztma) {
  int g = 0, per = 0;
  cgf::persistent_grid((long long)d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS) * batch, ZPShape<N>::MINB, &g, &per);
  const dim3 grid(g), block(ZPShape<N>::THREADS);
  const size_t sm = ZPShape<N>::smem;
  if constexpr (ZPShape<N>::TMA_OK) {
    if (ztma) {
      if (record)
        cgf::launch(kfp_zpass_p<N, true, false, true>, grid, block, sm, st, d, t, m, src, rec, ctl, n_local, record, p,
                    S0, batch, per, *ztma);
      else
        cgf::launch(kfp_zpass_p<N, false, false, true>, grid, block, sm, st, d, t, m, src, rec, ctl, n_local, record,
                    p, S0, batch, per, *ztma);
      return;
    }
  }
  if (record)
    cgf::launch(kfp_zpass_p<N, true>, grid, block, sm, st, d, t, m, src, rec, ctl, n_local, record, p, S0, batch, per,
                kNoZTma);
  else
    cgf::launch(kfp_zpass_p<N, false>, grid, block, sm, st, d, t, m, src, rec, ctl, n_local, record, p, S0, batch,
                per, kNoZTma);
}

template <int N>
void zp_run_fwd(const Dims& d, const Tables& t, const MediumDev& m, float* p, float2* S0, int batch,
                cudaStream_t st) {
  int g = 0, per = 0;
  cgf::persistent_grid((long long)d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS) * batch, ZPShape<N>::MINB, &g, &per);
  SourceDev src;
  memset(&src, 0, sizeof(src));
  RecordDev rec;
  memset(&rec, 0, sizeof(rec));
  rec.spp = 1;
  cgf::launch(kfp_zpass_p<N, false, true>, dim3(g), dim3(ZPShape<N>::THREADS), ZPShape<N>::smem, st, d, t, m, src,
              rec, (const long long*)nullptr, 0, 0, p, S0, batch, per, kNoZTma);
}

template <typename K>
static bool zp_allow(K kernel, int bytes) {
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess;
}

template <int N>
int zp_prepare() {
  const int sm = (int)ZPShape<N>::smem;
  bool ok = zp_allow(kfp_zpass_u<N>, sm) && zp_allow(kfp_zpass_p<N, false, true>, sm) &&
            zp_allow(kfp_zpass_p<N, true>, sm) && zp_allow(kfp_zpass_p<N, false>, sm);
  if constexpr (ZPShape<N>::TMA_OK)
    ok = ok && zp_allow(kfp_zpass_u<N, true>, sm) && zp_allow(kfp_zpass_p<N, true, false, true>, sm) &&
         zp_allow(kfp_zpass_p<N, false, false, true>, sm);
  return ok ? 0 : -1;
}

// one-tile-per-CTA z-passes (N of CG_FAST_SIZES, any ny)
template <int N>
void zt_run_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
              int batch, cudaStream_t st) {
  const dim3 grid((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), batch);
  cgf::launch(kf_zpass_u<N>, grid, dim3(CG_THREADS), ZShape<N>::smem, st, d, t, m, u, S0, S1, S2);
}

template <int N>
void zt_run_p(int mode, const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src, const RecordDev& rec,
              const long long* ctl, int n_local, int record, float* p, float2* S0, int batch, cudaStream_t st) {
  const dim3 grid((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), batch);
  if (mode == 0)
    cgf::launch(kf_zpass_p<N, 0>, grid, dim3(CG_THREADS), ZShape<N>::smem, st, d, t, m, src, rec, ctl, n_local,
                record, p, S0);
  else if (mode == 1)
    cgf::launch(kf_zpass_p<N, 1>, grid, dim3(CG_THREADS), ZShape<N>::smem, st, d, t, m, src, rec, ctl, n_local,
                record, p, S0);
  else
    cgf::launch(kf_zpass_p<N, 2>, grid, dim3(CG_THREADS), ZShape<N>::smem, st, d, t, m, src, rec, ctl, n_local,
                record, p, S0);
}

template <int N>
int zt_prepare() {
  const int sm = (int)ZShape<N>::smem;
  return (cudaFuncSetAttribute(kf_zpass_u<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess ||
          cudaFuncSetAttribute(kf_zpass_p<N, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess ||
          cudaFuncSetAttribute(kf_zpass_p<N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess ||
          cudaFuncSetAttribute(kf_zpass_p<N, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) != cudaSuccess)
             ? -1
             : 0;
}

#define CG_ZP_INSTANTIATE(n)                                                                                       \
  template void zp_run_u<n>(const Dims&, const Tables&, const MediumDev&, float*, float2*, float2*, float2*, int,  \
                            cudaStream_t, const ZTma*);                                                            \
  template void zp_run_p<n>(const Dims&, const Tables&, const MediumDev&, const SourceDev&, const RecordDev&,     \
                            const long long*, int, int, float*, float2*, int, cudaStream_t, const ZTma*);         \
  template void zp_run_fwd<n>(const Dims&, const Tables&, const MediumDev&, float*, float2*, int, cudaStream_t); \
  template int zp_prepare<n>();
#define CG_ZT_INSTANTIATE(n)                                                                                       \
  template void zt_run_u<n>(const Dims&, const Tables&, const MediumDev&, float*, float2*, float2*, float2*, int,  \
                            cudaStream_t);                                                                         \
  template void zt_run_p<n>(int, const Dims&, const Tables&, const MediumDev&, const SourceDev&, const RecordDev&, \
                            const long long*, int, int, float*, float2*, int, cudaStream_t);                      \
  template int zt_prepare<n>();
