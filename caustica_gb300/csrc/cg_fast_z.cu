// Size-specialised z-passes (nz = N known at compile time).
//
// Tile = (batch member, x, 32 consecutive y). Real rows y0+2p and y0+2p+1
// form complex pencil p (p = threadIdx / 16); s = threadIdx % 16 runs along
// the pencil. The inverse (complex-to-real) transform is an (A, B) fft2, the
// forward one a (B, A) fft2, so the values produced by the inverse arrive in
// exactly the registers the forward transform reads; the pointwise update
// runs in between, on cells (x, y, s + A b) with coalesced row accesses.
// Half spectra are staged through shared memory in both directions (the
// spectral layout has y fastest, the real layout z fastest).
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
__device__ __forceinline__ void z_split_store(float2* xb, const float2 (&X)[Split<N>::A], float2* __restrict__ S,
                                              const Dims& d, int x, int y0, int p, int s, const float* mk) {
  constexpr int A = Split<N>::A, B = Split<N>::B, NH = N / 2 + 1;
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
  float2* tw = sm;        // (A, B) order: inverse transforms
  float2* twf = sm + N;   // (B, A) order: forward transforms
  float4* stg4 = reinterpret_cast<float4*>(sm + Z::OFF_STG);
  float2* xb = sm + Z::OFF_STG;
  cgf::fill_twt<A, B>(tw, t.twz);
  cgf::fill_twt<B, A>(twf, t.twz);
  const int s = threadIdx.x & 15, p = threadIdx.x >> 4;
  const RowEx<A, B> exi{sm + Z::OFF_EX + p * Z::EX};
  const RowEx<B, A> exf{sm + Z::OFF_EX + p * Z::EX};
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

// mode 0: forward transform of p only; 2: inverse only into p; 1: full update
template <int N>
__global__ void __launch_bounds__(CG_THREADS, CG_FAST_MINB) kf_zpass_p(int mode, Dims d, Tables t, MediumDev m, SourceDev src,
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
  cgf::fill_twt<A, B>(tw, t.twz);
  cgf::fill_twt<B, A>(twf, t.twz);
  if (threadIdx.x == 0) s_peak = 0u;
  const int s = threadIdx.x & 15, p = threadIdx.x >> 4;
  const RowEx<A, B> exi{sm + Z::OFF_EX + p * Z::EX};
  const RowEx<B, A> exf{sm + Z::OFF_EX + p * Z::EX};
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
  if (mode == 0) {
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      w[b] = make_float2(va ? pb[rowa + n] : 0.f, vb ? pb[rowb + n] : 0.f);
    });
  } else {
    float4* tab_s = reinterpret_cast<float4*>(sm + Z::OFF_TAB);
    uint8_t* lab_s = reinterpret_cast<uint8_t*>(tab_s + 256);
    const bool lab = (mode == 1) && z_stage_labels<N>(lab_s, tab_s, m, d, x, y0);
    const uint8_t* la = lab_s + (2 * p) * N;
    const uint8_t* lb = la + N;
    z_stage<N>(stg4, S, d, x, y0, nullptr);
    // this thread's pressures load while the inverse transform runs
    float pa[B], pbv[B];
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int n = s + A * b;
      pa[b] = (mode == 1 && s < A && va) ? __ldg(pb + rowa + n) : 0.f;
      pbv[b] = (mode == 1 && s < A && vb) ? __ldg(pb + rowb + n) : 0.f;
    });
    __syncthreads();
    float2 v[A];
    z_inputs<N>(v, stg4, p, s);
    fft2<A, B, true>(v, w, s, tw, exi);
    if (mode == 2) {
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
  float2 X[A];
  fft2<B, A, false>(w, X, s, twf, exf);
  z_split_store<N>(xb, X, S, d, x, y0, p, s, nullptr);
}

bool fast_zpass_u(const Dims& d, const Tables& t, const MediumDev& m, float* u, float2* S0, float2* S1, float2* S2,
                  int batch, cudaStream_t st) {
  const dim3 grid((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), batch);
  switch (d.nz) {
#define CASE(n)                                                                       \
  case n:                                                                             \
    kf_zpass_u<n><<<grid, CG_THREADS, ZShape<n>::smem, st>>>(d, t, m, u, S0, S1, S2); \
    return true;
    CG_FAST_SIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

bool fast_zpass_p(int mode, const Dims& d, const Tables& t, const MediumDev& m, const SourceDev& src,
                  const RecordDev& rec, const long long* ctl, int n_local, int record, float* p, float2* S0,
                  int batch, cudaStream_t st) {
  const dim3 grid((unsigned)(d.nx * ((d.ny + CG_ZROWS - 1) / CG_ZROWS)), batch);
  switch (d.nz) {
#define CASE(n)                                                                                            \
  case n:                                                                                                  \
    kf_zpass_p<n><<<grid, CG_THREADS, ZShape<n>::smem, st>>>(mode, d, t, m, src, rec, ctl, n_local, record, \
                                                              p, S0);                                      \
    return true;
    CG_FAST_SIZES(CASE)
#undef CASE
    default:
      return false;
  }
}

int fast_prepare_z() {
#define SET(n)                                                                                          \
  if (cudaFuncSetAttribute(kf_zpass_u<n>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ZShape<n>::smem) != \
          cudaSuccess ||                                                                                \
      cudaFuncSetAttribute(kf_zpass_p<n>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ZShape<n>::smem) != \
          cudaSuccess)                                                                                  \
    return -1;
  CG_FAST_SIZES(SET)
#undef SET
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
