// Fused transverse (x, y) passes for square planes (nx == ny == N), GB300
// (sm_103a) thread-block clusters.
//
// One cluster of C CTAs owns one (kz plane, batch member). CTA `rank` holds
// rows x in [rank R, rank R + R), R = N / C, of three plane buffers in shared
// memory; the columns (fixed y, all x) are read and written across the
// cluster through distributed shared memory. A step's spectral chain
// between the two z-passes then costs one launch and one read / write of
// each spectrum instead of three launches:
//
//   grad:  rows     bS = FFT_y(S0)
//          columns  q = kappa/N FFT_x(bS);  bA = IFFT_x(q);  bB = IFFT_x(i k_x q)
//          rows     S1 = IFFT_y(bB);  S0 = IFFT_y(i k_y bA);  S2 = IFFT_y(bA)
//   div:   rows     bA = FFT_y(S1);  bB = i k_y FFT_y(S0) + FFT_y(S2)
//          columns  bS = IFFT_x(kappa/N (FFT_x(bB) + i k_x FFT_x(bA)))
//          rows     S0 = IFFT_y(bS)
//
// (the same arithmetic as the y-pass / x-pass sequence it replaces,
// engine.py:459-469). Every group of 16 threads owns one row in the row
// stages and one column in the column stage, so all threads run the same
// transforms and meet at every barrier. Rows are stored with the low four
// bits of y XOR-ed with the row index, which keeps both the row accesses and
// the strided column accesses free of bank conflicts.
//
// Opt-in (CG_FUSED_XY=1): on a 192^2 x 256 grid the pair takes 205 + 231 us
// against 94 + 104 us for the three-pass chains -- one 150 KB CTA per SM
// (12 warps), clusters of 8 that leave a quarter of the SMs idle, and the
// column gathers throttled in the load/store queue.
#include <cooperative_groups.h>

#include "cg_fast.cuh"
#include "cg_kspace.cuh"

namespace coop = cooperative_groups;
using cgf::fft2;
using cgf::RowEx;
using cgf::Split;
using cgf::static_for;

// cluster size per plane size: the three plane buffers and the transform
// scratch fit one CTA's shared memory
template <int N>
struct XYCluster;
template <>
struct XYCluster<64> {
  static constexpr int C = 2;
};
template <>
struct XYCluster<96> {
  static constexpr int C = 4;
};
template <>
struct XYCluster<128> {
  static constexpr int C = 8;
};
template <>
struct XYCluster<160> {
  static constexpr int C = 8;
};
template <>
struct XYCluster<192> {
  static constexpr int C = 8;
};

template <int N>
struct XYShape {
  static constexpr int C = XYCluster<N>::C, R = N / C, T = 16 * R;
  static constexpr int A = Split<N>::A, B = Split<N>::B;
  static constexpr int EX_F = RowEx<A, B>::SLAB, EX_I = RowEx<B, A>::SLAB;
  static constexpr int EX = EX_F > EX_I ? EX_F : EX_I;
  // twiddles (A, B) | twiddles (B, A) | bS | bA | bB | per-group transform scratch
  static constexpr size_t OFF_S = 2 * N, OFF_A = OFF_S + (size_t)R * N, OFF_B = OFF_A + (size_t)R * N;
  static constexpr size_t OFF_EX = OFF_B + (size_t)R * N;
  static constexpr size_t smem = sizeof(float2) * (OFF_EX + (size_t)R * EX);
  static_assert(N % C == 0 && N % 16 == 0 && Split<N>::ok, "unsupported plane size");
};

__device__ __forceinline__ int xy_swz(int r, int y) { return y ^ (r & 15); }

template <int N>
struct XYCtx {
  using X = XYShape<N>;
  static constexpr int A = X::A, B = X::B, R = X::R;
  coop::cluster_group cl;
  int rank, kz, s, g;
  float2 *tw, *twi, *bS, *bA, *bB;
  RowEx<A, B> ex;
  RowEx<B, A> exi;

  __device__ XYCtx(float2* sm, const Tables& t)
      : cl(coop::this_cluster()),
        rank((int)cl.block_rank()),
        kz((int)(blockIdx.x / X::C)),
        s(threadIdx.x & 15),
        g(threadIdx.x >> 4),
        tw(sm),
        twi(sm + N),
        bS(sm + X::OFF_S),
        bA(sm + X::OFF_A),
        bB(sm + X::OFF_B),
        ex{sm + X::OFF_EX + (threadIdx.x >> 4) * X::EX},
        exi{sm + X::OFF_EX + (threadIdx.x >> 4) * X::EX} {
    // nx == ny: the x and y twiddle tables hold the same values
    cgf::fill_twt<A, B>(tw, t.twy);
    cgf::fill_twt<B, A>(twi, t.twy);
  }

  // this group's row of a global spectrum (input distribution)
  __device__ __forceinline__ void load_row(float2 (&v)[A], const float2* __restrict__ S, long long base) const {
    static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      v[a] = (s < B) ? S[base + s + B * a] : make_float2(0.f, 0.f);
    });
  }
  __device__ __forceinline__ void store_row(float2* __restrict__ S, long long base, const float2 (&w)[B]) const {
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      S[base + s + A * b] = w[b];
    });
  }
  // this group's row of a plane buffer: output distribution in, input distribution out
  __device__ __forceinline__ void put_row(float2* buf, const float2 (&w)[B]) const {
    if (s < A) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      buf[g * N + xy_swz(g, s + A * b)] = w[b];
    });
  }
  __device__ __forceinline__ void get_row(float2 (&v)[A], const float2* buf) const {
    static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      v[a] = (s < B) ? buf[g * N + xy_swz(g, s + B * a)] : make_float2(0.f, 0.f);
    });
  }
  // column y of a plane buffer across the cluster
  __device__ __forceinline__ void gather_col(float2 (&v)[A], float2* buf, int y) {
    static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      float2 r = make_float2(0.f, 0.f);
      if (s < B) {
        const int x = s + B * a, owner = x / R, rr = x - owner * R;
        const float2* src = cl.map_shared_rank(buf, (unsigned)owner);
        r = src[rr * N + xy_swz(rr, y)];
      }
      v[a] = r;
    });
  }
  // after an inverse (B, A) transform thread s < B owns z[a] = element s + B a
  __device__ __forceinline__ void scatter_col(float2* buf, int y, const float2 (&z)[A]) {
    if (s < B) static_for<0, A>([&](auto ai) {
      constexpr int a = decltype(ai)::value;
      const int x = s + B * a, owner = x / R, rr = x - owner * R;
      float2* dst = cl.map_shared_rank(buf, (unsigned)owner);
      dst[rr * N + xy_swz(rr, y)] = z[a];
    });
  }
};

template <int N>
__global__ void __launch_bounds__(XYShape<N>::T, 1) kc_xy_grad(Dims d, Tables t, float kcoef, float invN,
                                                                float2* __restrict__ S0, float2* __restrict__ S1,
                                                                float2* __restrict__ S2) {
  using X = XYShape<N>;
  constexpr int A = X::A, B = X::B;
  extern __shared__ float2 sm[];
  XYCtx<N> c(sm, t);
  const int s = c.s;
  const long long mb = (long long)blockIdx.y * d.nspec;
  const int xr = c.rank * X::R + c.g;                 // this group's row
  const long long rbase = mb + ((long long)xr * d.nzh + c.kz) * N;
  const int y = c.rank * X::R + c.g;                  // this group's column
  __syncthreads();
  float2 v[A], w[B], z[A];
  // rows: bS = FFT_y(S0)
  c.load_row(v, S0, rbase);
  fft2<A, B, false>(v, w, s, c.tw, c.ex);
  c.put_row(c.bS, w);
  c.cl.sync();
  // columns: q = kappa/N FFT_x(bS); bA = IFFT_x(q); bB = IFFT_x(i kx q)
  c.gather_col(v, c.bS, y);
  fft2<A, B, false>(v, w, s, c.tw, c.ex);
  const float kyz2 = t.ky2[y] + t.kz2[c.kz];
  static_for<0, B>([&](auto bi) {
    constexpr int b = decltype(bi)::value;
    const int k = (s < A) ? s + A * b : 0;
    w[b] = c_scale(w[b], sinc_a2(kcoef * (t.kx2[k] + kyz2)) * invN);
  });
#pragma unroll 1
  for (int o = 0; o < 2; ++o) {
    if (o == 1) static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      const int k = (s < A) ? s + A * b : 0;
      w[b] = c_muli(c_scale(w[b], t.kx[k]));
    });
    fft2<B, A, true>(w, z, s, c.twi, c.exi);
    c.scatter_col(o == 0 ? c.bA : c.bB, y, z);
  }
  c.cl.sync();
  // rows: S1 = IFFT_y(bB); S0 = IFFT_y(i ky bA); S2 = IFFT_y(bA)
  c.get_row(v, c.bB);
  fft2<A, B, true>(v, w, s, c.tw, c.ex);
  c.store_row(S1, rbase, w);
  c.get_row(v, c.bA);
  float2 gk[A];
  static_for<0, A>([&](auto ai) {
    constexpr int a = decltype(ai)::value;
    const float k = (s < B) ? t.ky[s + B * a] : 0.f;
    gk[a] = c_muli(c_scale(v[a], k));
  });
  fft2<A, B, true>(gk, w, s, c.tw, c.ex);
  c.store_row(S0, rbase, w);
  fft2<A, B, true>(v, w, s, c.tw, c.ex);
  c.store_row(S2, rbase, w);
}

template <int N>
__global__ void __launch_bounds__(XYShape<N>::T, 1) kc_xy_div(Dims d, Tables t, float kcoef, float invN,
                                                               float2* __restrict__ S0, float2* __restrict__ S1,
                                                               float2* __restrict__ S2) {
  using X = XYShape<N>;
  constexpr int A = X::A, B = X::B;
  extern __shared__ float2 sm[];
  XYCtx<N> c(sm, t);
  const int s = c.s;
  const long long mb = (long long)blockIdx.y * d.nspec;
  const int xr = c.rank * X::R + c.g;
  const long long rbase = mb + ((long long)xr * d.nzh + c.kz) * N;
  const int y = c.rank * X::R + c.g;
  __syncthreads();
  float2 v[A], w[B], z[A], h[B];
  // rows: bA = FFT_y(S1); bB = i ky FFT_y(S0) + FFT_y(S2)
  c.load_row(v, S1, rbase);
  fft2<A, B, false>(v, w, s, c.tw, c.ex);
  c.put_row(c.bA, w);
  c.load_row(v, S0, rbase);
  fft2<A, B, false>(v, w, s, c.tw, c.ex);
  static_for<0, B>([&](auto bi) {
    constexpr int b = decltype(bi)::value;
    const float k = (s < A) ? t.ky[s + A * b] : 0.f;
    h[b] = c_muli(c_scale(w[b], k));
  });
  c.load_row(v, S2, rbase);
  fft2<A, B, false>(v, w, s, c.tw, c.ex);
  static_for<0, B>([&](auto bi) { w[decltype(bi)::value] = c_add(w[decltype(bi)::value], h[decltype(bi)::value]); });
  c.put_row(c.bB, w);
  c.cl.sync();
  // columns: bS = IFFT_x(kappa/N (FFT_x(bB) + i kx FFT_x(bA)))
  c.gather_col(v, c.bA, y);
  fft2<A, B, false>(v, w, s, c.tw, c.ex);
  static_for<0, B>([&](auto bi) { h[decltype(bi)::value] = w[decltype(bi)::value]; });
  c.gather_col(v, c.bB, y);
  fft2<A, B, false>(v, w, s, c.tw, c.ex);
  const float kyz2 = t.ky2[y] + t.kz2[c.kz];
  static_for<0, B>([&](auto bi) {
    constexpr int b = decltype(bi)::value;
    const int k = (s < A) ? s + A * b : 0;
    w[b] = c_scale(c_add(w[b], c_muli(c_scale(h[b], t.kx[k]))), sinc_a2(kcoef * (t.kx2[k] + kyz2)) * invN);
  });
  fft2<B, A, true>(w, z, s, c.twi, c.exi);
  c.scatter_col(c.bS, y, z);
  c.cl.sync();
  // rows: S0 = IFFT_y(bS)
  c.get_row(v, c.bS);
  fft2<A, B, true>(v, w, s, c.tw, c.ex);
  c.store_row(S0, rbase, w);
}

template <int N>
static cudaError_t xy_launch(bool grad, const Dims& d, const Tables& t, float kcoef, float invN, float2* S0,
                             float2* S1, float2* S2, int batch, cudaStream_t st) {
  using X = XYShape<N>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(X::C * d.nzh), (unsigned)batch, 1);
  cfg.blockDim = dim3(X::T, 1, 1);
  cfg.dynamicSmemBytes = X::smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = X::C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return grad ? cudaLaunchKernelEx(&cfg, kc_xy_grad<N>, d, t, kcoef, invN, S0, S1, S2)
              : cudaLaunchKernelEx(&cfg, kc_xy_div<N>, d, t, kcoef, invN, S0, S1, S2);
}

// Shared memory and a cluster placement check, once per size: 1 when the
// fused kernels of size N can run on this device.
template <int N>
static int xy_prepare() {
  using X = XYShape<N>;
  if (cudaFuncSetAttribute(kc_xy_grad<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)X::smem) != cudaSuccess ||
      cudaFuncSetAttribute(kc_xy_div<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)X::smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(X::C, 1, 1);
  cfg.blockDim = dim3(X::T, 1, 1);
  cfg.dynamicSmemBytes = X::smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = X::C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n1 = 0, n2 = 0;
  if (cudaOccupancyMaxActiveClusters(&n1, kc_xy_grad<N>, &cfg) != cudaSuccess ||
      cudaOccupancyMaxActiveClusters(&n2, kc_xy_div<N>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (n1 > 0 && n2 > 0) ? 1 : 0;
}

#define CG_XY_SIZES(X) X(64) X(96) X(128) X(160) X(192)

// 1 when the fused pair applies to this grid on the current device
int fused_xy_supported(const Dims& d) {
  if (d.nx != d.ny) return 0;
  switch (d.nx) {
#define CASE(n)                 \
  case n: {                     \
    static int ok = -1;         \
    if (ok < 0) ok = xy_prepare<n>(); \
    return ok;                  \
  }
    CG_XY_SIZES(CASE)
#undef CASE
    default:
      return 0;
  }
}

bool fused_xy(bool grad, const Dims& d, const Tables& t, float kcoef, float invN, float2* S0, float2* S1,
              float2* S2, int batch, cudaStream_t st) {
  if (d.nx != d.ny) return false;
  switch (d.nx) {
#define CASE(n) \
  case n:       \
    return xy_launch<n>(grad, d, t, kcoef, invN, S0, S1, S2, batch, st) == cudaSuccess;
    CG_XY_SIZES(CASE)
#undef CASE
    default:
      return false;
  }
}
