// Size-specialised pencil FFTs: register DFT codelets with compile-time
// twiddles and a two-level ("four-step") transform with one shared-memory
// exchange per pencil transform.
//
// A pencil of length N = A * B is held by B threads on input: thread s < B
// owns x[s + B a], a in [0, A). Phase 1 applies an A-point DFT in registers
// and the twiddle W_N^(s k1); the values go to shared memory as Y[k1][s];
// phase 2 thread s' < A reads Y[s'][n2], n2 in [0, B), and applies a B-point
// DFT, so thread s' ends up owning X[s' + A b], b in [0, B):
//   X[k1 + A k2] = sum_n2 W_N^(n2 k1) W_B^(n2 k2) sum_n1 x[B n1 + n2] W_A^(n1 k1).
// The output distribution of an (A, B) transform is the input distribution
// of a (B, A) transform, so a forward transform followed by an inverse one
// (or the reverse) needs no extra exchange.
//
// Register DFTs of composite size R = a b use the same decomposition inside
// one thread with compile-time twiddles W_R^m, evaluated by constexpr
// Taylor series of sin and cos (double precision, rounded once to float).
#pragma once

#include <stdlib.h>

#include <type_traits>
#include <utility>

#include "cg_common.cuh"

namespace cgf {

// ------------------------------------------------ compile-time sin/cos --
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double ct_sin_series(double x) {
  double x2 = x * x, term = x, sum = x;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}

constexpr double ct_cos_series(double x) {
  double x2 = x * x, term = 1.0, sum = 1.0;
  for (int k = 1; k < 16; ++k) {
    term *= -x2 / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}

// cos(2 pi m / R) and sin(2 pi m / R), exact at multiples of pi/2
constexpr double ct_cos2pi(int m, int R) {
  int q = ((m % R) + R) % R;
  if ((4 * q) % R == 0) {
    int quad = (4 * q) / R;
    return quad == 0 ? 1.0 : (quad == 2 ? -1.0 : 0.0);
  }
  double x = 2.0 * kPi * (double)q / (double)R;
  if (x > kPi) x -= 2.0 * kPi;
  return ct_cos_series(x);
}

constexpr double ct_sin2pi(int m, int R) {
  int q = ((m % R) + R) % R;
  if ((4 * q) % R == 0) {
    int quad = (4 * q) / R;
    return quad == 1 ? 1.0 : (quad == 3 ? -1.0 : 0.0);
  }
  double x = 2.0 * kPi * (double)q / (double)R;
  if (x > kPi) x -= 2.0 * kPi;
  return ct_sin_series(x);
}

// ------------------------------------------------------ static loops --
template <int I, int N, class F>
__host__ __device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

// v * W_R^m, forward W = exp(-2 pi i m / R), inverse its conjugate
template <int R, int M, bool INV>
__host__ __device__ __forceinline__ float2 twiddle_ct(float2 v) {
  constexpr double c = ct_cos2pi(M, R);
  constexpr double s = INV ? ct_sin2pi(M, R) : -ct_sin2pi(M, R);
  constexpr float cf = (float)c, sf = (float)s;
  if constexpr (cf == 1.0f && sf == 0.0f) return v;
  if constexpr (cf == -1.0f && sf == 0.0f) return make_float2(-v.x, -v.y);
  if constexpr (cf == 0.0f && sf == 1.0f) return make_float2(-v.y, v.x);
  if constexpr (cf == 0.0f && sf == -1.0f) return make_float2(v.y, -v.x);
  return make_float2(v.x * cf - v.y * sf, v.x * sf + v.y * cf);
}

template <bool INV>
__host__ __device__ __forceinline__ float2 rot(float2 a) {  // forward: -i a ; inverse: +i a
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

constexpr int ct_first_factor(int R) {
  return (R % 4 == 0 && R > 8) ? 4 : (R % 2 == 0 ? 2 : (R % 3 == 0 ? 3 : 5));
}

// ------------------------------------------------------- DFT codelets --
template <int R, bool INV>
struct Dft {
  static constexpr int A = ct_first_factor(R), B = R / A;
  __host__ __device__ __forceinline__ static void run(float2* v) {
    static_for<0, B>([&](auto bi) {
      constexpr int b = decltype(bi)::value;
      float2 t[A];
      static_for<0, A>([&](auto ai) { t[decltype(ai)::value] = v[B * decltype(ai)::value + b]; });
      Dft<A, INV>::run(t);
      static_for<0, A>([&](auto ai) {
        constexpr int a = decltype(ai)::value;
        v[B * a + b] = twiddle_ct<R, a * b, INV>(t[a]);
      });
    });
    static_for<0, A>([&](auto ki) { Dft<B, INV>::run(v + B * decltype(ki)::value); });
    float2 o[R];
    static_for<0, A>([&](auto k1i) {
      static_for<0, B>([&](auto k2i) {
        constexpr int k1 = decltype(k1i)::value, k2 = decltype(k2i)::value;
        o[k1 + A * k2] = v[B * k1 + k2];
      });
    });
    static_for<0, R>([&](auto i) { v[decltype(i)::value] = o[decltype(i)::value]; });
  }
};

template <bool INV>
struct Dft<1, INV> {
  __host__ __device__ __forceinline__ static void run(float2*) {}
};

template <bool INV>
struct Dft<2, INV> {
  __host__ __device__ __forceinline__ static void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = c_add(a, b);
    v[1] = c_sub(a, b);
  }
};

template <bool INV>
struct Dft<3, INV> {
  __host__ __device__ __forceinline__ static void run(float2* v) {
    const float h = 0.86602540378443864676f;
    float2 t = c_add(v[1], v[2]);
    float2 d = c_sub(v[1], v[2]);
    float2 m = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
    float2 r = rot<INV>(c_scale(d, h));
    v[0] = c_add(v[0], t);
    v[1] = c_add(m, r);
    v[2] = c_sub(m, r);
  }
};

template <bool INV>
struct Dft<4, INV> {
  __host__ __device__ __forceinline__ static void run(float2* v) {
    float2 t0 = c_add(v[0], v[2]);
    float2 t1 = c_sub(v[0], v[2]);
    float2 t2 = c_add(v[1], v[3]);
    float2 t3 = rot<INV>(c_sub(v[1], v[3]));
    v[0] = c_add(t0, t2);
    v[2] = c_sub(t0, t2);
    v[1] = c_add(t1, t3);
    v[3] = c_sub(t1, t3);
  }
};

template <bool INV>
struct Dft<5, INV> {
  __host__ __device__ __forceinline__ static void run(float2* v) {
    const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
    const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
    float2 t1 = c_add(v[1], v[4]);
    float2 t2 = c_add(v[2], v[3]);
    float2 t3 = c_sub(v[1], v[4]);
    float2 t4 = c_sub(v[2], v[3]);
    float2 y0 = c_add(v[0], c_add(t1, t2));
    float2 b1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    float2 b2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    float2 e1 = make_float2(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    float2 e2 = make_float2(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    float2 r1 = rot<INV>(e1);
    float2 r2 = rot<INV>(e2);
    v[0] = y0;
    v[1] = c_add(b1, r1);
    v[4] = c_sub(b1, r1);
    v[2] = c_add(b2, r2);
    v[3] = c_sub(b2, r2);
  }
};

template <bool INV>
struct Dft<8, INV> {
  __host__ __device__ __forceinline__ static void run(float2* v) {
    const float r2 = 0.70710678118654752440f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    o[1] = INV ? make_float2(r2 * (o[1].x - o[1].y), r2 * (o[1].x + o[1].y))
               : make_float2(r2 * (o[1].x + o[1].y), r2 * (o[1].y - o[1].x));
    o[2] = rot<INV>(o[2]);
    o[3] = INV ? make_float2(-r2 * (o[3].x + o[3].y), r2 * (o[3].x - o[3].y))
               : make_float2(r2 * (o[3].y - o[3].x), -r2 * (o[3].x + o[3].y));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = c_add(e[k], o[k]);
      v[k + 4] = c_sub(e[k], o[k]);
    }
  }
};

// ------------------------------------------------ two-level transform --
// Split of a pencil length N into (A, B): B = gcd(N, 16), A = N / B.
constexpr int ct_gcd(int a, int b) { return b == 0 ? a : ct_gcd(b, a % b); }
template <int N>
struct Split {
  static constexpr int B = ct_gcd(N, 16);
  static constexpr int A = N / B;
  static constexpr bool ok = (A <= 16);
};

// Pencil split of the size-specialised passes: (A, B) with B threads
// holding A values on input and A threads holding B values on output.
// Lengths 16 x (<= 16) use Split<N> on 16 threads per pencil; 320 = 16 x 20
// and 400 = 20 x 20 run on 20 threads per pencil, 512 = 32 x 16 (Split<512>)
// and 640 = 32 x 20 on 32.
template <int N>
struct PSplit {
  static constexpr int A = Split<N>::A, B = Split<N>::B;
  static constexpr int TPP = A > B ? A : B;  // threads per pencil
};
template <>
struct PSplit<320> {
  static constexpr int A = 16, B = 20, TPP = 20;
};
template <>
struct PSplit<400> {
  static constexpr int A = 20, B = 20, TPP = 20;
};
template <>
struct PSplit<640> {
  static constexpr int A = 32, B = 20, TPP = 32;
};

// Odd leading dimension >= n (bank-conflict-free strided access).
constexpr int ct_odd(int n) { return (n % 2) ? n : n + 1; }

// Exchange-buffer indexers. Row tiles: 16 pencils along threadIdx / 16, the
// within-pencil index s along the lanes. Column tiles: pencils along the
// lanes (threadIdx % 16).
// WARP: every thread of the pencil sits in one warp (threads per pencil
// divide 32 and pencils are consecutive in threadIdx), so the exchange of a
// pencil's own slab needs only a warp barrier. Hazards between pencils
// (staging buffers shared by a whole tile) keep their block barriers.
template <int A, int B, bool WARP = false>
struct RowEx {
  float2* base;  // this pencil's slab
  static constexpr int LD = ct_odd(B);
  static constexpr int SLAB = A * LD;
  static constexpr bool kWarp = WARP;
  __device__ __forceinline__ float2& at(int k1, int n2) const { return base[k1 * LD + n2]; }
};

template <int A, int B, int P = 16>
struct ColEx {
  float2* base;  // + lane pencil
  static constexpr int SLAB = 0;
  static constexpr bool kWarp = false;  // a column pencil spans the whole block
  __device__ __forceinline__ float2& at(int k1, int n2) const { return base[(k1 * B + n2) * P]; }
};

template <class Ex>
__device__ __forceinline__ void ex_sync() {
  if constexpr (Ex::kWarp)
    __syncwarp();
  else
    __syncthreads();
}

// Twiddle table of an (A, B) transform in the order the threads read it:
// twt[k1 * B + s] = exp(-2 pi i s k1 / N) (lanes run over s: conflict free).
template <int A, int B>
__device__ __forceinline__ void fill_twt(float2* twt, const float2* __restrict__ tw_lin) {
  for (int i = threadIdx.x; i < A * B; i += blockDim.x) {
    const int k1 = i / B, s = i - k1 * B;
    twt[i] = tw_lin[s * k1];
  }
}

// (A, B) transform of one pencil: thread s (< B) holds v[a] = x[s + B a];
// afterwards thread s (< A) holds w[b] = X[s + A b]. `twt` is the table laid
// out by fill_twt<A, B>. Every thread of the block calls it.
template <int A, int B, bool INV, class Ex>
__device__ __forceinline__ void fft2(const float2 (&v_in)[A], float2 (&w)[B], int s, const float2* __restrict__ twt,
                                     const Ex& ex) {
  if (s < B) {
    float2 v[A];
    static_for<0, A>([&](auto i) { v[decltype(i)::value] = v_in[decltype(i)::value]; });
    Dft<A, INV>::run(v);
    static_for<0, A>([&](auto ki) {
      constexpr int k1 = decltype(ki)::value;
      float2 y = v[k1];
      if constexpr (k1 > 0) {
        float2 t = twt[k1 * B + s];
        if (INV) t.y = -t.y;
        y = c_mul(y, t);
      }
      ex.at(k1, s) = y;
    });
  }
  ex_sync<Ex>();
  if (s < A) {
    static_for<0, B>([&](auto bi) { w[decltype(bi)::value] = ex.at(s, decltype(bi)::value); });
    Dft<B, INV>::run(w);
  }
  ex_sync<Ex>();
}

// Asynchronous 16-byte global -> shared copy (L2 only), completed by
// cp_async_wait0 and made visible to the block by a following barrier.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Tensor-map (TMA) copies completed on a shared-memory mbarrier. One thread
// arms the barrier with the byte count it expects and issues the copies;
// every consumer waits on the barrier's phase parity.
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase with the given parity, giving up after `limit` polls
// (each poll may suspend the thread for a short while); false when it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int limit = 1 << 20) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// generic-proxy accesses of this thread before asynchronous-proxy ones after
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
// A 3-D box of the tensor map at `map` (global memory) into shared memory at
// `dst` (aligned to the swizzle span), counted on `bar`.
__device__ __forceinline__ void tma_load_3d(void* dst, const void* map, unsigned long long* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_addr(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
      : "memory");
}

// Programmatic dependent launch: a pass lets the next one launch as soon as
// all of its own CTAs are running (pdl_trigger), and waits for the previous
// pass to complete and its writes to be visible (pdl_wait) before its first
// access to any field or spectrum; only constant tables are read before.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// Launch with programmatic stream serialisation (CG_PDL=0 turns it off).
inline bool pdl_enabled() {
  static int on = -1;
  if (on < 0) {
    const char* e = getenv("CG_PDL");
    on = (e && e[0] == '0') ? 0 : 1;
  }
  return on != 0;
}
template <typename... KArgs, typename... Args>
inline void launch(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// SM count of the current device (cached; 152 on GB300 if the query fails).
inline int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n < 1)
      n = 152;
  }
  return n;
}

// Persistent grid over `total` equal work items: about `per_sm` CTAs per SM,
// each a contiguous run of *per_cta items, none empty.
inline void persistent_grid(long long total, int per_sm, int* grid, int* per_cta) {
  const long long slots = (long long)sm_count() * per_sm;
  const long long g0 = total < slots ? total : slots;
  const long long per = (total + g0 - 1) / g0;
  *per_cta = (int)per;
  *grid = (int)((total + per - 1) / per);
}

}  // namespace cgf
