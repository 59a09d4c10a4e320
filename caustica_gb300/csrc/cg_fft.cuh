// Pencil FFT engine: mixed-radix (2,3,4,5,8) Stockham autosort on tiles of
// C pencils held in shared memory.
//
// Layout: element n of pencil c sits at buf[n * ld + c]. Consecutive lanes
// own consecutive pencils, so every stage's loads and stores are unit-stride
// across a half-warp and bank-conflict free whatever the radix pattern.
//
// Stage (Stockham, decimation in time; radix R, Ns = product of the radices
// already applied, M = N / R):
//   for j in [0, M): k = j mod Ns
//     v[q] = in[j + q M] * W_{Ns R}^{k q}        (q = 0 .. R-1)
//     v    = DFT_R(v)
//     out[(j - k) R + k + q Ns] = v[q]
// (Stockham's autosort form as given by Govindaraju et al., "High performance
// discrete Fourier transforms on graphics processors", SC 2008.)
//
// Twiddles come from one table tw[m] = exp(-2 pi i m / N), m in [0, N), built
// in FP64 on the device at set-up; W_{Ns R}^{k q} = tw[k q N / (Ns R)].
// Forward = exp(-i...), inverse = exp(+i...), both unnormalised.
#pragma once

#include "cg_common.cuh"

namespace cgfft {

template <bool INV>
__device__ __forceinline__ float2 tw_get(const float2* tw, int m) {
  float2 w = tw[m];
  return INV ? make_float2(w.x, -w.y) : w;
}

// forward: multiply by -i ; inverse: multiply by +i
template <bool INV>
__device__ __forceinline__ float2 rot90(float2 a) {
  return INV ? c_muli(a) : c_mulmi(a);
}

template <bool INV>
__device__ __forceinline__ void bfly2(float2* v) {
  float2 a = v[0], b = v[1];
  v[0] = c_add(a, b);
  v[1] = c_sub(a, b);
}

template <bool INV>
__device__ __forceinline__ void bfly3(float2* v) {
  // W3 = -1/2 -/+ i sqrt(3)/2
  const float h = 0.86602540378443864676f;
  float2 t = c_add(v[1], v[2]);
  float2 s = c_sub(v[1], v[2]);
  float2 y0 = c_add(v[0], t);
  float2 m = make_float2(v[0].x - 0.5f * t.x, v[0].y - 0.5f * t.y);
  float2 r = rot90<INV>(c_scale(s, h));  // -/+ i h s
  v[0] = y0;
  v[1] = c_add(m, r);
  v[2] = c_sub(m, r);
}

template <bool INV>
__device__ __forceinline__ void bfly4(float2* v) {
  float2 t0 = c_add(v[0], v[2]);
  float2 t1 = c_sub(v[0], v[2]);
  float2 t2 = c_add(v[1], v[3]);
  float2 t3 = rot90<INV>(c_sub(v[1], v[3]));
  v[0] = c_add(t0, t2);
  v[2] = c_sub(t0, t2);
  v[1] = c_add(t1, t3);
  v[3] = c_sub(t1, t3);
}

template <bool INV>
__device__ __forceinline__ void bfly5(float2* v) {
  // cos/sin of 2 pi/5 and 4 pi/5
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
  float2 r1 = rot90<INV>(e1);  // -/+ i e1
  float2 r2 = rot90<INV>(e2);
  v[0] = y0;
  v[1] = c_add(b1, r1);
  v[4] = c_sub(b1, r1);
  v[2] = c_add(b2, r2);
  v[3] = c_sub(b2, r2);
}

template <bool INV>
__device__ __forceinline__ void bfly8(float2* v) {
  const float r2 = 0.70710678118654752440f;
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  bfly4<INV>(e);
  bfly4<INV>(o);
  // W8^1 = (1 -/+ i)/sqrt2, W8^2 = -/+ i, W8^3 = (-1 -/+ i)/sqrt2
  float2 w1 = INV ? make_float2(r2, r2) : make_float2(r2, -r2);
  float2 w3 = INV ? make_float2(-r2, r2) : make_float2(-r2, -r2);
  o[1] = c_mul(o[1], w1);
  o[2] = rot90<INV>(o[2]);
  o[3] = c_mul(o[3], w3);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = c_add(e[k], o[k]);
    v[k + 4] = c_sub(e[k], o[k]);
  }
}

template <int R, bool INV>
__device__ __forceinline__ void bfly(float2* v) {
  if constexpr (R == 2) bfly2<INV>(v);
  else if constexpr (R == 3) bfly3<INV>(v);
  else if constexpr (R == 4) bfly4<INV>(v);
  else if constexpr (R == 5) bfly5<INV>(v);
  else bfly8<INV>(v);
}

template <int R, bool INV>
__device__ __forceinline__ void stage(const float2* __restrict__ in, float2* __restrict__ out, int ld,
                                      const float2* __restrict__ tw, int N, int Ns, int c, int g, int G) {
  const int M = N / R;
  const int tstep = N / (Ns * R);
  for (int j = g; j < M; j += G) {
    const int k = j % Ns;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = in[(j + q * M) * ld + c];
    if (Ns > 1) {
#pragma unroll
      for (int q = 1; q < R; ++q) v[q] = c_mul(v[q], tw_get<INV>(tw, k * q * tstep));
    }
    bfly<R, INV>(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) out[(base + q * Ns) * ld + c] = v[q];
  }
}

// Transform the C pencils of the tile in `a` (scratch `b`, same size).
// Every thread of the block must call it; thread (c, g) = (tid % C, tid / C).
// Returns the buffer that holds the result (a or b).
template <bool INV>
__device__ float2* tile_fft(float2* a, float2* b, int ld, const float2* __restrict__ tw, const AxisPlan& pl,
                            int c, int g, int G) {
  const int N = pl.n;
  int Ns = 1;
  for (int s = 0; s < pl.nstages; ++s) {
    const int R = pl.radix[s];
    switch (R) {
      case 8: stage<8, INV>(a, b, ld, tw, N, Ns, c, g, G); break;
      case 4: stage<4, INV>(a, b, ld, tw, N, Ns, c, g, G); break;
      case 2: stage<2, INV>(a, b, ld, tw, N, Ns, c, g, G); break;
      case 3: stage<3, INV>(a, b, ld, tw, N, Ns, c, g, G); break;
      default: stage<5, INV>(a, b, ld, tw, N, Ns, c, g, G); break;
    }
    __syncthreads();
    float2* t = a;
    a = b;
    b = t;
    Ns *= R;
  }
  return a;
}

}  // namespace cgfft
