// Pennes bioheat sub-step with CEM43 dose for GB300 (sm_103a).
//
// Reference: thermal/pennes.py:608-649 (loop body), :404-426 (faces and
// walls), thermal/dose.py:74-89 (rate). Per sub-step, for every cell:
//   work  = sum_axes [ kf_hi (th_up - th) - kf_lo (th - th_dn) ]   (faces that exist)
//         + walls (Dirichlet) + q - perf th - perf_offset
//   th'   = th + work * coeff            coeff = dt_sub / (rho C)
//   thmax = max(thmax, th')
//   dose += (R^(43 - T') + R^(43 - T)) * half_dt_min       (Kahan-compensated)
// The accumulation follows the reference's order (axis by axis: the face
// above, then the face below; walls; q; perfusion) with explicit
// round-to-nearest operations, so the temperature equals the reference's
// float32 NumPy result.
#include <stdlib.h>
#include <string.h>

#include "caustica_gb300.h"
#include "cg_common.cuh"
#include "cg_fast.cuh"

struct PennesDev {
  int nx, ny, nz;
  const float* kfx;  // [(nx-1)][ny][nz]
  const float* kfy;  // [nx][(ny-1)][nz]
  const float* kfz;  // [nx][ny][(nz-1)]
  const float* walls;  // 6 planes: x lo, x hi [ny*nz], y lo, y hi [nx*nz], z lo, z hi [nx*ny]
  const float* perf;
  const float* coeff;
  const float* q;
  const float* poff;
  int dirichlet, dose;
  float theta_wall, t_ref, half_dt_min;
  // label mode: per-material (k, dt_sub/(rho C), w_b rho_b C_b, perfusion offset)
  const uint8_t* labels;
  const float4* ltab;
  float inv_dx2;
  int has_poff;
  int wall_axes;  // label mode: bit a set when axis a has Dirichlet walls
  // label mode with at most CG_PENNES_FTAB materials: the face conductance of
  // every (lower, upper) material pair, formed once with face_k
  const float* ftab;
  int nlab;
};

#define CG_PENNES_FTAB 32

// Harmonic-mean face conductance over dx^2 with the reference's float32
// operation order: ((2 lo) hi / (lo + hi)) inv_dx2 (pennes.py:404-412).
__device__ __forceinline__ float face_k(float lo, float hi, float inv_dx2) {
  return __fmul_rn(__fdiv_rn(__fmul_rn(__fmul_rn(2.0f, lo), hi), __fadd_rn(lo, hi)), inv_dx2);
}

__device__ __forceinline__ float cem43_rate_dev(float T) {
  // R^(43 - T) with R = 0.5 above 43 C, 0.25 at or below (dose.py:74-89):
  // 0.5^e = 2^-e, 0.25^e = 2^-2e.
  float e = __fsub_rn(43.0f, T);
  return (T > 43.0f) ? exp2f(-e) : exp2f(-2.0f * e);
}

// One cell of the sub-step; (x, y, z) its coordinates, i its linear index.
__device__ __forceinline__ void pennes_cell(const PennesDev& P, const float* __restrict__ th, float* __restrict__ thn,
                                            float* thmax, float* dose, float* dcomp, const float4* tab,
                                            const float* ft, long long i, int x, int y, int z) {
  const long long sx = (long long)P.ny * P.nz, sy = P.nz;
  const float t0 = th[i];
  const bool lab = P.labels != nullptr;
  const int lme = lab ? P.labels[i] : 0;
  const float4 me = lab ? tab[lme] : make_float4(0.f, 0.f, 0.f, 0.f);
  // face conductance between lower-index material a and upper-index b
  auto fk = [&](int a, int b) {
    return ft ? ft[a * P.nlab + b] : face_k(tab[a].x, tab[b].x, P.inv_dx2);
  };
  float w = 0.0f;
  // axis x: face above (x, x+1) then face below (x-1, x)
  if (x + 1 < P.nx) {
    const float kf = lab ? fk(lme, P.labels[i + sx]) : P.kfx[((long long)x * P.ny + y) * P.nz + z];
    w = __fadd_rn(w, __fmul_rn(__fsub_rn(th[i + sx], t0), kf));
  }
  if (x > 0) {
    const float kf = lab ? fk(P.labels[i - sx], lme) : P.kfx[((long long)(x - 1) * P.ny + y) * P.nz + z];
    w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, th[i - sx]), kf));
  }
  if (y + 1 < P.ny) {
    const float kf = lab ? fk(lme, P.labels[i + sy]) : P.kfy[((long long)x * (P.ny - 1) + y) * P.nz + z];
    w = __fadd_rn(w, __fmul_rn(__fsub_rn(th[i + sy], t0), kf));
  }
  if (y > 0) {
    const float kf = lab ? fk(P.labels[i - sy], lme) : P.kfy[((long long)x * (P.ny - 1) + (y - 1)) * P.nz + z];
    w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, th[i - sy]), kf));
  }
  if (z + 1 < P.nz) {
    const float kf = lab ? fk(lme, P.labels[i + 1]) : P.kfz[((long long)x * P.ny + y) * (P.nz - 1) + z];
    w = __fadd_rn(w, __fmul_rn(__fsub_rn(th[i + 1], t0), kf));
  }
  if (z > 0) {
    const float kf = lab ? fk(P.labels[i - 1], lme) : P.kfz[((long long)x * P.ny + y) * (P.nz - 1) + (z - 1)];
    w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, th[i - 1]), kf));
  }
  if (P.dirichlet) {
    const long long pyz = (long long)P.ny * P.nz, pxz = (long long)P.nx * P.nz, pxy = (long long)P.nx * P.ny;
    const float* W = P.walls;
    const float dwall = __fsub_rn(P.theta_wall, t0);
    // 2 k_edge / dx^2 (pennes.py:414-426); label mode: walls only on the grid's own axes
    const float wk = lab ? __fmul_rn(__fmul_rn(2.0f, me.x), P.inv_dx2) : 0.f;
    const bool wx = !lab || (P.wall_axes & 1), wy = !lab || (P.wall_axes & 2), wz = !lab || (P.wall_axes & 4);
    if (wx && x == 0) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[(long long)y * P.nz + z], dwall));
    if (wx && x == P.nx - 1) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[pyz + (long long)y * P.nz + z], dwall));
    if (!lab) W += 2 * pyz;
    if (wy && y == 0) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[(long long)x * P.nz + z], dwall));
    if (wy && y == P.ny - 1) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[pxz + (long long)x * P.nz + z], dwall));
    if (!lab) W += 2 * pxz;
    if (wz && z == 0) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[(long long)x * P.ny + y], dwall));
    if (wz && z == P.nz - 1) w = __fadd_rn(w, __fmul_rn(lab ? wk : W[pxy + (long long)x * P.ny + y], dwall));
  }
  if (P.q) w = __fadd_rn(w, P.q[i]);
  if (lab) {
    if (me.z != 0.0f || P.has_poff) {
      w = __fsub_rn(w, __fmul_rn(me.z, t0));
      if (P.has_poff) w = __fsub_rn(w, me.w);
    }
    w = __fmul_rn(w, me.y);
  } else {
    if (P.perf) {
      w = __fsub_rn(w, __fmul_rn(P.perf[i], t0));
      if (P.poff) w = __fsub_rn(w, P.poff[i]);
    }
    w = __fmul_rn(w, P.coeff[i]);
  }
  const float t1 = __fadd_rn(t0, w);
  thn[i] = t1;
  const float tm = thmax[i];
  thmax[i] = (t1 > tm || t1 != t1) ? t1 : tm;
  if (P.dose) {
    const float r_new = cem43_rate_dev(__fadd_rn(t1, P.t_ref));
    const float r_old = cem43_rate_dev(__fadd_rn(t0, P.t_ref));
    const float inc = __fmul_rn(__fadd_rn(r_new, r_old), P.half_dt_min);
    // Kahan: true dose = s - c
    const float sd = dose[i], c = dcomp[i];
    const float yk = __fsub_rn(inc, c);
    const float tk = __fadd_rn(sd, yk);
    dcomp[i] = __fsub_rn(__fsub_rn(tk, sd), yk);
    dose[i] = tk;
  }
}

// One sub-step on dense per-cell coefficient maps (label media take the
// streaming kernels below). Block (32, PENNES_ROWS): each warp walks one
// (x, y) row along z, so accesses along z are coalesced and the coordinates
// need no 64-bit division; the rows of a block are consecutive in y, so the
// y-neighbours of most cells are already in L1.
#define PENNES_ROWS 8
__global__ void __launch_bounds__(32 * PENNES_ROWS) k_pennes_step(PennesDev P, const float* __restrict__ th,
                                                                  float* __restrict__ thn, float* thmax, float* dose,
                                                                  float* dcomp) {
  __shared__ float4 tab[256];
  __shared__ float ft_s[CG_PENNES_FTAB * CG_PENNES_FTAB];
  const int tid = threadIdx.y * 32 + threadIdx.x;
  if (P.labels)
    for (int i = tid; i < 256; i += 32 * PENNES_ROWS) tab[i] = P.ltab[i];
  if (P.ftab)
    for (int i = tid; i < P.nlab * P.nlab; i += 32 * PENNES_ROWS) ft_s[i] = P.ftab[i];
  __syncthreads();
  const float* ft = P.ftab ? ft_s : nullptr;
  const long long nrows = (long long)P.nx * P.ny;
  for (long long row = (long long)blockIdx.x * PENNES_ROWS + threadIdx.y; row < nrows;
       row += (long long)gridDim.x * PENNES_ROWS) {
    const int x = (int)(row / P.ny), y = (int)(row - (long long)x * P.ny);
    const long long base = row * P.nz;
    for (int z = threadIdx.x; z < P.nz; z += 32)
      pennes_cell(P, th, thn, thmax, dose, dcomp, tab, ft, base + z, x, y, z);
  }
}

// R^(43 - T) for the streaming kernel: the same exponent as cem43_rate_dev,
// 2^v by the hardware ex2.approx.f32 (PTX ISA; subnormal results kept).
__device__ __forceinline__ float cem43_rate_fast(float T) {
  const float e = __fsub_rn(43.0f, T);
  const float v = (T > 43.0f) ? -e : -2.0f * e;
  float r;
  asm("ex2.approx.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

// Label-mode sub-step that streams along x: block (PS_Z, PS_Y) owns a z-y
// tile and walks xs consecutive x planes, keeping each cell's x-1 / x / x+1
// temperatures and labels in registers and the current plane (with its
// one-cell y/z halo) in a double-buffered shared tile, so every temperature
// and label is read from memory about once and each plane needs one barrier.
// The loads are software-pipelined one plane ahead (halo, q, running maximum,
// dose and its compensation for plane x + 1, and temperature/label of plane
// x + 2 are issued before plane x is computed). FT: face conductances from
// the material-pair table; DOSE: CEM43 accumulation; DIR: Dirichlet walls.
// The temperature arithmetic is pennes_cell's, in the same order.
#define PS_Z 32
#define PS_Y 8
template <bool FT, bool DOSE, bool DIR>
__global__ void __launch_bounds__(PS_Z * PS_Y) k_pennes_stream(PennesDev P, int xs, const float* __restrict__ th,
                                                               float* __restrict__ thn, float* __restrict__ thmax,
                                                               float* __restrict__ dose, float* __restrict__ dcomp) {
  __shared__ float4 tab[256];
  __shared__ float ft_s[FT ? CG_PENNES_FTAB * CG_PENNES_FTAB : 1];
  constexpr int TW = PS_Z + 2, TS = (PS_Y + 2) * TW;  // plane tile row width and size
  __shared__ float tpl[2 * TS];
  __shared__ uint8_t lpl[2 * TS];
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * PS_Z + tz;
  for (int i = tid; i < 256; i += PS_Z * PS_Y) tab[i] = P.ltab[i];
  if (FT)
    for (int i = tid; i < P.nlab * P.nlab; i += PS_Z * PS_Y) ft_s[i] = P.ftab[i];
  const int nlab = P.nlab;
  const int z = blockIdx.x * PS_Z + tz, y = blockIdx.y * PS_Y + ty;
  const int x0 = blockIdx.z * xs, x1 = min(P.nx, x0 + xs);
  const bool in = z < P.nz && y < P.ny;
  const long long sx = (long long)P.ny * P.nz;
  const int c0 = in ? y * P.nz + z : 0;  // offset of (y, z) inside a plane
  auto fk = [&](int a, int b) { return FT ? ft_s[a * nlab + b] : face_k(tab[a].x, tab[b].x, P.inv_dx2); };
  // Halo duty of this thread: at most one y-side and one z-side neighbour
  // outside the tile (offset 0 = none) and its slot in the plane tile.
  int hy = 0, hz = 0, hys = 0, hzs = 0;
  if (in) {
    if (ty == 0 && y > 0) hy = -P.nz, hys = tz + 1;
    if (ty == PS_Y - 1 && y + 1 < P.ny) hy = P.nz, hys = (PS_Y + 1) * TW + tz + 1;
    if (tz == 0 && z > 0) hz = -1, hzs = (ty + 1) * TW;
    if (tz == PS_Z - 1 && z + 1 < P.nz) hz = 1, hzs = (ty + 1) * TW + PS_Z + 1;
  }
  const int me_s = (ty + 1) * TW + tz + 1;
  const bool ylo = y > 0, yhi = y + 1 < P.ny, zlo = z > 0, zhi = z + 1 < P.nz;
  // registers of plane x: own x-1 / x / x+1 values, halo, per-cell state
  float tp = 0.f, tc = 0.f, tn = 0.f, hyt = 0.f, hzt = 0.f, aq = 0.f, am = 0.f, ad = 0.f, ac = 0.f;
  int lp = 0, lc = 0, ln = 0, hyl = 0, hzl = 0;
  if (in) {
    const long long o = x0 * sx;
    const float* t_ = th + o;
    const uint8_t* l_ = P.labels + o;
    tc = t_[c0];
    lc = l_[c0];
    if (x0 > 0) tp = t_[c0 - sx], lp = l_[c0 - sx];
    if (x0 + 1 < P.nx) tn = t_[c0 + sx], ln = l_[c0 + sx];
    if (hy) hyt = t_[c0 + hy], hyl = l_[c0 + hy];
    if (hz) hzt = t_[c0 + hz], hzl = l_[c0 + hz];
    if (P.q) aq = P.q[o + c0];
    am = thmax[o + c0];
    if (DOSE) ad = dose[o + c0], ac = dcomp[o + c0];
  }
  for (int x = x0; x < x1; ++x) {
    // plane x and x + 1 bases are block-uniform; per-thread offsets are 32-bit
    const long long o = (long long)x * sx;
    float* tb = tpl + ((x - x0) & 1) * TS;
    uint8_t* lb = lpl + ((x - x0) & 1) * TS;
    // this buffer was last read two planes ago, before the previous barrier
    tb[me_s] = tc;
    lb[me_s] = (uint8_t)lc;
    if (hy) tb[hys] = hyt, lb[hys] = (uint8_t)hyl;
    if (hz) tb[hzs] = hzt, lb[hzs] = (uint8_t)hzl;
    __syncthreads();
    // issue plane x + 1's loads (and x + 2's temperature / label)
    float nq = 0.f, nm = 0.f, nd = 0.f, nc = 0.f, nhyt = 0.f, nhzt = 0.f, tnn = 0.f;
    int nhyl = 0, nhzl = 0, lnn = 0;
    if (in && x + 1 < x1) {
      const float* t1_ = th + (o + sx);
      const uint8_t* l1_ = P.labels + (o + sx);
      if (hy) nhyt = t1_[c0 + hy], nhyl = l1_[c0 + hy];
      if (hz) nhzt = t1_[c0 + hz], nhzl = l1_[c0 + hz];
      if (P.q) nq = (P.q + (o + sx))[c0];
      nm = (thmax + (o + sx))[c0];
      if (DOSE) nd = (dose + (o + sx))[c0], nc = (dcomp + (o + sx))[c0];
      if (x + 2 < P.nx) tnn = (t1_ + sx)[c0], lnn = (l1_ + sx)[c0];
    }
    if (in) {
      const float t0 = tc;
      const int lme = lc;
      const float4 me = tab[lme];
      float w = 0.0f;
      if (x + 1 < P.nx) w = __fadd_rn(w, __fmul_rn(__fsub_rn(tn, t0), fk(lme, ln)));
      if (x > 0) w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, tp), fk(lp, lme)));
      if (yhi) w = __fadd_rn(w, __fmul_rn(__fsub_rn(tb[me_s + TW], t0), fk(lme, lb[me_s + TW])));
      if (ylo) w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, tb[me_s - TW]), fk(lb[me_s - TW], lme)));
      if (zhi) w = __fadd_rn(w, __fmul_rn(__fsub_rn(tb[me_s + 1], t0), fk(lme, lb[me_s + 1])));
      if (zlo) w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, tb[me_s - 1]), fk(lb[me_s - 1], lme)));
      if (DIR) {
        const float dwall = __fsub_rn(P.theta_wall, t0);
        const float wk = __fmul_rn(__fmul_rn(2.0f, me.x), P.inv_dx2);
        const bool wx = P.wall_axes & 1, wy = P.wall_axes & 2, wz = P.wall_axes & 4;
        if (wx && x == 0) w = __fadd_rn(w, __fmul_rn(wk, dwall));
        if (wx && x == P.nx - 1) w = __fadd_rn(w, __fmul_rn(wk, dwall));
        if (wy && !ylo) w = __fadd_rn(w, __fmul_rn(wk, dwall));
        if (wy && !yhi) w = __fadd_rn(w, __fmul_rn(wk, dwall));
        if (wz && !zlo) w = __fadd_rn(w, __fmul_rn(wk, dwall));
        if (wz && !zhi) w = __fadd_rn(w, __fmul_rn(wk, dwall));
      }
      if (P.q) w = __fadd_rn(w, aq);
      if (me.z != 0.0f || P.has_poff) {
        w = __fsub_rn(w, __fmul_rn(me.z, t0));
        if (P.has_poff) w = __fsub_rn(w, me.w);
      }
      w = __fmul_rn(w, me.y);
      const float t1 = __fadd_rn(t0, w);
      (thn + o)[c0] = t1;
      (thmax + o)[c0] = (t1 > am || t1 != t1) ? t1 : am;
      if (DOSE) {
        const float r_new = cem43_rate_fast(__fadd_rn(t1, P.t_ref));
        const float r_old = cem43_rate_fast(__fadd_rn(t0, P.t_ref));
        const float inc = __fmul_rn(__fadd_rn(r_new, r_old), P.half_dt_min);
        const float yk = __fsub_rn(inc, ac);
        const float tk = __fadd_rn(ad, yk);
        (dcomp + o)[c0] = __fsub_rn(__fsub_rn(tk, ad), yk);
        (dose + o)[c0] = tk;
      }
    }
    // rotate to plane x + 1
    tp = tc, lp = lc, tc = tn, lc = ln, tn = tnn, ln = lnn;
    hyt = nhyt, hyl = nhyl, hzt = nhzt, hzl = nhzl;
    aq = nq, am = nm, ad = nd, ac = nc;
  }
}

// The streaming sub-step for an even nz: each thread owns a z-pair of cells,
// so per-cell state moves as float2 (labels as a 16-bit pair) and a cell's
// z-neighbour inside the pair is a register. Block (PP_Z, PP_Y) covers 2 PP_Z
// z by PP_Y y; the shared plane tile keeps the pair columns 8-byte aligned
// (interior from column 2, halo columns 1 and 2 PP_Z + 2). Per cell the
// arithmetic is pennes_cell's, in the same order.
#define PP_Z 16
#define PP_Y 16
template <bool FT, bool DOSE, bool DIR>
__global__ void __launch_bounds__(PP_Z * PP_Y) k_pennes_stream2(PennesDev P, int xs, const float* __restrict__ th,
                                                                float* __restrict__ thn, float* __restrict__ thmax,
                                                                float* __restrict__ dose, float* __restrict__ dcomp) {
  __shared__ float4 tab[256];
  __shared__ float ft_s[FT ? CG_PENNES_FTAB * CG_PENNES_FTAB : 1];
  constexpr int TW = 2 * PP_Z + 4, TS = (PP_Y + 2) * TW;  // plane tile row width and size
  __shared__ __align__(16) float tpl[2 * TS];
  __shared__ __align__(16) uint8_t lpl[2 * TS];
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * PP_Z + tz;
  for (int i = tid; i < 256; i += PP_Z * PP_Y) tab[i] = P.ltab[i];
  if (FT)
    for (int i = tid; i < P.nlab * P.nlab; i += PP_Z * PP_Y) ft_s[i] = P.ftab[i];
  const int nlab = P.nlab;
  const int z = blockIdx.x * 2 * PP_Z + 2 * tz, y = blockIdx.y * PP_Y + ty;
  const int x0 = blockIdx.z * xs, x1 = min(P.nx, x0 + xs);
  const bool in = z < P.nz && y < P.ny;  // nz is even, so z + 1 < nz too
  const long long sx = (long long)P.ny * P.nz;
  const int c0 = in ? y * P.nz + z : 0;  // offset of (y, z) inside a plane (even)
  auto fk = [&](int a, int b) { return FT ? ft_s[a * nlab + b] : face_k(tab[a].x, tab[b].x, P.inv_dx2); };
  auto ld2 = [](const float* p) { return *reinterpret_cast<const float2*>(p); };
  auto ldl = [](const uint8_t* p) { return (int)*reinterpret_cast<const uint16_t*>(p); };
  // Halo duty: at most one y-side pair and one z-side cell outside the tile
  // (offset 0 = none) and its slot in the plane tile.
  int hy = 0, hz = 0, hys = 0, hzs = 0;
  if (in) {
    if (ty == 0 && y > 0) hy = -P.nz, hys = 2 + 2 * tz;
    if (ty == PP_Y - 1 && y + 1 < P.ny) hy = P.nz, hys = (PP_Y + 1) * TW + 2 + 2 * tz;
    if (tz == 0 && z > 0) hz = -1, hzs = (ty + 1) * TW + 1;
    if (tz == PP_Z - 1 && z + 2 < P.nz) hz = 2, hzs = (ty + 1) * TW + 2 * PP_Z + 2;
  }
  const int me_s = (ty + 1) * TW + 2 + 2 * tz;
  const bool ylo = y > 0, yhi = y + 1 < P.ny, zlo = z > 0, zhi = z + 2 < P.nz;
  float2 tp = {0.f, 0.f}, tc = {0.f, 0.f}, tn = {0.f, 0.f}, hyt = {0.f, 0.f}, aq = {0.f, 0.f}, am = {0.f, 0.f},
         ad = {0.f, 0.f}, ac = {0.f, 0.f};
  float hzt = 0.f;
  int lp = 0, lc = 0, ln = 0, hyl = 0, hzl = 0;  // label pairs: low byte = cell z
  if (in) {
    const long long o = x0 * sx;
    const float* t_ = th + o;
    const uint8_t* l_ = P.labels + o;
    tc = ld2(t_ + c0);
    lc = ldl(l_ + c0);
    if (x0 > 0) tp = ld2(t_ + (c0 - sx)), lp = ldl(l_ + (c0 - sx));
    if (x0 + 1 < P.nx) tn = ld2(t_ + (c0 + sx)), ln = ldl(l_ + (c0 + sx));
    if (hy) hyt = ld2(t_ + (c0 + hy)), hyl = ldl(l_ + (c0 + hy));
    if (hz) hzt = t_[c0 + hz], hzl = l_[c0 + hz];
    if (P.q) aq = ld2(P.q + (o + c0));
    am = ld2(thmax + (o + c0));
    if (DOSE) ad = ld2(dose + (o + c0)), ac = ld2(dcomp + (o + c0));
  }
  for (int x = x0; x < x1; ++x) {
    const long long o = (long long)x * sx;
    float* tb = tpl + ((x - x0) & 1) * TS;
    uint8_t* lb = lpl + ((x - x0) & 1) * TS;
    // this buffer was last read two planes ago, before the previous barrier
    *reinterpret_cast<float2*>(tb + me_s) = tc;
    *reinterpret_cast<uint16_t*>(lb + me_s) = (uint16_t)lc;
    if (hy) *reinterpret_cast<float2*>(tb + hys) = hyt, *reinterpret_cast<uint16_t*>(lb + hys) = (uint16_t)hyl;
    if (hz) tb[hzs] = hzt, lb[hzs] = (uint8_t)hzl;
    __syncthreads();
    // issue plane x + 1's loads (and x + 2's temperature / labels)
    float2 nq = {0.f, 0.f}, nm = {0.f, 0.f}, nd = {0.f, 0.f}, nc = {0.f, 0.f}, nhyt = {0.f, 0.f}, tnn = {0.f, 0.f};
    float nhzt = 0.f;
    int nhyl = 0, nhzl = 0, lnn = 0;
    if (in && x + 1 < x1) {
      const float* t1_ = th + (o + sx);
      const uint8_t* l1_ = P.labels + (o + sx);
      if (hy) nhyt = ld2(t1_ + (c0 + hy)), nhyl = ldl(l1_ + (c0 + hy));
      if (hz) nhzt = t1_[c0 + hz], nhzl = l1_[c0 + hz];
      if (P.q) nq = ld2(P.q + (o + sx) + c0);
      nm = ld2(thmax + (o + sx) + c0);
      if (DOSE) nd = ld2(dose + (o + sx) + c0), nc = ld2(dcomp + (o + sx) + c0);
      if (x + 2 < P.nx) tnn = ld2(t1_ + sx + c0), lnn = ldl(l1_ + sx + c0);
    }
    if (in) {
      const float2 tyh = ld2(tb + me_s + TW), tyl = ld2(tb + me_s - TW);
      const int lyh = ldl(lb + me_s + TW), lyl = ldl(lb + me_s - TW);
      float r[2];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int sh = 8 * k;
        const float t0 = k ? tc.y : tc.x;
        const int lme = (lc >> sh) & 0xff;
        const float4 me = tab[lme];
        float w = 0.0f;
        if (x + 1 < P.nx) w = __fadd_rn(w, __fmul_rn(__fsub_rn(k ? tn.y : tn.x, t0), fk(lme, (ln >> sh) & 0xff)));
        if (x > 0) w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, k ? tp.y : tp.x), fk((lp >> sh) & 0xff, lme)));
        if (yhi) w = __fadd_rn(w, __fmul_rn(__fsub_rn(k ? tyh.y : tyh.x, t0), fk(lme, (lyh >> sh) & 0xff)));
        if (ylo) w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, k ? tyl.y : tyl.x), fk((lyl >> sh) & 0xff, lme)));
        if (k == 0) {
          // z + 1 is the pair's other cell; z - 1 comes from the tile
          w = __fadd_rn(w, __fmul_rn(__fsub_rn(tc.y, t0), fk(lme, (lc >> 8) & 0xff)));
          if (zlo) w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, tb[me_s - 1]), fk(lb[me_s - 1], lme)));
        } else {
          if (zhi) w = __fadd_rn(w, __fmul_rn(__fsub_rn(tb[me_s + 2], t0), fk(lme, lb[me_s + 2])));
          w = __fsub_rn(w, __fmul_rn(__fsub_rn(t0, tc.x), fk(lc & 0xff, lme)));
        }
        if (DIR) {
          const float dwall = __fsub_rn(P.theta_wall, t0);
          const float wk = __fmul_rn(__fmul_rn(2.0f, me.x), P.inv_dx2);
          const bool wx = P.wall_axes & 1, wy = P.wall_axes & 2, wz = P.wall_axes & 4;
          if (wx && x == 0) w = __fadd_rn(w, __fmul_rn(wk, dwall));
          if (wx && x == P.nx - 1) w = __fadd_rn(w, __fmul_rn(wk, dwall));
          if (wy && !ylo) w = __fadd_rn(w, __fmul_rn(wk, dwall));
          if (wy && !yhi) w = __fadd_rn(w, __fmul_rn(wk, dwall));
          if (wz && k == 0 && !zlo) w = __fadd_rn(w, __fmul_rn(wk, dwall));
          if (wz && k == 1 && !zhi) w = __fadd_rn(w, __fmul_rn(wk, dwall));
        }
        if (P.q) w = __fadd_rn(w, k ? aq.y : aq.x);
        if (me.z != 0.0f || P.has_poff) {
          w = __fsub_rn(w, __fmul_rn(me.z, t0));
          if (P.has_poff) w = __fsub_rn(w, me.w);
        }
        w = __fmul_rn(w, me.y);
        r[k] = __fadd_rn(t0, w);
      }
      *reinterpret_cast<float2*>(thn + o + c0) = make_float2(r[0], r[1]);
      *reinterpret_cast<float2*>(thmax + o + c0) = make_float2((r[0] > am.x || r[0] != r[0]) ? r[0] : am.x,
                                                               (r[1] > am.y || r[1] != r[1]) ? r[1] : am.y);
      if (DOSE) {
        float nds[2], ncs[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const float r_new = cem43_rate_fast(__fadd_rn(r[k], P.t_ref));
          const float r_old = cem43_rate_fast(__fadd_rn(k ? tc.y : tc.x, P.t_ref));
          const float inc = __fmul_rn(__fadd_rn(r_new, r_old), P.half_dt_min);
          const float sd = k ? ad.y : ad.x, cc = k ? ac.y : ac.x;
          const float yk = __fsub_rn(inc, cc);
          const float tk = __fadd_rn(sd, yk);
          ncs[k] = __fsub_rn(__fsub_rn(tk, sd), yk);
          nds[k] = tk;
        }
        *reinterpret_cast<float2*>(dcomp + o + c0) = make_float2(ncs[0], ncs[1]);
        *reinterpret_cast<float2*>(dose + o + c0) = make_float2(nds[0], nds[1]);
      }
    }
    // rotate to plane x + 1
    tp = tc, lp = lc, tc = tn, lc = ln, tn = tnn, ln = lnn;
    hyt = nhyt, hyl = nhyl, hzt = nhzt, hzl = nhzl;
    aq = nq, am = nm, ad = nd, ac = nc;
  }
}

template <bool FT, bool DOSE, bool DIR>
static void launch_stream_k(bool pair, const PennesDev& P, dim3 g, dim3 b, cudaStream_t st, int xs, const float* th,
                            float* thn, float* thmax, float* dose, float* dcomp) {
  if (pair)
    k_pennes_stream2<FT, DOSE, DIR><<<g, b, 0, st>>>(P, xs, th, thn, thmax, dose, dcomp);
  else
    k_pennes_stream<FT, DOSE, DIR><<<g, b, 0, st>>>(P, xs, th, thn, thmax, dose, dcomp);
}

template <bool FT, bool DOSE>
static void launch_stream_dir(bool pair, const PennesDev& P, dim3 g, dim3 b, cudaStream_t st, int xs,
                              const float* th, float* thn, float* thmax, float* dose, float* dcomp) {
  if (P.dirichlet)
    launch_stream_k<FT, DOSE, true>(pair, P, g, b, st, xs, th, thn, thmax, dose, dcomp);
  else
    launch_stream_k<FT, DOSE, false>(pair, P, g, b, st, xs, th, thn, thmax, dose, dcomp);
}

static void launch_stream(bool pair, const PennesDev& P, dim3 g, dim3 b, cudaStream_t st, int xs, const float* th,
                          float* thn, float* thmax, float* dose, float* dcomp) {
  if (P.ftab) {
    if (P.dose)
      launch_stream_dir<true, true>(pair, P, g, b, st, xs, th, thn, thmax, dose, dcomp);
    else
      launch_stream_dir<true, false>(pair, P, g, b, st, xs, th, thn, thmax, dose, dcomp);
  } else {
    if (P.dose)
      launch_stream_dir<false, true>(pair, P, g, b, st, xs, th, thn, thmax, dose, dcomp);
    else
      launch_stream_dir<false, false>(pair, P, g, b, st, xs, th, thn, thmax, dose, dcomp);
  }
}

// Face conductances of every (lower, upper) material pair (label mode).
__global__ void k_pennes_faces(const float4* ltab, int n, float inv_dx2, float* ftab) {
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) ftab[i] = face_k(ltab[i / n].x, ltab[i % n].x, inv_dx2);
}

// flag bit 0 cleared: a non-finite temperature; bit 1 cleared: a non-finite dose
__global__ void k_pennes_finite(const float* th, const float* dose, long long n, int* flag) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (!isfinite(th[i])) atomicAnd(flag, ~1);
    if (dose && !isfinite(dose[i])) atomicAnd(flag, ~2);
  }
}

struct cg_pennes {
  cg_pennes_config cfg;
  long long ncell;
  float* th[2] = {nullptr, nullptr};
  int cur = 0;
  float* thmax = nullptr;
  float* dose = nullptr;
  float* dcomp = nullptr;
  float *kfx = nullptr, *kfy = nullptr, *kfz = nullptr, *walls = nullptr;
  float *perf = nullptr, *coeff = nullptr, *q = nullptr, *poff = nullptr;
  int* flag = nullptr;
  uint8_t* labels = nullptr;
  float4* ltab = nullptr;
  float* ftab = nullptr;
  int nlab = 0;
  float inv_dx2 = 0.f;
  int lab_poff = 0, wall_axes = 7;
  int has_coef = 0, has_state = 0;
  cudaStream_t stream = nullptr;
};

static void pennes_free(cg_pennes* h) {
  if (!h) return;
  void* ptrs[] = {h->th[0], h->th[1], h->thmax, h->dose, h->dcomp, h->kfx, h->kfy, h->kfz,
                  h->walls, h->perf, h->coeff, h->q, h->poff, h->flag, h->labels, h->ltab, h->ftab};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

static int palloc(float** p, long long n) {
  if (n < 1) n = 1;
  cudaError_t e = cudaMalloc((void**)p, sizeof(float) * (size_t)n);
  if (e != cudaSuccess) {
    cg_set_error("cudaMalloc of %lld floats failed: %s", n, cudaGetErrorString(e));
    *p = nullptr;
    return CG_ERR_OOM;
  }
  return CG_OK;
}

extern "C" int cg_pennes_create(const cg_pennes_config* cfg, cg_pennes** out) {
  CG_REQUIRE(cfg && out, "null argument");
  *out = nullptr;
  CG_REQUIRE(cfg->nx >= 1 && cfg->ny >= 1 && cfg->nz >= 1, "invalid thermal grid %dx%dx%d", cfg->nx, cfg->ny, cfg->nz);
  // the streaming kernels address a cell inside its x plane with 32-bit offsets
  CG_REQUIRE((long long)cfg->ny * cfg->nz < (1LL << 31), "thermal grid %dx%dx%d: an x plane (ny x nz) must hold "
             "fewer than 2^31 cells", cfg->nx, cfg->ny, cfg->nz);
  cg_pennes* h = new cg_pennes();
  h->cfg = *cfg;
  const long long nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
  h->ncell = nx * ny * nz;
  int rc = CG_OK;
  if ((rc = palloc(&h->th[0], h->ncell)) || (rc = palloc(&h->th[1], h->ncell)) || (rc = palloc(&h->thmax, h->ncell)) ||
      (rc = palloc(&h->dose, h->ncell)) || (rc = palloc(&h->dcomp, h->ncell)) ||
      (rc = palloc(&h->kfx, (nx - 1) * ny * nz)) || (rc = palloc(&h->kfy, nx * (ny - 1) * nz)) ||
      (rc = palloc(&h->kfz, nx * ny * (nz - 1))) || (rc = palloc(&h->walls, 2 * (ny * nz + nx * nz + nx * ny))) ||
      (rc = palloc(&h->perf, h->ncell)) || (rc = palloc(&h->coeff, h->ncell)) || (rc = palloc(&h->q, h->ncell)) ||
      (rc = palloc(&h->poff, h->ncell))) {
    pennes_free(h);
    return rc;
  }
  cudaError_t e = cudaMalloc((void**)&h->flag, sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    cg_set_error("pennes set-up: %s", cudaGetErrorString(e));
    pennes_free(h);
    return CG_ERR_CUDA;
  }
  *out = h;
  return CG_OK;
}

extern "C" int cg_pennes_destroy(cg_pennes* h) {
  if (h) {
    cudaStreamSynchronize(h->stream);
    pennes_free(h);
  }
  return CG_OK;
}

static int copy_opt(float* dst, const float* src, long long n, int* present, cudaStream_t st) {
  *present = src != nullptr;
  if (!src || n <= 0) return CG_OK;
  CG_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(float) * (size_t)n, cudaMemcpyDefault, st));
  return CG_OK;
}

extern "C" int cg_pennes_set_coefficients(cg_pennes* h, const float* kf_x, const float* kf_y, const float* kf_z,
                                          const float* walls, const float* perf, const float* coeff,
                                          const float* q, const float* perf_offset) {
  CG_REQUIRE(h && coeff, "null argument");
  const long long nx = h->cfg.nx, ny = h->cfg.ny, nz = h->cfg.nz;
  CG_REQUIRE(nx == 1 || kf_x, "kf_x is required when nx > 1");
  CG_REQUIRE(ny == 1 || kf_y, "kf_y is required when ny > 1");
  CG_REQUIRE(nz == 1 || kf_z, "kf_z is required when nz > 1");
  CG_REQUIRE(!h->cfg.dirichlet || walls, "a Dirichlet solve needs the wall planes");
  int pr = 0, has_walls = 0, has_perf = 0, has_q = 0, has_poff = 0;
  int rc;
  if ((rc = copy_opt(h->kfx, kf_x, (nx - 1) * ny * nz, &pr, h->stream)) ||
      (rc = copy_opt(h->kfy, kf_y, nx * (ny - 1) * nz, &pr, h->stream)) ||
      (rc = copy_opt(h->kfz, kf_z, nx * ny * (nz - 1), &pr, h->stream)) ||
      (rc = copy_opt(h->walls, walls, 2 * (ny * nz + nx * nz + nx * ny), &has_walls, h->stream)) ||
      (rc = copy_opt(h->perf, perf, h->ncell, &has_perf, h->stream)) ||
      (rc = copy_opt(h->coeff, coeff, h->ncell, &pr, h->stream)) ||
      (rc = copy_opt(h->q, q, h->ncell, &has_q, h->stream)) ||
      (rc = copy_opt(h->poff, perf_offset, h->ncell, &has_poff, h->stream)))
    return rc;
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->has_coef = 1 | (has_perf << 1) | (has_q << 2) | (has_poff << 3);
  return CG_OK;
}

extern "C" int cg_pennes_set_labels(cg_pennes* h, const uint8_t* labels, int n_labels, const float* table,
                                     float inv_dx2, int has_perf_offset, int wall_axes, const float* q) {
  CG_REQUIRE(h && labels && table, "null argument");
  CG_REQUIRE(n_labels >= 1 && n_labels <= 256, "n_labels must be 1..256, got %d", n_labels);
  if (!h->labels) {
    CG_CUDA_TRY(cudaMalloc((void**)&h->labels, (size_t)h->ncell));
    CG_CUDA_TRY(cudaMalloc((void**)&h->ltab, 256 * sizeof(float4)));
    CG_CUDA_TRY(cudaMalloc((void**)&h->ftab, sizeof(float) * CG_PENNES_FTAB * CG_PENNES_FTAB));
  }
  float4 tab[256];
  memset(tab, 0, sizeof(tab));
  for (int i = 0; i < n_labels; ++i) tab[i] = make_float4(table[4 * i], table[4 * i + 1], table[4 * i + 2], table[4 * i + 3]);
  CG_CUDA_TRY(cudaMemcpyAsync(h->labels, labels, (size_t)h->ncell, cudaMemcpyDefault, h->stream));
  CG_CUDA_TRY(cudaMemcpyAsync(h->ltab, tab, sizeof(tab), cudaMemcpyHostToDevice, h->stream));
  if (q) CG_CUDA_TRY(cudaMemcpyAsync(h->q, q, sizeof(float) * (size_t)h->ncell, cudaMemcpyDefault, h->stream));
  h->nlab = n_labels <= CG_PENNES_FTAB ? n_labels : 0;
  if (h->nlab) k_pennes_faces<<<1, 256, 0, h->stream>>>(h->ltab, h->nlab, inv_dx2, h->ftab);
  CG_CUDA_TRY(cudaGetLastError());
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->inv_dx2 = inv_dx2;
  h->lab_poff = has_perf_offset;
  h->wall_axes = wall_axes;
  h->has_coef = 1 | (q ? 4 : 0);
  return CG_OK;
}

extern "C" int cg_pennes_set_state(cg_pennes* h, const float* theta, const float* theta_max, const float* dose) {
  CG_REQUIRE(h && theta && theta_max, "null argument");
  const size_t n = (size_t)h->ncell;
  h->cur = 0;
  CG_CUDA_TRY(cudaMemcpyAsync(h->th[0], theta, 4 * n, cudaMemcpyDefault, h->stream));
  CG_CUDA_TRY(cudaMemcpyAsync(h->thmax, theta_max, 4 * n, cudaMemcpyDefault, h->stream));
  if (dose) CG_CUDA_TRY(cudaMemcpyAsync(h->dose, dose, 4 * n, cudaMemcpyDefault, h->stream));
  else CG_CUDA_TRY(cudaMemsetAsync(h->dose, 0, 4 * n, h->stream));
  CG_CUDA_TRY(cudaMemsetAsync(h->dcomp, 0, 4 * n, h->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->has_state = 1;
  return CG_OK;
}

// dst = src + off (float32, round to nearest; off = -t_ref gives the host's
// float32 T - t_ref bit for bit, off = +t_ref its theta + t_ref); dst2 gets a copy.
__global__ void k_pennes_offset(const float* __restrict__ src, float* __restrict__ dst, float* __restrict__ dst2,
                                long long n, float off) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = __fadd_rn(src[i], off);
    dst[i] = v;
    if (dst2) dst2[i] = v;
  }
}

extern "C" int cg_pennes_set_temperature(cg_pennes* h, const float* T, const float* dose, int* finite) {
  CG_REQUIRE(h && T && finite, "null argument");
  const size_t n = (size_t)h->ncell;
  h->cur = 0;
  // T lands in the second state buffer, theta = T - t_ref in the first and in theta_max
  CG_CUDA_TRY(cudaMemcpyAsync(h->th[1], T, 4 * n, cudaMemcpyDefault, h->stream));
  k_pennes_offset<<<2048, 256, 0, h->stream>>>(h->th[1], h->th[0], h->thmax, h->ncell, -h->cfg.t_ref);
  CG_CUDA_TRY(cudaGetLastError());
  if (dose) CG_CUDA_TRY(cudaMemcpyAsync(h->dose, dose, 4 * n, cudaMemcpyDefault, h->stream));
  else CG_CUDA_TRY(cudaMemsetAsync(h->dose, 0, 4 * n, h->stream));
  CG_CUDA_TRY(cudaMemsetAsync(h->dcomp, 0, 4 * n, h->stream));
  const int all = 3;
  CG_CUDA_TRY(cudaMemcpyAsync(h->flag, &all, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  k_pennes_finite<<<1024, 256, 0, h->stream>>>(h->th[0], nullptr, h->ncell, h->flag);
  CG_CUDA_TRY(cudaGetLastError());
  int v = 0;
  CG_CUDA_TRY(cudaMemcpyAsync(&v, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  *finite = v & 1;
  h->has_state = 1;
  return CG_OK;
}

static PennesDev make_dev(const cg_pennes* h) {
  PennesDev P;
  P.nx = h->cfg.nx; P.ny = h->cfg.ny; P.nz = h->cfg.nz;
  P.kfx = h->kfx; P.kfy = h->kfy; P.kfz = h->kfz; P.walls = h->walls;
  P.perf = (h->has_coef & 2) ? h->perf : nullptr;
  P.coeff = h->coeff;
  P.q = (h->has_coef & 4) ? h->q : nullptr;
  P.poff = (h->has_coef & 8) ? h->poff : nullptr;
  P.dirichlet = h->cfg.dirichlet;
  P.dose = h->cfg.dose;
  P.theta_wall = h->cfg.theta_wall;
  P.t_ref = h->cfg.t_ref;
  P.half_dt_min = h->cfg.half_dt_min;
  P.labels = h->labels;
  P.ltab = h->ltab;
  P.inv_dx2 = h->inv_dx2;
  P.has_poff = h->lab_poff;
  P.wall_axes = h->wall_axes;
  P.ftab = (h->labels && h->nlab) ? h->ftab : nullptr;
  P.nlab = h->nlab;
  return P;
}

extern "C" int cg_pennes_run(cg_pennes* h, int n_sub) {
  CG_REQUIRE(h, "null handle");
  CG_REQUIRE(h->has_coef && h->has_state, "set coefficients and state before running");
  CG_REQUIRE(n_sub >= 0, "n_sub must be >= 0");
  const PennesDev P = make_dev(h);
  const dim3 block(32, PENNES_ROWS);
  long long blocks = ((long long)h->cfg.nx * h->cfg.ny + PENNES_ROWS - 1) / PENNES_ROWS;
  if (blocks > 152 * 64) blocks = 152 * 64;
  // label mode streams along x; z-pairs when nz is even (CG_PENNES_PAIR=0
  // keeps single cells). x planes per block: 16, or 8 when 16 leaves fewer
  // than four waves of 4 resident blocks on every SM (CG_PENNES_XS pins it).
  static const int xs_pin = [] {
    const char* e = getenv("CG_PENNES_XS");
    return e ? atoi(e) : 0;
  }();
  static const bool pair_ok = [] {
    const char* e = getenv("CG_PENNES_PAIR");
    return !(e && atoi(e) == 0);
  }();
  const bool pair = pair_ok && h->cfg.nz % 2 == 0;
  const int tzc = pair ? 2 * PP_Z : PS_Z, tyc = pair ? PP_Y : PS_Y;
  const dim3 sblock(pair ? PP_Z : PS_Z, tyc);
  const long long tiles_zy = (long long)((h->cfg.nz + tzc - 1) / tzc) * ((h->cfg.ny + tyc - 1) / tyc);
  const int xs = xs_pin > 0 ? xs_pin : (tiles_zy * ((h->cfg.nx + 15) / 16) >= 4LL * 4 * cgf::sm_count() ? 16 : 8);
  const dim3 sgrid((unsigned)((h->cfg.nz + tzc - 1) / tzc), (unsigned)((h->cfg.ny + tyc - 1) / tyc),
                   (unsigned)((h->cfg.nx + xs - 1) / xs));
  for (int i = 0; i < n_sub; ++i) {
    if (P.labels)
      launch_stream(pair, P, sgrid, sblock, h->stream, xs, h->th[h->cur], h->th[1 - h->cur], h->thmax, h->dose, h->dcomp);
    else
      k_pennes_step<<<(unsigned)blocks, block, 0, h->stream>>>(P, h->th[h->cur], h->th[1 - h->cur], h->thmax,
                                                               h->dose, h->dcomp);
    h->cur = 1 - h->cur;
  }
  CG_CUDA_TRY(cudaGetLastError());
  return CG_OK;
}

extern "C" int cg_pennes_timed_run(cg_pennes* h, int n_sub, float* ms) {
  CG_REQUIRE(h && ms, "null argument");
  cudaEvent_t a, b;
  CG_CUDA_TRY(cudaEventCreate(&a));
  CG_CUDA_TRY(cudaEventCreate(&b));
  CG_CUDA_TRY(cudaEventRecord(a, h->stream));
  const int rc = cg_pennes_run(h, n_sub);
  CG_CUDA_TRY(cudaEventRecord(b, h->stream));
  CG_CUDA_TRY(cudaEventSynchronize(b));
  CG_CUDA_TRY(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return rc;
}

extern "C" int cg_pennes_check_finite(cg_pennes* h, int* finite) {
  CG_REQUIRE(h && finite, "null argument");
  const int one = 3;
  CG_CUDA_TRY(cudaMemcpyAsync(h->flag, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  k_pennes_finite<<<1024, 256, 0, h->stream>>>(h->th[h->cur], h->cfg.dose ? h->dose : nullptr, h->ncell, h->flag);
  CG_CUDA_TRY(cudaGetLastError());
  int v = 0;
  CG_CUDA_TRY(cudaMemcpyAsync(&v, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  *finite = v;
  return CG_OK;
}

extern "C" int cg_pennes_get_temperature(cg_pennes* h, float* T, float* T_max, float* dose) {
  CG_REQUIRE(h, "null handle");
  const size_t n = (size_t)h->ncell;
  float* scratch = h->th[1 - h->cur];  // rewritten in full by the next sub-step
  if (T) {
    k_pennes_offset<<<2048, 256, 0, h->stream>>>(h->th[h->cur], scratch, nullptr, h->ncell, h->cfg.t_ref);
    CG_CUDA_TRY(cudaGetLastError());
    CG_CUDA_TRY(cudaMemcpyAsync(T, scratch, 4 * n, cudaMemcpyDefault, h->stream));
  }
  if (T_max) {
    k_pennes_offset<<<2048, 256, 0, h->stream>>>(h->thmax, scratch, nullptr, h->ncell, h->cfg.t_ref);
    CG_CUDA_TRY(cudaGetLastError());
    CG_CUDA_TRY(cudaMemcpyAsync(T_max, scratch, 4 * n, cudaMemcpyDefault, h->stream));
  }
  if (dose) CG_CUDA_TRY(cudaMemcpyAsync(dose, h->dose, 4 * n, cudaMemcpyDefault, h->stream));
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return CG_OK;
}

extern "C" int cg_pennes_get_state(cg_pennes* h, float* theta, float* theta_max, float* dose) {
  CG_REQUIRE(h, "null handle");
  const size_t n = (size_t)h->ncell;
  CG_CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (theta) CG_CUDA_TRY(cudaMemcpy(theta, h->th[h->cur], 4 * n, cudaMemcpyDefault));
  if (theta_max) CG_CUDA_TRY(cudaMemcpy(theta_max, h->thmax, 4 * n, cudaMemcpyDefault));
  if (dose) CG_CUDA_TRY(cudaMemcpy(dose, h->dose, 4 * n, cudaMemcpyDefault));
  return CG_OK;
}
