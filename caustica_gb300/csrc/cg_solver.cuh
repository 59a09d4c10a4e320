// Host-side solver handle shared by the k-space translation units.
#pragma once

#include "cg_kspace.cuh"

struct cg_solver {
  Dims d;
  int B;
  AxisPlan px, py, pz;
  int spp, max_periods, nh, harm[CG_MAX_H];
  double kcoef;
  float invN;
  int nonlinear;
  // device memory
  float* p = nullptr;
  float* u = nullptr;
  float2* S0 = nullptr;
  float2* S1 = nullptr;
  float2* S2 = nullptr;
  float2 *twx = nullptr, *twy = nullptr, *twz = nullptr;
  float *kx = nullptr, *ky = nullptr, *kz = nullptr, *kx2 = nullptr, *ky2 = nullptr, *kz2 = nullptr;
  float *sx = nullptr, *sy = nullptr, *sz = nullptr;
  uint8_t* labels = nullptr;
  float4* ltab = nullptr;
  float *dtr = nullptr, *rc2 = nullptr, *ab = nullptr, *b2 = nullptr;
  int* src_ptr = nullptr;
  int* src_z = nullptr;
  float *src_ac = nullptr, *src_as = nullptr;
  int n_src = 0;
  float4* drive = nullptr;
  int n_drive = 0;
  float *bins = nullptr, *comp = nullptr, *pmax = nullptr;
  unsigned int* peaks = nullptr;
  int* harm_dev = nullptr;
  long long* ctl = nullptr;
  long long nrec = 0;
  int rec_lo[3], rec_hi[3], conv_lo[3], conv_hi[3];
  int has_medium = 0;
  cudaStream_t stream = nullptr;
  size_t smem_y = 0, smem_x = 0, smem_z = 0;
  int fused_xy = 0;  // the transverse passes run as two cluster launches per step
  int zpers = 1;     // persistent z-passes (where the grid allows)
  // x-slabs of the plane-local passes: > 1 runs [y, z, y] slab by slab so
  // each slab's spectra and fields stay in L2 between its three passes; the
  // pressure spectrum between steps is then y- and z-transformed
  int slabs = 1;
  // tensor-map staging of the persistent z-tiles: the encoded descriptors of
  // S1, S0, S2 (host memory; each launch passes them by value) with the
  // device flag a staging wait raises when it gives up, whether they exist
  // on this grid, and whether the step uses them
  ZTma ztma_host = {};
  int ztma_ok = 0;
  int* ztma_err = nullptr;
  int ztma = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one period, record off/on
  // phasors of the last finalize, [B][nh][nrec], kept for device post-processing
  float2* ph = nullptr;
  int ph_valid = 0;
  // post-processing scratch (focal metrics, heating coefficients), grown on demand
  void* post = nullptr;
  size_t post_bytes = 0;
};

// Grow the handle's post-processing scratch to at least `bytes`.
int cg_solver_post_scratch(cg_solver* s, size_t bytes);

