// Size-specialised y-/x-pass launchers for lengths 8, 16, 24, 32, 48, 64.
#include "cg_fast_yx.cuh"

CG_YX_INSTANTIATE(8)
CG_YX_INSTANTIATE(16)
CG_YX_INSTANTIATE(24)
CG_YX_INSTANTIATE(32)
CG_YX_INSTANTIATE(48)
CG_YX_INSTANTIATE(64)
