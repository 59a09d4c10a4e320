// Size-specialised y-/x-pass launchers for lengths 96, 128, 160.
#include "cg_fast_yx.cuh"

CG_YX_INSTANTIATE(96)
CG_YX_INSTANTIATE(128)
CG_YX_INSTANTIATE(160)
