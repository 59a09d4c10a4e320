// Size-specialised y-/x-pass launchers for lengths 192, 256.
#include "cg_fast_yx.cuh"

CG_YX_INSTANTIATE(192)
CG_YX_INSTANTIATE(256)
