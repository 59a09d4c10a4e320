// Size-specialised y-/x-pass launchers for lengths 512.
#include "cg_fast_yx.cuh"

CG_YX_INSTANTIATE(512)
