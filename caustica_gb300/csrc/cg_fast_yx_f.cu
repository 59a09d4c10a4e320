// Size-specialised y-/x-pass launchers for lengths 640.
#include "cg_fast_yx.cuh"

CG_YX_INSTANTIATE(640)
