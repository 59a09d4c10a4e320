// Size-specialised y-/x-pass launchers for lengths 320, 400.
#include "cg_fast_yx.cuh"

CG_YX_INSTANTIATE(320)
CG_YX_INSTANTIATE(400)
