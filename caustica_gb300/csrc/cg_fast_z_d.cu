// Size-specialised z-pass launchers for lengths 320, 400.
#include "cg_fast_z.cuh"

CG_ZP_INSTANTIATE(320)
CG_ZP_INSTANTIATE(400)
