// Size-specialised z-pass launchers for lengths 192, 256.
#include "cg_fast_z.cuh"

CG_ZP_INSTANTIATE(192)
CG_ZP_INSTANTIATE(256)
CG_ZT_INSTANTIATE(192)
CG_ZT_INSTANTIATE(256)
