// Size-specialised z-pass launchers for lengths 512.
#include "cg_fast_z.cuh"

CG_ZP_INSTANTIATE(512)
