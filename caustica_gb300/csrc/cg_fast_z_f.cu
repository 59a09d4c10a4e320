// Size-specialised z-pass launchers for lengths 640.
#include "cg_fast_z.cuh"

CG_ZP_INSTANTIATE(640)
