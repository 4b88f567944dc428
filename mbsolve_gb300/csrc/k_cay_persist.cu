// Persistent kernels of the FP32 Cayley solvers for 4-6 levels (their own
// translation unit, compiled in parallel with k_cay456.cu, which registers
// the launch per level of the same shapes).
#include "inst.cuh"

MBG_REG_CAY_PONLY(float, 4, 1, 128)
MBG_REG_CAY_PONLY(float, 5, 1, 128)
MBG_REG_CAY_PONLY(float, 6, 1, 128)
