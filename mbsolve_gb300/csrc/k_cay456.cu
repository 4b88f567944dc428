// 4- to 6-level Cayley kernels.
#include "inst.cuh"
MBG_REG_CAY(float, 4, 1, 128)
MBG_REG_CAY(double, 4, 1, 128)
MBG_REG_CAY(float, 5, 1, 128)
MBG_REG_CAY(double, 5, 1, 128)
MBG_REG_CAY(float, 6, 1, 128)
MBG_REG_CAY(double, 6, 1, 128)
