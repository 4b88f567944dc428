// 2- and 3-level Cayley kernels.
#include "inst.cuh"
MBG_REG_CAY(float, 2, 1, 128)
MBG_REG_CAY(float, 2, 2, 256)
MBG_REG_CAY(float, 2, 4, 256)
MBG_REG_CAY(double, 2, 1, 128)
MBG_REG_CAY(double, 2, 2, 256)
MBG_REG_CAY(float, 3, 1, 128)
MBG_REG_CAY(float, 3, 1, 256)
MBG_REG_CAY(float, 3, 2, 128)
MBG_REG_CAY(double, 3, 1, 128)
