// 3-level coherence-vector kernels (V = 8).
#include "inst.cuh"
MBG_REG_CVR(float, 3, 1, 128)
MBG_REG_CVR(float, 3, 2, 128)
MBG_REG_CVR(float, 3, 2, 256)
MBG_REG_CVR(double, 3, 1, 128)
MBG_REG_CVR(double, 3, 2, 128)
