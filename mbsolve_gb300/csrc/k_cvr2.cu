// 2-level coherence-vector kernels (V = 3).
#include "inst.cuh"
MBG_REG_CVR(float, 2, 1, 128)
MBG_REG_CVR(float, 2, 2, 128)
MBG_REG_CVR(float, 2, 2, 256)
MBG_REG_CVR(float, 2, 4, 128)
MBG_REG_CVR_P(float, 2, 4, 256)
MBG_REG_CVR(float, 2, 8, 128)
MBG_REG_CVR(float, 2, 8, 256)
MBG_REG_CVR(double, 2, 1, 128)
MBG_REG_CVR(double, 2, 2, 128)
MBG_REG_CVR(double, 2, 2, 256)
MBG_REG_CVR(double, 2, 4, 256)
