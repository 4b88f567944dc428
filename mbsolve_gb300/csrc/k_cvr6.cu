// 6-level coherence-vector kernels (V = 35).
#include "inst.cuh"
MBG_REG_CVR_TC_P(6)
MBG_REG_CVR(float, 6, 1, 256)
MBG_REG_CVR(double, 6, 1, 128)
