// 4- and 5-level coherence-vector kernels (V = 15, 24).
#include "inst.cuh"
MBG_REG_CVR_TC_P(4)
MBG_REG_CVR(float, 4, 1, 256)
MBG_REG_CVR(double, 4, 1, 128)
MBG_REG_CVR_TC_P(5)
MBG_REG_CVR(float, 5, 1, 256)
MBG_REG_CVR(double, 5, 1, 128)
