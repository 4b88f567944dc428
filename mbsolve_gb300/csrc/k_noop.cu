// Maxwell-only kernels (algo_lindblad_noop.hpp).
#include "inst.cuh"
MBG_REG_NOOP(float, 4, 256)
MBG_REG_NOOP(float, 8, 256)
MBG_REG_NOOP(float, 8, 128)
MBG_REG_NOOP(double, 2, 256)
MBG_REG_NOOP(double, 4, 256)
