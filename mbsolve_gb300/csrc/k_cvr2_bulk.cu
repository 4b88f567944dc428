// 2-level FP32 coherence-vector kernels with bulk-copy (TMA) staging of the
// tile state (not the default; MBG_TILE_STAGING=bulk selects them).
#include "inst.cuh"
MBG_REG_CVR2_BULK(1, 128)
MBG_REG_CVR2_BULK(2, 128)
MBG_REG_CVR2_BULK(2, 256)
MBG_REG_CVR2_BULK(4, 128)
MBG_REG_CVR2_BULK(4, 256)
MBG_REG_CVR2_BULK(8, 128)
MBG_REG_CVR2_BULK(8, 256)
