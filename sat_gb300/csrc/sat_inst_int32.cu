// Kernel instantiations for 32-bit integer input (i32 -> i32, f64; u32 -> u32).
#include "sat_inst.cuh"
SG_TABLE(int32,
         SG_ALL(int32_t, int32_t, uint32_t, SG_I32, SG_I32, 0),
         SG_ALL(int32_t, double, double, SG_I32, SG_F64, 0),
         SG_ALL(uint32_t, uint32_t, uint32_t, SG_U32, SG_U32, 0),
         SG_SCANS(int32_t, int32_t, uint32_t, SG_I32, SG_I32),
         SG_SCANS(int32_t, double, double, SG_I32, SG_F64),
         SG_SCANS(uint32_t, uint32_t, uint32_t, SG_U32, SG_U32))
