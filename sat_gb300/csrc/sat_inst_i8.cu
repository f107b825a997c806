// Kernel instantiations for 8-bit signed input (i8 -> i32, f32, f64).
#include "sat_inst.cuh"
SG_TABLE(i8,
         SG_ALL(int8_t, int32_t, uint32_t, SG_I8, SG_I32, 0),
         SG_ALL(int8_t, float, float, SG_I8, SG_F32, 0),
         SG_ALL(int8_t, float, satgb::CF32, SG_I8, SG_F32, 1),
         SG_ALL(int8_t, double, double, SG_I8, SG_F64, 0),
         SG_SCANS(int8_t, int32_t, uint32_t, SG_I8, SG_I32),
         SG_TALL(int8_t, int32_t, uint32_t, SG_I8, SG_I32),
         SG_TALL(int8_t, float, float, SG_I8, SG_F32),
         SG_SCANS(int8_t, float, float, SG_I8, SG_F32),
         SG_SCANS(int8_t, double, double, SG_I8, SG_F64))
