// Kernel instantiations for 8-bit unsigned input (u8 -> u32, f32, f64).
#include "sat_inst.cuh"
SG_TABLE(u8,
         SG_ALL(uint8_t, uint32_t, uint32_t, SG_U8, SG_U32, 0),
         SG_ALL(uint8_t, float, float, SG_U8, SG_F32, 0),
         SG_ALL(uint8_t, float, satgb::CF32, SG_U8, SG_F32, 1),
         SG_ALL(uint8_t, double, double, SG_U8, SG_F64, 0),
         SG_SCANS(uint8_t, uint32_t, uint32_t, SG_U8, SG_U32),
         SG_TALL(uint8_t, uint32_t, uint32_t, SG_U8, SG_U32),
         SG_TALL(uint8_t, float, float, SG_U8, SG_F32),
         SG_SCANS(uint8_t, float, float, SG_U8, SG_F32),
         SG_SCANS(uint8_t, double, double, SG_U8, SG_F64))
