// Kernel instantiations for f32 input (f32 -> f32 plain and compensated, f64).
#include "sat_inst.cuh"
SG_TABLE(f32,
         SG_ALL(float, float, float, SG_F32, SG_F32, 0),
         SG_ALL(float, float, satgb::CF32, SG_F32, SG_F32, 1),
         SG_ALL(float, double, double, SG_F32, SG_F64, 0),
         SG_SCANS(float, float, float, SG_F32, SG_F32),
         SG_SCANS(float, double, double, SG_F32, SG_F64))
