// Kernel instantiations for f64 input (f64 -> f64).
#include "sat_inst.cuh"
SG_TABLE(f64, SG_ALL(double, double, double, SG_F64, SG_F64, 0),
         SG_SCANS(double, double, double, SG_F64, SG_F64))
