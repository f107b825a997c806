// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes the reference's own CPU integral image (pengdada/SAT,
// integralImage/integralImage.h) through extern "C" symbols so that the test
// suite and the golden-vector script can run the reference itself.  Nothing is
// copied: the reference header is included from the reference checkout at
// build time (see oracle/Makefile) and the result goes to oracle/_ref/, which
// is never committed.
//
//   ref_serial_<in>_<out>    -> IntegralImageSerial<TSrc,TDst>   (integralImage.h:105-124)
//   ref_parallel_<t>_<t>     -> IntegralImageParallel<T,T>       (integralImage.h:129-146)
//   ref_allrow_<in>_<out>    -> IntegralImageAllRow<TSrc,TDst>   (integralImage.h:148-160),
//                               the row scan (IntegralRow on every row)
//   ref_allrow_t_<in>_<out>  -> IntegralImageAllRow then Transpose (integralImage.h:280-288),
//                               the check of SerielScan::TestX (BRLT-Scan.cu:176-180)
//   ref_colscan_<in>_<out>   -> IntegralStride down every column (integralImage.h:91-101)
//
// IntegralImageParallel only compiles when TSrc == TDst (its dead line :134
// assigns `const TDst* p0 = src`), so it is exported for the matching pairs.
#include "integralImage.h"

#define SERIAL(NAME, TS, TD)                                             \
  extern "C" void ref_serial_##NAME(const TS* s, TD* d, int w, int h) { \
    IntegralImageSerial<TS, TD>(s, d, w, h);                            \
  }
#define PARALLEL(NAME, T)                                                  \
  extern "C" void ref_parallel_##NAME(const T* s, T* d, int w, int h) {   \
    IntegralImageParallel<T, T>(s, d, w, h);                              \
  }

#define SCANS(NAME, TS, TD)                                                         \
  extern "C" void ref_allrow_##NAME(const TS* s, TD* d, int w, int h) {            \
    IntegralImageAllRow<TS, TD>(s, d, w, h);                                       \
  }                                                                                \
  extern "C" void ref_allrow_t_##NAME(const TS* s, TD* tmp, TD* d, int w, int h) { \
    IntegralImageAllRow<TS, TD>(s, tmp, w, h);                                     \
    Transpose<TD, TD>(tmp, w, h, d, h, w);                                         \
  }                                                                                \
  extern "C" void ref_colscan_##NAME(const TS* s, TD* d, int w, int h) {           \
    for (int x = 0; x < w; ++x) IntegralStride<TS, TD>(s + x, w, d + x, w, h);     \
  }

SERIAL(u8_u32, unsigned char, unsigned int)
SERIAL(u8_f32, unsigned char, float)
SERIAL(u8_f64, unsigned char, double)
SERIAL(i8_i32, char, int)
SERIAL(i8_f32, char, float)
SERIAL(i8_f64, char, double)
SERIAL(i32_i32, int, int)
SERIAL(i32_f64, int, double)
SERIAL(u32_u32, unsigned int, unsigned int)
SERIAL(f32_f32, float, float)
SERIAL(f32_f64, float, double)
SERIAL(f64_f64, double, double)

PARALLEL(u32_u32, unsigned int)
PARALLEL(i32_i32, int)
PARALLEL(f32_f32, float)
PARALLEL(f64_f64, double)

SCANS(u8_u32, unsigned char, unsigned int)
SCANS(u8_f32, unsigned char, float)
SCANS(u8_f64, unsigned char, double)
SCANS(i8_i32, char, int)
SCANS(i8_f32, char, float)
SCANS(i8_f64, char, double)
SCANS(i32_i32, int, int)
SCANS(i32_f64, int, double)
SCANS(u32_u32, unsigned int, unsigned int)
SCANS(f32_f32, float, float)
SCANS(f32_f64, float, double)
SCANS(f64_f64, double, double)
