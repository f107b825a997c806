/*
 * sat_oracle.c -- CPU oracle for the summed-area-table (SAT) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker, never the product:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load the library built from it.  The CUDA library never links it and has
 * no CPU fallback.
 *
 * It restates, in plain C, the reference's CPU integral image
 * (integralImage/integralImage.h of pengdada/SAT):
 *
 *   - oracle_sat_serial_*   follows IntegralImageSerial  (integralImage.h:105-124):
 *       row 0 is a running sum; every later row is its own running row sum
 *       added to the output row above; all arithmetic is done in the output
 *       type, so 32-bit integer outputs wrap modulo 2^32.
 *   - oracle_sat_parallel_* follows IntegralImageParallel (integralImage.h:129-146):
 *       an OpenMP pass of row prefix sums (IntegralRow, :74-82) followed by an
 *       OpenMP pass of column prefix sums (IntegralStride, :90-100), in place
 *       on the output.  The reference only compiles it when the input and
 *       output types match (dead line :134); the restatement widens while it
 *       reads, which is what the reference's row pass does for matching types.
 *
 * and adds what the reference does not have but the tests need:
 *
 *   - oracle_sat_dd_*        an FP64 oracle: forward or reverse (suffix) SAT
 *       accumulated in double-double (Knuth TwoSum) and rounded once to
 *       double, so it is exact to about 2^-100 relative to SAT(|a|);
 *   - oracle_sat_abs_dd_*    SAT(|a|) in the same arithmetic (the error
 *       denominator for signed data);
 *   - oracle_err_stats_*     max/mean relative error against the FP64 oracle;
 *   - oracle_gen_*           a counter-based input generator (splitmix64 of
 *       seed and linear index) identical to the numpy one in oracle.py.
 *
 * Pitches are in elements, as in the reference (GpuData::DataPitch,
 * cudaLib.cuh:178-180).
 */
#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Serial SAT: IntegralImageSerial (integralImage.h:105-124).         */
/* ACC is the arithmetic type (uint32_t for both 32-bit integer       */
/* outputs so that overflow is the defined mod-2^32 wrap), CVT turns  */
/* one input element into ACC.                                        */
/* ------------------------------------------------------------------ */
#define DEF_SERIAL(NAME, TIN, TOUT, ACC, CVT)                                   \
  void oracle_sat_serial_##NAME(const TIN* src, int64_t in_pitch, TOUT* dst,    \
                                int64_t out_pitch, int64_t w, int64_t h) {      \
    if (w <= 0 || h <= 0) return;                                               \
    ACC sum = 0;                                                                \
    for (int64_t x = 0; x < w; ++x) {                                           \
      sum += CVT(src[x]);                                                       \
      dst[x] = (TOUT)sum;                                                       \
    }                                                                           \
    for (int64_t y = 1; y < h; ++y) {                                           \
      const TIN* s = src + y * in_pitch;                                        \
      TOUT* d = dst + y * out_pitch;                                            \
      const TOUT* up = dst + (y - 1) * out_pitch;                               \
      sum = 0;                                                                  \
      for (int64_t x = 0; x < w; ++x) {                                         \
        sum += CVT(s[x]);                                                       \
        d[x] = (TOUT)((ACC)up[x] + sum);                                        \
      }                                                                         \
    }                                                                           \
  }

/* ------------------------------------------------------------------ */
/* Parallel SAT: IntegralImageParallel (integralImage.h:129-146).     */
/* ------------------------------------------------------------------ */
#define DEF_PARALLEL(NAME, TIN, TOUT, ACC, CVT)                                 \
  void oracle_sat_parallel_##NAME(const TIN* src, int64_t in_pitch, TOUT* dst,  \
                                  int64_t out_pitch, int64_t w, int64_t h,      \
                                  int nthreads) {                               \
    if (w <= 0 || h <= 0) return;                                               \
    if (nthreads <= 0) nthreads = 1;                                            \
    _Pragma("omp parallel for num_threads(nthreads) schedule(static)")          \
    for (int64_t y = 0; y < h; ++y) {                                           \
      const TIN* s = src + y * in_pitch;                                        \
      TOUT* d = dst + y * out_pitch;                                            \
      ACC sum = 0;                                                              \
      for (int64_t x = 0; x < w; ++x) {                                         \
        sum += CVT(s[x]);                                                       \
        d[x] = (TOUT)sum;                                                       \
      }                                                                         \
    }                                                                           \
    _Pragma("omp parallel for num_threads(nthreads) schedule(static)")          \
    for (int64_t x = 0; x < w; ++x) {                                           \
      ACC sum = 0;                                                              \
      TOUT* d = dst + x;                                                        \
      for (int64_t y = 0; y < h; ++y, d += out_pitch) {                         \
        sum += (ACC)(*d);                                                       \
        *d = (TOUT)sum;                                                         \
      }                                                                         \
    }                                                                           \
  }

#define CV_U(x) ((uint32_t)(x))
#define CV_I8(x) ((uint32_t)(int32_t)(x)) /* sign-extend, then wrap as u32 */
#define CV_F(x) ((float)(x))
#define CV_D(x) ((double)(x))

/* The type pairs the reference dispatches (ScanRow-BRLT.cu:274-376 and the
 * matching blocks of BRLT-Scan.cu / ScanRowColumn.cu), plus u32->u32, the
 * TDst->TDst second-pass instantiation. */
#define FOR_EACH_PAIR(M)                                   \
  M(u8_u32, uint8_t, uint32_t, uint32_t, CV_U)              \
  M(u8_f32, uint8_t, float, float, CV_F)                    \
  M(u8_f64, uint8_t, double, double, CV_D)                  \
  M(i8_i32, int8_t, int32_t, uint32_t, CV_I8)               \
  M(i8_f32, int8_t, float, float, CV_F)                     \
  M(i8_f64, int8_t, double, double, CV_D)                   \
  M(i32_i32, int32_t, int32_t, uint32_t, CV_U)              \
  M(i32_f64, int32_t, double, double, CV_D)                 \
  M(u32_u32, uint32_t, uint32_t, uint32_t, CV_U)            \
  M(f32_f32, float, float, float, CV_F)                     \
  M(f32_f64, float, double, double, CV_D)                   \
  M(f64_f64, double, double, double, CV_D)

FOR_EACH_PAIR(DEF_SERIAL)
FOR_EACH_PAIR(DEF_PARALLEL)

/* ------------------------------------------------------------------ */
/* Row-only and column-only scans: IntegralRow / IntegralStride        */
/* (integralImage.h:74-101) applied to every row (stride 1) or every   */
/* column (stride = pitch), as IncrementScanX/Y compute them.          */
/* ------------------------------------------------------------------ */
#define DEF_SCANS(NAME, TIN, TOUT, ACC, CVT)                                     \
  void oracle_scan_rows_##NAME(const TIN* src, int64_t in_pitch, TOUT* dst,      \
                               int64_t out_pitch, int64_t w, int64_t h) {        \
    for (int64_t y = 0; y < h; ++y) {                                            \
      ACC sum = 0;                                                               \
      for (int64_t x = 0; x < w; ++x) {                                          \
        sum += CVT(src[y * in_pitch + x]);                                       \
        dst[y * out_pitch + x] = (TOUT)sum;                                      \
      }                                                                          \
    }                                                                            \
  }                                                                              \
  void oracle_scan_cols_##NAME(const TIN* src, int64_t in_pitch, TOUT* dst,      \
                               int64_t out_pitch, int64_t w, int64_t h) {        \
    for (int64_t x = 0; x < w; ++x) {                                            \
      ACC sum = 0;                                                               \
      for (int64_t y = 0; y < h; ++y) {                                          \
        sum += CVT(src[y * in_pitch + x]);                                       \
        dst[y * out_pitch + x] = (TOUT)sum;                                      \
      }                                                                          \
    }                                                                            \
  }

FOR_EACH_PAIR(DEF_SCANS)

/* ------------------------------------------------------------------ */
/* Reverse (suffix) SAT, the adjoint of the forward SAT:              */
/*   R(y,x) = sum_{j>=y, i>=x} a(j,i),                                */
/* computed in the same serial order mirrored (last row first, each   */
/* row right to left), in the output type.                            */
/* ------------------------------------------------------------------ */
#define DEF_REVERSE(NAME, TIN, TOUT, ACC, CVT)                                  \
  void oracle_sat_reverse_##NAME(const TIN* src, int64_t in_pitch, TOUT* dst,   \
                                 int64_t out_pitch, int64_t w, int64_t h) {     \
    if (w <= 0 || h <= 0) return;                                               \
    for (int64_t y = h - 1; y >= 0; --y) {                                      \
      const TIN* s = src + y * in_pitch;                                        \
      TOUT* d = dst + y * out_pitch;                                            \
      const TOUT* dn = (y + 1 < h) ? dst + (y + 1) * out_pitch : NULL;          \
      ACC sum = 0;                                                              \
      for (int64_t x = w - 1; x >= 0; --x) {                                    \
        sum += CVT(s[x]);                                                       \
        d[x] = dn ? (TOUT)((ACC)dn[x] + sum) : (TOUT)sum;                       \
      }                                                                         \
    }                                                                           \
  }
FOR_EACH_PAIR(DEF_REVERSE)

/* ------------------------------------------------------------------ */
/* FP64 oracle in double-double arithmetic.                           */
/* TwoSum: Knuth, TAOCP vol. 2, 4.2.2; used as the accurate summation */
/* of Ogita, Rump & Oishi, "Accurate sum and dot product" (2005).     */
/* ------------------------------------------------------------------ */
typedef struct { double hi, lo; } dd_t;

static inline dd_t dd_add_d(dd_t a, double b) {
  double s = a.hi + b;
  double bb = s - a.hi;
  double err = (a.hi - (s - bb)) + (b - bb);
  double lo = a.lo + err;
  double hi = s + lo; /* renormalise */
  lo = lo - (hi - s);
  dd_t r = {hi, lo};
  return r;
}

static inline dd_t dd_add(dd_t a, dd_t b) {
  dd_t r = dd_add_d(a, b.hi);
  return dd_add_d(r, b.lo);
}

/* Forward or reverse SAT of one plane in double-double; `absval` sums |a|.
 * colacc holds w double-double column accumulators. */
#define DEF_DD(NAME, TIN)                                                        \
  static void sat_dd_core_##NAME(const TIN* src, int64_t in_pitch, double* dst, \
                                 int64_t out_pitch, int64_t w, int64_t h,       \
                                 int reverse, int absval, dd_t* colacc) {       \
    for (int64_t x = 0; x < w; ++x) { colacc[x].hi = 0.0; colacc[x].lo = 0.0; } \
    for (int64_t k = 0; k < h; ++k) {                                           \
      int64_t y = reverse ? (h - 1 - k) : k;                                    \
      const TIN* s = src + y * in_pitch;                                        \
      double* d = dst + y * out_pitch;                                          \
      dd_t row = {0.0, 0.0};                                                    \
      for (int64_t q = 0; q < w; ++q) {                                         \
        int64_t x = reverse ? (w - 1 - q) : q;                                  \
        double v = (double)s[x];                                                \
        if (absval) v = fabs(v);                                                \
        row = dd_add_d(row, v);                                                 \
        colacc[x] = dd_add(colacc[x], row);                                     \
        d[x] = colacc[x].hi + colacc[x].lo;                                     \
      }                                                                         \
    }                                                                           \
  }                                                                             \
  int oracle_sat_dd_##NAME(const TIN* src, int64_t in_pitch, double* dst,       \
                           int64_t out_pitch, int64_t w, int64_t h,             \
                           int reverse, int absval, void* scratch) {            \
    if (w <= 0 || h <= 0) return 0;                                             \
    sat_dd_core_##NAME(src, in_pitch, dst, out_pitch, w, h, reverse, absval,    \
                       (dd_t*)scratch);                                         \
    return 0;                                                                   \
  }

DEF_DD(u8, uint8_t)
DEF_DD(i8, int8_t)
DEF_DD(u32, uint32_t)
DEF_DD(i32, int32_t)
DEF_DD(f32, float)
DEF_DD(f64, double)

/* ------------------------------------------------------------------ */
/* Error statistics of a float SAT against the FP64 oracle.           */
/* out[0] = max |S-S64|/|S64|  (over |S64| > 0)                        */
/* out[1] = mean of the same                                          */
/* out[2] = max |S-S64|/SAT(|a|)64  (over SAT(|a|) > 0)               */
/* out[3] = mean of the same                                          */
/* ------------------------------------------------------------------ */
#define DEF_ERR(NAME, T)                                                        \
  void oracle_err_stats_##NAME(const T* s, int64_t s_pitch, const double* r,    \
                               const double* rabs, int64_t w, int64_t h,        \
                               double* out) {                                   \
    double mx = 0, sm = 0, mxa = 0, sma = 0;                                    \
    int64_t n = 0, na = 0;                                                      \
    for (int64_t y = 0; y < h; ++y) {                                           \
      for (int64_t x = 0; x < w; ++x) {                                         \
        double ref = r[y * w + x];                                              \
        double e = fabs((double)s[y * s_pitch + x] - ref);                      \
        if (ref != 0.0) {                                                       \
          double q = e / fabs(ref);                                             \
          if (q > mx) mx = q;                                                   \
          sm += q; ++n;                                                         \
        }                                                                       \
        if (rabs) {                                                             \
          double d = rabs[y * w + x];                                           \
          if (d > 0.0) {                                                        \
            double q = e / d;                                                   \
            if (q > mxa) mxa = q;                                               \
            sma += q; ++na;                                                     \
          }                                                                     \
        }                                                                       \
      }                                                                         \
    }                                                                           \
    out[0] = mx; out[1] = n ? sm / (double)n : 0.0;                             \
    out[2] = mxa; out[3] = na ? sma / (double)na : 0.0;                         \
  }
DEF_ERR(f32, float)
DEF_ERR(f64, double)

/* ------------------------------------------------------------------ */
/* Counter-based generator: z = splitmix64(seed * 2^32 + ... )        */
/* element i of stream `seed` is splitmix64_mix(seed_key + (i+1)*G)   */
/* with G the golden-ratio increment, i.e. the i-th output of a       */
/* splitmix64 generator started at seed_key (Steele, Lea & Flood,     */
/* "Fast splittable pseudorandom number generators", 2014).           */
/* ------------------------------------------------------------------ */
#define SM_GAMMA 0x9E3779B97F4A7C15ULL

static inline uint64_t sm_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

static inline uint64_t sm_key(uint64_t seed) { return sm_mix(seed ^ 0x5A7A5A7A5A7A5A7AULL); }

static inline uint64_t sm_at(uint64_t key, uint64_t i) { return sm_mix(key + (i + 1) * SM_GAMMA); }

void oracle_gen_u8(uint64_t seed, int64_t n, uint8_t* out) {
  uint64_t k = sm_key(seed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) out[i] = (uint8_t)(sm_at(k, (uint64_t)i) >> 56);
}

void oracle_gen_u32(uint64_t seed, int64_t n, uint32_t* out) {
  uint64_t k = sm_key(seed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) out[i] = (uint32_t)(sm_at(k, (uint64_t)i) >> 32);
}

/* uniform [0,1) with 24 random bits: exact in f32 */
void oracle_gen_f32_uniform(uint64_t seed, int64_t n, float* out) {
  uint64_t k = sm_key(seed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    out[i] = (float)(sm_at(k, (uint64_t)i) >> 40) * (1.0f / 16777216.0f);
}

/* uniform [0,1) with 53 random bits */
void oracle_gen_f64_uniform(uint64_t seed, int64_t n, double* out) {
  uint64_t k = sm_key(seed);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    out[i] = (double)(sm_at(k, (uint64_t)i) >> 11) * (1.0 / 9007199254740992.0);
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
