// sat_types.cuh -- arithmetic types, conversions and look-back status words
// shared by the SAT kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace satgb {

// Compensated f32 value: s is the running sum, e the accumulated rounding
// error of every addition that produced s (exact per step by TwoSum).  The
// represented value is s + e, rounded once when the result is stored.
struct CF32 {
  float s, e;
};

// Knuth's TwoSum (TAOCP vol. 2, 4.2.2, Theorem B): s + err == a + b exactly,
// with s = fl(a + b), for any a, b (no ordering precondition).  The compensated
// path is compiled without fast-math, so the compiler keeps this sequence.
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return s;
}

// ---------------------------------------------------------------------------
// Arithmetic traits.  K = number of 32-bit payload words in a status word set.
// ---------------------------------------------------------------------------
template <class A>
struct Ar;

template <>
struct Ar<uint32_t> {
  static constexpr int K = 1;
  __device__ __forceinline__ static uint32_t zero() { return 0u; }
  __device__ __forceinline__ static uint32_t add(uint32_t a, uint32_t b) { return a + b; }
  __device__ __forceinline__ static uint32_t shfl_up(uint32_t a, int d, int w = 32) { return __shfl_up_sync(0xffffffffu, a, d, w); }
  __device__ __forceinline__ static uint32_t shfl_down(uint32_t a, int d, int w = 32) { return __shfl_down_sync(0xffffffffu, a, d, w); }
  __device__ __forceinline__ static uint32_t shfl(uint32_t a, int l) { return __shfl_sync(0xffffffffu, a, l); }
  __device__ __forceinline__ static void to_words(uint32_t a, uint32_t* w) { w[0] = a; }
  __device__ __forceinline__ static uint32_t from_words(const uint32_t* w) { return w[0]; }
};

template <>
struct Ar<float> {
  static constexpr int K = 1;
  __device__ __forceinline__ static float zero() { return 0.f; }
  __device__ __forceinline__ static float add(float a, float b) { return __fadd_rn(a, b); }
  __device__ __forceinline__ static float shfl_up(float a, int d, int w = 32) { return __shfl_up_sync(0xffffffffu, a, d, w); }
  __device__ __forceinline__ static float shfl_down(float a, int d, int w = 32) { return __shfl_down_sync(0xffffffffu, a, d, w); }
  __device__ __forceinline__ static float shfl(float a, int l) { return __shfl_sync(0xffffffffu, a, l); }
  __device__ __forceinline__ static void to_words(float a, uint32_t* w) { w[0] = __float_as_uint(a); }
  __device__ __forceinline__ static float from_words(const uint32_t* w) { return __uint_as_float(w[0]); }
};

template <>
struct Ar<double> {
  static constexpr int K = 2;
  __device__ __forceinline__ static double zero() { return 0.0; }
  __device__ __forceinline__ static double add(double a, double b) { return __dadd_rn(a, b); }
  __device__ __forceinline__ static double shfl_up(double a, int d, int w = 32) { return __shfl_up_sync(0xffffffffu, a, d, w); }
  __device__ __forceinline__ static double shfl_down(double a, int d, int w = 32) { return __shfl_down_sync(0xffffffffu, a, d, w); }
  __device__ __forceinline__ static double shfl(double a, int l) { return __shfl_sync(0xffffffffu, a, l); }
  __device__ __forceinline__ static void to_words(double a, uint32_t* w) {
    unsigned long long b = (unsigned long long)__double_as_longlong(a);
    w[0] = (uint32_t)b;
    w[1] = (uint32_t)(b >> 32);
  }
  __device__ __forceinline__ static double from_words(const uint32_t* w) {
    return __longlong_as_double((long long)(((unsigned long long)w[1] << 32) | w[0]));
  }
};

template <>
struct Ar<CF32> {
  static constexpr int K = 2;
  __device__ __forceinline__ static CF32 zero() { return CF32{0.f, 0.f}; }
  __device__ __forceinline__ static CF32 add(CF32 a, CF32 b) {
    float err;
    float s = two_sum(a.s, b.s, err);
    return CF32{s, __fadd_rn(__fadd_rn(a.e, b.e), err)};
  }
  __device__ __forceinline__ static CF32 shfl_up(CF32 a, int d, int w = 32) {
    return CF32{__shfl_up_sync(0xffffffffu, a.s, d, w), __shfl_up_sync(0xffffffffu, a.e, d, w)};
  }
  __device__ __forceinline__ static CF32 shfl_down(CF32 a, int d, int w = 32) {
    return CF32{__shfl_down_sync(0xffffffffu, a.s, d, w), __shfl_down_sync(0xffffffffu, a.e, d, w)};
  }
  __device__ __forceinline__ static CF32 shfl(CF32 a, int l) {
    return CF32{__shfl_sync(0xffffffffu, a.s, l), __shfl_sync(0xffffffffu, a.e, l)};
  }
  __device__ __forceinline__ static void to_words(CF32 a, uint32_t* w) {
    w[0] = __float_as_uint(a.s);
    w[1] = __float_as_uint(a.e);
  }
  __device__ __forceinline__ static CF32 from_words(const uint32_t* w) {
    return CF32{__uint_as_float(w[0]), __uint_as_float(w[1])};
  }
};

// ---------------------------------------------------------------------------
// Input -> accumulator and accumulator -> output conversions.
// Integer outputs accumulate in uint32_t: mod-2^32 wrap is then defined, and
// for i32 outputs the bits equal two's-complement wrapping int arithmetic.
// ---------------------------------------------------------------------------
template <class A, class TIn>
struct Cvt;
template <class TIn>
struct Cvt<uint32_t, TIn> {
  __device__ __forceinline__ static uint32_t in(TIn x) { return (uint32_t)x; }
};
template <>
struct Cvt<uint32_t, int8_t> {
  __device__ __forceinline__ static uint32_t in(int8_t x) { return (uint32_t)(int32_t)x; }
};
template <class TIn>
struct Cvt<float, TIn> {
  __device__ __forceinline__ static float in(TIn x) { return (float)x; }
};
template <class TIn>
struct Cvt<double, TIn> {
  __device__ __forceinline__ static double in(TIn x) { return (double)x; }
};
template <class TIn>
struct Cvt<CF32, TIn> {
  __device__ __forceinline__ static CF32 in(TIn x) { return CF32{(float)x, 0.f}; }
};

// acc + one input element.  The compensated accumulator's element carries no
// error term, so a TwoSum of the sums and one add of the errors do: one add
// fewer per element than the general pair + pair addition.
template <class A, class TIn>
struct AddIn {
  __device__ __forceinline__ static A add(A acc, TIn x) { return Ar<A>::add(acc, Cvt<A, TIn>::in(x)); }
};
template <class TIn>
struct AddIn<CF32, TIn> {
  __device__ __forceinline__ static CF32 add(CF32 acc, TIn x) {
    float err;
    const float s = two_sum(acc.s, (float)x, err);
    return CF32{s, __fadd_rn(acc.e, err)};
  }
};

template <class TOut, class A>
struct OutCvt;
template <>
struct OutCvt<uint32_t, uint32_t> {
  __device__ __forceinline__ static uint32_t out(uint32_t a) { return a; }
};
template <>
struct OutCvt<int32_t, uint32_t> {
  __device__ __forceinline__ static int32_t out(uint32_t a) { return (int32_t)a; }
};
template <>
struct OutCvt<float, float> {
  __device__ __forceinline__ static float out(float a) { return a; }
};
template <>
struct OutCvt<double, double> {
  __device__ __forceinline__ static double out(double a) { return a; }
};
template <>
struct OutCvt<float, CF32> {
  __device__ __forceinline__ static float out(CF32 a) { return __fadd_rn(a.s, a.e); }
};

// ---------------------------------------------------------------------------
// Look-back status words.  Every 32-bit payload travels in its own 64-bit
// word whose high half is a tag: ((epoch mod 2^30-1) + 1) << 2 | state, state
// 1 = aggregate (this tile's own sum), 2 = inclusive (everything up to and
// including this tile).  A word is written with one 64-bit store, so a reader
// never sees a tag with another publication's payload; a multi-word value is
// accepted only when all its words carry the same valid tag.  Zeroed memory
// (tag 0) and words of earlier launches (other epoch) read as "not ready", so
// the status arrays never need clearing between launches.
// ---------------------------------------------------------------------------
constexpr uint32_t kStateAgg = 1u;
constexpr uint32_t kStateInc = 2u;

__device__ __forceinline__ uint32_t make_tag(uint32_t epoch, uint32_t state) {
  return (((epoch % 0x3fffffffu) + 1u) << 2) | state;
}

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <class A>
__device__ __forceinline__ void publish(unsigned long long* words, A val, uint32_t tag) {
  constexpr int K = Ar<A>::K;
  uint32_t p[K];
  Ar<A>::to_words(val, p);
#pragma unroll
  for (int k = 0; k < K; ++k) st_relaxed_u64(words + k, ((unsigned long long)tag << 32) | p[k]);
}

// Workspace header (device memory, zero-initialised once at allocation).
// `error` belongs to the running launch: once set, every bounded wait of that
// launch gives up at once, so the launch ends quickly.  The last CTA of the
// launch moves it to `sticky` (kept until the host reads and clears it) and
// resets it, so one timed-out launch never cuts short the waits of the next.
struct WsHeader {
  unsigned long long ticket; // next tile ticket of the running launch
  uint32_t done;             // CTAs that finished the running launch
  uint32_t epoch;            // launch counter; advanced by the last CTA of each launch
  uint32_t error;            // 0, or a device error code (kDevErrTimeout) of the running launch
  uint32_t error_tile;       // tile that recorded it
  uint32_t sticky;           // the first error of the launches since the host last cleared it
  uint32_t sticky_tile;      // tile that recorded it
  uint32_t pad[8];
};
static_assert(sizeof(WsHeader) == 64, "header is one 64-byte block");

constexpr uint32_t kDevErrTimeout = 7u; // == SATGB_ERR_TIMEOUT

}  // namespace satgb
