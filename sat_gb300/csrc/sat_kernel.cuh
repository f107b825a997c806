// sat_kernel.cuh -- single-pass tiled summed-area table with decoupled
// look-back in both tile directions.
//
// Replaces the reference's two-launch algorithms (pengdada/SAT
// integralImage/ScanRow-BRLT.cu:24-180 blockScan x2, BRLT-Scan.cu:15-127
// serielScan x2, ScanRowColumn.cu:16-268 ScanX + ScanY), which each move
// in + 3*out bytes, with one launch that reads each input element once and
// writes each output element once.
//
// Decomposition.  The image is cut into TH x TW tiles.  For a tile with
// origin (x0, y0):
//
//   S(y,x) = L(y,x)                             local SAT of the tile
//          + sum_{y0<=j<=y} rowleft(j)          rowleft(j)  = sum_{i<x0} a(j,i)
//          + sum_{x0<=i<=x} colabove(i)         colabove(i) = sum_{j<y0} a(j,i)
//          + corner                             corner      = sum_{j<y0,i<x0} a(j,i)
//
// rowleft and colabove come from vector look-backs over the tiles to the left
// and above (each tile publishes its row sums and column sums as an
// "aggregate", then the running sums including itself as "inclusive"), and
// corner from a scalar look-back over the tiles above, whose aggregate is
// u = sum_j rowleft(j) of that tile and whose inclusive value is its own
// corner + u.
//
// Order.  Tiles are handed out by an atomic ticket along anti-diagonals
// (tx + ty ascending, then ty ascending).  A tile's left and upper neighbours
// lie on the previous diagonal, so they were handed out a whole diagonal
// earlier and the chains of tiles that wait on each other stay a few
// diagonals long (row-major order would chain every tile of a tile row).  Every
// tile a tile waits on has a smaller ticket and is held by a running CTA that
// never waits on a larger ticket, so the persistent grid cannot deadlock.
//
// The reverse (suffix) SAT mirrors every step: tickets run from the last
// tile, look-backs go right and down, scans run right-to-left and
// bottom-to-top.
//
// CTA structure (NW warps).  Each tile's input reaches a ring of S
// shared-memory stages through one 2-D TMA load (the tensor map clips at the
// image edges and fills zeros), S tiles ahead of the one being computed; an
// mbarrier per stage signals arrival.  One thread that is idle during the
// look-back phase (the producer) takes the tickets -- one atomic kept in
// flight a whole tile ahead -- and refills the stage the CTA has just read,
// so ticket and load latencies overlap the look-back waits.  Images whose rows
// are not 16-byte aligned are read straight from global memory instead.  Warp w owns
// tile rows [w*RPW, (w+1)*RPW), lane l owns CPT = 16/sizeof(TOut) adjacent
// columns [l*CPT, (l+1)*CPT), so each output row segment is one 16-byte
// store and a warp writes 512 contiguous bytes per row.  Row scans: in-thread,
// then a Kogge-Stone warp scan of the per-thread totals; column scans:
// in-thread over the warp's rows, then a cross-warp carry through shared
// memory.  After the local phase, consumer threads [0, TW) run the column
// look-back (one column each) while threads [TW, TW+TH) run the row look-back
// (one row each), each group synchronising on its own named barrier.  Shared
// vectors indexed by column use slot c*32+lane for column l*CPT+c, which
// keeps the shared accesses of the hot loop bank-conflict free.
#pragma once
#include <cuda.h>

#include "sat_types.cuh"

namespace satgb {

// One image, or a stack of `planes` equally sized images at a fixed stride
// (the planes of an N x C x H x W tensor), each with its own SAT.
struct ImageDesc {
  CUtensorMap tmap_in;  // 3-D tiled map (x, y, plane) of the input (valid when flags & kInTma)
  CUtensorMap tmap_out; // 3-D tiled map of the output (valid when flags & kOutTma)
  const void* in;
  void* out;
  int64_t in_pitch;  // elements
  int64_t out_pitch; // elements
  int64_t width, height;
  int64_t planes;          // >= 1
  int64_t in_plane;        // plane stride of the input, elements
  int64_t out_plane;       // plane stride of the output, elements
  int64_t tiles_per_plane; // ntx * nty
  int64_t tile_base; // global index of the image's first tile
  // Columns the tensor maps cover: the width rounded down to whole 16-byte
  // chunks.  TMA moves whole chunks, so a map that reached into a row's last,
  // partial chunk could write the caller's row padding; the columns past the
  // map ([tma_*_w, width)) are loaded and stored with plain accesses.
  int64_t tma_in_w, tma_out_w;
  int32_t ntx, nty;  // tiles across / down (per plane)
  uint32_t flags;    // kInVec | kOutVec | kInTma | kOutTma
  uint32_t pad;
};
constexpr uint32_t kInVec = 1u;  // every thread's CPT-element input row segment is vector-aligned
constexpr uint32_t kOutVec = 2u; // every 16-byte output row segment is aligned
constexpr uint32_t kInTma = 4u;  // tmap_in is valid: tiles arrive by TMA
constexpr uint32_t kOutTma = 8u; // tmap_out is valid: results leave by TMA

struct SatParams {
  ImageDesc img0;          // the image when n_images == 1
  const ImageDesc* images; // device table when n_images > 1
  int64_t n_images;
  int64_t n_tiles;
  unsigned long long* row_words;
  unsigned long long* col_words;
  unsigned long long* corner_words;
  WsHeader* ws;
  int64_t wait_limit_ns;
  int64_t stall_tile; // test knob: this tile never publishes (-1: none)
  // Batches: the tile of each ticket, (image << 40) | (ty << 20) | tx, in an
  // order whose every tile comes after the tiles it depends on (nullptr: the
  // images one after the other, each in the kernel's own order).
  const unsigned long long* order;
};

// Pipeline depth.  A stage holds one tile from its TMA load until its TMA
// store has read the results back out of it (or, for the register kernel,
// until the output phase has read the input), so a CTA cycles through S
// stages: as many as fit in its share of the SM's 227 KB of shared memory
// (CTAS CTAs per SM) next to its static shared memory, between 2 and 6.
template <int STAGE_BYTES, int STATIC_BYTES, int CTAS>
struct Stages {
  static constexpr int budget = (CTAS == 1 ? 232448 : 115712) - STATIC_BYTES; // per-CTA limit, 1 or 2 CTAs per SM
  static constexpr int fit = budget / STAGE_BYTES;
  static constexpr int value = fit < 2 ? 2 : (fit > 6 ? 6 : fit);
};

template <int BYTES>
struct VecT;
template <>
struct VecT<1> { using T = unsigned char; };
template <>
struct VecT<2> { using T = unsigned short; };
template <>
struct VecT<4> { using T = unsigned int; };
template <>
struct VecT<8> { using T = uint2; };
template <>
struct VecT<16> { using T = uint4; };

template <class TIn, int CPT>
__device__ __forceinline__ void load_seg(const TIn* p, bool vec, int nvalid, TIn (&x)[CPT]) {
  if (vec) {
    using V = typename VecT<CPT * sizeof(TIn)>::T;
    union {
      V v;
      TIn e[CPT];
    } u;
    u.v = __ldcs(reinterpret_cast<const V*>(p));
#pragma unroll
    for (int c = 0; c < CPT; ++c) x[c] = u.e[c];
  } else {
#pragma unroll
    for (int c = 0; c < CPT; ++c) x[c] = (c < nvalid) ? __ldcs(p + c) : TIn(0);
  }
}

// One thread's CPT input elements of one row, kept packed in registers
// (a single 32-bit register for four 8-bit pixels).
template <class TIn, int CPT>
struct RowSeg {
  using V = typename VecT<CPT * sizeof(TIn)>::T;
  union {
    V v;
    TIn e[CPT];
  } u;
};

template <class TIn, int CPT>
__device__ __forceinline__ void load_seg_smem(const TIn* p, TIn (&x)[CPT]) {
  using V = typename VecT<CPT * sizeof(TIn)>::T;
  union {
    V v;
    TIn e[CPT];
  } u;
  u.v = *reinterpret_cast<const V*>(p);
#pragma unroll
  for (int c = 0; c < CPT; ++c) x[c] = u.e[c];
}

template <class TOut, int CPT>
__device__ __forceinline__ void store_seg(TOut* p, bool vec, int nvalid, const TOut (&o)[CPT]) {
  if (vec) {
    static_assert(CPT * sizeof(TOut) == 16, "16-byte segments");
    union {
      uint4 v;
      TOut e[CPT];
    } u;
#pragma unroll
    for (int c = 0; c < CPT; ++c) u.e[c] = o[c];
    __stcs(reinterpret_cast<uint4*>(p), u.v);
  } else if (CPT * sizeof(TOut) == 16 && nvalid == CPT && ((uintptr_t)p % 16) == 0) {
    // rows whose pitch is not a multiple of 16 bytes: this row's segment may still be aligned
    union {
      uint4 v;
      TOut e[CPT];
    } u;
#pragma unroll
    for (int c = 0; c < CPT; ++c) u.e[c] = o[c];
    __stcs(reinterpret_cast<uint4*>(p), u.v);
  } else if (CPT * sizeof(TOut) == 16 && nvalid == CPT && ((uintptr_t)p % 8) == 0) {
    union {
      uint2 v[2];
      TOut e[CPT];
    } u;
#pragma unroll
    for (int c = 0; c < CPT; ++c) u.e[c] = o[c];
    __stcs(reinterpret_cast<uint2*>(p), u.v[0]);
    __stcs(reinterpret_cast<uint2*>(p) + 1, u.v[1]);
  } else {
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (c < nvalid) __stcs(p + c, o[c]);
  }
}

// One row segment of CPT input elements from global memory when the caller's
// rows are not vector-aligned (packed rows of odd widths, offset views): four
// 1-byte pixels come from the one or two aligned 32-bit words that hold them
// (both inside the buffer: each holds a byte of the segment), a 16-byte
// segment of wider types by one vector load when this row happens to be
// aligned; else element by element.  Elements past nvalid are zero.
template <class TIn, int CPT>
__device__ __forceinline__ void load_seg_unaligned(const TIn* p, int nvalid, TIn (&x)[CPT]) {
  if (sizeof(TIn) == 1 && CPT == 4) {
    const uintptr_t a = (uintptr_t)p;
    const unsigned off = (unsigned)(a & 3u);
    const uint32_t* wp = reinterpret_cast<const uint32_t*>(a - off);
    const uint32_t lo = __ldcs(wp);
    const uint32_t hi = (off + (unsigned)nvalid > 4u) ? __ldcs(wp + 1) : 0u;
    uint32_t v = __funnelshift_r(lo, hi, off * 8u);
    if (nvalid < 4) v &= (1u << (8 * nvalid)) - 1u;
    union {
      uint32_t w;
      TIn e[4];
    } u;
    u.w = v;
#pragma unroll
    for (int c = 0; c < CPT; ++c) x[c] = u.e[c < 4 ? c : 0];
  } else if (nvalid == CPT && ((uintptr_t)p % (CPT * sizeof(TIn))) == 0) {
    load_seg<TIn, CPT>(p, true, CPT, x);
  } else {
#pragma unroll
    for (int c = 0; c < CPT; ++c) x[c] = (c < nvalid) ? __ldcs(p + c) : TIn(0);
  }
}

// Cold paths, kept out of line so the tile loop stays small: a thread moves
// its own RPW x CPT block between global memory and its slots of the stage
// (row stride TW elements).  fill: rows [0, rows) and columns [c0, nvalid)
// come from global memory, columns below c0 are left as they are (TMA filled
// them), everything else becomes zero.  drain: the block's valid part
// (rows [0, rows), columns [c0, nvalid)) goes to global memory.
template <class TIn, int CPT, int RPW, int TW>
__device__ __noinline__ void stage_fill(TIn* sb, const TIn* g, long long pitch, int rows, int nvalid, int c0,
                                        bool vec) {
  // every row's loads first, then the shared-memory stores, so the loads overlap
  RowSeg<TIn, CPT> seg[RPW];
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    TIn x[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) x[c] = TIn(0);
    if (c0 > 0) load_seg_smem<TIn, CPT>(sb + r * TW, x);
    if (r < rows && nvalid > 0) {
      if (vec && c0 == 0 && nvalid == CPT) {
        load_seg<TIn, CPT>(g + r * pitch, true, CPT, x);
      } else if (c0 == 0) {
        load_seg_unaligned<TIn, CPT>(g + r * pitch, nvalid, x);
      } else {
#pragma unroll
        for (int c = 0; c < CPT; ++c)
          if (c >= c0) x[c] = (c < nvalid) ? __ldcs(g + r * pitch + c) : TIn(0);
      }
    } else {
#pragma unroll
      for (int c = 0; c < CPT; ++c)
        if (c >= c0) x[c] = TIn(0);
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c) seg[r].u.e[c] = x[c];
  }
#pragma unroll
  for (int r = 0; r < RPW; ++r) *reinterpret_cast<typename RowSeg<TIn, CPT>::V*>(sb + r * TW) = seg[r].u.v;
}

template <class TOut, int CPT, int RPW, int TW, bool REV>
__device__ __noinline__ void stage_drain(const TOut* so, TOut* g, long long pitch, int rows, int nvalid, int c0,
                                         bool vec) {
  for (int r = 0; r < rows && r < RPW; ++r) {
    TOut o[CPT];
    load_seg_smem<TOut, CPT>(so + r * TW, o);
    if (vec && c0 == 0 && nvalid == CPT) {
      store_seg<TOut, CPT>(g + r * pitch, true, CPT, o);
    } else {
#pragma unroll
      for (int c = 0; c < CPT; ++c)
        if (c >= c0 && c < nvalid) __stcs(g + r * pitch + c, o[c]);
    }
  }
}

// ---------------------------------------------------------------------------
// mbarrier / TMA / named-barrier helpers (inline PTX)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, int x, int y, int z, uint32_t src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(z), "r"(src)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Waits until every bulk store this thread committed has finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Waits until every bulk store this thread committed is complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Shared-memory loads and stores the compiler may not cache or reorder
// (values handed between warps without a barrier).
template <class T>
__device__ __forceinline__ T vload(const T* p) {
  T r;
  const volatile uint32_t* src = reinterpret_cast<const volatile uint32_t*>(p);
  uint32_t* dst = reinterpret_cast<uint32_t*>(&r);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(T) / 4); ++i) dst[i] = src[i];
  return r;
}
template <class T>
__device__ __forceinline__ void vstore(T* p, const T& v) {
  volatile uint32_t* dst = reinterpret_cast<volatile uint32_t*>(p);
  const uint32_t* src = reinterpret_cast<const uint32_t*>(&v);
#pragma unroll
  for (int i = 0; i < (int)(sizeof(T) / 4); ++i) dst[i] = src[i];
}

// Records a device error (first one wins) in the workspace header.
__device__ __forceinline__ void record_error(const SatParams& P, long long tile) {
  if (atomicCAS(&P.ws->error, 0u, kDevErrTimeout) == 0u) P.ws->error_tile = (uint32_t)tile;
}

// End of a launch, called by thread 0 of every CTA after its last tile: the
// last CTA to get here resets the ticket and the CTA count, moves a recorded
// error to the sticky word (and clears it for the next launch) and advances
// the epoch, which invalidates every status word of this launch.
__device__ __forceinline__ void finish_launch(const SatParams& P, uint32_t epoch) {
  __threadfence();
  const uint32_t prev = atomicAdd(&P.ws->done, 1u);
  if (prev == gridDim.x - 1) {
    __threadfence();
    const uint32_t err = ld_relaxed_u32(&P.ws->error);
    if (err != 0u) {
      if (P.ws->sticky == 0u) {
        P.ws->sticky = err;
        P.ws->sticky_tile = P.ws->error_tile;
      }
      P.ws->error = 0u;
      P.ws->error_tile = 0u;
    }
    P.ws->ticket = 0ull;
    P.ws->done = 0u;
    P.ws->epoch = epoch + 1u;
    __threadfence();
  }
}

// Bounded wait for an mbarrier phase; false (and an error recorded) when the
// wait limit runs out.
static __device__ __noinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, const SatParams& P, long long tile) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_timer_ns();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 63u &&
        ((long long)(global_timer_ns() - t0) > P.wait_limit_ns || ld_relaxed_u32(&P.ws->error) != 0u)) {
      record_error(P, tile);
      return false;
    }
  }
}

// Ticket -> tile.  Tiles of one image are ordered by anti-diagonal d = tx+ty,
// then by ty; P(d) = number of tiles on diagonals < d.
__device__ __forceinline__ long long diag_prefix(long long d, long long ntx, long long nty) {
  const long long a = ntx < nty ? ntx : nty;
  const long long b = ntx < nty ? nty : ntx;
  if (d <= a) return d * (d + 1) / 2;
  if (d <= b) return a * (a + 1) / 2 + (d - a) * a;
  const long long m = ntx + nty - 1 - d;
  return ntx * nty - m * (m + 1) / 2;
}

__device__ __forceinline__ void diag_tile(long long k, int ntx, int nty, int& tx, int& ty) {
  long long lo = 0, hi = (long long)ntx + nty - 2; // largest d with P(d) <= k
  while (lo < hi) {
    const long long mid = (lo + hi + 1) >> 1;
    if (diag_prefix(mid, ntx, nty) <= k) lo = mid;
    else hi = mid - 1;
  }
  const long long d = lo;
  const long long i = k - diag_prefix(d, ntx, nty);
  const long long ty_min = d - (ntx - 1) > 0 ? d - (ntx - 1) : 0;
  ty = (int)(ty_min + i);
  tx = (int)(d - ty);
}

// Windowed look-back.  The look-back thread of a vector element (or of the
// corner) reads the status words of W predecessors at once -- one round trip
// for W tiles.  It walks the window from the nearest predecessor, summing
// aggregates until it meets an inclusive value; when it reaches a predecessor
// that has published nothing yet, it reads the window again, now starting at
// that predecessor.  So an inclusive value W tiles back is found in one round
// trip as long as the tiles in between have published their aggregates, which
// they do right after their local phase.  The first window is read one local
// phase ahead of its use (before the next tile's local phase), so that round
// trip overlaps work and the values it sees are recent.  Measured at 8192^2
// (f32, u8 -> u32): windows of 1 or 2 predecessors beat 4 by ~1.5 % and 6 or 8
// lose 2-5 %: the inclusive value is nearly always one or two tiles back, and
// wider windows only add loads; 8-byte accumulators see no difference.
template <class A>
struct EarlyWin {
  static constexpr int W = Ar<A>::K == 1 ? 2 : 3;
  unsigned long long w[W][Ar<A>::K];
};

template <class A>
__device__ __forceinline__ void early_read(EarlyWin<A>& e, const unsigned long long* base, long long stride,
                                           int steps, int first = 0) {
  constexpr int K = Ar<A>::K;
#pragma unroll
  for (int q = 0; q < EarlyWin<A>::W; ++q) {
#pragma unroll
    for (int k = 0; k < K; ++k)
      e.w[q][k] = (first + q < steps) ? ld_relaxed_u64(base + (first + q + 1) * stride + k) : 0ull;
  }
}

// 0 = not published yet, else kStateAgg / kStateInc with the value in `val`.
template <class A>
__device__ __forceinline__ uint32_t decode_word(const unsigned long long (&w)[Ar<A>::K], uint32_t tagA, uint32_t tagI,
                                                A& val) {
  constexpr int K = Ar<A>::K;
  const uint32_t tag = (uint32_t)(w[0] >> 32);
  bool ok = (tag == tagA || tag == tagI);
  uint32_t pl[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    ok = ok && ((uint32_t)(w[k] >> 32) == tag);
    pl[k] = (uint32_t)w[k];
  }
  if (!ok) return 0u;
  val = Ar<A>::from_words(pl);
  return tag & 3u;
}

template <class A>
__device__ __forceinline__ A resolve(EarlyWin<A>& e, const unsigned long long* base, long long stride, int steps,
                                     uint32_t tagA, uint32_t tagI, const SatParams& P, long long tile) {
  constexpr int W = EarlyWin<A>::W;
  A acc = Ar<A>::zero();
  int i = 0; // predecessors already accounted for
  unsigned long long t0 = 0;
  unsigned ns = 0;
  for (uint32_t round = 0;; ++round) {
    bool progressed = false;
#pragma unroll
    for (int q = 0; q < W; ++q) {
      if (i >= steps) return acc;
      A val;
      const uint32_t st = decode_word<A>(e.w[q], tagA, tagI, val);
      if (!st) break;
      acc = Ar<A>::add(val, acc);
      ++i;
      progressed = true;
      if (st == kStateInc) return acc;
    }
    if (i >= steps) return acc;
    if (!progressed) {
      // the nearest open predecessor has published nothing yet: back off, bounded
      if (t0 == 0) t0 = global_timer_ns();
      if (ns) __nanosleep(ns);
      ns = ns ? (ns < 256 ? 2 * ns : ns) : 32;
      if ((round & 7u) == 7u &&
          ((long long)(global_timer_ns() - t0) > P.wait_limit_ns || ld_relaxed_u32(&P.ws->error) != 0u)) {
        record_error(P, tile);
        return acc;
      }
    }
    early_read<A>(e, base, stride, steps, i);
  }
}

// resolve() for N elements of one thread at once (a look-back thread that owns
// several columns or rows of a tile): every round walks each open element's
// window, then re-reads the windows of all elements still open together, so
// their round trips overlap instead of following one another.  Element i's
// status words start at base0 + i * elem_step.
template <class A, int N>
__device__ __forceinline__ void resolve_n(EarlyWin<A> (&e)[N], const unsigned long long* base0, long long elem_step,
                                          long long stride, int steps, uint32_t tagA, uint32_t tagI,
                                          const SatParams& P, long long tile, A (&acc)[N]) {
  constexpr int W = EarlyWin<A>::W;
  int idx[N];
  uint32_t open = 0;
#pragma unroll
  for (int n = 0; n < N; ++n) {
    acc[n] = Ar<A>::zero();
    idx[n] = 0;
    if (steps > 0) open |= 1u << n;
  }
  unsigned long long t0 = 0;
  unsigned ns = 0;
  for (uint32_t round = 0; open; ++round) {
    bool progressed = false;
#pragma unroll
    for (int n = 0; n < N; ++n) {
      if (!(open & (1u << n))) continue;
#pragma unroll
      for (int q = 0; q < W; ++q) {
        A val;
        const uint32_t st = decode_word<A>(e[n].w[q], tagA, tagI, val);
        if (!st) break;
        acc[n] = Ar<A>::add(val, acc[n]);
        ++idx[n];
        progressed = true;
        if (st == kStateInc || idx[n] >= steps) {
          open &= ~(1u << n);
          break;
        }
      }
    }
    if (!open) break;
    if (!progressed) {
      if (t0 == 0) t0 = global_timer_ns();
      if (ns) __nanosleep(ns);
      ns = ns ? (ns < 256 ? 2 * ns : ns) : 32;
      if ((round & 7u) == 7u &&
          ((long long)(global_timer_ns() - t0) > P.wait_limit_ns || ld_relaxed_u32(&P.ws->error) != 0u)) {
        record_error(P, tile);
        return;
      }
    }
#pragma unroll
    for (int n = 0; n < N; ++n)
      if (open & (1u << n)) early_read<A>(e[n], base0 + n * elem_step, stride, steps, idx[n]);
  }
}

// The fields of an image descriptor a tile needs, in registers.  For a single
// image they are read straight from the kernel parameter (constant bank);
// only batched launches read the descriptor table in global memory.
struct ImageView {
  const void* in;
  void* out;
  int64_t in_pitch, out_pitch, width, height, in_plane, out_plane, tma_in_w, tma_out_w;
  int32_t ntx, nty;
  uint32_t flags;
};

__device__ __forceinline__ ImageView image_view(const SatParams& P, int img) {
  ImageView v;
  if (P.n_images == 1) {
    v.in = P.img0.in;
    v.out = P.img0.out;
    v.in_pitch = P.img0.in_pitch;
    v.out_pitch = P.img0.out_pitch;
    v.width = P.img0.width;
    v.height = P.img0.height;
    v.in_plane = P.img0.in_plane;
    v.out_plane = P.img0.out_plane;
    v.tma_in_w = P.img0.tma_in_w;
    v.tma_out_w = P.img0.tma_out_w;
    v.ntx = P.img0.ntx;
    v.nty = P.img0.nty;
    v.flags = P.img0.flags;
  } else {
    const ImageDesc* D = &P.images[img];
    v.in = D->in;
    v.out = D->out;
    v.in_pitch = D->in_pitch;
    v.out_pitch = D->out_pitch;
    v.width = D->width;
    v.height = D->height;
    v.in_plane = D->in_plane;
    v.out_plane = D->out_plane;
    v.tma_in_w = D->tma_in_w;
    v.tma_out_w = D->tma_out_w;
    v.ntx = D->ntx;
    v.nty = D->nty;
    v.flags = D->flags;
  }
  return v;
}

// DIRECT: results go from registers straight to global memory, so a stage
// holds only the tile's input (tall tiles of 1-byte pixels then fit).
template <class TIn, class TOut, class A, int RPW, int NW, int CTAS, bool DIRECT = false>
struct TileShape {
  static constexpr int CPT = 16 / (int)sizeof(TOut);
  static constexpr int TW = 32 * CPT;
  static constexpr int TH = NW * RPW;
  static constexpr int IN_BYTES = TH * TW * (int)sizeof(TIn); // what the TMA load brings
  static constexpr int STAGE_BYTES =
      TH * TW * (int)(DIRECT || sizeof(TIn) > sizeof(TOut) ? sizeof(TIn) : sizeof(TOut));
  // static shared memory of the kernel (s_tr, s_colp, the vectors), roughly
  // rows per transpose pass: two passes when two CTAs share an SM, to halve the scratch
  static constexpr int RP = (CTAS == 2 && RPW == 8) ? 4 : RPW;
  static constexpr int STATIC_BYTES = (NW * RP * 32 + 2 * NW * TW + 4 * TH + 2 * NW + TW) * (int)sizeof(A) + 256;
  static constexpr int S = Stages<STAGE_BYTES, STATIC_BYTES, CTAS>::value;
  static constexpr int DYN_SMEM = S * STAGE_BYTES;
  static constexpr int THREADS = NW * 32;
};

// A ticket mapped to its tile (t = -1: the tickets are exhausted).
struct TilePlan {
  long long t; // spatial tile index (status words)
  int tx, ty, img, pl;
};

// Maps ticket `tk` to its tile.
// Tile orders inside a plane: anti-diagonal for the SAT (both neighbours
// precede a tile by about a diagonal); row-major when tiles depend only on the
// tile above (column scan) -- the order whose concurrent tiles lie closest in
// memory.
constexpr int kOrderDiag = 0;
constexpr int kOrderRows = 1;

template <bool REV, int ORDER = kOrderDiag>
__device__ __noinline__ TilePlan plan_tile(const SatParams& P, unsigned long long tk) {
  TilePlan tp;
  tp.t = -1;
  tp.tx = tp.ty = tp.img = tp.pl = 0;
  if ((long long)tk >= P.n_tiles) return tp;
  const long long q = REV ? (P.n_tiles - 1 - (long long)tk) : (long long)tk;
  if (P.order) {
    const unsigned long long e = P.order[q];
    tp.img = (int)(e >> 40);
    tp.ty = (int)((e >> 20) & 0xFFFFFu);
    tp.tx = (int)(e & 0xFFFFFu);
    tp.pl = 0;
    tp.t = P.images[tp.img].tile_base + (long long)tp.ty * P.images[tp.img].ntx + tp.tx;
    return tp;
  }
  int img = 0;
  if (P.n_images > 1) {
    int lo = 0, hi = (int)P.n_images - 1; // last image with tile_base <= q
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (P.images[mid].tile_base <= q) lo = mid;
      else hi = mid - 1;
    }
    img = lo;
  }
  const ImageDesc* D = (P.n_images == 1) ? &P.img0 : &P.images[img];
  const int ntx = D->ntx, nty = D->nty;
  // planes one after the other; anti-diagonal order inside a plane
  const long long local = q - D->tile_base;
  const long long pl = local / D->tiles_per_plane;
  int tx, ty;
  const long long li = local - pl * D->tiles_per_plane;
  if (ORDER == kOrderRows) {
    ty = (int)(li / ntx);
    tx = (int)(li - (long long)ty * ntx);
  } else {
    diag_tile(li, ntx, nty, tx, ty);
  }
  tp.t = D->tile_base + pl * D->tiles_per_plane + (long long)ty * ntx + tx;
  tp.tx = tx;
  tp.ty = ty;
  tp.img = img;
  tp.pl = (int)pl;
  return tp;
}

// Publishes a planned tile to the CTA (shared tile info of stage `st`) and
// starts its input on its way into the stage (TMA, or a bare arrive for
// images read from global memory; a bare arrive with tile -1 at the end).
template <class TIn, int TW, int TH, int STAGE_BYTES>
__device__ __forceinline__ void issue_tile(const SatParams& P, const TilePlan& tp, int st, TIn* stage_ptr,
                                           long long* s_tile, int* s_img, int* s_tx, int* s_ty, int* s_pl,
                                           unsigned long long* s_full) {
  const uint32_t bar = smem_u32(&s_full[st]);
  s_tile[st] = tp.t;
  s_img[st] = tp.img;
  s_tx[st] = tp.tx;
  s_ty[st] = tp.ty;
  s_pl[st] = tp.pl;
  if (tp.t < 0) {
    mbar_arrive(bar);
    return;
  }
  const ImageDesc* D = (P.n_images == 1) ? &P.img0 : &P.images[tp.img];
  if (D->flags & kInTma) {
    mbar_arrive_expect_tx(bar, (uint32_t)STAGE_BYTES);
    tma_load_3d(smem_u32(stage_ptr), &D->tmap_in, tp.tx * TW, tp.ty * TH, tp.pl, bar);
  } else {
    mbar_arrive(bar);
  }
}

// Takes ticket `tk`, maps it to a tile and starts its input on its way into
// stage `st`.  Returns false once the tickets are exhausted (the stage then
// carries -1).
template <class TIn, bool REV, int TW, int TH, int STAGE_BYTES, int ORDER = kOrderDiag>
__device__ __noinline__ bool produce(const SatParams& P, unsigned long long tk, int st, TIn* stage_ptr,
                                        long long* s_tile, int* s_img, int* s_tx, int* s_ty, int* s_pl,
                                        unsigned long long* s_full) {
  const TilePlan tp = plan_tile<REV, ORDER>(P, tk);
  issue_tile<TIn, TW, TH, STAGE_BYTES>(P, tp, st, stage_ptr, s_tile, s_img, s_tx, s_ty, s_pl, s_full);
  return tp.t >= 0;
}

// ---------------------------------------------------------------------------
// The tile kernel.  Tiles are software-pipelined through the CTA: iteration k
// runs the local phase of tile k+1, then the look-back of tile k, then the
// output phase of tile k, so the round trips of tile k's look-back overlap
// tile k+1's local work.
//
//  A  (tile k+1) aggregates: each thread sums its CPT-column x RPW-row block by
//     columns (colp) and by rows (rowp).  A transpose through shared memory
//     turns the 32 lanes' row partials of each row into the exclusive prefix E
//     over the lanes (kept in registers until the output phase) and the row
//     total.  Column partials and row totals go to shared memory.
//  B  threads [0,TW): sum tile k+1's column partials into its column
//     aggregate (published at once) and turn them into the exclusive prefix
//     over warps C_w; then finish tile k's column look-back and publish its
//     inclusive column sums.  Threads [TW,TW+TH) do the same for rows, then
//     scan tile k's rowleft over its rows (RL) and form u = sum rowleft, the
//     corner aggregate.  A spare warp resolves tile k's corner (so the
//     corner's inclusive value corner + u is published right away); a spare
//     thread takes tickets and starts TMA loads.
//  D  (tile k) output: warp w forms the SAT row just above its rows,
//        Top_w(x) = corner + RL(above the warp) + sum_{x0<=i<=x} (colabove(i) + C_w(i)),
//     then walks its rows once: run = rowleft(y) + E(y) + in-thread row
//     prefix, acc(x) += run.  Results go back into the tile's stage and leave
//     by one TMA store (or by plain stores for images TMA cannot address);
//     with DIRECT they go from registers straight to global memory, one
//     16-byte segment per thread and row, and the stages hold input only.
//
// The reverse (suffix) SAT runs every scan in the opposite direction.
// ---------------------------------------------------------------------------
// What the tile kernel computes: the SAT, or only its column scan (each
// column's prefix sums: the reference's ScanY, IncrementScanY.cu:10-126),
// which keeps the column look-back and no corner.  The row-only scan (ScanX,
// IncrementScanX.cu:12-113) needs no look-back and has its own kernel
// (scan_rows_t.cu).
constexpr int kKindSat = 0;
constexpr int kKindCols = 2;

template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB, int KIND = kKindSat,
          bool DIRECT = false>
__global__ void __launch_bounds__(NW * 32, MINB) sat_tile_kernel(const __grid_constant__ SatParams P) {
  using SH = TileShape<TIn, TOut, A, RPW, NW, MINB, DIRECT>;
  constexpr int CPT = SH::CPT;
  constexpr int TW = SH::TW;
  constexpr int TH = SH::TH;
  constexpr int S = SH::S;
  constexpr int NC = NW * 32;
  constexpr int STAGE_ELEMS = SH::STAGE_BYTES / (int)sizeof(TIn); // stage stride in input elements
  constexpr int SPARE = NC - (TW + TH);
  static_assert(SPARE >= 64, "threads for rows, columns, the corner warp and the producer");
  static_assert(TH % 32 == 0 && TW % 32 == 0, "groups are whole warps");
  static_assert(32 % RPW == 0, "rows per warp divide the warp");
  static_assert(S >= 3, "a stage for the tile in output, one in the local phase, one loading");
  constexpr int CW = (TW + TH) / 32; // corner warp
  constexpr int PT = NC - 1;         // producer thread (in the last warp, never the corner warp)
  static_assert(CW < NW - 1, "corner warp and producer warp differ");
  constexpr int RP = SH::RP;         // rows per transpose pass
  constexpr int LPR = 32 / RP;       // transpose-scan: lanes per row ...
  constexpr int CH = RP;             // ... and values per lane
  constexpr int K = Ar<A>::K;
  constexpr bool WIDEN = !DIRECT && sizeof(TIn) < sizeof(TOut); // outputs overlap other threads' inputs in the stage
  constexpr int ORDER = KIND == kKindCols ? kOrderRows : kOrderDiag;
  using AR = Ar<A>;

  extern __shared__ __align__(128) unsigned char dsmem[];
  TIn* stages = reinterpret_cast<TIn*>(dsmem);

  __shared__ A s_tr[NW][RP][32];    // per-warp transpose scratch (index lane ^ row: conflict free)
  __shared__ A s_colp[2][NW][TW];   // per warp: raw column partials (by slot); then the exclusive prefix over warps
  __shared__ A s_rowagg[TH];        // row totals of the tile in the local phase
  // row look-back results, by tile parity: tile k+1's are made while tile k's are used
  __shared__ A s_rowleft[2][TH];    // rowleft of each row
  __shared__ A s_RLw[2][NW];        // per warp: the scan over its 32-row group of rowleft, at the row before the warp
  __shared__ A s_rlw[2][TH / 32];   // per 32-row group: the sum of rowleft
  __shared__ A s_colabove[TW];      // its column look-back result (by slot)
  __shared__ A s_corner;
  __shared__ A s_u[2];              // u = sum of rowleft (the corner aggregate), by tile parity
  __shared__ int s_cnt_row;         // arrivals of the row warps
  __shared__ long long s_tile[S];   // spatial tile index per stage (-1: no more tiles)
  __shared__ int s_img[S];
  __shared__ int s_tx[S], s_ty[S], s_pl[S];
  __shared__ __align__(8) unsigned long long s_full[S];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t epoch = ld_relaxed_u32(&P.ws->epoch);
  const uint32_t tagA = make_tag(epoch, kStateAgg);
  const uint32_t tagI = make_tag(epoch, kStateInc);

  unsigned long long pending = 0; // producer thread: the next ticket, fetched a tile ahead
  bool producing = true;          // producer thread: tickets not yet exhausted
  if (tid == 0) {
    s_cnt_row = 0;
  }
  if (tid == PT) {
#pragma unroll
    for (int s = 0; s < S; ++s) mbar_init(smem_u32(&s_full[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
#pragma unroll
    for (int s = 0; s < S - 1; ++s) {
      if (producing)
        producing = produce<TIn, REV, TW, TH, SH::IN_BYTES, ORDER>(P, atomicAdd(&P.ws->ticket, 1ull), s,
                                                            stages + s * STAGE_ELEMS, s_tile, s_img, s_tx, s_ty,
                                                            s_pl, s_full);
    }
    if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
  }
  __syncthreads();

  // ---- per-tile state carried from the local phase to the output phase ---------
  struct Tile {
    long long t;
    int tx, ty, img, p;
  };
  Tile nxt, cur;
  A E_nxt[RPW], E_cur[RPW];
  A agg_cur = AR::zero(); // this thread's element of the current tile's aggregate (column or row groups)
  const unsigned long long* lb_base = nullptr;
  long long lb_stride = 0;
  int lb_steps = 0;

  // phase A for the tile in stage kk % S; false when the tickets ran out
  auto phase_a = [&](int kk) -> bool {
    const int st = kk % S;
    mbar_wait_bounded(smem_u32(&s_full[st]), (kk / S) & 1, P, -1);
    nxt.t = s_tile[st];
    if (nxt.t < 0) return false;
    nxt.tx = s_tx[st];
    nxt.ty = s_ty[st];
    nxt.img = s_img[st];
    nxt.p = s_pl[st];
    const ImageView D = image_view(P, nxt.img);
    const uint32_t flags = D.flags;
    const long long x0 = (long long)nxt.tx * TW, y0 = (long long)nxt.ty * TH;
    const long long xt = x0 + (long long)lane * CPT;
    const long long rem = D.width - xt;
    const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);
    TIn* sb = stages + st * STAGE_ELEMS + (warp * RPW) * TW + lane * CPT;
    A colp[CPT], rowp[RPW];
#pragma unroll
    for (int c = 0; c < CPT; ++c) colp[c] = AR::zero();
    const bool tma = flags & kInTma;
    const TIn* gin = static_cast<const TIn*>(D.in) + (long long)nxt.p * D.in_plane + (y0 + warp * RPW) * D.in_pitch + xt;
    const bool vin = (flags & kInVec) && nvalid == CPT;
    const bool tail_in = tma && nvalid > 0 && xt + nvalid > D.tma_in_w;
    if (!tma || tail_in) {
      // no TMA for this image, or columns past the map (they arrived as zeros)
      const long long rows = D.height - (y0 + warp * RPW);
      const int c0 = tma ? (int)(D.tma_in_w - xt > 0 ? D.tma_in_w - xt : 0) : 0;
      stage_fill<TIn, CPT, RPW, TW>(sb, gin, D.in_pitch, rows < 0 ? 0 : (rows > RPW ? RPW : (int)rows), nvalid, c0,
                                    vin);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); // before TMA refills the stage
    }
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      RowSeg<TIn, CPT> x;
      x.u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
      A rs = AR::zero();
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        colp[c] = AddIn<A, TIn>::add(colp[c], x.u.e[c]);
        rs = AddIn<A, TIn>::add(rs, x.u.e[c]);
      }
      rowp[r] = rs;
    }
    // row partials -> exclusive prefix over the lanes (E) and the row totals,
    // RP rows per pass through the transpose scratch (not for the column scan)
#pragma unroll
    for (int h = 0; h < (KIND == kKindCols ? 0 : RPW / RP); ++h) {
#pragma unroll
      for (int r = 0; r < RP; ++r) s_tr[warp][r][lane ^ r] = rowp[h * RP + r];
      __syncwarp();
      {
        const int r = lane / LPR, q = lane % LPR;
        A tot = AR::zero();
#pragma unroll
        for (int i = 0; i < CH; ++i) tot = AR::add(tot, s_tr[warp][r][(q * CH + (REV ? CH - 1 - i : i)) ^ r]);
        A incl = tot;
#pragma unroll
        for (int d = 1; d < LPR; d <<= 1) {
          const A o = REV ? AR::shfl_down(incl, d, LPR) : AR::shfl_up(incl, d, LPR);
          if (REV ? (q + d < LPR) : (q >= d)) incl = AR::add(o, incl);
        }
        A ex = REV ? AR::shfl_down(incl, 1, LPR) : AR::shfl_up(incl, 1, LPR);
        if (q == (REV ? LPR - 1 : 0)) ex = AR::zero();
#pragma unroll
        for (int i = 0; i < CH; ++i) {
          const int idx = (q * CH + (REV ? CH - 1 - i : i)) ^ r;
          const A vv = s_tr[warp][r][idx];
          s_tr[warp][r][idx] = ex;
          ex = AR::add(ex, vv);
        }
        if (q == (REV ? 0 : LPR - 1)) s_rowagg[warp * RPW + h * RP + r] = incl;
      }
      __syncwarp();
#pragma unroll
      for (int r = 0; r < RP; ++r) E_nxt[h * RP + r] = s_tr[warp][r][lane ^ r];
      if (RPW / RP > 1) __syncwarp();
    }
#pragma unroll
    for (int c = 0; c < CPT; ++c) s_colp[kk & 1][warp][c * 32 + lane] = colp[c];
    return true;
  };

  // publish the new tile's aggregate (column or row element), start its look-back window
  auto start_lookback = [&](int kk) {
    const long long t = nxt.t;
    const ImageView D = image_view(P, nxt.img);
    const int ntx = D.ntx, nty = D.nty;
    const bool stall = (t == P.stall_tile);
    if (tid < TW) {
      const int j = tid;
      A ac = AR::zero();
#pragma unroll
      for (int w = 0; w < NW; ++w) ac = AR::add(ac, s_colp[kk & 1][w][j]);
      if ((REV ? (nxt.ty > 0) : (nxt.ty < nty - 1)) && !stall)
        publish<A>(P.col_words + ((unsigned long long)t * TW + j) * K, ac, tagA);
      A run = AR::zero();
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        const int w = REV ? NW - 1 - i : i;
        const A b = s_colp[kk & 1][w][j];
        s_colp[kk & 1][w][j] = run;
        run = AR::add(run, b);
      }
      agg_cur = ac;
      lb_base = P.col_words + ((unsigned long long)t * TW + j) * K;
      lb_stride = (REV ? 1 : -1) * (long long)ntx * TW * K;
      lb_steps = REV ? (nty - 1 - nxt.ty) : nxt.ty;
    } else if (tid < TW + TH) {
      const int yy = tid - TW;
      if (KIND != kKindCols && (REV ? (nxt.tx > 0) : (nxt.tx < ntx - 1)) && !stall)
        publish<A>(P.row_words + ((unsigned long long)t * TH + yy) * K, s_rowagg[yy], tagA);
    } else if (warp == CW && lane == 0) {
      lb_base = P.corner_words + (unsigned long long)t * K;
      lb_stride = (REV ? 1 : -1) * (long long)ntx * K;
      lb_steps = REV ? (nty - 1 - nxt.ty) : nxt.ty;
    }
  };

  // iteration k = -1 only runs the local phase of tile 0 (one copy of each
  // phase in the code keeps the loop small)
  bool have = true;
  for (int k = -1;; ++k) {
    const int st = (k + S) % S;
    A my_agg = AR::zero();
    EarlyWin<A> my_win; // look-back window of the current tile (columns, rows or the corner)
    const unsigned long long* my_base = lb_base;
    const long long my_stride = lb_stride;
    const int my_steps = lb_steps;
    if (k >= 0) {
      if (!have) break;
      cur = nxt;
#pragma unroll
      for (int r = 0; r < RPW; ++r) E_cur[r] = E_nxt[r];
      my_agg = agg_cur;
      // the current tile's first column / corner look-back window: read now,
      // used after A(k+1), so the round trip overlaps the local phase
      if ((tid < TW) || (KIND == kKindSat && warp == CW && lane == 0))
        early_read<A>(my_win, my_base, my_stride, my_steps);
    }
    // Row threads run the row look-back of the NEXT tile (k+1) in this
    // iteration, right after its local phase: its u (the corner aggregate)
    // then goes out without waiting for this CTA's corner of tile k.
    long long rt = -1;
    int rtx = 0, rty = 0, rntx = 1, rnty = 1;
    if (KIND != kKindCols && tid >= TW && tid < TW + TH) {
      const int sn = (k + 1) % S; // tile k+1's stage: filled at least one iteration ago
      rt = s_tile[sn];
      if (rt >= 0) {
        rtx = s_tx[sn];
        rty = s_ty[sn];
        const ImageView Dn = image_view(P, s_img[sn]);
        rntx = Dn.ntx;
        rnty = Dn.nty;
        my_base = P.row_words + ((unsigned long long)rt * TH + (tid - TW)) * K;
        early_read<A>(my_win, my_base, (REV ? 1 : -1) * (long long)TH * K, REV ? (rntx - 1 - rtx) : rtx);
      }
    }

    // ---- A(k+1) ----------------------------------------------------------------
    const bool have_next = phase_a(k + 1);
    __syncthreads();

    // ---- B: the next tile's aggregates and row look-back, the current tile's
    //      column and corner look-backs ------------------------------------------
    const bool has_cur = k >= 0;
    const long long t = has_cur ? cur.t : -1;
    const bool stall = (t == P.stall_tile);
    bool pub_col = false;
    if (has_cur) {
      const ImageView D = image_view(P, cur.img);
      pub_col = REV ? (cur.ty > 0) : (cur.ty < D.nty - 1);
    }
    if (have_next) start_lookback(k + 1);
    // one look-back call site for the three roles (columns, rows, corner)
    A got = AR::zero();
    const bool lb_row = tid >= TW && tid < TW + TH && rt >= 0;
    const bool lb_cur =
        has_cur && ((tid < TW) || (KIND == kKindSat && warp == CW && lane == 0));
    if (lb_row || lb_cur) {
      const long long stride = lb_row ? (REV ? 1 : -1) * (long long)TH * K : my_stride;
      const int steps = lb_row ? (REV ? (rntx - 1 - rtx) : rtx) : my_steps;
      got = resolve<A>(my_win, my_base, stride, steps, tagA, tagI, P, lb_row ? rt : t);
    }
    if (tid < TW) {
      if (!has_cur) {
        // nothing to do for the columns before the first tile
      } else {
        const A above = got;
        if (pub_col && !stall)
          publish<A>(P.col_words + ((unsigned long long)t * TW + tid) * K, AR::add(above, my_agg), tagI);
        s_colabove[tid] = above;
      }
    } else if (tid < TW + TH) {
      if (rt >= 0) {
      const int yy = tid - TW;
      const int nb = (k + 1) & 1;
      const bool rstall = (rt == P.stall_tile);
      const A left = got;
      if ((REV ? (rtx > 0) : (rtx < rntx - 1)) && !rstall)
        publish<A>(P.row_words + ((unsigned long long)rt * TH + yy) * K, AR::add(left, s_rowagg[yy]), tagI);
      s_rowleft[nb][yy] = left;
      // scan of rowleft over this warp's 32 rows, in scan order; the group sum
      A incl = left;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const A o = REV ? AR::shfl_down(incl, d) : AR::shfl_up(incl, d);
        if (REV ? (lane + d < 32) : (lane >= d)) incl = AR::add(o, incl);
      }
      if (REV ? (yy % RPW == 0 && yy > 0) : ((yy + 1) % RPW == 0 && yy + 1 < TH))
        s_RLw[nb][REV ? yy / RPW - 1 : (yy + 1) / RPW] = incl;
      if (lane == (REV ? 0 : 31)) s_rlw[nb][yy / 32] = incl;
      __syncwarp();
      if (lane == 0) {
        // the last row warp to get here forms u = sum of rowleft and publishes it
        // as the next tile's corner aggregate
        __threadfence_block();
        if (atomicAdd(&s_cnt_row, 1) == TH / 32 - 1) {
          __threadfence_block();
          s_cnt_row = 0;
          A u = AR::zero();
#pragma unroll
          for (int g = 0; g < TH / 32; ++g) u = AR::add(u, vload(&s_rlw[nb][g]));
          s_u[nb] = u;
          if (KIND == kKindSat && (REV ? (rty > 0) : (rty < rnty - 1)) && !rstall)
            publish<A>(P.corner_words + (unsigned long long)rt * K, u, tagA);
        }
      }
      }
    } else if (warp == CW) {
      if (lane == 0 && has_cur) {
        // corner of tile k; its u was formed in the previous iteration
        s_corner = got;
        if (KIND == kKindSat && pub_col && !stall)
          publish<A>(P.corner_words + (unsigned long long)t * K, AR::add(got, s_u[k & 1]), tagI);
      }
    } else if (tid == PT && producing && has_cur) {
      // tile k+S-1 into the stage whose store (tile k-1) has finished reading it
      const int ps = (st + S - 1) % S;
      bulk_wait_read_all();
      producing = produce<TIn, REV, TW, TH, SH::IN_BYTES, ORDER>(P, pending, ps, stages + ps * STAGE_ELEMS, s_tile, s_img,
                                                          s_tx, s_ty, s_pl, s_full);
      if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
    }
    __syncthreads();
    if (!has_cur) {
      have = have_next;
      continue;
    }

    // ---- D(k): scan with the carries injected, results out ---------------------
    {
      const ImageView D = image_view(P, cur.img);
      const uint32_t flags = D.flags;
      const long long x0 = (long long)cur.tx * TW, y0 = (long long)cur.ty * TH;
      const long long xt = x0 + (long long)lane * CPT;
      const long long rem = D.width - xt;
      const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);
      const A corner = s_corner;
      A top[CPT];
      {
        const bool has_prev = REV ? (warp < NW - 1) : (warp > 0);
        A rl_prev = AR::zero();
        if (has_prev) {
          // RL of the row just outside the warp: its group's scan plus the groups before it
          const int yp = REV ? (warp + 1) * RPW : warp * RPW - 1;
          rl_prev = s_RLw[k & 1][warp];
#pragma unroll
          for (int g = 0; g < TH / 32; ++g)
            if (REV ? (g > yp / 32) : (g < yp / 32)) rl_prev = AR::add(s_rlw[k & 1][g], rl_prev);
        }
        A cp[CPT];
#pragma unroll
        for (int i = 0; i < CPT; ++i) {
          const int c = REV ? CPT - 1 - i : i;
          cp[c] = AR::add(s_colabove[c * 32 + lane], s_colp[k & 1][warp][c * 32 + lane]);
          if (i) cp[c] = AR::add(cp[REV ? c + 1 : c - 1], cp[c]);
        }
        A incl = cp[REV ? 0 : CPT - 1];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const A o = REV ? AR::shfl_down(incl, d) : AR::shfl_up(incl, d);
          if (REV ? (lane + d < 32) : (lane >= d)) incl = AR::add(o, incl);
        }
        A ex = REV ? AR::shfl_down(incl, 1) : AR::shfl_up(incl, 1);
        if (lane == (REV ? 31 : 0)) ex = AR::zero();
        const A base = AR::add(AR::add(corner, rl_prev), ex);
#pragma unroll
        for (int c = 0; c < CPT; ++c) top[c] = AR::add(base, cp[c]);
        if (KIND == kKindCols) {
          // column scan: each column's carry only (no prefix over the columns)
#pragma unroll
          for (int c = 0; c < CPT; ++c) top[c] = AR::add(s_colabove[c * 32 + lane], s_colp[k & 1][warp][c * 32 + lane]);
        }
      }
      TIn* sb = stages + st * STAGE_ELEMS + (warp * RPW) * TW + lane * CPT;
      TOut* so = reinterpret_cast<TOut*>(stages + st * STAGE_ELEMS) + (warp * RPW) * TW + lane * CPT;
      const bool tma_out = flags & kOutTma;
      RowSeg<TIn, CPT> raw[WIDEN ? RPW : 1];
      if (WIDEN) {
        // wider outputs overwrite other threads' inputs: read all inputs first
#pragma unroll
        for (int r = 0; r < (WIDEN ? RPW : 1); ++r)
          raw[r].u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
        __syncthreads();
      }
      const int64_t out_pitch = D.out_pitch;
      const int64_t height = D.height;
      const bool vout = (flags & kOutVec) && nvalid == CPT;
      TOut* out = static_cast<TOut*>(D.out) + (long long)cur.p * D.out_plane + (y0 + warp * RPW) * out_pitch + xt;
      const bool tail_out = tma_out && nvalid > 0 && xt + nvalid > D.tma_out_w;
#pragma unroll
      for (int i = 0; i < RPW; ++i) {
        const int r = REV ? RPW - 1 - i : i;
        RowSeg<TIn, CPT> x;
        if (WIDEN) x = raw[WIDEN ? r : 0];
        else x.u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
        A run = AR::add(E_cur[r], s_rowleft[k & 1][warp * RPW + r]);
        union {
          uint4 v;
          TOut e[CPT];
        } o;
#pragma unroll
        for (int ii = 0; ii < CPT; ++ii) {
          const int c = REV ? CPT - 1 - ii : ii;
          const A a = Cvt<A, TIn>::in(x.u.e[c]);
          if (KIND == kKindCols) {
            top[c] = AR::add(top[c], a);
            o.e[c] = OutCvt<TOut, A>::out(top[c]);
          } else {
            run = AR::add(run, a);
            if (KIND == kKindSat) top[c] = AR::add(top[c], run);
            o.e[c] = OutCvt<TOut, A>::out(top[c]);
          }
        }
        if (DIRECT) {
          if (y0 + warp * RPW + r < height && nvalid > 0) store_seg<TOut, CPT>(out + r * out_pitch, vout, nvalid, o.e);
        } else {
          *reinterpret_cast<uint4*>(so + r * TW) = o.v;
        }
      }
      if (!DIRECT && (!tma_out || tail_out)) {
        // no TMA for this image, or columns past the map: plain stores
        const long long rows = height - (y0 + warp * RPW);
        const int c0 = tma_out ? (int)(D.tma_out_w - xt > 0 ? D.tma_out_w - xt : 0) : 0;
        stage_drain<TOut, CPT, RPW, TW, REV>(so, out, out_pitch, rows < 0 ? 0 : (rows > RPW ? RPW : (int)rows),
                                             nvalid, c0, vout);
      }
      // end of the tile: shared vectors may be reused; with TMA output one bulk
      // tensor store moves the tile out (clipped at the image edges) and drains
      // while the CTA goes on with the next tiles.  The stage is written by the
      // generic proxy and next read or overwritten by TMA: order the two.
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (!DIRECT && tma_out && tid == PT) {
        const CUtensorMap* map = (P.n_images == 1) ? &P.img0.tmap_out : &P.images[cur.img].tmap_out;
        tma_store_3d(map, cur.tx * TW, cur.ty * TH, cur.p, smem_u32(stages + st * STAGE_ELEMS));
      }
    }
    have = have_next;
  }
  if (tid == PT) bulk_wait_all(); // stores read shared memory until they complete

  // ---- end of launch: the last CTA resets the ticket and advances the epoch --
  __syncthreads();
  if (tid == 0) finish_launch(P, epoch);
}

}  // namespace satgb
