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

struct ImageDesc {
  CUtensorMap tmap_in; // 2-D tiled map of the input (valid when flags & kInTma)
  const void* in;
  void* out;
  int64_t in_pitch;  // elements
  int64_t out_pitch; // elements
  int64_t width, height;
  int64_t tile_base; // global index of the image's first tile
  int32_t ntx, nty;  // tiles across / down
  uint32_t flags;    // kInVec | kOutVec | kInTma
  uint32_t pad;
};
constexpr uint32_t kInVec = 1u;  // every thread's CPT-element input row segment is vector-aligned
constexpr uint32_t kOutVec = 2u; // every 16-byte output row segment is aligned
constexpr uint32_t kInTma = 4u;  // tmap_in is valid: tiles arrive by TMA

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
};

// Pipeline depth: enough stages for ~64 KB of input in flight per CTA.
template <int STAGE_BYTES>
struct Stages {
  static constexpr int value = STAGE_BYTES >= 32768 ? 2 : (STAGE_BYTES >= 16384 ? 3 : 4);
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
  } else {
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      if (c < nvalid) __stcs(p + c, o[c]);
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
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Records a device error (first one wins) in the workspace header.
__device__ __forceinline__ void record_error(const SatParams& P, long long tile) {
  if (atomicCAS(&P.ws->error, 0u, kDevErrTimeout) == 0u) P.ws->error_tile = (uint32_t)tile;
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

// Spins until the K-word status value at `w` is valid for this launch.
// The wait is bounded: after wait_limit_ns (or when another wait of this
// launch already failed) it records SATGB_ERR_TIMEOUT in the workspace
// header, returns a zero "inclusive" value and lets the kernel run to its end,
// so the context stays usable and the host reports the error.
template <class A>
__device__ __noinline__ uint32_t wait_read(const unsigned long long* w, uint32_t tag_agg,
                                           uint32_t tag_inc, A& val, const SatParams& P,
                                           long long tile) {
  uint32_t st = try_read<A>(w, tag_agg, tag_inc, val);
  if (st) return st;
  const unsigned long long t0 = global_timer_ns();
  unsigned ns = 20;
  for (uint32_t it = 0;; ++it) {
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
    st = try_read<A>(w, tag_agg, tag_inc, val);
    if (st) return st;
    if ((it & 15u) == 15u) {
      bool give_up = ld_relaxed_u32(&P.ws->error) != 0u ||
                     (long long)(global_timer_ns() - t0) > P.wait_limit_ns || it > (1u << 26);
      if (give_up) {
        record_error(P, tile);
        val = Ar<A>::zero();
        return kStateInc;
      }
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

// Windowed look-back.  At the start of a tile the look-back thread of a vector
// element (or of the corner) loads the status words of its W nearest
// predecessors -- one round trip that overlaps the tile's local phase.  After
// the local phase, resolve() walks those values (aggregates are summed until an
// inclusive value is found) and only goes back to memory, with waiting reads,
// for predecessors that were not ready or lie beyond the window.
template <class A>
struct EarlyWin {
  static constexpr int W = Ar<A>::K == 1 ? 3 : 2;
  unsigned long long w[W][Ar<A>::K];
};

template <class A>
__device__ __forceinline__ void early_read(EarlyWin<A>& e, const unsigned long long* base, long long stride,
                                           int steps) {
  constexpr int K = Ar<A>::K;
#pragma unroll
  for (int i = 0; i < EarlyWin<A>::W; ++i) {
#pragma unroll
    for (int k = 0; k < K; ++k) e.w[i][k] = (i < steps) ? ld_relaxed_u64(base + (i + 1) * stride + k) : 0ull;
  }
}

template <class A>
__device__ __forceinline__ A resolve(const EarlyWin<A>& e, const unsigned long long* base, long long stride,
                                     int steps, uint32_t tagA, uint32_t tagI, const SatParams& P, long long tile) {
  constexpr int K = Ar<A>::K;
  A acc = Ar<A>::zero();
  int i = 0;
#pragma unroll
  for (int q = 0; q < EarlyWin<A>::W; ++q) {
    if (i != q || q >= steps) break;
    const uint32_t tag = (uint32_t)(e.w[q][0] >> 32);
    bool ok = (tag == tagA || tag == tagI);
    uint32_t pl[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      ok = ok && ((uint32_t)(e.w[q][k] >> 32) == tag);
      pl[k] = (uint32_t)e.w[q][k];
    }
    if (!ok) break;
    acc = Ar<A>::add(Ar<A>::from_words(pl), acc);
    if (tag == tagI) return acc;
    ++i;
  }
  for (; i < steps; ++i) {
    A val;
    const uint32_t sr = wait_read<A>(base + (i + 1) * stride, tagA, tagI, val, P, tile);
    acc = Ar<A>::add(val, acc);
    if (sr == kStateInc) break;
  }
  return acc;
}

template <class TIn, class TOut, class A, int RPW, int NW>
struct TileShape {
  static constexpr int CPT = 16 / (int)sizeof(TOut);
  static constexpr int TW = 32 * CPT;
  static constexpr int TH = NW * RPW;
  static constexpr int STAGE_BYTES = TH * TW * (int)sizeof(TIn);
  static constexpr int S = Stages<STAGE_BYTES>::value;
  static constexpr int DYN_SMEM = S * STAGE_BYTES;
  static constexpr int THREADS = NW * 32;
};

// Takes ticket `tk`, maps it to a tile and starts its input on its way into
// stage `st` (TMA, or a bare arrive for images read from global memory).
// Returns false once the tickets are exhausted (the stage then carries -1).
template <class TIn, bool REV, int TW, int TH, int STAGE_BYTES>
__device__ __forceinline__ bool produce(const SatParams& P, unsigned long long tk, int st, TIn* stage_ptr,
                                        long long* s_tile, int* s_img, int* s_tx, int* s_ty,
                                        unsigned long long* s_full) {
  const uint32_t bar = smem_u32(&s_full[st]);
  if ((long long)tk >= P.n_tiles) {
    s_tile[st] = -1;
    mbar_arrive(bar);
    return false;
  }
  const long long q = REV ? (P.n_tiles - 1 - (long long)tk) : (long long)tk;
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
  int tx, ty;
  diag_tile(q - D->tile_base, ntx, nty, tx, ty);
  s_tile[st] = D->tile_base + (long long)ty * ntx + tx;
  s_img[st] = img;
  s_tx[st] = tx;
  s_ty[st] = ty;
  if (D->flags & kInTma) {
    mbar_arrive_expect_tx(bar, (uint32_t)STAGE_BYTES);
    tma_load_2d(smem_u32(stage_ptr), &D->tmap_in, tx * TW, ty * TH, bar);
  } else {
    mbar_arrive(bar);
  }
  return true;
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB>
__global__ void __launch_bounds__(NW * 32, MINB) sat_tile_kernel(const __grid_constant__ SatParams P) {
  using SH = TileShape<TIn, TOut, A, RPW, NW>;
  constexpr int CPT = SH::CPT;
  constexpr int TW = SH::TW;
  constexpr int TH = SH::TH;
  constexpr int S = SH::S;
  constexpr int NC = NW * 32;
  constexpr int STAGE_ELEMS = TH * TW;
  constexpr int PT = NC - 1; // producer thread: idle in the look-back phase when TW + TH < NC
  // corner look-back thread: a spare thread when there is one, else thread 0 after its column
  constexpr int CT = (TW + TH < NC - 1) ? TW + TH : 0;
  static_assert(TW + TH <= NC, "one thread per row and per column of the tile");
  static_assert(TH % 32 == 0 && TW % 32 == 0, "groups are whole warps");
  constexpr int K = Ar<A>::K;
  using AR = Ar<A>;

  extern __shared__ __align__(128) unsigned char dsmem[];
  TIn* stages = reinterpret_cast<TIn*>(dsmem);

  __shared__ A s_bot[2][NW][TW];    // per warp: column sums of its row-scanned rows, then the cross-warp carry
  __shared__ A s_colraw[2][NW][TW]; // per warp: column sums of the raw input
  __shared__ A s_rowagg[2][TH];     // row sums of the tile
  __shared__ A s_rowleft[TH];       // row look-back result
  __shared__ A s_RL[TH];            // scan over the tile's rows of rowleft
  __shared__ A s_colabove[TW];      // column look-back result (by slot)
  __shared__ A s_CA[TW];            // scan over the tile's columns of colabove (by slot)
  __shared__ A s_corner, s_u;
  __shared__ long long s_tile[S];   // spatial tile index per stage (-1: no more tiles)
  __shared__ int s_img[S];
  __shared__ int s_tx[S], s_ty[S];
  __shared__ __align__(8) unsigned long long s_full[S];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t epoch = ld_relaxed_u32(&P.ws->epoch);
  const uint32_t tagA = make_tag(epoch, kStateAgg);
  const uint32_t tagI = make_tag(epoch, kStateInc);

  unsigned long long pending = 0; // producer thread: the next ticket, fetched a tile ahead
  bool producing = true;
  if (tid == PT) {
#pragma unroll
    for (int s = 0; s < S; ++s) mbar_init(smem_u32(&s_full[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
#pragma unroll
    for (int s = 0; s < S; ++s) {
      if (producing)
        producing = produce<TIn, REV, TW, TH, SH::STAGE_BYTES>(P, atomicAdd(&P.ws->ticket, 1ull), s,
                                                               stages + s * STAGE_ELEMS, s_tile, s_img, s_tx,
                                                               s_ty, s_full);
    }
    if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
  }
  __syncthreads();

  {
    for (int k = 0;; ++k) {
      const int st = k % S;
      const int buf = k & 1;
      mbar_wait_bounded(smem_u32(&s_full[st]), (k / S) & 1, P, -1);
      const long long t = s_tile[st];
      if (t < 0) break;
      const int tx = s_tx[st], ty = s_ty[st];
      const ImageDesc* Dp = (P.n_images == 1) ? &P.img0 : &P.images[s_img[st]];
      const int64_t width = Dp->width, height = Dp->height;
      const int64_t out_pitch = Dp->out_pitch;
      const int ntx = Dp->ntx, nty = Dp->nty;
      const uint32_t flags = Dp->flags;

      const long long x0 = (long long)tx * TW;
      const long long y0 = (long long)ty * TH;
      const long long xt = x0 + (long long)lane * CPT;
      const long long rem = width - xt;
      const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);

      // early look-back reads: the W nearest predecessors of this thread's element
      const int col_steps = REV ? (nty - 1 - ty) : ty;
      const int row_steps = REV ? (ntx - 1 - tx) : tx;
      EarlyWin<A> early, early_c;
      const unsigned long long* lb_base = nullptr;
      long long lb_stride = 0;
      int lb_steps = 0;
      if (tid < TW) {
        lb_base = P.col_words + ((unsigned long long)t * TW + tid) * K;
        lb_stride = (REV ? 1 : -1) * (long long)ntx * TW * K;
        lb_steps = col_steps;
      } else if (tid < TW + TH) {
        lb_base = P.row_words + ((unsigned long long)t * TH + (tid - TW)) * K;
        lb_stride = (REV ? 1 : -1) * (long long)TH * K;
        lb_steps = row_steps;
      }
      if (lb_base) early_read<A>(early, lb_base, lb_stride, lb_steps);
      const unsigned long long* cb_base = P.corner_words + (unsigned long long)t * K;
      const long long cb_stride = (REV ? 1 : -1) * (long long)ntx * K;
      if (tid == CT) early_read<A>(early_c, cb_base, cb_stride, col_steps);

      // ---- phase A: load, local row scans, local column scans ---------------
      A v[RPW][CPT];
      A colraw[CPT];
#pragma unroll
      for (int c = 0; c < CPT; ++c) colraw[c] = AR::zero();
      if (flags & kInTma) {
        const TIn* sb = stages + st * STAGE_ELEMS + (warp * RPW) * TW + lane * CPT;
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          TIn x[CPT];
          load_seg_smem<TIn, CPT>(sb + r * TW, x);
#pragma unroll
          for (int c = 0; c < CPT; ++c) {
            v[r][c] = Cvt<A, TIn>::in(x[c]);
            colraw[c] = AR::add(colraw[c], v[r][c]);
          }
        }
      } else {
        const TIn* in = static_cast<const TIn*>(Dp->in);
        const int64_t in_pitch = Dp->in_pitch;
        const bool vin = (flags & kInVec) && nvalid == CPT;
#pragma unroll
        for (int r = 0; r < RPW; ++r) {
          const long long y = y0 + warp * RPW + r;
          TIn x[CPT];
          if (y < height && nvalid > 0) {
            load_seg<TIn, CPT>(in + y * in_pitch + xt, vin, nvalid, x);
          } else {
#pragma unroll
            for (int c = 0; c < CPT; ++c) x[c] = TIn(0);
          }
#pragma unroll
          for (int c = 0; c < CPT; ++c) {
            v[r][c] = Cvt<A, TIn>::in(x[c]);
            colraw[c] = AR::add(colraw[c], v[r][c]);
          }
        }
      }
      // row scans, all RPW rows interleaved step by step (independent chains)
      A incl[RPW];
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
#pragma unroll
        for (int i = 1; i < CPT; ++i) {
          const int c = REV ? CPT - 1 - i : i;
          const int p = REV ? c + 1 : c - 1;
          v[r][c] = AR::add(v[r][p], v[r][c]);
        }
        incl[r] = v[r][REV ? 0 : CPT - 1];
      }
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        A o[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) o[r] = REV ? AR::shfl_down(incl[r], d) : AR::shfl_up(incl[r], d);
        if (REV ? (lane + d < 32) : (lane >= d)) {
#pragma unroll
          for (int r = 0; r < RPW; ++r) incl[r] = AR::add(o[r], incl[r]);
        }
      }
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const A ex = REV ? AR::shfl_down(incl[r], 1) : AR::shfl_up(incl[r], 1);
        if (lane != (REV ? 31 : 0)) {
#pragma unroll
          for (int c = 0; c < CPT; ++c) v[r][c] = AR::add(ex, v[r][c]);
        }
        if (lane == (REV ? 0 : 31)) s_rowagg[buf][warp * RPW + r] = incl[r];
      }
#pragma unroll
      for (int i = 1; i < RPW; ++i) {
        const int r = REV ? RPW - 1 - i : i;
        const int p = REV ? r + 1 : r - 1;
#pragma unroll
        for (int c = 0; c < CPT; ++c) v[r][c] = AR::add(v[p][c], v[r][c]);
      }
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        s_bot[buf][warp][c * 32 + lane] = v[REV ? 0 : RPW - 1][c];
        s_colraw[buf][warp][c * 32 + lane] = colraw[c];
      }
      __syncthreads(); // stage st has been read by every thread: the producer may refill it

      // ---- phases B+C: look-backs (column group | row group), vector scans ------
      const bool pub_row = REV ? (tx > 0) : (tx < ntx - 1);
      const bool pub_col = REV ? (ty > 0) : (ty < nty - 1);
      const bool stall = (t == P.stall_tile);
      if (tid == PT && TW + TH < NC) {
        // producer: tile k+S into the stage just read; fetch the ticket after it
        if (producing) {
          producing = produce<TIn, REV, TW, TH, SH::STAGE_BYTES>(P, pending, st, stages + st * STAGE_ELEMS, s_tile,
                                                                 s_img, s_tx, s_ty, s_full);
          if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
        }
      } else if (CT != 0 && tid == CT) {
        // corner look-back over the tiles above (scalar)
        s_corner = resolve<A>(early_c, cb_base, cb_stride, col_steps, tagA, tagI, P, t);
      } else if (tid < TW) {
        const int j = tid; // column slot
        A ac = AR::zero();
#pragma unroll
        for (int w = 0; w < NW; ++w) ac = AR::add(ac, s_colraw[buf][w][j]);
        unsigned long long* mine = P.col_words + ((unsigned long long)t * TW + j) * K;
        if (pub_col && !stall) publish<A>(mine, ac, tagA);
        A run = AR::zero();
#pragma unroll
        for (int i = 0; i < NW; ++i) {
          const int w = REV ? NW - 1 - i : i;
          const A b = s_bot[buf][w][j];
          s_bot[buf][w][j] = run;
          run = AR::add(run, b);
        }
        const A above = resolve<A>(early, lb_base, lb_stride, lb_steps, tagA, tagI, P, t);
        if (pub_col && !stall) publish<A>(mine, AR::add(above, ac), tagI);
        s_colabove[j] = above;
        if (CT == 0 && j == 0) s_corner = resolve<A>(early_c, cb_base, cb_stride, col_steps, tagA, tagI, P, t);
        named_sync(2, TW);
        if (tid < 32) {
          // inclusive scan of colabove over the tile's columns, in scan order
          A loc[CPT];
#pragma unroll
          for (int i = 0; i < CPT; ++i) {
            const int slot = REV ? (CPT - 1 - i) * 32 + (31 - lane) : i * 32 + lane;
            loc[i] = s_colabove[slot];
            if (i) loc[i] = AR::add(loc[i - 1], loc[i]);
          }
          A incl = loc[CPT - 1];
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            const A o = AR::shfl_up(incl, d);
            if (lane >= d) incl = AR::add(o, incl);
          }
          const A ex = AR::shfl_up(incl, 1);
#pragma unroll
          for (int i = 0; i < CPT; ++i) {
            const int slot = REV ? (CPT - 1 - i) * 32 + (31 - lane) : i * 32 + lane;
            s_CA[slot] = lane ? AR::add(ex, loc[i]) : loc[i];
          }
        }
      } else if (tid < TW + TH) {
        const int yy = tid - TW; // tile row
        const A ar = s_rowagg[buf][yy];
        unsigned long long* mine = P.row_words + ((unsigned long long)t * TH + yy) * K;
        if (pub_row && !stall) publish<A>(mine, ar, tagA);
        const A left = resolve<A>(early, lb_base, lb_stride, lb_steps, tagA, tagI, P, t);
        if (pub_row && !stall) publish<A>(mine, AR::add(left, ar), tagI);
        s_rowleft[yy] = left;
        named_sync(3, TH);
        if (tid < TW + 32) {
          // inclusive scan of rowleft over the tile's rows, in scan order; u = total
          constexpr int PER = TH / 32;
          A loc[PER];
#pragma unroll
          for (int i = 0; i < PER; ++i) {
            const int q = lane * PER + i;
            loc[i] = s_rowleft[REV ? TH - 1 - q : q];
            if (i) loc[i] = AR::add(loc[i - 1], loc[i]);
          }
          A incl = loc[PER - 1];
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            const A o = AR::shfl_up(incl, d);
            if (lane >= d) incl = AR::add(o, incl);
          }
          const A ex = AR::shfl_up(incl, 1);
#pragma unroll
          for (int i = 0; i < PER; ++i) {
            const int q = lane * PER + i;
            s_RL[REV ? TH - 1 - q : q] = lane ? AR::add(ex, loc[i]) : loc[i];
          }
          if (lane == 31) {
            s_u = incl; // u = sum of rowleft over the tile: the corner aggregate
            if (pub_col && !stall) publish<A>(P.corner_words + (unsigned long long)t * K, incl, tagA);
          }
        }
        if (tid == PT && TW + TH == NC && producing) {
          // producer when no thread is idle: after its own row look-back
          producing = produce<TIn, REV, TW, TH, SH::STAGE_BYTES>(P, pending, st, stages + st * STAGE_ELEMS, s_tile,
                                                                 s_img, s_tx, s_ty, s_full);
          if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
        }
      }
      __syncthreads();

      // ---- phase D: add the carries and store ---------------------------------
      const A corner = s_corner;
      if (tid == 0 && pub_col && !stall)
        publish<A>(P.corner_words + (unsigned long long)t * K, AR::add(corner, s_u), tagI);
      A colterm[CPT];
#pragma unroll
      for (int c = 0; c < CPT; ++c)
        colterm[c] = AR::add(AR::add(s_bot[buf][warp][c * 32 + lane], s_CA[c * 32 + lane]), corner);
      TOut* out = static_cast<TOut*>(Dp->out) + (y0 + warp * RPW) * out_pitch + xt;
      const bool vout = (flags & kOutVec) && nvalid == CPT;
#pragma unroll
      for (int r = 0; r < RPW; ++r) {
        const long long y = y0 + warp * RPW + r;
        if (y < height && nvalid > 0) {
          const A rt = s_RL[warp * RPW + r];
          TOut o[CPT];
#pragma unroll
          for (int c = 0; c < CPT; ++c) o[c] = OutCvt<TOut, A>::out(AR::add(AR::add(v[r][c], rt), colterm[c]));
          store_seg<TOut, CPT>(out, vout, nvalid, o);
        }
        out += out_pitch;
      }
    }
  }

  // ---- end of launch: the last CTA resets the ticket and advances the epoch --
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const uint32_t prev = atomicAdd(&P.ws->done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      P.ws->ticket = 0ull;
      P.ws->done = 0u;
      P.ws->epoch = epoch + 1u;
      __threadfence();
    }
  }
}

}  // namespace satgb
