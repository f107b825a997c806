// sat_kernel.cuh -- single-pass tiled summed-area table with decoupled
// look-back in both tile directions.
//
// Replaces the reference's two-launch algorithms (pengdada/SAT
// integralImage/ScanRow-BRLT.cu:24-180 blockScan x2, BRLT-Scan.cu:15-127
// serielScan x2, ScanRowColumn.cu:16-268 ScanX + ScanY), which each move
// in + 3*out bytes, with one launch that reads each input element once and
// writes each output element once.
//
// Decomposition.  The image is cut into TH x TW tiles (row-major order inside
// each image, images one after the other).  For a tile with origin (x0, y0):
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
// corner + u.  Tiles are handed out by an atomic ticket in that same order,
// so every tile a tile waits on is held by a running CTA that never waits on
// a later tile: the persistent grid cannot deadlock, whatever its size.
//
// The reverse (suffix) SAT uses the mirror image of every step: tickets run
// from the last tile, look-backs go right and down, scans run right-to-left
// and bottom-to-top.
//
// Thread layout (NW warps): warp w owns tile rows [w*RPW, (w+1)*RPW), lane l
// owns CPT = 16/sizeof(TOut) adjacent columns [l*CPT, (l+1)*CPT), so each
// output row segment is one 16-byte store and a warp writes 512 contiguous
// bytes per row.  Row scans: in-thread, then a Kogge-Stone warp scan of the
// per-thread totals.  Column scans: in-thread over the warp's RPW rows, then a
// cross-warp carry through shared memory.  Shared vectors that are indexed by
// column use slot c*32+lane for column l*CPT+c, which makes every shared
// access of the hot loop bank-conflict free.
#pragma once
#include "sat_types.cuh"

namespace satgb {

struct ImageDesc {
  const void* in;
  void* out;
  int64_t in_pitch;  // elements
  int64_t out_pitch; // elements
  int64_t width, height;
  int64_t tile_base; // global index of the image's first tile
  int32_t ntx, nty;  // tiles across / down
  uint32_t flags;    // kInVec | kOutVec
  uint32_t pad;
};
constexpr uint32_t kInVec = 1u;  // every thread's CPT-element input row segment is vector-aligned
constexpr uint32_t kOutVec = 2u; // every 16-byte output row segment is aligned

struct SatParams {
  const ImageDesc* images; // device table when n_images > 1
  ImageDesc img0;          // the image when n_images == 1
  int64_t n_images;
  int64_t n_tiles;
  unsigned long long* row_words;
  unsigned long long* col_words;
  unsigned long long* corner_words;
  WsHeader* ws;
  int64_t wait_limit_ns;
  int64_t stall_tile; // test knob: this tile never publishes (-1: none)
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
    if (ns < 512) ns <<= 1;
    st = try_read<A>(w, tag_agg, tag_inc, val);
    if (st) return st;
    if ((it & 15u) == 15u) {
      bool give_up = ld_relaxed_u32(&P.ws->error) != 0u ||
                     (long long)(global_timer_ns() - t0) > P.wait_limit_ns || it > (1u << 26);
      if (give_up) {
        if (atomicCAS(&P.ws->error, 0u, kDevErrTimeout) == 0u) P.ws->error_tile = (uint32_t)tile;
        val = Ar<A>::zero();
        return kStateInc;
      }
    }
  }
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NW>
__global__ void __launch_bounds__(NW * 32) sat_tile_kernel(const __grid_constant__ SatParams P) {
  constexpr int CPT = 16 / (int)sizeof(TOut);
  constexpr int TW = 32 * CPT;
  constexpr int TH = NW * RPW;
  constexpr int NT = NW * 32;
  static_assert(TW + TH <= NT, "one thread per row and per column of the tile");
  static_assert(TH % 32 == 0, "row vector is scanned by one warp");
  constexpr int K = Ar<A>::K;
  using AR = Ar<A>;

  __shared__ A s_bot[NW][TW];    // per warp: column sums of its row-scanned rows, then the cross-warp carry
  __shared__ A s_colraw[NW][TW]; // per warp: column sums of the raw input
  __shared__ A s_rowagg[TH];     // row sums of the tile
  __shared__ A s_rowleft[TH];    // row look-back result
  __shared__ A s_RL[TH];         // scan over the tile's rows of rowleft
  __shared__ A s_colabove[TW];   // column look-back result (by slot)
  __shared__ A s_CA[TW];         // scan over the tile's columns of colabove (by slot)
  __shared__ A s_corner;
  __shared__ long long s_tile;
  __shared__ int s_img;

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t epoch = ld_relaxed_u32(&P.ws->epoch);
  const uint32_t tagA = make_tag(epoch, kStateAgg);
  const uint32_t tagI = make_tag(epoch, kStateInc);

  for (;;) {
    if (tid == 0) {
      const unsigned long long tk = atomicAdd(&P.ws->ticket, 1ull);
      long long t = -1;
      int img = 0;
      if ((long long)tk < P.n_tiles) {
        t = REV ? (P.n_tiles - 1 - (long long)tk) : (long long)tk;
        if (P.n_images > 1) {
          int lo = 0, hi = (int)P.n_images - 1; // last image with tile_base <= t
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (P.images[mid].tile_base <= t) lo = mid;
            else hi = mid - 1;
          }
          img = lo;
        }
      }
      s_tile = t;
      s_img = img;
    }
    __syncthreads();
    const long long t = s_tile;
    if (t < 0) break;
    const ImageDesc D = (P.n_images == 1) ? P.img0 : P.images[s_img];

    const long long lt = t - D.tile_base;
    const int ty = (int)(lt / D.ntx);
    const int tx = (int)(lt - (long long)ty * D.ntx);
    const long long x0 = (long long)tx * TW;
    const long long y0 = (long long)ty * TH;
    const long long xt = x0 + (long long)lane * CPT;
    const long long rem = D.width - xt;
    const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);
    const bool vin = (D.flags & kInVec) && nvalid == CPT;
    const bool vout = (D.flags & kOutVec) && nvalid == CPT;
    const TIn* __restrict__ in = static_cast<const TIn*>(D.in);
    TOut* __restrict__ out = static_cast<TOut*>(D.out);

    // ---- phase A: load, local row scans, local column scans ---------------
    A v[RPW][CPT];
    A colraw[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c) colraw[c] = AR::zero();
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const long long y = y0 + warp * RPW + r;
      TIn x[CPT];
      if (y < D.height && nvalid > 0) {
        load_seg<TIn, CPT>(in + y * D.in_pitch + xt, vin, nvalid, x);
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
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
#pragma unroll
      for (int i = 1; i < CPT; ++i) {
        const int c = REV ? CPT - 1 - i : i;
        const int p = REV ? c + 1 : c - 1;
        v[r][c] = AR::add(v[r][p], v[r][c]);
      }
      A incl = v[r][REV ? 0 : CPT - 1];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const A o = REV ? AR::shfl_down(incl, d) : AR::shfl_up(incl, d);
        if (REV ? (lane + d < 32) : (lane >= d)) incl = AR::add(o, incl);
      }
      const A ex = REV ? AR::shfl_down(incl, 1) : AR::shfl_up(incl, 1);
      if (lane != (REV ? 31 : 0)) {
#pragma unroll
        for (int c = 0; c < CPT; ++c) v[r][c] = AR::add(ex, v[r][c]);
      }
      if (lane == (REV ? 0 : 31)) s_rowagg[warp * RPW + r] = incl;
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
      s_bot[warp][c * 32 + lane] = v[REV ? 0 : RPW - 1][c];
      s_colraw[warp][c * 32 + lane] = colraw[c];
    }
    __syncthreads();

    // ---- phase B: publish aggregates, vector look-backs, publish inclusive --
    const bool pub_row = REV ? (tx > 0) : (tx < D.ntx - 1);
    const bool pub_col = REV ? (ty > 0) : (ty < D.nty - 1);
    const bool stall = (t == P.stall_tile);
    if (tid < TW) {
      const int j = tid; // column slot
      A ac = AR::zero();
#pragma unroll
      for (int w = 0; w < NW; ++w) ac = AR::add(ac, s_colraw[w][j]);
      A run = AR::zero();
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        const int w = REV ? NW - 1 - i : i;
        const A b = s_bot[w][j];
        s_bot[w][j] = run;
        run = AR::add(run, b);
      }
      unsigned long long* mine = P.col_words + ((unsigned long long)t * TW + j) * K;
      if (pub_col && !stall) publish<A>(mine, ac, tagA);
      A above = AR::zero();
      const int steps = REV ? (D.nty - 1 - ty) : ty;
      long long nb = t;
      for (int s = 0; s < steps; ++s) {
        nb += REV ? D.ntx : -D.ntx;
        A val;
        const uint32_t st = wait_read<A>(P.col_words + ((unsigned long long)nb * TW + j) * K, tagA, tagI, val, P, t);
        above = AR::add(val, above);
        if (st == kStateInc) break;
      }
      if (pub_col && !stall) publish<A>(mine, AR::add(above, ac), tagI);
      s_colabove[j] = above;
    } else if (tid < TW + TH) {
      const int yy = tid - TW; // tile row
      const A ar = s_rowagg[yy];
      unsigned long long* mine = P.row_words + ((unsigned long long)t * TH + yy) * K;
      if (pub_row && !stall) publish<A>(mine, ar, tagA);
      A left = AR::zero();
      const int steps = REV ? (D.ntx - 1 - tx) : tx;
      long long nb = t;
      for (int s = 0; s < steps; ++s) {
        nb += REV ? 1 : -1;
        A val;
        const uint32_t st = wait_read<A>(P.row_words + ((unsigned long long)nb * TH + yy) * K, tagA, tagI, val, P, t);
        left = AR::add(val, left);
        if (st == kStateInc) break;
      }
      if (pub_row && !stall) publish<A>(mine, AR::add(left, ar), tagI);
      s_rowleft[yy] = left;
    }
    __syncthreads();

    // ---- phase C: corner look-back; scans of the look-back vectors ----------
    if (warp == 0) {
      A part = AR::zero();
#pragma unroll
      for (int k = lane; k < TH; k += 32) part = AR::add(part, s_rowleft[k]);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) part = AR::add(part, AR::shfl_down(part, d));
      if (lane == 0) {
        const A u = part;
        unsigned long long* mine = P.corner_words + (unsigned long long)t * K;
        if (pub_col && !stall) publish<A>(mine, u, tagA);
        A corner = AR::zero();
        const int steps = REV ? (D.nty - 1 - ty) : ty;
        long long nb = t;
        for (int s = 0; s < steps; ++s) {
          nb += REV ? D.ntx : -D.ntx;
          A val;
          const uint32_t st = wait_read<A>(P.corner_words + (unsigned long long)nb * K, tagA, tagI, val, P, t);
          corner = AR::add(val, corner);
          if (st == kStateInc) break;
        }
        if (pub_col && !stall) publish<A>(mine, AR::add(corner, u), tagI);
        s_corner = corner;
      }
    } else if (warp == 1) {
      // inclusive scan of rowleft over the tile's rows, in scan order
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
    } else if (warp == 2) {
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
    __syncthreads();

    // ---- phase D: add the carries and store ---------------------------------
    const A corner = s_corner;
    A colterm[CPT];
#pragma unroll
    for (int c = 0; c < CPT; ++c)
      colterm[c] = AR::add(AR::add(s_bot[warp][c * 32 + lane], s_CA[c * 32 + lane]), corner);
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const long long y = y0 + warp * RPW + r;
      if (y < D.height && nvalid > 0) {
        const A rt = s_RL[warp * RPW + r];
        TOut o[CPT];
#pragma unroll
        for (int c = 0; c < CPT; ++c) o[c] = OutCvt<TOut, A>::out(AR::add(AR::add(v[r][c], rt), colterm[c]));
        store_seg<TOut, CPT>(out + y * D.out_pitch + xt, vout, nvalid, o);
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
