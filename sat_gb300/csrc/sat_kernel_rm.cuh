// sat_kernel_rm.cuh -- the row-major warp-specialized tile loop (configuration 6).
//
// Same tiles, warp roles and direct stores as the warp-specialized kernel
// (sat_kernel_ws.cuh), with the tiles handed out in row-major order (the order
// whose concurrent tiles lie closest in memory) and carries that need no chain
// along a tile row:
//
//   rowleft(j)  = sum of the row aggregates (row sums) of every tile to the
//                 left in the same tile row.  A tile publishes its row sums as
//                 soon as its local phase is done and never an inclusive value;
//                 the row-group thread of row j reads all its predecessors'
//                 words in a few batched loads.  In row-major order those tiles
//                 were handed out just before this one, so they are all in
//                 flight or done: there is no dependency chain along the row.
//   V(x)        = S(y0 - 1, x), the SAT row just above the tile over its
//                 columns, from a vertical decoupled look-back whose
//                 aggregate is the tile's own contribution to its bottom row,
//                 u + sum_{x0<=i<=x} colsum(i) with u = sum_j rowleft(j), and
//                 whose inclusive value is the tile's bottom SAT row.  The tile
//                 above was handed out a whole tile row earlier, so the first
//                 window nearly always holds its inclusive value.
//
// Then, for the rows y of the tile (rows below y0, columns x of the tile):
//   S(y, x) = V(x) + sum_{y0<=j<=y} (rowleft(j) + sum_{x0<=i<=x} a(j, i)),
// so no corner carry is needed.  The reverse (suffix) SAT mirrors every step
// (tiles from the last, rows of tiles from the right, the look-back downward).
//
// Roles (one CTA per SM):
//   NWC compute warps   local phase of tile k+1, output phase of tile k
//   column group        TW threads: exclusive prefix of the column partials
//                       over the compute warps (by slot), then one column per
//                       thread in column order: the tile's column-sum prefix,
//                       its aggregate (once u is in) and the vertical look-back
//   row group           TH threads, one row each: the row aggregate out, the
//                       sum of the predecessors' aggregates, the scan of
//                       rowleft over the tile's rows and u
//   producer warp       tickets and stage refills
#pragma once
#include "sat_kernel_ws.cuh"

namespace satgb {

template <class TIn, class TOut, class A, int RPW, int NWC>
struct TileShapeRM {
  static constexpr int CPT = 16 / (int)sizeof(TOut);
  static constexpr int TW = 32 * CPT;
  static constexpr int TH = NWC * RPW;
  static constexpr int NCW = TW / 32;
  static constexpr int NRW = TH / 32;
  static constexpr int RP = RPW > 4 ? 4 : RPW;
  static constexpr int IN_BYTES = TH * TW * (int)sizeof(TIn);
  static constexpr int STAGE_BYTES = IN_BYTES; // direct stores: a stage holds the input only
  static constexpr int STATIC_BYTES =
      (NWC * RP * 32 + 2 * NWC * TW + 2 * TH + 2 * TW + 2 * TH + 2 * NWC + 2 * NRW + 2 * NCW + TW + 8) *
          (int)sizeof(A) +
      512;
  static constexpr int S = Stages<STAGE_BYTES, STATIC_BYTES, 1>::value;
  static constexpr int DYN_SMEM = S * STAGE_BYTES;
  static constexpr int THREADS = (NWC + NCW + NRW + 1) * 32;
};

constexpr int kBarU = 7;    // the row group's u is in (row group arrives, column group waits)
constexpr int kBarCols = 8; // the column group's exchanges among its warps

// Sum of the aggregates (status words at first + i * stride, i < count) of
// the tiles before this one in its tile row, in batches of loads so the
// round trips overlap; a word not yet published is read again (bounded wait).
template <class A>
__device__ __forceinline__ A sum_row_aggregates(const unsigned long long* first, long long stride, int count,
                                                uint32_t tagA, uint32_t tagI, const SatParams& P, long long tile) {
  constexpr int K = Ar<A>::K;
  constexpr int B = K == 1 ? 16 : 8;
  A acc = Ar<A>::zero();
  int i = 0;
  unsigned long long t0 = 0;
  unsigned ns = 0;
  for (uint32_t round = 0; i < count; ++round) {
    unsigned long long w[B][K];
#pragma unroll
    for (int q = 0; q < B; ++q)
#pragma unroll
      for (int k = 0; k < K; ++k) w[q][k] = (i + q < count) ? ld_relaxed_u64(first + (long long)(i + q) * stride + k) : 0ull;
    int got = 0;
    bool open = true;
#pragma unroll
    for (int q = 0; q < B; ++q) {
      if (!open || i + q >= count) break;
      A v;
      if (decode_word<A>(w[q], tagA, tagI, v)) {
        acc = Ar<A>::add(acc, v);
        ++got;
      } else {
        open = false;
      }
    }
    i += got;
    if (i < count && got < B) {
      if (t0 == 0) t0 = global_timer_ns();
      if (!got) {
        if (ns) __nanosleep(ns);
        ns = ns ? (ns < 256 ? 2 * ns : ns) : 32;
      }
      if ((round & 7u) == 7u &&
          ((long long)(global_timer_ns() - t0) > P.wait_limit_ns || ld_relaxed_u32(&P.ws->error) != 0u)) {
        record_error(P, tile);
        return acc;
      }
    }
  }
  return acc;
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NWC>
__global__ void __launch_bounds__(TileShapeRM<TIn, TOut, A, RPW, NWC>::THREADS, 1)
    sat_tile_kernel_rm(const __grid_constant__ SatParams P) {
  using SH = TileShapeRM<TIn, TOut, A, RPW, NWC>;
  constexpr int CPT = SH::CPT;
  constexpr int TW = SH::TW;
  constexpr int TH = SH::TH;
  constexpr int S = SH::S;
  constexpr int NCW = SH::NCW, NRW = SH::NRW;
  constexpr int STAGE_ELEMS = SH::STAGE_BYTES / (int)sizeof(TIn);
  constexpr int WCOL = NWC, WROW = NWC + NCW, WPROD = NWC + NCW + NRW;
  constexpr int NAGG = (NWC + NCW + NRW) * 32;
  constexpr int RP = SH::RP;
  constexpr int LPR = 32 / RP;
  constexpr int CH = RP;
  static_assert(TW % 32 == 0 && TH % 32 == 0, "look-back groups are whole warps");
  static_assert(RPW % RP == 0 && 32 % RP == 0, "whole transpose passes");
  static_assert(S >= 3, "stages for the tile in output, the one in the local phase and one loading");
  constexpr int K = Ar<A>::K;
  using AR = Ar<A>;

  extern __shared__ __align__(128) unsigned char dsmem[];
  TIn* stages = reinterpret_cast<TIn*>(dsmem);

  __shared__ A s_tr[NWC][RP][32];   // compute warps: transpose scratch
  __shared__ A s_colp[2][NWC][TW];  // column partials by slot, then their exclusive prefix over the warps
  __shared__ A s_rowagg[2][TH];     // row totals
  __shared__ A s_vab[2][TW];        // V(x): the SAT row above the tile (by slot)
  __shared__ A s_rowleft[2][TH];    // rowleft of each row
  __shared__ A s_rlprev[2][NWC];    // per compute warp: sum of rowleft over the rows before it (scan order)
  __shared__ A s_rwt[2][NRW];       // row group: per-warp sums of rowleft
  __shared__ A s_cwt[2][NCW];       // column group: per-warp sums of the column sums
  __shared__ A s_csum[TW];          // column sums of the tile, by slot
  __shared__ A s_u[2];              // u = sum of rowleft
  __shared__ long long s_tile[S];
  __shared__ int s_img[S];
  __shared__ int s_tx[S], s_ty[S], s_pl[S];
  __shared__ __align__(8) unsigned long long s_full[S];
  __shared__ __align__(8) unsigned long long s_done[S]; // the output phase has read the stage

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t epoch = ld_relaxed_u32(&P.ws->epoch);
  const uint32_t tagA = make_tag(epoch, kStateAgg);
  const uint32_t tagI = make_tag(epoch, kStateInc);

  // ---- prologue: the producer fills every stage ---------------------------------
  bool producing = true;
  unsigned long long pending = 0;
  if (warp == WPROD && lane == 0) {
#pragma unroll
    for (int s = 0; s < S; ++s) {
      mbar_init(smem_u32(&s_full[s]), 1);
      mbar_init(smem_u32(&s_done[s]), NWC);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int s = 0; s < S && producing; ++s) {
      const TilePlan tp = plan_tile<REV, kOrderRows>(P, atomicAdd(&P.ws->ticket, 1ull));
      issue_tile<TIn, TW, TH, SH::IN_BYTES>(P, tp, s, stages + s * STAGE_ELEMS, s_tile, s_img, s_tx, s_ty, s_pl,
                                           s_full);
      if (tp.t < 0) producing = false;
    }
    if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
  }
  __syncthreads();

  if (warp == WPROD && lane == 0) {
    // ---- producer: each stage is refilled once the output phase has read it -----
    TilePlan next;
    bool have_next = false;
    if (producing) {
      next = plan_tile<REV, kOrderRows>(P, pending);
      have_next = true;
      if (next.t >= 0) pending = atomicAdd(&P.ws->ticket, 1ull);
    }
    for (int k = 0; have_next; ++k) {
      const int st = k % S;
      mbar_wait_bounded(smem_u32(&s_done[st]), (k / S) & 1, P, -1);
      issue_tile<TIn, TW, TH, SH::IN_BYTES>(P, next, st, stages + st * STAGE_ELEMS, s_tile, s_img, s_tx, s_ty, s_pl,
                                           s_full);
      have_next = false;
      if (next.t >= 0) {
        next = plan_tile<REV, kOrderRows>(P, pending);
        have_next = true;
        if (next.t >= 0) pending = atomicAdd(&P.ws->ticket, 1ull);
      }
    }
  }

  if (warp < NWC) {
    // ---- compute warps ----------------------------------------------------------
    A E_nxt[RPW], E_cur[RPW];
    auto local_phase = [&](int kk) -> bool {
      const int st = kk % S;
      mbar_wait_bounded(smem_u32(&s_full[st]), (kk / S) & 1, P, -1);
      if (s_tile[st] < 0) return false;
      const ImageView D = image_view(P, s_img[st]);
      const long long x0 = (long long)s_tx[st] * TW, y0 = (long long)s_ty[st] * TH;
      const long long xt = x0 + (long long)lane * CPT;
      const long long rem = D.width - xt;
      const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);
      TIn* sb = stages + st * STAGE_ELEMS + (warp * RPW) * TW + lane * CPT;
      const bool tma = D.flags & kInTma;
      if (!tma || (nvalid > 0 && xt + nvalid > D.tma_in_w)) {
        const TIn* gin = static_cast<const TIn*>(D.in) + (long long)s_pl[st] * D.in_plane +
                         (y0 + warp * RPW) * D.in_pitch + xt;
        const long long rows = D.height - (y0 + warp * RPW);
        const int c0 = tma ? (int)(D.tma_in_w - xt > 0 ? D.tma_in_w - xt : 0) : 0;
        stage_fill<TIn, CPT, RPW, TW>(sb, gin, D.in_pitch, rows < 0 ? 0 : (rows > RPW ? RPW : (int)rows), nvalid,
                                      c0, (D.flags & kInVec) != 0);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      }
      A colp[CPT], rowp[RPW];
#pragma unroll
      for (int c = 0; c < CPT; ++c) colp[c] = AR::zero();
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
#pragma unroll
      for (int h = 0; h < RPW / RP; ++h) {
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
          if (q == (REV ? 0 : LPR - 1)) s_rowagg[kk & 1][warp * RPW + h * RP + r] = incl;
        }
        __syncwarp();
#pragma unroll
        for (int r = 0; r < RP; ++r) E_nxt[h * RP + r] = s_tr[warp][r][lane ^ r];
        __syncwarp();
      }
#pragma unroll
      for (int c = 0; c < CPT; ++c) s_colp[kk & 1][warp][c * 32 + lane] = colp[c];
      return true;
    };

    bool have = local_phase(0);
    named_arrive(kBarAgg0, NAGG);
    for (int k = 0; have; ++k) {
      const int st = k % S;
#pragma unroll
      for (int r = 0; r < RPW; ++r) E_cur[r] = E_nxt[r];
      const bool have_next = local_phase(k + 1);
      named_arrive(kBarAgg0 + ((k + 1) & 1), NAGG);
      named_sync(kBarCar0 + (k & 1), NAGG); // tile k's carries are in

      // ---- output phase of tile k (results straight to global memory) ---------
      const ImageView D = image_view(P, s_img[st]);
      const uint32_t flags = D.flags;
      const long long x0 = (long long)s_tx[st] * TW, y0 = (long long)s_ty[st] * TH;
      const long long xt = x0 + (long long)lane * CPT;
      const long long rem = D.width - xt;
      const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);
      const int kb = k & 1;
      TIn* sb = stages + st * STAGE_ELEMS + (warp * RPW) * TW + lane * CPT;
      RowSeg<TIn, CPT> xin[RPW];
#pragma unroll
      for (int r = 0; r < RPW; ++r) xin[r].u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&s_done[st])); // the stage goes back to the producer
      A top[CPT];
      {
        // the SAT row just above the warp's rows: V(x) + RL_w + sum_{x0<=i<=x} C_w(i)
        A cp[CPT];
#pragma unroll
        for (int i = 0; i < CPT; ++i) {
          const int c = REV ? CPT - 1 - i : i;
          cp[c] = s_colp[kb][warp][c * 32 + lane];
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
        const A base = AR::add(s_rlprev[kb][warp], ex);
#pragma unroll
        for (int c = 0; c < CPT; ++c) top[c] = AR::add(AR::add(s_vab[kb][c * 32 + lane], base), cp[c]);
      }
      const bool vout = (flags & kOutVec) && nvalid == CPT;
      TOut* out = static_cast<TOut*>(D.out) + (long long)s_pl[st] * D.out_plane + (y0 + warp * RPW) * D.out_pitch + xt;
#pragma unroll
      for (int i = 0; i < RPW; ++i) {
        const int r = REV ? RPW - 1 - i : i;
        A run = AR::add(E_cur[r], s_rowleft[kb][warp * RPW + r]);
        TOut o[CPT];
#pragma unroll
        for (int ii = 0; ii < CPT; ++ii) {
          const int c = REV ? CPT - 1 - ii : ii;
          run = AddIn<A, TIn>::add(run, xin[r].u.e[c]);
          top[c] = AR::add(top[c], run);
          o[c] = OutCvt<TOut, A>::out(top[c]);
        }
        if (y0 + warp * RPW + r < D.height && nvalid > 0) store_seg<TOut, CPT>(out + r * D.out_pitch, vout, nvalid, o);
      }
      have = have_next;
    }
  }

  if (warp >= WCOL && warp < WROW) {
    // ---- column group ------------------------------------------------------------
    const int j = tid - WCOL * 32;                // slot (partials) and column (look-back) index
    const int cw = warp - WCOL;                   // warp within the group
    const int jslot = (j % CPT) * 32 + j / CPT;   // slot of column j
    for (int k = 0;; ++k) {
      const int st = k % S;
      mbar_wait_bounded(smem_u32(&s_full[st]), (k / S) & 1, P, -1);
      const long long t = s_tile[st];
      if (t < 0) {
        named_sync(kBarAgg0 + (k & 1), NAGG);
        break;
      }
      const int kb = k & 1;
      const int ty = s_ty[st];
      const ImageView D = image_view(P, s_img[st]);
      const int ntx = D.ntx, nty = D.nty;
      const bool pub = (REV ? (ty > 0) : (ty < nty - 1)) && t != P.stall_tile;
      const long long vstride = (REV ? 1 : -1) * (long long)ntx * TW * K;
      const int vsteps = REV ? (nty - 1 - ty) : ty;
      unsigned long long* base = P.col_words + ((unsigned long long)t * TW + j) * K; // column j's words
      EarlyWin<A> win[1];
      early_read<A>(win[0], base, vstride, vsteps);
      named_sync(kBarAgg0 + kb, NAGG); // tile k's partials are in
      // (a) by slot: exclusive prefix of the partials over the compute warps, the column sum
      {
        A v[NWC];
#pragma unroll
        for (int w = 0; w < NWC; ++w) v[w] = s_colp[kb][w][j];
        A run = AR::zero();
#pragma unroll
        for (int i = 0; i < NWC; ++i) {
          const int w = REV ? NWC - 1 - i : i;
          s_colp[kb][w][j] = run;
          run = AR::add(run, v[w]);
        }
        s_csum[j] = run;
      }
      named_sync(kBarCols, NCW * 32);
      // (b) by column: inclusive prefix of the column sums over the tile's columns (scan order)
      A cs = s_csum[jslot];
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const A o = REV ? AR::shfl_down(cs, d) : AR::shfl_up(cs, d);
        if (REV ? (lane + d < 32) : (lane >= d)) cs = AR::add(o, cs);
      }
      if (NCW > 1) {
        if (lane == (REV ? 0 : 31)) s_cwt[kb][cw] = cs;
        named_sync(kBarCols, NCW * 32);
        A before = AR::zero();
#pragma unroll
        for (int i = 0; i < NCW; ++i) {
          const int w = REV ? NCW - 1 - i : i;
          if (REV ? (w > cw) : (w < cw)) before = AR::add(before, s_cwt[kb][w]);
        }
        cs = AR::add(before, cs);
      }
      named_sync(kBarU, (NCW + NRW) * 32); // u is in
      const A agg = AR::add(vload(&s_u[kb]), cs);
      if (pub) publish<A>(base, agg, tagA);
      A vab[1];
      resolve_n<A, 1>(win, base, 0, vstride, vsteps, tagA, tagI, P, t, vab);
      if (pub) publish<A>(base, AR::add(vab[0], agg), tagI);
      s_vab[kb][jslot] = vab[0];
      __syncwarp();
      named_arrive(kBarCar0 + kb, NAGG);
    }
  }

  if (warp >= WROW && warp < WPROD) {
    // ---- row group: one row per thread ---------------------------------------------
    const int y = tid - WROW * 32;
    const int rw = warp - WROW;
    for (int k = 0;; ++k) {
      const int st = k % S;
      mbar_wait_bounded(smem_u32(&s_full[st]), (k / S) & 1, P, -1);
      const long long t = s_tile[st];
      if (t < 0) {
        named_sync(kBarAgg0 + (k & 1), NAGG);
        break;
      }
      const int kb = k & 1;
      const int tx = s_tx[st];
      const ImageView D = image_view(P, s_img[st]);
      const int ntx = D.ntx;
      const bool pub = (REV ? (tx > 0) : (tx < ntx - 1)) && t != P.stall_tile;
      unsigned long long* base = P.row_words + ((unsigned long long)t * TH + y) * K;
      named_sync(kBarAgg0 + kb, NAGG);
      const A agg = s_rowagg[kb][y];
      if (pub) publish<A>(base, agg, tagA);
      // rowleft: the aggregates of every tile before this one in its tile row
      const int npred = REV ? (ntx - 1 - tx) : tx;
      const A left = sum_row_aggregates<A>(base + (REV ? 1 : -1) * (long long)TH * K, (REV ? 1 : -1) * (long long)TH * K,
                                           npred, tagA, tagI, P, t);
      s_rowleft[kb][y] = left;
      A incl = left;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const A o = REV ? AR::shfl_down(incl, d) : AR::shfl_up(incl, d);
        if (REV ? (lane + d < 32) : (lane >= d)) incl = AR::add(o, incl);
      }
      if (NRW > 1) {
        if (lane == (REV ? 0 : 31)) s_rwt[kb][rw] = incl;
        named_sync(kBarRows, NRW * 32);
        A before = AR::zero();
#pragma unroll
        for (int i = 0; i < NRW; ++i) {
          const int w = REV ? NRW - 1 - i : i;
          if (REV ? (w > rw) : (w < rw)) before = AR::add(before, s_rwt[kb][w]);
        }
        incl = AR::add(before, incl);
      }
      if (!REV && (y + 1) % RPW == 0 && y + 1 < TH) s_rlprev[kb][(y + 1) / RPW] = incl;
      if (REV && y % RPW == 0 && y > 0) s_rlprev[kb][y / RPW - 1] = incl;
      if (y == (REV ? TH - 1 : 0)) s_rlprev[kb][REV ? NWC - 1 : 0] = AR::zero();
      if (y == (REV ? 0 : TH - 1)) vstore(&s_u[kb], incl);
      __syncwarp();
      named_arrive(kBarU, (NCW + NRW) * 32);
      named_arrive(kBarCar0 + kb, NAGG);
    }
  }

  // ---- end of launch -----------------------------------------------------------
  __syncthreads();
  if (tid == 0) finish_launch(P, epoch);
}

}  // namespace satgb
