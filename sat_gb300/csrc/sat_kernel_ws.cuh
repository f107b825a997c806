// sat_kernel_ws.cuh -- the warp-specialized tile loop.
//
// Same decomposition, tickets, status words and look-backs as sat_tile_kernel
// (sat_kernel.cuh); the work of a tile is split between warps that never wait
// on one another at a CTA-wide barrier:
//
//   NWC compute warps   the local phase of tile k+1 (partials, the lanes' row
//                       prefix E in registers), then the output phase of
//                       tile k from its TMA stage, results back into the stage
//   column warp         column sums over the compute warps: the column
//                       aggregate out at once, the exclusive prefix over the
//                       warps, the column look-back; lane 0 the corner look-back
//   row warp            row aggregates out, the row look-back, the scan of
//                       rowleft over the tile's rows and u = sum rowleft (the
//                       corner aggregate of the tile below)
//   store warp          one TMA tensor store per tile, and the refill of the
//                       stage it has read with the tile S ahead; tickets
//
// Hand-offs: named barriers AGG[2] (compute warps arrive when a tile's
// partials are in shared memory, the look-back warps wait) and CAR[2] (the
// look-back warps arrive when a tile's carries are in shared memory, the
// compute warps wait), two of each by tile parity: a barrier is used again two
// tiles later, when every participant has provably passed its previous phase.
// Per stage, an mbarrier "done" (each compute warp arrives when its rows of the
// tile's results are in the stage, the store warp waits); the compute warps
// may run up to S-1 tiles ahead of the store warp, which an mbarrier's phase
// parity tolerates and a named barrier would not.
// The look-back of tile k therefore runs while the compute warps finish tile
// k-1 and compute tile k+1's partials, and the TMA ring runs S-1 tiles ahead
// of the compute warps because a stage is refilled as soon as its store has
// read it.
//
// Shared vectors written by the look-back warps for tile k live in buffers
// indexed k & 1; the compute warps' partials likewise, so the look-back warps
// may read tile k's while the compute warps write tile k+1's.
#pragma once
#include "sat_kernel.cuh"

namespace satgb {

template <class TIn, class TOut, class A, int RPW, int NWC>
struct TileShapeWS {
  static constexpr int CPT = 16 / (int)sizeof(TOut);
  static constexpr int TW = 32 * CPT;
  static constexpr int TH = NWC * RPW;
  static constexpr int IN_BYTES = TH * TW * (int)sizeof(TIn);
  static constexpr int STAGE_BYTES = TH * TW * (int)(sizeof(TIn) > sizeof(TOut) ? sizeof(TIn) : sizeof(TOut));
  static constexpr int STATIC_BYTES =
      (NWC * RPW * 32 + 2 * NWC * TW + 2 * TH + 2 * TW + 2 * TH + 2 * NWC + 8) * (int)sizeof(A) + 512;
  static constexpr int S = Stages<STAGE_BYTES, STATIC_BYTES, 1>::value;
  static constexpr int DYN_SMEM = S * STAGE_BYTES;
  static constexpr int THREADS = (NWC + 3) * 32;
};

// named barrier ids (0 is __syncthreads)
constexpr int kBarAgg0 = 1; // + (k & 1)
constexpr int kBarCar0 = 3; // + (k & 1)
constexpr int kBarWiden = 5;

__device__ __forceinline__ void named_arrive(int id, int nthreads) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NWC>
__global__ void __launch_bounds__((NWC + 3) * 32, 1) sat_tile_kernel_ws(const __grid_constant__ SatParams P) {
  using SH = TileShapeWS<TIn, TOut, A, RPW, NWC>;
  constexpr int CPT = SH::CPT;
  constexpr int TW = SH::TW;
  constexpr int TH = SH::TH;
  constexpr int S = SH::S;
  constexpr int STAGE_ELEMS = SH::STAGE_BYTES / (int)sizeof(TIn);
  constexpr int WCOL = NWC, WROW = NWC + 1, WSTORE = NWC + 2; // warp roles
  constexpr int NAGG = (NWC + 2) * 32;   // compute + look-back warps
  constexpr int COLS_PER_LANE = TW / 32; // column warp: slots lane + 32 i
  constexpr int ROWS_PER_LANE = TH / 32; // row warp: rows lane * ROWS_PER_LANE + i
  static_assert(TW % 32 == 0 && TH % 32 == 0, "look-back warps hold whole lanes' worth");
  static_assert(32 % RPW == 0, "rows per warp divide the warp");
  static_assert(S >= 3, "stages for the tile in output, the one in the local phase and one loading");
  constexpr int LPR = 32 / RPW; // transpose-scan: lanes per row ...
  constexpr int CH = RPW;       // ... and values per lane
  constexpr int K = Ar<A>::K;
  constexpr bool WIDEN = sizeof(TIn) < sizeof(TOut);
  using AR = Ar<A>;

  extern __shared__ __align__(128) unsigned char dsmem[];
  TIn* stages = reinterpret_cast<TIn*>(dsmem);

  __shared__ A s_tr[NWC][RPW][32];   // compute warps: transpose scratch (lane ^ row: conflict free)
  __shared__ A s_colp[2][NWC][TW];   // per tile parity and warp: column partials, then their exclusive prefix over the warps
  __shared__ A s_rowagg[2][TH];      // row totals
  __shared__ A s_colabove[2][TW];    // column look-back results (by slot)
  __shared__ A s_rowleft[2][TH];     // row look-back results
  __shared__ A s_rlprev[2][NWC];     // per compute warp: sum of rowleft over the rows before it (scan order)
  __shared__ A s_corner[2], s_u[2];
  __shared__ int s_cnt_corner[2];    // arrivals of {corner, u} per tile parity
  __shared__ long long s_tile[S];    // spatial tile index per stage (-1: no more tiles)
  __shared__ int s_img[S];
  __shared__ int s_tx[S], s_ty[S], s_pl[S];
  __shared__ __align__(8) unsigned long long s_full[S];
  __shared__ __align__(8) unsigned long long s_done[S]; // the stage's results are complete

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t epoch = ld_relaxed_u32(&P.ws->epoch);
  const uint32_t tagA = make_tag(epoch, kStateAgg);
  const uint32_t tagI = make_tag(epoch, kStateInc);

  // ---- prologue: the store warp fills every stage -----------------------------
  if (tid < 2) s_cnt_corner[tid] = 0;
  int issued = 0;                 // store warp, lane 0: tiles handed to the CTA
  bool producing = true;          // ... tickets not yet exhausted
  unsigned long long pending = 0; // ... the next ticket, fetched a tile ahead
  if (warp == WSTORE && lane == 0) {
#pragma unroll
    for (int s = 0; s < S; ++s) {
      mbar_init(smem_u32(&s_full[s]), 1);
      mbar_init(smem_u32(&s_done[s]), NWC);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int s = 0; s < S && producing; ++s) {
      const TilePlan tp = plan_tile<REV>(P, atomicAdd(&P.ws->ticket, 1ull));
      issue_tile<TIn, TW, TH, SH::IN_BYTES>(P, tp, s, stages + s * STAGE_ELEMS, s_tile, s_img, s_tx, s_ty, s_pl,
                                           s_full);
      if (tp.t < 0) producing = false;
      else ++issued;
    }
    if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
  }
  __syncthreads();

  if (warp == WSTORE && lane == 0) {
    // ---- store thread: one store per tile, then the refill of its stage -------
    TilePlan next;
    bool have_next = false;
    if (producing) {
      next = plan_tile<REV>(P, pending);
      have_next = true;
      if (next.t >= 0) pending = atomicAdd(&P.ws->ticket, 1ull);
    }
    // Two stores in flight: after tile k's store is issued, the refill goes into
    // the stage of tile k-1, whose store has had a tile's time to read it.
    for (int k = 0; k <= issued; ++k) {
      if (k < issued) {
        const int st = k % S;
        mbar_wait_bounded(smem_u32(&s_done[st]), (k / S) & 1, P, -1); // tile k's results are in its stage
        const ImageDesc* D = (P.n_images == 1) ? &P.img0 : &P.images[s_img[st]];
        if (D->flags & kOutTma)
          tma_store_3d(&D->tmap_out, s_tx[st] * TW, s_ty[st] * TH, s_pl[st], smem_u32(stages + st * STAGE_ELEMS));
        asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); // all but the newest store have read
      } else {
        bulk_wait_read_all();
      }
      if (k >= 1 && have_next) {
        // tile (k-1)+S into the stage tile k-1 has left
        const int ps = (k - 1) % S;
        issue_tile<TIn, TW, TH, SH::IN_BYTES>(P, next, ps, stages + ps * STAGE_ELEMS, s_tile, s_img, s_tx, s_ty,
                                             s_pl, s_full);
        have_next = false;
        if (next.t >= 0) {
          ++issued;
          next = plan_tile<REV>(P, pending);
          have_next = true;
          if (next.t >= 0) pending = atomicAdd(&P.ws->ticket, 1ull);
        }
      }
    }
    bulk_wait_all();
  }

  if (warp < NWC) {
    // ---- compute warps ----------------------------------------------------------
    A E_nxt[RPW], E_cur[RPW];
    // local phase of tile kk: false when the tickets ran out (the look-back
    // warps still get their AGG arrival, to see the end)
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
        // no TMA for this image, or columns past the map (they arrived as zeros)
        const TIn* gin = static_cast<const TIn*>(D.in) + (long long)s_pl[st] * D.in_plane +
                         (y0 + warp * RPW) * D.in_pitch + xt;
        const long long rows = D.height - (y0 + warp * RPW);
        const int c0 = tma ? (int)(D.tma_in_w - xt > 0 ? D.tma_in_w - xt : 0) : 0;
        stage_fill<TIn, CPT, RPW, TW>(sb, gin, D.in_pitch, rows < 0 ? 0 : (rows > RPW ? RPW : (int)rows), nvalid,
                                      c0, (D.flags & kInVec) != 0);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); // before TMA reads or refills the stage
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
          const A a = Cvt<A, TIn>::in(x.u.e[c]);
          colp[c] = AR::add(colp[c], a);
          rs = AR::add(rs, a);
        }
        rowp[r] = rs;
      }
      // row partials -> exclusive prefix over the lanes (E) and the row totals
#pragma unroll
      for (int r = 0; r < RPW; ++r) s_tr[warp][r][lane ^ r] = rowp[r];
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
        if (q == (REV ? 0 : LPR - 1)) s_rowagg[kk & 1][warp * RPW + r] = incl;
      }
      __syncwarp();
#pragma unroll
      for (int r = 0; r < RPW; ++r) E_nxt[r] = s_tr[warp][r][lane ^ r];
      __syncwarp();
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

      // ---- output phase of tile k -----------------------------------------------
      const ImageView D = image_view(P, s_img[st]);
      const uint32_t flags = D.flags;
      const long long x0 = (long long)s_tx[st] * TW, y0 = (long long)s_ty[st] * TH;
      const long long xt = x0 + (long long)lane * CPT;
      const long long rem = D.width - xt;
      const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);
      const int kb = k & 1;
      A top[CPT];
      {
        A cp[CPT];
#pragma unroll
        for (int i = 0; i < CPT; ++i) {
          const int c = REV ? CPT - 1 - i : i;
          cp[c] = AR::add(s_colabove[kb][c * 32 + lane], s_colp[kb][warp][c * 32 + lane]);
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
        const A base = AR::add(AR::add(s_corner[kb], s_rlprev[kb][warp]), ex);
#pragma unroll
        for (int c = 0; c < CPT; ++c) top[c] = AR::add(base, cp[c]);
      }
      TIn* sb = stages + st * STAGE_ELEMS + (warp * RPW) * TW + lane * CPT;
      TOut* so = reinterpret_cast<TOut*>(stages + st * STAGE_ELEMS) + (warp * RPW) * TW + lane * CPT;
      const bool tma_out = flags & kOutTma;
      RowSeg<TIn, CPT> raw[WIDEN ? RPW : 1];
      if (WIDEN) {
        // wider outputs overwrite other threads' inputs: every compute warp reads first
#pragma unroll
        for (int r = 0; r < (WIDEN ? RPW : 1); ++r)
          raw[r].u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
        named_sync(kBarWiden, NWC * 32);
      }
#pragma unroll
      for (int i = 0; i < RPW; ++i) {
        const int r = REV ? RPW - 1 - i : i;
        RowSeg<TIn, CPT> x;
        if (WIDEN) x = raw[WIDEN ? r : 0];
        else x.u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
        A run = AR::add(E_cur[r], s_rowleft[kb][warp * RPW + r]);
        union {
          uint4 v;
          TOut e[CPT];
        } o;
#pragma unroll
        for (int ii = 0; ii < CPT; ++ii) {
          const int c = REV ? CPT - 1 - ii : ii;
          run = AR::add(run, Cvt<A, TIn>::in(x.u.e[c]));
          top[c] = AR::add(top[c], run);
          o.e[c] = OutCvt<TOut, A>::out(top[c]);
        }
        *reinterpret_cast<uint4*>(so + r * TW) = o.v;
      }
      const bool tail_out = tma_out && nvalid > 0 && xt + nvalid > D.tma_out_w;
      if (!tma_out || tail_out) {
        // no TMA for this image, or columns past the map: plain stores
        TOut* out = static_cast<TOut*>(D.out) + (long long)s_pl[st] * D.out_plane + (y0 + warp * RPW) * D.out_pitch + xt;
        const long long rows = D.height - (y0 + warp * RPW);
        const int c0 = tma_out ? (int)(D.tma_out_w - xt > 0 ? D.tma_out_w - xt : 0) : 0;
        stage_drain<TOut, CPT, RPW, TW, REV>(so, out, D.out_pitch, rows < 0 ? 0 : (rows > RPW ? RPW : (int)rows),
                                             nvalid, c0, (flags & kOutVec) && nvalid == CPT);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); // results to the TMA store
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&s_done[st]));
      have = have_next;
    }
  }

  if (warp == WCOL) {
    // ---- column warp: column aggregates, exclusive prefix over the warps, the
    //      column look-back; lane 0 also the corner ------------------------------
    for (int k = 0;; ++k) {
      named_sync(kBarAgg0 + (k & 1), NAGG); // tile k's partials are in
      const int st = k % S;
      const long long t = s_tile[st];
      if (t < 0) break;
      const int kb = k & 1;
      const int ty = s_ty[st];
      const ImageView D = image_view(P, s_img[st]);
      const int ntx = D.ntx, nty = D.nty;
      const bool pub_col = (REV ? (ty > 0) : (ty < nty - 1)) && t != P.stall_tile;
      const long long cstride = (REV ? 1 : -1) * (long long)ntx * TW * K;
      const int csteps = REV ? (nty - 1 - ty) : ty;
      EarlyWin<A> win[COLS_PER_LANE];
#pragma unroll
      for (int i = 0; i < COLS_PER_LANE; ++i)
        early_read<A>(win[i], P.col_words + ((unsigned long long)t * TW + lane + 32 * i) * K, cstride, csteps);
      EarlyWin<A> cwin;
      unsigned long long* cbase = P.corner_words + (unsigned long long)t * K;
      const long long kstride = (REV ? 1 : -1) * (long long)ntx * K;
      if (lane == 0) early_read<A>(cwin, cbase, kstride, csteps);
      A agg[COLS_PER_LANE];
#pragma unroll
      for (int i = 0; i < COLS_PER_LANE; ++i) {
        const int j = lane + 32 * i;
        A ac = AR::zero();
#pragma unroll
        for (int w = 0; w < NWC; ++w) ac = AR::add(ac, s_colp[kb][w][j]);
        if (pub_col) publish<A>(P.col_words + ((unsigned long long)t * TW + j) * K, ac, tagA);
        A run = AR::zero();
#pragma unroll
        for (int ii = 0; ii < NWC; ++ii) {
          const int w = REV ? NWC - 1 - ii : ii;
          const A b = s_colp[kb][w][j];
          s_colp[kb][w][j] = run;
          run = AR::add(run, b);
        }
        agg[i] = ac;
      }
      // all of this lane's columns resolve together (their round trips overlap)
      A above[COLS_PER_LANE];
      resolve_n<A, COLS_PER_LANE>(win, P.col_words + ((unsigned long long)t * TW + lane) * K, 32LL * K, cstride,
                                  csteps, tagA, tagI, P, t, above);
#pragma unroll
      for (int i = 0; i < COLS_PER_LANE; ++i) {
        const int j = lane + 32 * i;
        unsigned long long* base = P.col_words + ((unsigned long long)t * TW + j) * K;
        if (pub_col) publish<A>(base, AR::add(above[i], agg[i]), tagI);
        s_colabove[kb][j] = above[i];
      }
      if (lane == 0) {
        const A c = resolve<A>(cwin, cbase, kstride, csteps, tagA, tagI, P, t);
        vstore(&s_corner[kb], c);
        __threadfence_block();
        if (atomicAdd(&s_cnt_corner[kb], 1) == 1) {
          // u is in: this thread publishes corner + u
          __threadfence_block();
          s_cnt_corner[kb] = 0;
          if (pub_col) publish<A>(cbase, AR::add(c, vload(&s_u[kb])), tagI);
        }
      }
      __syncwarp();
      named_arrive(kBarCar0 + kb, NAGG);
    }
  }

  if (warp == WROW) {
    // ---- row warp: row aggregates, the row look-back, rowleft's scan and u ---
    for (int k = 0;; ++k) {
      named_sync(kBarAgg0 + (k & 1), NAGG);
      const int st = k % S;
      const long long t = s_tile[st];
      if (t < 0) break;
      const int kb = k & 1;
      const int tx = s_tx[st], ty = s_ty[st];
      const ImageView D = image_view(P, s_img[st]);
      const int ntx = D.ntx, nty = D.nty;
      const bool stall = (t == P.stall_tile);
      const bool pub_row = (REV ? (tx > 0) : (tx < ntx - 1)) && !stall;
      const bool pub_col = (REV ? (ty > 0) : (ty < nty - 1)) && !stall;
      const long long rstride = (REV ? 1 : -1) * (long long)TH * K;
      const int rsteps = REV ? (ntx - 1 - tx) : tx;
      EarlyWin<A> win[ROWS_PER_LANE];
      A agg[ROWS_PER_LANE], left[ROWS_PER_LANE];
#pragma unroll
      for (int i = 0; i < ROWS_PER_LANE; ++i) {
        const int y = lane * ROWS_PER_LANE + i;
        unsigned long long* base = P.row_words + ((unsigned long long)t * TH + y) * K;
        early_read<A>(win[i], base, rstride, rsteps);
        agg[i] = s_rowagg[kb][y];
        if (pub_row) publish<A>(base, agg[i], tagA);
      }
      resolve_n<A, ROWS_PER_LANE>(win, P.row_words + ((unsigned long long)t * TH + lane * ROWS_PER_LANE) * K, K,
                                  rstride, rsteps, tagA, tagI, P, t, left);
#pragma unroll
      for (int i = 0; i < ROWS_PER_LANE; ++i) {
        const int y = lane * ROWS_PER_LANE + i;
        unsigned long long* base = P.row_words + ((unsigned long long)t * TH + y) * K;
        if (pub_row) publish<A>(base, AR::add(left[i], agg[i]), tagI);
        s_rowleft[kb][y] = left[i];
      }
      // inclusive scan of rowleft over the tile's rows, in scan order
      A incl[ROWS_PER_LANE];
      A tsum = AR::zero();
#pragma unroll
      for (int ii = 0; ii < ROWS_PER_LANE; ++ii) {
        const int i = REV ? ROWS_PER_LANE - 1 - ii : ii;
        tsum = AR::add(tsum, left[i]);
        incl[i] = tsum;
      }
      A lsum = tsum; // inclusive over the lanes (scan order)
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const A o = REV ? AR::shfl_down(lsum, d) : AR::shfl_up(lsum, d);
        if (REV ? (lane + d < 32) : (lane >= d)) lsum = AR::add(o, lsum);
      }
      A lex = REV ? AR::shfl_down(lsum, 1) : AR::shfl_up(lsum, 1);
      if (lane == (REV ? 31 : 0)) lex = AR::zero();
#pragma unroll
      for (int i = 0; i < ROWS_PER_LANE; ++i) {
        incl[i] = AR::add(lex, incl[i]);
        const int y = lane * ROWS_PER_LANE + i;
        // rowleft summed over the rows before compute warp w (scan order)
        if (!REV && (y + 1) % RPW == 0 && y + 1 < TH) s_rlprev[kb][(y + 1) / RPW] = incl[i];
        if (REV && y % RPW == 0 && y > 0) s_rlprev[kb][y / RPW - 1] = incl[i];
      }
      if (lane == 0) s_rlprev[kb][REV ? NWC - 1 : 0] = AR::zero();
      // u = sum of rowleft: the corner aggregate of the tile below
      if (lane == (REV ? 0 : 31)) {
        const A u = incl[REV ? 0 : ROWS_PER_LANE - 1];
        unsigned long long* cw = P.corner_words + (unsigned long long)t * K;
        if (pub_col) publish<A>(cw, u, tagA);
        vstore(&s_u[kb], u);
        __threadfence_block();
        if (atomicAdd(&s_cnt_corner[kb], 1) == 1) {
          // the corner is in: this thread publishes corner + u
          __threadfence_block();
          s_cnt_corner[kb] = 0;
          if (pub_col) publish<A>(cw, AR::add(vload(&s_corner[kb]), u), tagI);
        }
      }
      __syncwarp();
      named_arrive(kBarCar0 + kb, NAGG);
    }
  }

  // ---- end of launch: the last CTA resets the ticket and advances the epoch --
  __syncthreads();
  if (tid == 0) finish_launch(P, epoch);
}

}  // namespace satgb
