// sat_kernel_ws.cuh -- the warp-specialized tile loop.
//
// Same decomposition, tickets, status words and look-backs as sat_tile_kernel
// (sat_kernel.cuh); the work of a tile is split between warp groups that never
// wait on one another at a CTA-wide barrier:
//
//   NWC compute warps   the local phase of tile k+1 (partials, the lanes' row
//                       prefix E in registers), then the output phase of
//                       tile k from its TMA stage
//   column group        TW / 32 warps, one column per thread: the column
//                       aggregate out at once, the exclusive prefix over the
//                       compute warps, the column look-back; thread 0 also
//                       the corner look-back
//   row group           TH / 32 warps, one row per thread: the row aggregate
//                       out, the row look-back, the scan of rowleft over the
//                       tile's rows and u = sum rowleft (the corner aggregate
//                       of the tile below)
//   store warp          tickets and stage refills; without DIRECT also one TMA
//                       tensor store per tile
//
// Every look-back thread owns one element, so a tile's look-back costs one
// round trip to L2 (plus waits for late predecessors) instead of one per
// element a thread owns; the look-back threads read their first window as
// soon as the tile's input has arrived, before its partials are ready.
//
// Results leave in one of two ways.  Without DIRECT they go back into the
// tile's stage and one TMA store moves them out; the stage is refilled once
// that store has read it.  With DIRECT each thread stores its 16-byte row
// segments straight from registers, and the stage (input only) goes back to
// the producer as soon as the output phase has read it: the refill is no longer
// held up by the output phase and its store, so the TMA ring keeps the loads a
// whole tile further ahead of the compute warps.
//
// Hand-offs: named barriers AGG[2] (compute warps arrive when a tile's
// partials are in shared memory, the look-back groups wait) and CAR[2] (the
// look-back groups arrive when a tile's carries are in shared memory, the
// compute warps wait), two of each by tile parity: a barrier is used again two
// tiles later, when every participant has provably passed its previous phase.
// Per stage, an mbarrier "done" (each compute warp arrives when its rows of the
// tile's results are in the stage -- with DIRECT, when it has read the stage --
// and the store warp waits); the compute warps may run up to S-1 tiles ahead
// of the store warp, which an mbarrier's phase parity tolerates and a named
// barrier would not.
//
// Shared vectors written by the look-back groups for tile k live in buffers
// indexed k & 1; the compute warps' partials likewise.  A group starts on
// tile k+1 only after every compute warp has arrived at AGG(k+1), i.e. has
// finished its output phase of tile k-1, the last reader of buffer (k+1) & 1.
#pragma once
#include "sat_kernel.cuh"

namespace satgb {

// DIRECT: results go from registers straight to global memory (16-byte
// stores, one per thread and row), so a stage holds only the tile's input.
// CTAS: CTAs per SM the shared memory is split between.
template <class TIn, class TOut, class A, int RPW, int NWC, bool DIRECT = false, int CTAS = 1>
struct TileShapeWS {
  static constexpr int CPT = 16 / (int)sizeof(TOut);
  static constexpr int TW = 32 * CPT;
  static constexpr int TH = NWC * RPW;
  static constexpr int NCW = TW / 32;          // column-group warps
  static constexpr int NRW = TH / 32;          // row-group warps
  static constexpr int RP = RPW > 4 ? 4 : RPW; // rows per pass of the lanes' row transpose
  static constexpr int IN_BYTES = TH * TW * (int)sizeof(TIn);
  static constexpr int STAGE_BYTES =
      TH * TW * (int)(DIRECT || sizeof(TIn) > sizeof(TOut) ? sizeof(TIn) : sizeof(TOut));
  static constexpr int STATIC_BYTES =
      (NWC * RP * 32 + 2 * NWC * TW + 2 * TH + 2 * TW + 2 * TH + 2 * NWC + 2 * NRW + 8) * (int)sizeof(A) + 512;
  static constexpr int S = Stages<STAGE_BYTES, STATIC_BYTES, CTAS>::value;
  static constexpr int DYN_SMEM = S * STAGE_BYTES;
  static constexpr int THREADS = (NWC + NCW + NRW + 1) * 32;
};

// named barrier ids (0 is __syncthreads)
constexpr int kBarAgg0 = 1; // + (k & 1)
constexpr int kBarCar0 = 3; // + (k & 1)
constexpr int kBarWiden = 5;
constexpr int kBarRows = 6; // the row group's scan across its warps

__device__ __forceinline__ void named_arrive(int id, int nthreads) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NWC, bool DIRECT = false, int CTAS = 1>
__global__ void __launch_bounds__(TileShapeWS<TIn, TOut, A, RPW, NWC, DIRECT, CTAS>::THREADS, CTAS)
    sat_tile_kernel_ws(const __grid_constant__ SatParams P) {
  using SH = TileShapeWS<TIn, TOut, A, RPW, NWC, DIRECT, CTAS>;
  constexpr int CPT = SH::CPT;
  constexpr int TW = SH::TW;
  constexpr int TH = SH::TH;
  constexpr int S = SH::S;
  constexpr int NCW = SH::NCW, NRW = SH::NRW;
  constexpr int STAGE_ELEMS = SH::STAGE_BYTES / (int)sizeof(TIn);
  constexpr int WCOL = NWC, WROW = NWC + NCW, WSTORE = NWC + NCW + NRW; // first warp of each role
  constexpr int NAGG = (NWC + NCW + NRW) * 32;                           // compute + look-back warps
  constexpr int RP = SH::RP;   // rows per transpose pass ...
  constexpr int LPR = 32 / RP; // ... lanes per row ...
  constexpr int CH = RP;       // ... and values per lane
  static_assert(TW % 32 == 0 && TH % 32 == 0, "look-back groups are whole warps");
  static_assert(RPW % RP == 0 && 32 % RP == 0, "whole transpose passes");
  static_assert(S >= 3, "stages for the tile in output, the one in the local phase and one loading");
  constexpr int K = Ar<A>::K;
  constexpr bool WIDEN = !DIRECT && sizeof(TIn) < sizeof(TOut); // outputs overlap other threads' inputs in the stage
  using AR = Ar<A>;

  extern __shared__ __align__(128) unsigned char dsmem[];
  TIn* stages = reinterpret_cast<TIn*>(dsmem);

  __shared__ A s_tr[NWC][RP][32];    // compute warps: transpose scratch (lane ^ row: conflict free)
  __shared__ A s_colp[2][NWC][TW];   // per tile parity and warp: column partials, then their exclusive prefix over the warps
  __shared__ A s_rowagg[2][TH];      // row totals
  __shared__ A s_colabove[2][TW];    // column look-back results (by slot)
  __shared__ A s_rowleft[2][TH];     // row look-back results
  __shared__ A s_rlprev[2][NWC];     // per compute warp: sum of rowleft over the rows before it (scan order)
  __shared__ A s_rwt[2][NRW];        // row group: sum of rowleft over each warp's 32 rows
  __shared__ A s_corner[2], s_u[2];
  __shared__ int s_cnt_corner[2];    // arrivals of {corner, u} per tile parity
  __shared__ long long s_tile[S];    // spatial tile index per stage (-1: no more tiles)
  __shared__ int s_img[S];
  __shared__ int s_tx[S], s_ty[S], s_pl[S];
  __shared__ __align__(8) unsigned long long s_full[S];
  // the stage's results are complete (DIRECT: the stage has been read and may be refilled)
  __shared__ __align__(8) unsigned long long s_done[S];

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

  if (DIRECT && warp == WSTORE && lane == 0) {
    // ---- producer thread: each stage is refilled once the output phase of its
    //      tile has read it --------------------------------------------------------
    TilePlan next;
    bool have_next = false;
    if (producing) {
      next = plan_tile<REV>(P, pending);
      have_next = true;
      if (next.t >= 0) pending = atomicAdd(&P.ws->ticket, 1ull);
    }
    for (int k = 0; have_next; ++k) {
      // tile k is a real tile (the one S ahead of it is still to come): its
      // output phase arrives on the stage's barrier
      const int st = k % S;
      mbar_wait_bounded(smem_u32(&s_done[st]), (k / S) & 1, P, -1);
      issue_tile<TIn, TW, TH, SH::IN_BYTES>(P, next, st, stages + st * STAGE_ELEMS, s_tile, s_img, s_tx, s_ty, s_pl,
                                           s_full);
      have_next = false;
      if (next.t >= 0) {
        next = plan_tile<REV>(P, pending);
        have_next = true;
        if (next.t >= 0) pending = atomicAdd(&P.ws->ticket, 1ull);
      }
    }
  }

  if (!DIRECT && warp == WSTORE && lane == 0) {
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
    // groups still get their AGG arrival, to see the end)
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
          colp[c] = AddIn<A, TIn>::add(colp[c], x.u.e[c]);
          rs = AddIn<A, TIn>::add(rs, x.u.e[c]);
        }
        rowp[r] = rs;
      }
      // row partials -> exclusive prefix over the lanes (E) and the row totals,
      // RP rows per pass through the transpose scratch
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
      if (DIRECT) {
        // every input row of the thread into registers, the stage back to the
        // producer, then the results straight to global memory
        RowSeg<TIn, CPT> xin[RPW];
#pragma unroll
        for (int r = 0; r < RPW; ++r) xin[r].u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&s_done[st]));
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
        continue;
      }
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
          run = AddIn<A, TIn>::add(run, x.u.e[c]);
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

  if (warp >= WCOL && warp < WROW) {
    // ---- column group: one column (slot) per thread; thread 0 also the corner --
    const int j = tid - WCOL * 32;
    for (int k = 0;; ++k) {
      const int st = k % S;
      // the tile is known once its input has arrived: read the first look-back
      // windows now, so that round trip overlaps the compute warps' local phase
      mbar_wait_bounded(smem_u32(&s_full[st]), (k / S) & 1, P, -1);
      const long long t = s_tile[st];
      if (t < 0) {
        named_sync(kBarAgg0 + (k & 1), NAGG); // the compute warps' last arrival
        break;
      }
      const int kb = k & 1;
      const int ty = s_ty[st];
      const ImageView D = image_view(P, s_img[st]);
      const int ntx = D.ntx, nty = D.nty;
      const bool pub_col = (REV ? (ty > 0) : (ty < nty - 1)) && t != P.stall_tile;
      const long long cstride = (REV ? 1 : -1) * (long long)ntx * TW * K;
      const int csteps = REV ? (nty - 1 - ty) : ty;
      unsigned long long* base = P.col_words + ((unsigned long long)t * TW + j) * K;
      EarlyWin<A> win[1];
      early_read<A>(win[0], base, cstride, csteps);
      EarlyWin<A> cwin[1];
      unsigned long long* cbase = P.corner_words + (unsigned long long)t * K;
      const long long kstride = (REV ? 1 : -1) * (long long)ntx * K;
      if (j == 0) early_read<A>(cwin[0], cbase, kstride, csteps);
      named_sync(kBarAgg0 + kb, NAGG); // tile k's partials are in
      // the column's partials of every compute warp: all loads first, then the
      // exclusive prefix over the warps (scan order) and the aggregate
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
      const A agg = run;
      if (pub_col) publish<A>(base, agg, tagA);
      A above[1];
      resolve_n<A, 1>(win, base, 0, cstride, csteps, tagA, tagI, P, t, above);
      if (pub_col) publish<A>(base, AR::add(above[0], agg), tagI);
      s_colabove[kb][j] = above[0];
      if (j == 0) {
        A c[1];
        resolve_n<A, 1>(cwin, cbase, 0, kstride, csteps, tagA, tagI, P, t, c);
        vstore(&s_corner[kb], c[0]);
        __threadfence_block();
        if (atomicAdd(&s_cnt_corner[kb], 1) == 1) {
          // u is in: this thread publishes corner + u
          __threadfence_block();
          s_cnt_corner[kb] = 0;
          if (pub_col) publish<A>(cbase, AR::add(c[0], vload(&s_u[kb])), tagI);
        }
      }
      __syncwarp();
      named_arrive(kBarCar0 + kb, NAGG);
    }
  }

  if (warp >= WROW && warp < WSTORE) {
    // ---- row group: one row per thread; rowleft's scan over the tile's rows and u
    const int y = tid - WROW * 32; // the thread's row
    const int rw = warp - WROW;    // its warp within the group
    for (int k = 0;; ++k) {
      const int st = k % S;
      mbar_wait_bounded(smem_u32(&s_full[st]), (k / S) & 1, P, -1);
      const long long t = s_tile[st];
      if (t < 0) {
        named_sync(kBarAgg0 + (k & 1), NAGG);
        break;
      }
      const int kb = k & 1;
      const int tx = s_tx[st], ty = s_ty[st];
      const ImageView D = image_view(P, s_img[st]);
      const int ntx = D.ntx, nty = D.nty;
      const bool stall = (t == P.stall_tile);
      const bool pub_row = (REV ? (tx > 0) : (tx < ntx - 1)) && !stall;
      const bool pub_col = (REV ? (ty > 0) : (ty < nty - 1)) && !stall;
      const long long rstride = (REV ? 1 : -1) * (long long)TH * K;
      const int rsteps = REV ? (ntx - 1 - tx) : tx;
      unsigned long long* base = P.row_words + ((unsigned long long)t * TH + y) * K;
      EarlyWin<A> win[1];
      early_read<A>(win[0], base, rstride, rsteps);
      named_sync(kBarAgg0 + kb, NAGG);
      const A agg = s_rowagg[kb][y];
      if (pub_row) publish<A>(base, agg, tagA);
      A left[1];
      resolve_n<A, 1>(win, base, 0, rstride, rsteps, tagA, tagI, P, t, left);
      if (pub_row) publish<A>(base, AR::add(left[0], agg), tagI);
      s_rowleft[kb][y] = left[0];
      // inclusive scan of rowleft over the tile's rows, in scan order: within
      // the warp, then across the group's warps
      A incl = left[0];
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
      // rowleft summed over the rows before compute warp w (scan order)
      if (!REV && (y + 1) % RPW == 0 && y + 1 < TH) s_rlprev[kb][(y + 1) / RPW] = incl;
      if (REV && y % RPW == 0 && y > 0) s_rlprev[kb][y / RPW - 1] = incl;
      if (y == (REV ? TH - 1 : 0)) s_rlprev[kb][REV ? NWC - 1 : 0] = AR::zero();
      // u = sum of rowleft: the corner aggregate of the tile below
      if (y == (REV ? 0 : TH - 1)) {
        const A u = incl;
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
