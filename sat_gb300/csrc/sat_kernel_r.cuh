// sat_kernel_r.cuh -- the tile loop with each tile's inputs held in registers
// from the local phase to the output phase.
//
// Same decomposition, tickets, status words and look-backs as
// sat_tile_kernel (sat_kernel.cuh); a different CTA design:
//
//  * Several small CTAs per SM (typically two of 8 warps), each running one
//    tile at a time: local phase, look-back, output phase.  While one CTA
//    waits for its look-back round trip the other computes, so the latency is
//    hidden without software pipelining inside a CTA.
//  * A thread loads its RPW x CPT block of the tile from the TMA stage into
//    registers once; the output phase works from those registers.  The stage
//    is free for the next TMA load as soon as the local phase is over, so the
//    ring of S stages runs S tiles ahead.
//  * Results leave by 16-byte streaming stores straight from registers: a
//    warp writes 512 contiguous bytes of each of its rows.
//  * The first look-back window is read when the tile arrives, so its round
//    trip overlaps the local phase.
//
// Per tile and element: one shared-memory read of the input (plus the TMA
// write), one global store; the transposes add one shared write and read per
// thread and row.
#pragma once
#include "sat_kernel.cuh"

namespace satgb {

template <class TIn, class TOut, class A, int RPW, int NW, int CTAS>
struct TileShapeR {
  static constexpr int CPT = 16 / (int)sizeof(TOut);
  static constexpr int TW = 32 * CPT;
  static constexpr int TH = NW * RPW;
  static constexpr int IN_BYTES = TH * TW * (int)sizeof(TIn);
  static constexpr int STAGE_BYTES = IN_BYTES; // stages hold inputs only
  static constexpr int STATIC_BYTES = (NW * RPW * 32 + NW * TW + 4 * TH + TW) * (int)sizeof(A) + 512;
  static constexpr int S = Stages<STAGE_BYTES, STATIC_BYTES, CTAS>::value;
  static constexpr int DYN_SMEM = S * STAGE_BYTES;
  static constexpr int THREADS = NW * 32;
};

template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB>
__global__ void __launch_bounds__(NW * 32, MINB) sat_tile_kernel_r(const __grid_constant__ SatParams P) {
  using SH = TileShapeR<TIn, TOut, A, RPW, NW, MINB>;
  constexpr int CPT = SH::CPT;
  constexpr int TW = SH::TW;
  constexpr int TH = SH::TH;
  constexpr int S = SH::S;
  constexpr int NC = NW * 32;
  constexpr int STAGE_ELEMS = SH::STAGE_BYTES / (int)sizeof(TIn);
  static_assert(NC - (TW + TH) >= 64, "threads for rows, columns, the corner warp and the producer");
  static_assert(TH % 32 == 0 && TW % 32 == 0, "groups are whole warps");
  static_assert(32 % RPW == 0, "rows per warp divide the warp");
  static_assert(S >= 2, "one stage in use, one loading");
  constexpr int CW = (TW + TH) / 32; // corner warp
  constexpr int PT = NC - 1;         // producer thread (last warp, never the corner warp)
  static_assert(CW < NW - 1, "corner warp and producer warp differ");
  constexpr int LPR = 32 / RPW; // transpose-scan: lanes per row ...
  constexpr int CH = RPW;       // ... and values per lane
  constexpr int K = Ar<A>::K;
  using AR = Ar<A>;

  extern __shared__ __align__(128) unsigned char dsmem[];
  TIn* stages = reinterpret_cast<TIn*>(dsmem);

  __shared__ A s_tr[NW][RPW][32]; // per-warp transpose scratch (index lane ^ row: conflict free)
  __shared__ A s_colp[NW][TW];    // per warp: column partials (by slot); then the exclusive prefix over warps
  __shared__ A s_rowagg[TH];      // row totals
  __shared__ A s_rowleft[TH];     // row look-back result
  __shared__ A s_RL[TH];          // its scan over each 32-row group
  __shared__ A s_rlw[TH / 32];    // per 32-row group: the sum of rowleft
  __shared__ A s_colabove[TW];    // column look-back result (by slot)
  __shared__ A s_corner, s_u;
  __shared__ int s_cnt_row, s_cnt_corner; // arrivals of the row warps / of {rows, corner}
  __shared__ long long s_tile[S];         // spatial tile index per stage (-1: no more tiles)
  __shared__ int s_img[S];
  __shared__ int s_tx[S], s_ty[S], s_pl[S];
  __shared__ __align__(8) unsigned long long s_full[S];

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint32_t epoch = ld_relaxed_u32(&P.ws->epoch);
  const uint32_t tagA = make_tag(epoch, kStateAgg);
  const uint32_t tagI = make_tag(epoch, kStateInc);
  const bool is_col = tid < TW;
  const bool is_row = !is_col && tid < TW + TH;
  const bool is_cor = warp == CW && lane == 0;

  unsigned long long pending = 0; // producer thread: the next ticket, fetched a tile ahead
  bool producing = true;
  if (tid == 0) {
    s_cnt_row = 0;
    s_cnt_corner = 0;
  }
  if (tid == PT) {
#pragma unroll
    for (int s = 0; s < S; ++s) mbar_init(smem_u32(&s_full[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
#pragma unroll
    for (int s = 0; s < S; ++s) {
      if (producing)
        producing = produce<TIn, REV, TW, TH, SH::IN_BYTES>(P, atomicAdd(&P.ws->ticket, 1ull), s,
                                                            stages + s * STAGE_ELEMS, s_tile, s_img, s_tx, s_ty,
                                                            s_pl, s_full);
    }
    if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
  }
  __syncthreads();

  for (int k = 0;; ++k) {
    const int st = k % S;
    mbar_wait_bounded(smem_u32(&s_full[st]), (k / S) & 1, P, -1);
    const long long t = s_tile[st];
    if (t < 0) break;
    const int tx = s_tx[st], ty = s_ty[st], img = s_img[st], pl = s_pl[st];
    const ImageView D = image_view(P, img);
    const int ntx = D.ntx, nty = D.nty;
    const bool stall = (t == P.stall_tile);
    const bool pub_row = REV ? (tx > 0) : (tx < ntx - 1);
    const bool pub_col = REV ? (ty > 0) : (ty < nty - 1);

    // look-back role of this thread; its first window is read now, so the
    // round trip overlaps the local phase
    const unsigned long long* lb_base = nullptr;
    long long lb_stride = 0;
    int lb_steps = 0;
    if (is_col) {
      lb_base = P.col_words + ((unsigned long long)t * TW + tid) * K;
      lb_stride = (REV ? 1 : -1) * (long long)ntx * TW * K;
      lb_steps = REV ? (nty - 1 - ty) : ty;
    } else if (is_row) {
      lb_base = P.row_words + ((unsigned long long)t * TH + (tid - TW)) * K;
      lb_stride = (REV ? 1 : -1) * (long long)TH * K;
      lb_steps = REV ? (ntx - 1 - tx) : tx;
    } else if (is_cor) {
      lb_base = P.corner_words + (unsigned long long)t * K;
      lb_stride = (REV ? 1 : -1) * (long long)ntx * K;
      lb_steps = REV ? (nty - 1 - ty) : ty;
    }
    EarlyWin<A> win;
    if (is_col || is_row || is_cor) early_read<A>(win, lb_base, lb_stride, lb_steps);

    // ---- local phase: the thread's block into registers, partial sums ---------
    const long long x0 = (long long)tx * TW, y0 = (long long)ty * TH;
    const long long xt = x0 + (long long)lane * CPT;
    const long long rem = D.width - xt;
    const int nvalid = rem <= 0 ? 0 : (rem >= CPT ? CPT : (int)rem);
    const long long rows_left = D.height - (y0 + warp * RPW);
    const int nrows = rows_left <= 0 ? 0 : (rows_left >= RPW ? RPW : (int)rows_left);
    TIn* sb = stages + st * STAGE_ELEMS + (warp * RPW) * TW + lane * CPT;
    {
      const bool tma = D.flags & kInTma;
      if (!tma || (nvalid > 0 && xt + nvalid > D.tma_in_w)) {
        // no TMA for this image, or columns past the map (they arrived as zeros)
        const TIn* gin =
            static_cast<const TIn*>(D.in) + (long long)pl * D.in_plane + (y0 + warp * RPW) * D.in_pitch + xt;
        const int c0 = tma ? (int)(D.tma_in_w - xt > 0 ? D.tma_in_w - xt : 0) : 0;
        stage_fill<TIn, CPT, RPW, TW>(sb, gin, D.in_pitch, nrows, nvalid, c0, (D.flags & kInVec) != 0);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); // before TMA refills the stage
      }
    }
    RowSeg<TIn, CPT> x[RPW];
#pragma unroll
    for (int r = 0; r < RPW; ++r) x[r].u.v = *reinterpret_cast<const typename RowSeg<TIn, CPT>::V*>(sb + r * TW);
    A colp[CPT], rowp[RPW];
#pragma unroll
    for (int c = 0; c < CPT; ++c) colp[c] = AR::zero();
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      A rs = AR::zero();
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        colp[c] = AddIn<A, TIn>::add(colp[c], x[r].u.e[c]);
        rs = AddIn<A, TIn>::add(rs, x[r].u.e[c]);
      }
      rowp[r] = rs;
    }
    // row partials -> exclusive prefix over the lanes (E) and the row totals
    A E[RPW];
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
      if (q == (REV ? 0 : LPR - 1)) s_rowagg[warp * RPW + r] = incl;
    }
    __syncwarp();
#pragma unroll
    for (int r = 0; r < RPW; ++r) E[r] = s_tr[warp][r][lane ^ r];
#pragma unroll
    for (int c = 0; c < CPT; ++c) s_colp[warp][c * 32 + lane] = colp[c];
    __syncthreads(); // partials complete; every thread is done with the stage

    // ---- look-back phase ----------------------------------------------------
    A my_agg = AR::zero();
    if (is_col) {
      // column aggregate out at once, then the exclusive prefix over the warps
      const int j = tid;
      A ac = AR::zero();
#pragma unroll
      for (int w = 0; w < NW; ++w) ac = AR::add(ac, s_colp[w][j]);
      if (pub_col && !stall) publish<A>(P.col_words + ((unsigned long long)t * TW + j) * K, ac, tagA);
      A run = AR::zero();
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        const int w = REV ? NW - 1 - i : i;
        const A b = s_colp[w][j];
        s_colp[w][j] = run;
        run = AR::add(run, b);
      }
      my_agg = ac;
    } else if (is_row) {
      my_agg = s_rowagg[tid - TW];
      if (pub_row && !stall) publish<A>(P.row_words + ((unsigned long long)t * TH + (tid - TW)) * K, my_agg, tagA);
    } else if (tid == PT && producing) {
      // refill the stage this tile came from: every thread has read it
      producing = produce<TIn, REV, TW, TH, SH::IN_BYTES>(P, pending, st, stages + st * STAGE_ELEMS, s_tile, s_img,
                                                          s_tx, s_ty, s_pl, s_full);
      if (producing) pending = atomicAdd(&P.ws->ticket, 1ull);
    }
    // one look-back call site for the three roles (columns, rows, corner)
    A got = AR::zero();
    if (is_col || is_row || is_cor) got = resolve<A>(win, lb_base, lb_stride, lb_steps, tagA, tagI, P, t);
    if (is_col) {
      if (pub_col && !stall) publish<A>(P.col_words + ((unsigned long long)t * TW + tid) * K, AR::add(got, my_agg), tagI);
      s_colabove[tid] = got;
    } else if (is_row) {
      const int yy = tid - TW;
      if (pub_row && !stall) publish<A>(P.row_words + ((unsigned long long)t * TH + yy) * K, AR::add(got, my_agg), tagI);
      s_rowleft[yy] = got;
      // scan of rowleft over this warp's 32 rows, in scan order; the group sum
      A incl = got;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const A o = REV ? AR::shfl_down(incl, d) : AR::shfl_up(incl, d);
        if (REV ? (lane + d < 32) : (lane >= d)) incl = AR::add(o, incl);
      }
      s_RL[yy] = incl;
      if (lane == (REV ? 0 : 31)) s_rlw[yy / 32] = incl;
      __syncwarp();
      if (lane == 0) {
        // the last row warp to get here publishes u = sum of rowleft, the corner
        // aggregate; the later of it and the corner thread publishes corner + u
        __threadfence_block();
        if (atomicAdd(&s_cnt_row, 1) == TH / 32 - 1) {
          __threadfence_block();
          s_cnt_row = 0;
          A u = AR::zero();
#pragma unroll
          for (int g = 0; g < TH / 32; ++g) u = AR::add(u, vload(&s_rlw[g]));
          vstore(&s_u, u);
          unsigned long long* cw = P.corner_words + (unsigned long long)t * K;
          if (pub_col && !stall) publish<A>(cw, u, tagA);
          __threadfence_block();
          if (atomicAdd(&s_cnt_corner, 1) == 1) {
            __threadfence_block();
            s_cnt_corner = 0;
            if (pub_col && !stall) publish<A>(cw, AR::add(vload(&s_corner), u), tagI);
          }
        }
      }
    } else if (is_cor) {
      vstore(&s_corner, got);
      __threadfence_block();
      if (atomicAdd(&s_cnt_corner, 1) == 1) {
        __threadfence_block();
        s_cnt_corner = 0;
        if (pub_col && !stall) publish<A>(P.corner_words + (unsigned long long)t * K, AR::add(got, vload(&s_u)), tagI);
      }
    }
    __syncthreads();

    // ---- output phase: carries in, scan from registers, stores out ------------
    A top[CPT];
    {
      const A corner = s_corner;
      const bool has_prev = REV ? (warp < NW - 1) : (warp > 0);
      A rl_prev = AR::zero();
      if (has_prev) {
        // RL of the row just outside the warp: its group's scan plus the groups before it
        const int yp = REV ? (warp + 1) * RPW : warp * RPW - 1;
        rl_prev = s_RL[yp];
#pragma unroll
        for (int g = 0; g < TH / 32; ++g)
          if (REV ? (g > yp / 32) : (g < yp / 32)) rl_prev = AR::add(s_rlw[g], rl_prev);
      }
      A cp[CPT];
#pragma unroll
      for (int i = 0; i < CPT; ++i) {
        const int c = REV ? CPT - 1 - i : i;
        cp[c] = AR::add(s_colabove[c * 32 + lane], s_colp[warp][c * 32 + lane]);
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
    }
    {
      const int64_t out_pitch = D.out_pitch;
      TOut* out = static_cast<TOut*>(D.out) + (long long)pl * D.out_plane + (y0 + warp * RPW) * out_pitch + xt;
      const bool vout = (D.flags & kOutVec) && nvalid == CPT && nrows == RPW;
#pragma unroll
      for (int i = 0; i < RPW; ++i) {
        const int r = REV ? RPW - 1 - i : i;
        A run = AR::add(E[r], s_rowleft[warp * RPW + r]);
        union {
          uint4 v;
          TOut e[CPT];
        } o;
#pragma unroll
        for (int ii = 0; ii < CPT; ++ii) {
          const int c = REV ? CPT - 1 - ii : ii;
          run = AddIn<A, TIn>::add(run, x[r].u.e[c]);
          top[c] = AR::add(top[c], run);
          o.e[c] = OutCvt<TOut, A>::out(top[c]);
        }
        if (vout) {
          __stcs(reinterpret_cast<uint4*>(out + r * out_pitch), o.v);
        } else if (r < nrows) {
#pragma unroll
          for (int c = 0; c < CPT; ++c)
            if (c < nvalid) __stcs(out + r * out_pitch + c, o.e[c]);
        }
      }
    }
  }

  // ---- end of launch: the last CTA resets the ticket and advances the epoch --
  __syncthreads();
  if (tid == 0) finish_launch(P, epoch);
}

}  // namespace satgb
