// recon.cu -- direct-DFT reconstruction (replaces imagerecon, vissGen10M_shade.cu:149-175,
// and the tiled optim2 form, vissGen10M_shade_optim2.cu:219-317).
//
// F_j = norm * sum_k [not masked] y_k exp(+2 pi i t_kj),  y_k = wgt_k V_k
//
// A work item is REC_PIX = 1024 pixels (4 per thread, fixed-point coordinates
// in registers) against one segment of visibility rows of one channel, streamed
// through shared memory in tiles of 2 REC_Q rows, 4 REC_Q with the geometric mask and
// no compensation (REC_Q or REC_Q / 2 on request).
// The phase of y_k is folded into the
// row's fixed-point bias (y e^{ix} = |y| e^{i(x + arg y)}), so a term is the
// same as in the vis kernel: 3 IMAD [+3 FFMA fractional uvw] [+3 FFMA
// compensated], turns -> angle, __sincosf, 2 FFMA with |y_k|.
// Masks:
//   GEOMETRIC: rows hidden from the whole pixel block are dropped when a tile is
//     loaded; the rest come in snapshot runs.  Per run the warp tests the cap
//     bounding its 128 pixels against the snapshot's cones (warp-uniform); where
//     that leaves the run open, every thread tests its pixels against the
//     snapshot's bounding cone and the warp votes: all occluded -> the run is
//     skipped, all visible -> unmasked loop, else the thread builds a per-pixel
//     satellite occlusion bitmask and tests each row's pair.
//   REF: the reference ratio mask can only fire on pixels (thetaP, phiP) with
//     1 <= thetaP <= tmax_k, 1 <= phiP <= pmax_k; tiles whose rows cannot touch
//     the item's pixels run unmasked.
// Persistent CTAs take items from an atomic counter, longest segments first.
// A channel split into several segments leaves partial sums per segment,
// reduced in a fixed order.
#include "viss_internal.cuh"

namespace viss {

// Exact decision near the limb (rare), out of line.
__device__ __noinline__ bool geo_exact_pix(const ReconParams& p, int j, int gidx) {
  count_limb(p.flags);
  return geo_occluded_exact(p.l[j], p.m[j], p.n[j], p.sat_pos + 3 * (int64_t)gidx, p.R);
}

template <bool FRAC, bool COMP>
__device__ __forceinline__ void rec_term(const int4& r0, const float4& r1, const float4& rf, float c, int A, int B,
                                         int C, float X, float Y, float Z, float lx, float ly, float lz, float& fr,
                                         float& fi) {
  const uint32_t q = (uint32_t)r0.x * (uint32_t)A + (uint32_t)r0.y * (uint32_t)B + (uint32_t)r0.z * (uint32_t)C +
                     (uint32_t)r0.w;
  float e = KM3PI;
  if (FRAC) e = fmaf(r1.x, X, fmaf(r1.y, Y, fmaf(r1.z, Z, e)));
  if (COMP) e = fmaf(rf.x, lx, fmaf(rf.y, ly, fmaf(rf.z, lz, e)));
  const float x = turns_to_angle(q, e);
  float sn, cs;
  __sincosf(x, &sn, &cs);
  fr = fmaf(c, cs, fr);
  fi = fmaf(c, sn, fi);
}

constexpr int RM_NONE = 0, RM_REF = 1, RM_GEO = 2;
constexpr int REC_SAT_CACHE = 512;   // satellite directions cached per tile (float4)
constexpr int REC_CONE_CACHE = 128;  // snapshot cones cached per tile

template <int RM, bool COMP, int Q>
struct RecSmem {
  int4 r0[Q];
  float4 r1[Q];
  float4 rf[COMP ? Q : 1];
  int4 win[RM == RM_REF ? Q : 1];
  uint32_t pm[RM == RM_GEO ? Q : 1];   // the row's two satellites as bits of its snapshot's satellites
  int snap[RM == RM_GEO ? Q : 1];
  int runend[RM == RM_GEO ? Q : 1];
  float4 sat[RM == RM_GEO ? REC_SAT_CACHE : 1];
  float4 cone[RM == RM_GEO ? 2 * REC_CONE_CACHE : 1];
  float4 wcap[RM == RM_GEO ? 2 * (REC_THREADS / 32) : 1];  // each warp's patch: {axis, cos r}, {sin r}
  int srange[2];
  int wkeep[(REC_THREADS / 32) * ((Q + REC_THREADS - 1) / REC_THREADS)];
  float4 acc[REC_PIX];            // running totals (re, im) and their Kahan compensation per pixel
};

template <int RM, bool FRAC, bool COMP, int Q>
__device__ __forceinline__ void recon_body(const ReconParams& p, RecSmem<RM, COMP, Q>& sm, int64_t pb, int64_t kb,
                                           int64_t ke, float2* out, float norm, bool direct) {
  constexpr int REC_LOAD = (Q + REC_THREADS - 1) / REC_THREADS;  // tile rows per thread in the load
  const int tid = threadIdx.x;
  // a warp owns 32 * REC_TJ consecutive positions: with the spatial order of
  // the geometric passes that is one compact patch of sky
  const int64_t j0 = pb * REC_PIX + (int64_t)tid * REC_TJ;
  int A[REC_TJ], B[REC_TJ], C[REC_TJ];
  float XF[REC_TJ], YF[REC_TJ], ZF[REC_TJ];
  float LX[REC_TJ], LY[REC_TJ], LZ[REC_TJ];
  int TP[REC_TJ], PP[REC_TJ];
  // running totals live in sm.acc; pixel directions (geometric) are re-read per snapshot run
#pragma unroll
  for (int i = 0; i < REC_TJ; ++i) {
    const int64_t pos = j0 + i;  // pixels padded to a whole block
    const int4 a = p.pix0[pos];
    A[i] = a.x; B[i] = a.y; C[i] = a.z;
    XF[i] = YF[i] = ZF[i] = 0.f;
    if (FRAC) {
      const int4 b = p.pix1[pos];
      XF[i] = __int_as_float(b.x); YF[i] = __int_as_float(b.y); ZF[i] = __int_as_float(b.z);
    }
    LX[i] = LY[i] = LZ[i] = 0.f;
    if (COMP) { const float4 lo = p.plo[pos]; LX[i] = lo.x; LY[i] = lo.y; LZ[i] = lo.z; }
    TP[i] = PP[i] = -1;
    if (RM == RM_REF) { const int2 qr = p.pqr[pos]; PP[i] = qr.x; TP[i] = qr.y; }
    sm.acc[tid * REC_TJ + i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  unsigned valid = 0;  // bit i: pixel i of this thread is a real pixel
#pragma unroll
  for (int i = 0; i < REC_TJ; ++i) valid |= (j0 + i < p.J ? 1u : 0u) << i;
  const int64_t jfirst = pb * REC_PIX;
  int64_t jlast = jfirst + REC_PIX - 1;
  if (jlast > p.J - 1) jlast = p.J - 1;

  // geometric: the block's bounding cone {axis, cos r, sin r}; a row whose snapshot
  // hides every pixel of the block is dropped from the tile, for all warps at once
  float4 bc0 = make_float4(0.f, 0.f, 0.f, -2.f);
  float bsin = 1.f;
  if (RM == RM_GEO) {
    bc0 = __ldg(p.bcones + 2 * pb);
    bsin = __ldg(p.bcones + 2 * pb + 1).x;
    // this warp's patch cap (read and written by this warp only)
    if ((tid & 31) < 2)
      sm.wcap[2 * (tid >> 5) + (tid & 31)] = __ldg(p.wcones + 2 * (pb * (REC_THREADS / 32) + (tid >> 5)) + (tid & 31));
    __syncwarp();
  }

  for (int64_t tile = kb; tile < ke; tile += Q) {
    int nq = (int)((ke - tile) < Q ? (ke - tile) : Q);
    __syncthreads();
    if (RM == RM_GEO && tid == 0) { sm.srange[0] = 0x7fffffff; sm.srange[1] = -1; }
    if (RM == RM_GEO) {
      // keep row tid unless its snapshot's all-occluded cone {a, cos ao} holds the whole
      // block: angle(axis, a) + r < ao, i.e. axis.a > cos(ao - r) = cos ao cos r + sin ao sin r
      // (REC_LOAD rows per thread, kept rows compacted in order)
      bool keep[REC_LOAD];
      int pk[REC_LOAD];
      unsigned bal[REC_LOAD];
#pragma unroll
      for (int h = 0; h < REC_LOAD; ++h) {
        const int r = h * REC_THREADS + tid;
        keep[h] = false;
        pk[h] = 0;
        if (r < nq) {
          pk[h] = p.rowsat[tile + r];
          const int sn = sat_gm(pk[h]) / p.nsat;
          const float4 sc = __ldg(p.scones + 2 * (int64_t)sn);
          keep[h] = true;
          if (sc.w <= 1.f && bc0.w >= -1.f && sc.w < bc0.w) {  // the cone is wider than the block
            const float cao = sc.w, sao = sqrtf(fmaxf(0.f, 1.f - cao * cao));
            const float lim = fmaf(cao, bc0.w, sao * bsin) + 1e-5f;
            const float d = fmaf(bc0.x, sc.x, fmaf(bc0.y, sc.y, bc0.z * sc.z));
            keep[h] = !(d > lim);
          }
        }
        bal[h] = __ballot_sync(0xffffffffu, keep[h]);
        if ((tid & 31) == 0) sm.wkeep[h * (REC_THREADS / 32) + (tid >> 5)] = __popc(bal[h]);
      }
      __syncthreads();
      int base = 0;
#pragma unroll
      for (int h = 0; h < REC_LOAD; ++h) {
        int off = base + __popc(bal[h] & ((1u << (tid & 31)) - 1u)), tot = 0;
#pragma unroll
        for (int w2 = 0; w2 < REC_THREADS / 32; ++w2) {
          const int c = sm.wkeep[h * (REC_THREADS / 32) + w2];
          if (w2 < (tid >> 5)) off += c;
          tot += c;
        }
        if (keep[h]) {
          const int64_t k = tile + h * REC_THREADS + tid;
          sm.r0[off] = p.rows0[k];
          sm.r1[off] = p.rows1[k];
          if (COMP) sm.rf[off] = p.rowsf[k];
          const int sn = sat_gm(pk[h]) / p.nsat;
          const int g0 = sn * p.nsat;
          sm.pm[off] = (1u << (sat_gm(pk[h]) - g0)) | (1u << (sat_gn(pk[h]) - g0));
          sm.snap[off] = sn;
          atomicMin(&sm.srange[0], sn);
          atomicMax(&sm.srange[1], sn);
        }
        base += tot;
      }
      nq = base;
      __syncthreads();
      if (nq == 0) continue;  // the block is hidden from every row of this tile
    }
    bool hit = false;
    for (int r = tid; r < (RM == RM_GEO ? 0 : nq); r += REC_THREADS) {
      const int64_t k = tile + r;
      sm.r0[r] = p.rows0[k];
      sm.r1[r] = p.rows1[k];
      if (COMP) sm.rf[r] = p.rowsf[k];
      if (RM == RM_REF) {
        const int4 wv = p.win[k];
        sm.win[r] = wv;
        if (wv.x >= 1 && wv.y >= 1) {
          const int64_t lo_idx = (int64_t)p.res + 1, hi_idx = (int64_t)wv.y * p.res + wv.x;
          if (lo_idx <= jlast && hi_idx >= jfirst) hit = true;
        }
      }
    }
    const bool masked_tile = __syncthreads_or(hit) != 0;
    float tr[REC_TJ], ti[REC_TJ];  // this tile's sums
#pragma unroll
    for (int i = 0; i < REC_TJ; ++i) tr[i] = ti[i] = 0.f;
    if (RM == RM_GEO) {
      const int s_lo = sm.srange[0], s_hi = sm.srange[1];
      const int nsn = s_hi - s_lo + 1;
      const bool cached = nsn <= REC_CONE_CACHE && nsn * p.nsat <= REC_SAT_CACHE;
      if (cached) {
        for (int t = tid; t < nsn * p.nsat; t += REC_THREADS) sm.sat[t] = p.satdir[(int64_t)s_lo * p.nsat + t];
        for (int t = tid; t < 2 * nsn; t += REC_THREADS) sm.cone[t] = p.scones[2 * (int64_t)s_lo + t];
      }
      for (int r = tid; r < nq; r += REC_THREADS) {
        const int sn = sm.snap[r];
        if (r == 0 || sm.snap[r - 1] != sn) {
          int e = r + 1;
          while (e < nq && sm.snap[e] == sn) ++e;
          sm.runend[r] = e;
        }
      }
      __syncthreads();
      for (int r = 0; r < nq;) {
        const int re = sm.runend[r];
        const int sn = sm.snap[r];
        const float4 c0 = cached ? sm.cone[2 * (sn - s_lo)] : __ldg(p.scones + 2 * (int64_t)sn);
        const float4 c1 = cached ? sm.cone[2 * (sn - s_lo) + 1] : __ldg(p.scones + 2 * (int64_t)sn + 1);
        // The warp's patch cap {a, r} against the snapshot's cones (warp-uniform):
        // all hidden when angle(a, c) + r < alpha_occ, i.e. a.c > cos(alpha_occ - r);
        // all visible when angle(a, c) - r > alpha_vis, i.e. a.c < cos(alpha_vis + r)
        // (alpha_vis + r < pi).  Margins of 1e-5 in the cosine; what the cap leaves
        // open the per-pixel vote decides, so the decisions are the vote's.
        const float4 wc = sm.wcap[2 * (tid >> 5)];
        const float ws = sm.wcap[2 * (tid >> 5) + 1].x;
        const float dw = fmaf(wc.x, c0.x, fmaf(wc.y, c0.y, wc.z * c0.z));
        bool wocc = false, wvis = false;
        if (wc.w >= -1.f) {
          wocc = c0.w <= 1.f && c0.w < wc.w && dw > fmaf(c0.w, wc.w, c1.y * ws) + 1e-5f;
          wvis = c1.x >= -1.f && fmaf(c1.z, wc.w, c1.x * ws) > 0.f && dw < fmaf(c1.x, wc.w, -c1.z * ws) - 1e-5f;
        }
        if (!wocc && !wvis) {
          bool all_vis = true, all_occ = true;
#pragma unroll
          for (int i = 0; i < REC_TJ; ++i) {
            const float4 g = __ldg(p.pgeo + j0 + i);
            const float d = fmaf(g.x, c0.x, fmaf(g.y, c0.y, g.z * c0.z));
            const bool v = (valid >> i) & 1u;
            all_vis &= !v || d < c1.x;
            all_occ &= !v || d > c0.w;
          }
          wocc = __all_sync(0xffffffffu, all_occ);
          wvis = __all_sync(0xffffffffu, all_vis);
        }
        if (wocc) { r = re; continue; }
        if (wvis) {
#pragma unroll 2
          for (int rr = r; rr < re; ++rr) {
            const int4 r0 = sm.r0[rr];
            const float4 r1 = sm.r1[rr];
            float4 rf = make_float4(0.f, 0.f, 0.f, 0.f);
            if (COMP) rf = sm.rf[rr];
#pragma unroll
            for (int i = 0; i < REC_TJ; ++i)
              rec_term<FRAC, COMP>(r0, r1, rf, r1.w, A[i], B[i], C[i], XF[i], YF[i], ZF[i], LX[i], LY[i], LZ[i],
                                   tr[i], ti[i]);
          }
        } else {
          // per-pixel satellite occlusion bits for snapshot sn
          uint32_t bits[REC_TJ];
          const int g0 = sn * p.nsat;
#pragma unroll
          for (int i = 0; i < REC_TJ; ++i) bits[i] = 0u;
#pragma unroll
          for (int i = 0; i < REC_TJ; ++i) {
            const float4 g = __ldg(p.pgeo + j0 + i);
            for (int sat = 0; sat < p.nsat; ++sat) {
              const float4 d = cached ? sm.sat[(sn - s_lo) * p.nsat + sat] : __ldg(p.satdir + g0 + sat);
              const float e = fmaf(g.x, d.x, fmaf(g.y, d.y, fmaf(g.z, d.z, d.w)));
              bool occ = e < 0.f;
              if (fabsf(e) < GEO_EPS && ((valid >> i) & 1u)) occ = geo_exact_pix(p, __float_as_int(g.w), g0 + sat);
              bits[i] |= (occ ? 1u : 0u) << sat;
            }
          }
#pragma unroll 2
          for (int rr = r; rr < re; ++rr) {
            const int4 r0 = sm.r0[rr];
            const float4 r1 = sm.r1[rr];
            float4 rf = make_float4(0.f, 0.f, 0.f, 0.f);
            if (COMP) rf = sm.rf[rr];
            const uint32_t pm = sm.pm[rr];
#pragma unroll
            for (int i = 0; i < REC_TJ; ++i) {
              const float c = (bits[i] & pm) ? 0.f : r1.w;
              rec_term<FRAC, COMP>(r0, r1, rf, c, A[i], B[i], C[i], XF[i], YF[i], ZF[i], LX[i], LY[i], LZ[i],
                                   tr[i], ti[i]);
            }
          }
        }
        r = re;
      }
    } else if (RM == RM_REF && masked_tile) {
      for (int rr = 0; rr < nq; ++rr) {
        const int4 r0 = sm.r0[rr];
        const float4 r1 = sm.r1[rr];
        float4 rf = make_float4(0.f, 0.f, 0.f, 0.f);
        if (COMP) rf = sm.rf[rr];
        const int4 wv = sm.win[rr];
#pragma unroll
        for (int i = 0; i < REC_TJ; ++i) {
          const bool skip = TP[i] >= 1 && TP[i] <= wv.x && PP[i] >= 1 && PP[i] <= wv.y;
          const float c = skip ? 0.f : r1.w;
          rec_term<FRAC, COMP>(r0, r1, rf, c, A[i], B[i], C[i], XF[i], YF[i], ZF[i], LX[i], LY[i], LZ[i], tr[i],
                               ti[i]);
        }
      }
    } else {
#pragma unroll 2
      for (int rr = 0; rr < nq; ++rr) {
        const int4 r0 = sm.r0[rr];
        const float4 r1 = sm.r1[rr];
        float4 rf = make_float4(0.f, 0.f, 0.f, 0.f);
        if (COMP) rf = sm.rf[rr];
#pragma unroll
        for (int i = 0; i < REC_TJ; ++i)
          rec_term<FRAC, COMP>(r0, r1, rf, r1.w, A[i], B[i], C[i], XF[i], YF[i], ZF[i], LX[i], LY[i], LZ[i], tr[i],
                               ti[i]);
      }
    }
#pragma unroll
    for (int i = 0; i < REC_TJ; ++i) {
      float4 t = sm.acc[tid * REC_TJ + i];  // owned by this thread alone
      kahan_add(t.x, t.z, tr[i]);
      kahan_add(t.y, t.w, ti[i]);
      sm.acc[tid * REC_TJ + i] = t;
    }
  }
  // F = norm * (-fr - i fi)  (the angle carried an extra half turn)
#pragma unroll
  for (int i = 0; i < REC_TJ; ++i) {
    const int64_t pos = j0 + i;
    const float4 t = sm.acc[tid * REC_TJ + i];
    const float fr = t.x, fi = t.y;
    if (pos < p.J) {
      if (direct) {
        const int64_t j = p.perm ? (int64_t)p.perm[pos] : pos;
        out[j] = make_float2(-fr * norm, -fi * norm);
      } else {
        out[pos] = make_float2(fr, fi);
      }
    }
  }
}

// Persistent: grid = resident CTAs; each CTA takes the next work item (segment,
// pixel block) from an atomic counter until none are left.  The counter is
// reset by the host before the launch; no CTA waits on another.
// Resident CTAs per SM the instances are compiled for.  The unmasked and REF-mask ones
// fit in 64 registers (a few spills in the REF one), and a fourth CTA hides their tile
// barriers better (10 MHz recon: unmasked 168.0 -> 162.4 ms, REF windows 168.3 -> 161.2);
// the geometric one needs 80 (at 64 it spills in its term loops: 163 -> 177 ms).
template <int RM>
constexpr int rec_min_blocks() { return RM != RM_GEO ? VISS_REC_MINB + 1 : VISS_REC_MINB; }

template <int RM, bool COMP, int Q>
__global__ void __launch_bounds__(REC_THREADS, rec_min_blocks<RM>()) recon_fast_kernel(const ReconParams p) {
  __shared__ RecSmem<RM, COMP, Q> sm;
  __shared__ int s_item;
  const bool frac = __ldg(p.flags + FLAG_FRAC) != 0;
  for (;;) {
    __syncthreads();  // everyone has read the previous item
    if (threadIdx.x == 0) s_item = atomicAdd(p.flags + FLAG_REC_COUNTER, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= p.nitems) break;
    const int seg = item / p.npb;
    const int64_t pb = item - (int64_t)seg * p.npb;
    const int ch = p.seg_ch[seg], slot = p.seg_slot[seg];
    const bool direct = slot < 0;
    float2* out = direct ? p.out + (int64_t)ch * p.J : p.partial + (int64_t)slot * p.J;
    if (frac) recon_body<RM, true, COMP, Q>(p, sm, pb, p.seg_lo[seg], p.seg_hi[seg], out, p.ch_norm[ch], direct);
    else recon_body<RM, false, COMP, Q>(p, sm, pb, p.seg_lo[seg], p.seg_hi[seg], out, p.ch_norm[ch], direct);
  }
}

template <int RM, bool COMP, int Q>
static void launch_tile(const ReconParams& p, int ctas_per_sm, cudaStream_t st) {
  const int g = persistent_grid(recon_fast_kernel<RM, COMP, Q>, REC_THREADS, ctas_per_sm, p.nitems);
  recon_fast_kernel<RM, COMP, Q><<<g, REC_THREADS, 0, st>>>(p);
}

// Row tiles of 2 REC_Q visibilities (the default; 4 REC_Q for the geometric mask without
// compensation), REC_Q or REC_Q / 2 (tuning).  Longer geometric tiles meet at the block
// barrier half as often and drop more hidden rows per load (10 MHz recon 163.0 -> 161.1
// ms; the satellite cache is halved to keep three CTAs per SM: 37 snapshots of 8
// satellites fit).  The compensated instance keeps 2 REC_Q: at 4 REC_Q its shared
// memory would leave two CTAs per SM.
template <int RM>
static void launch_rm(const ReconParams& p, int ctas_per_sm, bool comp, cudaStream_t st) {
  constexpr int QD = RM == RM_GEO ? 4 * REC_Q : 2 * REC_Q;
  if (p.row_tile == 1) {
    if (comp) launch_tile<RM, true, REC_Q / 2>(p, ctas_per_sm, st);
    else launch_tile<RM, false, REC_Q / 2>(p, ctas_per_sm, st);
  } else if (p.row_tile == 2) {
    if (comp) launch_tile<RM, true, 2 * REC_Q>(p, ctas_per_sm, st);
    else launch_tile<RM, false, QD>(p, ctas_per_sm, st);
  } else {
    if (comp) launch_tile<RM, true, REC_Q>(p, ctas_per_sm, st);
    else launch_tile<RM, false, REC_Q>(p, ctas_per_sm, st);
  }
}

int launch_recon_fast(const ReconParams& p, int ctas_per_sm, bool comp, cudaStream_t st) {
  if (p.nitems <= 0) return VISS_OK;
  switch (p.recon_mask) {
    case VISS_RECON_MASK_NONE: launch_rm<RM_NONE>(p, ctas_per_sm, comp, st); break;
    case VISS_RECON_MASK_REF: launch_rm<RM_REF>(p, ctas_per_sm, comp, st); break;
    case VISS_RECON_MASK_GEOMETRIC: launch_rm<RM_GEO>(p, ctas_per_sm, comp, st); break;
    default: return fail(VISS_ERR_INVALID, "unknown recon mask");
  }
  VISS_LAUNCH_CHECK("recon_fast_kernel");
  return VISS_OK;
}

// F[c] = norm_c * -(sum of channel c's partial slots), slots summed in order in double.
__global__ void recon_reduce_kernel(const RecReduceParams p) {
  const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (pos >= p.J || p.nslot[c] == 0) return;
  double sr = 0.0, si = 0.0;
  for (int s = 0; s < p.nslot[c]; ++s) {
    const float2 v = p.partial[(int64_t)(p.slot0[c] + s) * p.J + pos];
    sr += v.x;
    si += v.y;
  }
  const int64_t j = p.perm ? (int64_t)p.perm[pos] : pos;
  const double norm = p.norm[c];
  p.out[(int64_t)c * p.J + j] = make_float2((float)(-sr * norm), (float)(-si * norm));
}

int launch_recon_reduce(const RecReduceParams& p, cudaStream_t st) {
  if (p.J <= 0 || p.nch <= 0) return VISS_OK;
  recon_reduce_kernel<<<dim3((unsigned)((p.J + 255) / 256), (unsigned)p.nch), 256, 0, st>>>(p);
  VISS_LAUNCH_CHECK("recon_reduce_kernel");
  return VISS_OK;
}

// ---------------------------------------------------------------- plain
// The reference's plain recon, restated: one thread per pixel, FP32 phase
//   ph = u*l/d + v*m/d + w*(n + n_offset)/d,  x = +2 pi ph   (vissGen10M_shade.cu:169)
// precise sincosf, register accumulator (optim1, :235-271); reference ratio
// mask evaluated per term from r1 = M1/M2, r2 = M3/M4 (:166).
// F64 (the FP64-phase arm of precision sweeps): the phase in FP64, reduced to
// [-1/2, 1/2] turn in FP64, sincosf of the float angle, Kahan sums.
struct PlainRecArgs {
  const float *u, *v, *w, *wgt, *V, *l, *m, *n;
  const float* r1;
  const float* r2;
  const int32_t* snap;
  const int32_t* pair;
  const float* sat_pos;
  const float4* satdir;
  int64_t K, J;
  int nsat;
  int rmask;
  int res;
  float dl, dm, dn;
  float noff;
  double noff64;
  float norm;
  double R;
  float2* out;
  int* flags;  // near-limb count (may be null)
};

template <bool F64>
__global__ void recon_plain_kernel(const PlainRecArgs a) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.J) return;
  const float phiP = floorf((float)(j / a.res));
  const float thetaP = (float)j - phiP * (float)a.res;
  const float lj = a.l[j], mj = a.m[j], nj = a.n[j] + a.noff;
  // FP64-phase arm: l/d, m/d, (n + n_offset)/d in double
  const double ld = (double)a.l[j] / (double)a.dl, md = (double)a.m[j] / (double)a.dm;
  const double nd = ((double)a.n[j] + a.noff64) / (double)a.dn;
  const float p2 = 2.0f * (float)kPi;
  float fr = 0.f, fi = 0.f, cr = 0.f, ci = 0.f;
  for (int64_t k = 0; k < a.K; ++k) {
    if (a.rmask == VISS_RECON_MASK_REF) {
      const float t0 = a.r1[k], p0 = a.r2[k];
      if (fabsf(t0 - thetaP) < t0 && fabsf(p0 - phiP) < p0) continue;
    } else if (a.rmask == VISS_RECON_MASK_GEOMETRIC) {
      const int s = a.snap[k], pr = a.pair[k];
      const int64_t g1 = (int64_t)s * a.nsat + (pr & 0xffff), g2 = (int64_t)s * a.nsat + ((pr >> 16) & 0xffff);
      if (geo_test_plain(a.l[j], a.m[j], a.n[j], a.satdir[g1], a.sat_pos + 3 * g1, a.R, a.flags) ||
          geo_test_plain(a.l[j], a.m[j], a.n[j], a.satdir[g2], a.sat_pos + 3 * g2, a.R, a.flags))
        continue;
    }
    float sn, cs;
    if (F64) {
      const double t = fma((double)a.u[k], ld, fma((double)a.v[k], md, (double)a.w[k] * nd));
      sincosf((float)((t - rint(t)) * (2.0 * kPi)), &sn, &cs);
    } else {
      const float ph = a.u[k] * lj / a.dl + a.v[k] * mj / a.dm + a.w[k] * nj / a.dn;
      sincosf(p2 * ph, &sn, &cs);
    }
    const float wg = a.wgt ? a.wgt[k] : 1.0f;
    const float yr = wg * a.V[2 * k], yi = wg * a.V[2 * k + 1];
    if (F64) {
      kahan_add(fr, cr, yr * cs - yi * sn);
      kahan_add(fi, ci, yr * sn + yi * cs);
    } else {
      fr += yr * cs - yi * sn;
      fi += yr * sn + yi * cs;
    }
  }
  a.out[j] = make_float2(fr * a.norm, fi * a.norm);
}

int launch_recon_plain(const viss_dft_cfg& cfg, const viss_sky& sky, const viss_vis_set& vis,
                       const viss_geometry* geo, const float* V, const float* ratios, const float4* satdir,
                       const float* dlmn, float2* out, cudaStream_t st, int* flags) {
  PlainRecArgs a{};
  a.flags = flags;
  a.satdir = satdir;
  a.u = vis.u; a.v = vis.v; a.w = vis.w; a.wgt = vis.wgt; a.V = V;
  a.l = sky.l; a.m = sky.m; a.n = sky.n;
  a.r1 = ratios; a.r2 = ratios ? ratios + vis.K : nullptr;
  a.snap = vis.snap; a.pair = vis.pair;
  a.sat_pos = geo ? geo->sat_pos : nullptr;
  a.nsat = geo ? geo->nsat : 0;
  a.K = vis.K; a.J = sky.J;
  a.rmask = cfg.recon_mask;
  a.res = cfg.res > 0 ? cfg.res : 1;
  a.dl = dlmn[0]; a.dm = dlmn[1]; a.dn = dlmn[2];
  a.noff = (float)cfg.n_offset;
  a.noff64 = cfg.n_offset;
  a.norm = (float)cfg.norm;
  a.R = cfg.moon_radius_km;
  a.out = out;
  if (a.J <= 0) return VISS_OK;
  if (cfg.precision == VISS_PREC_F64_PHASE) recon_plain_kernel<true><<<(unsigned)((a.J + 255) / 256), 256, 0, st>>>(a);
  else recon_plain_kernel<false><<<(unsigned)((a.J + 255) / 256), 256, 0, st>>>(a);
  VISS_LAUNCH_CHECK("recon_plain_kernel");
  return VISS_OK;
}

}  // namespace viss
