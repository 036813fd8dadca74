// vis_dft.cu -- shaded visibility DFT (replaces visscal, vissGen10M_shade.cu:108-145).
//
// V_k = sum_j C_kj exp(-2 pi i t_kj),  t_kj = s (u_k l_j + v_k m_j + w_k (n_j + n_offset))
//
// Tiled kernel: a work item is VIS_ROWS = 1024 visibilities of one channel (4
// per thread, in registers) against one chunk of the sky, streamed through
// shared memory in tiles of VIS_P (or VIS_P / 2) pixels; every thread reads each pixel record
// as a broadcast.  Per term:
//   3 IMAD (phase mod 1 turn in 32-bit fixed point; exact for integer uvw)
//   [+3 FFMA for fractional uvw] [+3 FFMA compensation]
//   shift/or + 1 FFMA (turns -> angle), __sincosf (2 SFU ops), 2 FFMA (MAC).
// The occlusion predicate is evaluated inline per tile:
//   GEOMETRIC: pixels are classified against a cone bounding the shadow cones
//     of every satellite used by the CTA's rows -- all visible / all occluded /
//     mixed -- and compacted into a fast list (brightness or occluded value,
//     no per-term test) and a mixed list.  Each (mixed pixel, satellite of the
//     block's rows) pair is decided once per tile into shared-memory bits (in
//     double within GEO_EPS of the limb); a term ORs its row's two satellite
//     bits.  Blocks whose rows span too many satellites for the bits test the
//     row's two satellites per term instead.
//   REF_*: per-row window (row range x column range on the fine grid); a warp
//     none of whose 128 windows reaches the tile runs the unmasked loop.
// Pixel chunks give partial sums, reduced in a fixed order.
#include "viss_internal.cuh"

namespace viss {

template <bool FRAC, bool COMP>
__device__ __forceinline__ void vis_term(const int4& a, const int4& b, const float4& lo, float c, int U,
                                         int V, int W, float FU, float FV, float FW, int bias, float UF, float VF,
                                         float WF, float& ar, float& ai) {
  const uint32_t q = (uint32_t)U * (uint32_t)a.x + (uint32_t)V * (uint32_t)a.y + (uint32_t)W * (uint32_t)a.z +
                     (uint32_t)bias;
  float x;
  if (FRAC || COMP) {
    // fractional uvw [and the pixel fixed-point rounding], in FP32 radians (the row
    // coefficients carry the 2 pi), summed onto the angle's constant
    float e = KM3PI;
    if (FRAC) e = fmaf(FU, __int_as_float(b.x), fmaf(FV, __int_as_float(b.y), fmaf(FW, __int_as_float(b.z), e)));
    if (COMP) e = fmaf(UF, lo.x, fmaf(VF, lo.y, fmaf(WF, lo.z, e)));
    x = turns_to_angle(q, e);
  } else {
    x = turns_to_angle(q, KM3PI);
  }
  float sn, cs;
  __sincosf(x, &sn, &cs);
  ar = fmaf(c, cs, ar);
  ai = fmaf(c, sn, ai);
}

// Exact decision near the limb (rare): kept out of line so its double-precision
// registers do not weigh on the hot loops.
__device__ __noinline__ bool geo_exact_at(const VisParams& p, int j, int gidx) {
  count_limb(p.flags);
  return geo_occluded_exact(p.l[j], p.m[j], p.n[j], p.sat_pos + 3 * (int64_t)gidx, p.R);
}

// fast geometric test against one satellite: s_hat . p_hat + cos(alpha) < 0,
// re-decided exactly near the limb.
__device__ __forceinline__ bool geo_test(const float4& g, const float4& d, int gidx, const VisParams& p) {
  const float e = fmaf(g.x, d.x, fmaf(g.y, d.y, fmaf(g.z, d.z, d.w)));
  if (fabsf(e) >= GEO_EPS) return e < 0.f;
  return geo_exact_at(p, __float_as_int(g.w), gidx);
}

__device__ __noinline__ bool ref_hit_general(int4 wv, int64_t j, int res);

// REF window membership of fine pixel (q, r) / index j for window {lo_a, lo_b, M1, M2}.
__device__ __forceinline__ bool ref_hit(const int4& wv, int q, int r, int64_t j, int res) {
  if (wv.x > wv.y) return false;
  if (wv.z + 1 >= 0 && wv.w <= res) return q >= wv.x && q <= wv.y && r > wv.z && r < wv.w;
  return ref_hit_general(wv, j, res);
}

// windows whose column range is not inside one row
__device__ __noinline__ bool ref_hit_general(int4 wv, int64_t j, int res) {
  // exists lo in [lo_a, lo_b] with lo*res + M1 + 1 <= j < lo*res + M2
  const int64_t hi_num = j - wv.z - 1, lo_num = j - wv.w + 1;
  int64_t lo_max = hi_num >= 0 ? hi_num / res : -((-hi_num + res - 1) / res);     // floor
  int64_t lo_min = lo_num >= 0 ? (lo_num + res - 1) / res : -((-lo_num) / res);   // ceil
  if (lo_min < wv.x) lo_min = wv.x;
  if (lo_max > wv.y) lo_max = wv.y;
  return lo_min <= lo_max;
}

// Fine->coarse map: pixel j's value for window wv, exactly as the reference's
// member loop (mean over its fine members, the occluded value inside the window).
__device__ __noinline__ float ref_members_value(const FineMapDev& m, int4 wv, int64_t j, int res, float occ) {
  const int2 mm = m.mem[j];
  double sum = 0.0;
  for (int c = 0; c < mm.y; ++c) {
    const int i = m.members[mm.x + c];
    if (i < 0) {  // rejected index (flagged in the prep)
      sum = nan("");
      continue;
    }
    float ff = m.FF[i];
    if (m.trunc) ff = (float)(int)ff;
    bool hit = false;
    if (wv.x <= wv.y) {
      if (wv.z + 1 >= 0 && wv.w <= res) {
        const int q = i / res, r = i - q * res;
        hit = q >= wv.x && q <= wv.y && r > wv.z && r < wv.w;
      } else {
        hit = ref_hit_general(wv, i, res);
      }
    }
    sum += hit ? (double)occ : (double)ff;
  }
  return (float)(sum / (double)mm.y);  // 0/0 = NaN for an empty pixel, as the reference
}

// Fine->coarse map: the pixel's bounding box of members decides most terms
// (disjoint from the window: base brightness c0; inside it: occ); the rest
// take the exact member loop.
__device__ __forceinline__ float ref_map_value(const FineMapDev& m, const int4& wv, const int4& bx, float c0, float occ,
                                               int64_t j, int res) {
  if (wv.x > wv.y) return c0;
  if (wv.z + 1 >= 0 && wv.w <= res) {
    if (bx.y < wv.x || bx.x > wv.y || bx.w <= wv.z || bx.z >= wv.w) return c0;
    if (bx.x >= wv.x && bx.y <= wv.y && bx.z > wv.z && bx.w < wv.w) return occ;
  }
  return ref_members_value(m, wv, j, res, occ);
}

template <int MASK, bool COMP, int P>
struct VisSmem {
  static constexpr bool GEO = MASK == VISS_MASK_GEOMETRIC;
  static constexpr bool REF = MASK == VISS_MASK_REF_QUIRK || MASK == VISS_MASK_REF_INTENDED;
  int4 p0[P];
  int4 p1[P];
  float4 lo[COMP ? P : 1];
  float4 geo[GEO ? P : 1];
  int2 qr[REF ? P : 1];
  int4 win[REF ? VIS_ROWS : 1];   // the block's REF windows, read in masked tiles only
  int wcnt[VIS_THREADS / 32][2];
  float4 acc[VIS_ROWS];           // running totals (re, im) and their Kahan compensation per visibility
  uint32_t sbits[GEO ? VIS_SAT_WORDS : 1];  // [satellite][word]: bit b = mixed pixel 32*word + b occluded
};

template <int MASK, bool FRAC, bool COMP, int P>
__device__ __forceinline__ void vis_body(const VisParams& p, VisSmem<MASK, COMP, P>& sm, int64_t rb, int split, int ch,
                                         int64_t rb_first, int64_t row_first, int64_t nvalid) {
  constexpr bool GEO = MASK == VISS_MASK_GEOMETRIC;
  constexpr bool REF = MASK == VISS_MASK_REF_QUIRK || MASK == VISS_MASK_REF_INTENDED;
  int4* const s_p0 = sm.p0;
  int4* const s_p1 = sm.p1;
  float4* const s_lo = sm.lo;
  float4* const s_geo = sm.geo;
  int2* const s_qr = sm.qr;
  auto& s_wcnt = sm.wcnt;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t row0 = rb * VIS_ROWS;                   // padded row of this rowblock
  const int64_t local0 = (rb - rb_first) * VIS_ROWS;    // its first row within the channel
  const float* bright = p.bright ? p.bright + (int64_t)ch * p.J : nullptr;

  // Registers per visibility: fixed-point U,V,W [+ fractional F] [+ float U for
  // the compensation] and the two accumulators.  Satellite indices (geometric)
  // and windows (REF) are fetched only on the masked paths.
  int U[VIS_TK], V[VIS_TK], W[VIS_TK], BI[VIS_TK];
  float FU[VIS_TK], FV[VIS_TK], FW[VIS_TK];
  float UF[VIS_TK], VF[VIS_TK], WF[VIS_TK];
  float tr[VIS_TK], ti[VIS_TK];   // this tile's sums; running totals live in sm.acc
  bool any_win = false;
#pragma unroll
  for (int i = 0; i < VIS_TK; ++i) {
    const int64_t k = row0 + tid + i * VIS_THREADS;  // rows are padded to a whole block
    const int4 r0 = p.rows0[k];
    U[i] = r0.x; V[i] = r0.y; W[i] = r0.z; BI[i] = r0.w;
    FU[i] = FV[i] = FW[i] = 0.f;
    if (FRAC) {
      const float4 r1 = p.rows1[k];
      FU[i] = r1.x; FV[i] = r1.y; FW[i] = r1.z;
    }
    UF[i] = VF[i] = WF[i] = 0.f;
    if (COMP) {
      const float4 f = p.rowsf[k];
      UF[i] = f.x; VF[i] = f.y; WF[i] = f.z;
    }
    if (REF) {
      const int4 wv = p.win[k];
      sm.win[tid + i * VIS_THREADS] = wv;
      any_win |= wv.x <= wv.y && wv.z + 1 < wv.w;
    }
    sm.acc[tid + i * VIS_THREADS] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  float4 cone0 = make_float4(0.f, 0.f, 0.f, 2.f), cone1 = make_float4(-2.f, 0.f, 0.f, 0.f);
  if (GEO) {
    cone0 = p.cones[2 * rb];
    cone1 = p.cones[2 * rb + 1];
  }
  const int g_lo = __float_as_int(cone1.y), g_span = __float_as_int(cone1.z);  // the rows' satellites
  const float occ_val = p.occ_val;

  const int64_t jb = (int64_t)split * p.jchunk;
  int64_t je = jb + p.jchunk;
  if (je > p.J) je = p.J;

  for (int64_t tile = jb; tile < je; tile += P) {
    const int np = (int)((je - tile) < P ? (je - tile) : P);
    __syncthreads();  // previous tile fully consumed
#pragma unroll
    for (int i = 0; i < VIS_TK; ++i) tr[i] = ti[i] = 0.f;
    int nfast = np, nmix = 0;
    bool masked_tile = false;
    if (GEO) {
      // pass 1: classify against the block's bounding cone (only the class is
      // kept across the barrier); pass 2: re-read the records (L2) and place them.
      constexpr int Q = P / VIS_THREADS;
      unsigned cls = 0;  // 2 bits per slot: 1 fast, 2 mixed
#pragma unroll
      for (int qq = 0; qq < Q; ++qq) {
        const int i = tid + qq * VIS_THREADS;
        if (i < np) {
          const float4 g = p.pgeo[tile + i];
          const float d = fmaf(g.x, cone0.x, fmaf(g.y, cone0.y, g.z * cone0.z));
          if (d > cone0.w) cls |= (occ_val != 0.f ? 1u : 0u) << (2 * qq);  // occluded for every row
          else if (d < cone1.x) cls |= 1u << (2 * qq);                      // visible for every row
          else cls |= 2u << (2 * qq);
        }
      }
      unsigned bF[Q], bM[Q];
      int cf = 0, cm = 0;
#pragma unroll
      for (int qq = 0; qq < Q; ++qq) {
        bF[qq] = __ballot_sync(0xffffffffu, ((cls >> (2 * qq)) & 3u) == 1u);
        bM[qq] = __ballot_sync(0xffffffffu, ((cls >> (2 * qq)) & 3u) == 2u);
        cf += __popc(bF[qq]);
        cm += __popc(bM[qq]);
      }
      if (lane == 0) { s_wcnt[warp][0] = cf; s_wcnt[warp][1] = cm; }
      __syncthreads();
      int offF = 0, offM = 0, totF = 0, totM = 0;
#pragma unroll
      for (int w2 = 0; w2 < VIS_THREADS / 32; ++w2) {
        const int f = s_wcnt[w2][0], m = s_wcnt[w2][1];
        if (w2 < warp) { offF += f; offM += m; }
        totF += f; totM += m;
      }
      const unsigned lt = (1u << lane) - 1u;
#pragma unroll
      for (int qq = 0; qq < Q; ++qq) {
        const unsigned c = (cls >> (2 * qq)) & 3u;
        if (c) {
          const int64_t j = tile + tid + qq * VIS_THREADS;
          int4 a = p.pix0[j];
          if (bright) a.w = __float_as_int(bright[j]);
          const float4 g = p.pgeo[j];
          const float d = fmaf(g.x, cone0.x, fmaf(g.y, cone0.y, g.z * cone0.z));
          if (c == 1u && d > cone0.w) a.w = __float_as_int(occ_val);
          const int pos = c == 1u ? offF + __popc(bF[qq] & lt) : P - 1 - (offM + __popc(bM[qq] & lt));
          s_p0[pos] = a;
          if (FRAC) s_p1[pos] = p.pix1[j];
          if (COMP) s_lo[pos] = p.plo[j];
          if (c == 2u) s_geo[pos] = g;
        }
        offF += __popc(bF[qq]);
        offM += __popc(bM[qq]);
      }
      nfast = totF;
      nmix = totM;
      __syncthreads();
    } else {
      for (int i = tid; i < np; i += VIS_THREADS) {
        const int64_t j = tile + i;
        int4 a = p.pix0[j];
        if (bright) a.w = __float_as_int(bright[j]);
        s_p0[i] = a;
        if (FRAC) s_p1[i] = p.pix1[j];
        if (COMP) s_lo[i] = p.plo[j];
        if (REF) s_qr[i] = p.pqr[j];
      }
      bool hit = false;
      if (REF && any_win) {
        // bounding fine-index range of each window against [tile, tile + np)
#pragma unroll
        for (int i = 0; i < VIS_TK; ++i) {
          const int4 wv = sm.win[tid + i * VIS_THREADS];
          if (wv.x <= wv.y && wv.z + 1 < wv.w) {
            const int64_t lo_idx = (int64_t)wv.x * p.res + wv.z + 1;
            const int64_t hi_idx = (int64_t)wv.y * p.res + wv.w - 1;
            int64_t tlo = tile, thi = tile + np - 1;  // fine indices the tile's pixels cover
            if (p.use_map) {
              const int2 tr = p.map.tile_rng[tile / VIS_P];
              tlo = tr.x;
              thi = tr.y;
            } else if (p.ref_rng) {
              const int2 tr = p.ref_rng[tile / VIS_P];
              tlo = tr.x;
              thi = tr.y;
            }
            if (lo_idx <= thi && hi_idx >= tlo) hit = true;
          }
        }
      }
      // per warp: a warp none of whose 128 windows reaches the tile runs the unmasked loop
      __syncthreads();  // the tile's records are in shared memory
      masked_tile = __any_sync(0xffffffffu, hit);
    }

    if (!masked_tile) {
#pragma unroll 2
      for (int pi = 0; pi < nfast; ++pi) {
        const int4 a = s_p0[pi];
        int4 b = make_int4(0, 0, 0, 0);
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f);
        if (FRAC) b = s_p1[pi];
        if (COMP) lo = s_lo[pi];
        const float c = __int_as_float(a.w);
#pragma unroll
        for (int i = 0; i < VIS_TK; ++i)
          vis_term<FRAC, COMP>(a, b, lo, c, U[i], V[i], W[i], FU[i], FV[i], FW[i], BI[i], UF[i], VF[i], WF[i],
                               tr[i], ti[i]);
      }
    } else if (REF) {
      for (int pi = 0; pi < np; ++pi) {
        const int4 a = s_p0[pi];
        int4 b = make_int4(0, 0, 0, 0);
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f);
        if (FRAC) b = s_p1[pi];
        if (COMP) lo = s_lo[pi];
        const int2 qr = s_qr[pi];
        const float c0 = __int_as_float(a.w);
        int4 bx = make_int4(0, 0, 0, 0);
        if (p.use_map) bx = __ldg(p.map.box + tile + pi);
#pragma unroll
        for (int i = 0; i < VIS_TK; ++i) {
          const int4 wv = sm.win[tid + i * VIS_THREADS];
          const float c = p.use_map ? ref_map_value(p.map, wv, bx, c0, occ_val, tile + pi, p.res)
                                    : (ref_hit(wv, qr.x, qr.y, (int64_t)qr.x * p.res + qr.y, p.res) ? occ_val : c0);
          vis_term<FRAC, COMP>(a, b, lo, c, U[i], V[i], W[i], FU[i], FV[i], FW[i], BI[i], UF[i], VF[i], WF[i],
                               tr[i], ti[i]);
        }
      }
    }
    const int nwd = (nmix + 31) >> 5;
    if (GEO && nmix > 0 && g_span > 0 && g_span <= VIS_ROWS && g_span * nwd <= VIS_SAT_WORDS) {
      // Each (mixed pixel, satellite) decided once for the tile: span x nmix
      // tests instead of up to 2 x VIS_ROWS x nmix.  A warp per satellite, a
      // ballot per 32-pixel word.
      for (int s = warp; s < g_span; s += VIS_THREADS / 32) {
        const float4 d = __ldg(p.satdir + g_lo + s);
        for (int wd = 0; wd < nwd; ++wd) {
          const int mi = 32 * wd + lane;
          const bool occ = mi < nmix && geo_test(s_geo[P - 1 - mi], d, g_lo + s, p);
          const unsigned bits = __ballot_sync(0xffffffffu, occ);
          if (lane == 0) sm.sbits[s * nwd + wd] = bits;
        }
      }
      // word offsets of each row's two satellites (padding rows, outside the
      // block's range, read satellite g_lo; their sums are never stored)
      int so[VIS_TK];
#pragma unroll
      for (int i = 0; i < VIS_TK; ++i) {
        const int pk = __ldg(p.rowsat + row0 + tid + i * VIS_THREADS);
        int sa = sat_gm(pk) - g_lo, sb = sat_gn(pk) - g_lo;
        if ((unsigned)sa >= (unsigned)g_span) sa = 0;
        if ((unsigned)sb >= (unsigned)g_span) sb = 0;
        so[i] = sa * nwd | (sb * nwd) << 16;
      }
      __syncthreads();
      for (int wd = 0; wd < nwd; ++wd) {
        unsigned ob[VIS_TK];  // occluded from either satellite, 32 pixels per word
#pragma unroll
        for (int i = 0; i < VIS_TK; ++i) ob[i] = sm.sbits[(so[i] & 0xffff) + wd] | sm.sbits[(so[i] >> 16) + wd];
        const int nb = min(32, nmix - 32 * wd);
        for (int bi = 0; bi < nb; ++bi) {
          const int pi = P - 1 - (32 * wd + bi);
          const int4 a = s_p0[pi];
          int4 b = make_int4(0, 0, 0, 0);
          float4 lo = make_float4(0.f, 0.f, 0.f, 0.f);
          if (FRAC) b = s_p1[pi];
          if (COMP) lo = s_lo[pi];
          const float c0 = __int_as_float(a.w);
#pragma unroll
          for (int i = 0; i < VIS_TK; ++i) {
            const float c = (ob[i] >> bi) & 1u ? occ_val : c0;
            if (c != 0.f)
              vis_term<FRAC, COMP>(a, b, lo, c, U[i], V[i], W[i], FU[i], FV[i], FW[i], BI[i], UF[i], VF[i], WF[i],
                                   tr[i], ti[i]);
          }
        }
      }
    } else if (GEO && nmix > 0) {
      int gm[VIS_TK], gn[VIS_TK];
#pragma unroll
      for (int i = 0; i < VIS_TK; ++i) {
        const int64_t k = row0 + tid + i * VIS_THREADS;
        const int pk = __ldg(p.rowsat + k);
        gm[i] = sat_gm(pk);
        gn[i] = sat_gn(pk);
      }
      for (int mi = 0; mi < nmix; ++mi) {
        const int pi = P - 1 - mi;
        const int4 a = s_p0[pi];
        int4 b = make_int4(0, 0, 0, 0);
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f);
        if (FRAC) b = s_p1[pi];
        if (COMP) lo = s_lo[pi];
        const float4 g = s_geo[pi];
        const float c0 = __int_as_float(a.w);
#pragma unroll
        for (int i = 0; i < VIS_TK; ++i) {
          // the rows' satellite directions stay in L1 for the whole mixed list
          const bool occ = geo_test(g, __ldg(p.satdir + gm[i]), gm[i], p) || geo_test(g, __ldg(p.satdir + gn[i]), gn[i], p);
          const float c = occ ? occ_val : c0;
          if (c != 0.f)
            vis_term<FRAC, COMP>(a, b, lo, c, U[i], V[i], W[i], FU[i], FV[i], FW[i], BI[i], UF[i], VF[i], WF[i],
                                 tr[i], ti[i]);
        }
      }
    }
#pragma unroll
    for (int i = 0; i < VIS_TK; ++i) {
      float4 t = sm.acc[tid + i * VIS_THREADS];  // owned by this thread alone
      kahan_add(t.x, t.z, tr[i]);
      kahan_add(t.y, t.w, ti[i]);
      sm.acc[tid + i * VIS_THREADS] = t;
    }
  }

  // V = -ar + i ai  (the angle carried an extra half turn)
#pragma unroll
  for (int i = 0; i < VIS_TK; ++i) {
    const int64_t kl = local0 + tid + i * VIS_THREADS;
    const float4 t = sm.acc[tid + i * VIS_THREADS];
    const float ar = t.x, ai = t.y;
    if (kl < nvalid) {
      const int64_t k = row_first + kl;
      if (p.nsplit == 1) p.out[k] = make_float2(-ar, ai);
      else p.out[(int64_t)split * p.K + k] = make_float2(ar, ai);
    }
  }
}

// Integer-valued uvw (the reference's ceil(), MIncline:156-158) need no
// fractional term; the row prep sets flags[0] when any uvw is fractional and
// the kernel picks its loop from that flag (uniform branch, no host sync).
//
// Persistent: grid = resident CTAs; each CTA takes the next work item (rowblock,
// pixel chunk) from an atomic counter until none are left, so uneven items
// (channels, occluded fractions) balance without a wave tail.  The counter is
// reset by the host before the launch; no CTA ever waits on another.
template <int MASK, bool COMP, int P>
__global__ void __launch_bounds__(VIS_THREADS, VISS_VIS_MINB) vis_fast_kernel(const VisParams p) {
  __shared__ VisSmem<MASK, COMP, P> sm;
  __shared__ int s_item;
  const bool frac = __ldg(p.flags + FLAG_FRAC) != 0;
  for (;;) {
    __syncthreads();  // everyone has read the previous item
    if (threadIdx.x == 0) s_item = atomicAdd(p.flags + FLAG_VIS_COUNTER, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= p.nitems) break;
    const int64_t rb = item / p.nsplit;
    const int split = item - (int)(rb * p.nsplit);
    int ch = 0;
    while (ch + 1 < p.ch.nch && rb >= p.ch.rb_off[ch + 1]) ++ch;
    const int64_t nvalid = p.ch.row_off[ch + 1] - p.ch.row_off[ch];
    if (frac) vis_body<MASK, true, COMP, P>(p, sm, rb, split, ch, p.ch.rb_off[ch], p.ch.row_off[ch], nvalid);
    else vis_body<MASK, false, COMP, P>(p, sm, rb, split, ch, p.ch.rb_off[ch], p.ch.row_off[ch], nvalid);
  }
}

// Persistent grid: resident CTAs of this kernel (capped by ctas_per_sm) on every SM.
template <int MASK, bool COMP, int P>
static void launch_tile(const VisParams& p, int ctas_per_sm, cudaStream_t st) {
  const int g = persistent_grid(vis_fast_kernel<MASK, COMP, P>, VIS_THREADS, ctas_per_sm, p.nitems);
  vis_fast_kernel<MASK, COMP, P><<<g, VIS_THREADS, 0, st>>>(p);
}

// Sky tile of VIS_P pixels, or VIS_P / 2 (tuning): smaller tiles halve the shared
// memory per block and the granularity of the occlusion compaction.
template <int MASK>
static void launch_mask(const VisParams& p, int ctas_per_sm, bool comp, cudaStream_t st) {
  if (p.small_tile) {
    if (comp) launch_tile<MASK, true, VIS_P / 2>(p, ctas_per_sm, st);
    else launch_tile<MASK, false, VIS_P / 2>(p, ctas_per_sm, st);
  } else {
    if (comp) launch_tile<MASK, true, VIS_P>(p, ctas_per_sm, st);
    else launch_tile<MASK, false, VIS_P>(p, ctas_per_sm, st);
  }
}

int launch_vis_fast(const VisParams& p, int ctas_per_sm, bool comp, cudaStream_t st) {
  if (p.nitems <= 0) return VISS_OK;
  switch (p.mask) {
    case VISS_MASK_NONE: launch_mask<VISS_MASK_NONE>(p, ctas_per_sm, comp, st); break;
    case VISS_MASK_REF_QUIRK: launch_mask<VISS_MASK_REF_QUIRK>(p, ctas_per_sm, comp, st); break;
    case VISS_MASK_REF_INTENDED: launch_mask<VISS_MASK_REF_INTENDED>(p, ctas_per_sm, comp, st); break;
    case VISS_MASK_GEOMETRIC: launch_mask<VISS_MASK_GEOMETRIC>(p, ctas_per_sm, comp, st); break;
    default: return fail(VISS_ERR_INVALID, "unknown mask mode");
  }
  VISS_LAUNCH_CHECK("vis_fast_kernel");
  return VISS_OK;
}

__global__ void vis_reduce_kernel(const float2* __restrict__ part, int nsplit, int64_t K, float2* out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  double sr = 0.0, si = 0.0;
  for (int s = 0; s < nsplit; ++s) {
    const float2 v = part[(int64_t)s * K + k];
    sr += v.x;
    si += v.y;
  }
  out[k] = make_float2((float)-sr, (float)si);
}

int launch_vis_reduce(const float2* partial, int nsplit, int64_t K, float2* out, cudaStream_t st) {
  if (K <= 0) return VISS_OK;
  vis_reduce_kernel<<<(unsigned)((K + 255) / 256), 256, 0, st>>>(partial, nsplit, K, out);
  VISS_LAUNCH_CHECK("vis_reduce_kernel");
  return VISS_OK;
}

// ---------------------------------------------------------------- plain
// The reference's plain method, restated: one thread per visibility, the sky
// read from global memory, FP32 phase
//   ph = u*l/d + v*m/d + w*(n-1)/d,  x = -2 pi ph  (vissGen10M_shade.cu:137-138)
// with precise sincosf, accumulated in registers (optim1, :154-205), times the
// trailing exp(-2 pi i (1 + n_offset) w / d) (:143).  Masks as in the tiled kernel.
// F64 (the FP64-phase arm of precision sweeps): the whole phase
// (u l + v m + w (n + n_offset)) / d in FP64 (the trailing factor folded in),
// reduced to [-1/2, 1/2] turn in FP64, sincosf of the float angle, Kahan sums.
struct PlainVisArgs {
  const float *u, *v, *w, *l, *m, *n, *bright;
  const int32_t* shade;
  const int32_t* snap;
  const int32_t* pair;
  const float* sat_pos;
  const float4* satdir;
  int64_t K, J;
  int nsat;
  int mask;
  int res;
  int trunc;
  float occ;
  float dl, dm, dn;
  float trail;  // 1 + n_offset
  double R;
  double noff;  // n_offset (FP64-phase arm)
  float2* out;
  int* flags;  // near-limb count (may be null)
  const int32_t* widx;  // REF windows test widx[j] (NULL: j)
  // non-identity fine->coarse map: FF, NXq (float or int), countLoc
  const float* FF;
  const float* NXq_f;
  const int32_t* NXq_i;
  const int32_t* countLoc;
  int64_t X;
};

template <bool F64>
__global__ void vis_plain_kernel(const PlainVisArgs a) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.K) return;
  const float uk = a.u[k], vk = a.v[k], wk = a.w[k];
  // FP64-phase arm: u/d, v/d, w/d in double
  const double ud = (double)uk / (double)a.dl, vd = (double)vk / (double)a.dm, wd = (double)wk / (double)a.dn;
  float cr = 0.f, ci = 0.f;  // Kahan compensations (FP64-phase arm)
  int4 wv = make_int4(1, 0, 0, 0);
  if ((a.mask == VISS_MASK_REF_QUIRK || a.mask == VISS_MASK_REF_INTENDED) && a.shade) {
    const int M1 = a.shade[4 * k], M2 = a.shade[4 * k + 1], M3 = a.shade[4 * k + 2], M4 = a.shade[4 * k + 3];
    if (a.mask == VISS_MASK_REF_QUIRK) { if (M3 <= 0 && M4 >= 0) wv = make_int4(0, M4, M1, M2); }
    else if (M3 <= M4) wv = make_int4(M3, M4, M1, M2);
  }
  const bool geo = a.mask == VISS_MASK_GEOMETRIC;
  float4 d1 = make_float4(0.f, 0.f, 0.f, 0.f), d2 = d1;
  const float *p1 = nullptr, *p2 = nullptr;
  if (geo) {
    const int s = a.snap[k], pr = a.pair[k];
    const int64_t g1 = (int64_t)s * a.nsat + (pr & 0xffff), g2 = (int64_t)s * a.nsat + ((pr >> 16) & 0xffff);
    d1 = a.satdir[g1]; d2 = a.satdir[g2];
    p1 = a.sat_pos + 3 * g1; p2 = a.sat_pos + 3 * g2;
  }
  const float m2pi = -2.0f * (float)kPi;
  float ar = 0.f, ai = 0.f;
  int64_t start = 0;
  for (int64_t j = 0; j < a.J; ++j) {
    float c;
    if (a.countLoc) {
      // vissGen10M_shade.cu:123-135: C = mean over the pixel's fine members of FF, 240 inside the window
      const int cnt = a.countLoc[j];
      float sum = 0.f;
      for (int e = 0; e < cnt; ++e) {
        const int64_t loc = a.NXq_f ? (int64_t)a.NXq_f[start + e] : (int64_t)a.NXq_i[start + e];
        if (loc < 0 || loc >= a.X || start + e >= a.X) {  // outside the fine grid: no read, NaN
          sum = nanf("");
          continue;
        }
        float ff = a.FF[loc];
        if (a.trunc) ff = (float)(int)ff;
        if (wv.x <= wv.y && ref_hit_general(wv, loc, a.res)) ff = a.occ;
        sum += ff;
      }
      start += cnt;
      c = sum / (float)cnt;
    } else {
      c = a.bright[j];
      if (a.trunc) c = (float)(int)c;
    }
    if (a.countLoc) {
      if (geo) {
        const float sx = a.l[j], sy = a.m[j], sz = a.n[j];
        if (geo_test_plain(sx, sy, sz, d1, p1, a.R, a.flags) || geo_test_plain(sx, sy, sz, d2, p2, a.R, a.flags))
          c = a.occ;
      }
    } else if (wv.x <= wv.y) {
      const int64_t i = a.widx ? (int64_t)a.widx[j] : j;  // the fine index the window tests
      int64_t q = i / a.res, r = i - q * a.res;
      if (r < 0) { r += a.res; --q; }
      if (ref_hit(wv, (int)q, (int)r, i, a.res)) c = a.occ;
    } else if (geo) {
      const float sx = a.l[j], sy = a.m[j], sz = a.n[j];
      if (geo_test_plain(sx, sy, sz, d1, p1, a.R, a.flags) || geo_test_plain(sx, sy, sz, d2, p2, a.R, a.flags))
        c = a.occ;
    }
    float sn, cs;
    if (F64) {
      const double t = fma(ud, (double)a.l[j], fma(vd, (double)a.m[j], wd * ((double)a.n[j] + a.noff)));
      sincosf((float)((t - rint(t)) * (-2.0 * kPi)), &sn, &cs);
      kahan_add(ar, cr, c * cs);
      kahan_add(ai, ci, c * sn);
      continue;
    }
    const float ph = uk * a.l[j] / a.dl + vk * a.m[j] / a.dm + wk * (a.n[j] - 1.0f) / a.dn;
    sincosf(m2pi * ph, &sn, &cs);
    ar = fmaf(c, cs, ar);
    ai = fmaf(c, sn, ai);
  }
  if (F64) {  // the trailing factor is in the phase
    a.out[k] = make_float2(ar, ai);
    return;
  }
  float sn, cs;
  sincosf(m2pi * (a.trail * wk / a.dn), &sn, &cs);
  a.out[k] = make_float2(ar * cs - ai * sn, ar * sn + ai * cs);
}

int launch_vis_plain(const viss_dft_cfg& cfg, const viss_sky& sky, const viss_vis_set& vis,
                     const viss_geometry* geo, const float4* satdir, const float* dlmn, float2* out, cudaStream_t st,
                     const viss_fine_map* map, int* flags, const int32_t* widx) {
  PlainVisArgs a{};
  a.flags = flags;
  a.widx = widx;
  if (map) {
    a.FF = map->FF; a.NXq_f = map->NXq_f; a.NXq_i = map->NXq_i; a.countLoc = map->countLoc; a.X = map->X;
  }
  a.satdir = satdir;
  a.u = vis.u; a.v = vis.v; a.w = vis.w;
  a.l = sky.l; a.m = sky.m; a.n = sky.n; a.bright = sky.bright;
  a.shade = vis.shade; a.snap = vis.snap; a.pair = vis.pair;
  a.sat_pos = geo ? geo->sat_pos : nullptr;
  a.nsat = geo ? geo->nsat : 0;
  a.K = vis.K; a.J = sky.J;
  a.mask = cfg.mask_mode; a.res = cfg.res > 0 ? cfg.res : 1; a.trunc = cfg.trunc_brightness;
  a.occ = cfg.occluded_value;
  a.dl = dlmn[0]; a.dm = dlmn[1]; a.dn = dlmn[2];
  a.trail = (float)(1.0 + cfg.n_offset);
  a.noff = cfg.n_offset;
  a.R = cfg.moon_radius_km;
  a.out = out;
  if (a.K <= 0) return VISS_OK;
  if (cfg.precision == VISS_PREC_F64_PHASE) vis_plain_kernel<true><<<(unsigned)((a.K + 255) / 256), 256, 0, st>>>(a);
  else vis_plain_kernel<false><<<(unsigned)((a.K + 255) / 256), 256, 0, st>>>(a);
  VISS_LAUNCH_CHECK("vis_plain_kernel");
  return VISS_OK;
}

}  // namespace viss
