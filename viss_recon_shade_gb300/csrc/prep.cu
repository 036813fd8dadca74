// prep.cu -- per-pass preparation kernels: fixed-point pixel and visibility
// records, satellite directions and occlusion cones.  All O(J + K + S*nsat);
// the O(K*J) work is in vis_dft.cu and recon.cu.
#include <cfloat>

#include "viss_internal.cuh"

namespace viss {

// ------------------------------------------------------------- pixels
// Pixel j: phase coordinates x = s*l, y = s*m, z = s*(n + n_offset) in turns per
// wavelength, evaluated in double from the float inputs.
// Records are written at position `pos`; with a permutation the pixel at pos
// is perm[pos] (records keep the original index in rec1.w / geo.w).
__global__ void prep_pixels_kernel(PixPrepArgs a) {
  const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pos >= a.Jpad) return;
  if (pos >= a.J) {
    a.rec0[pos] = make_int4(0, 0, 0, 0);
    if (a.rec1) a.rec1[pos] = make_int4(0, 0, 0, (int)pos);
    if (a.lo) a.lo[pos] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.geo) a.geo[pos] = make_float4(0.f, 0.f, 0.f, __int_as_float((int)pos));
    if (a.qr) a.qr[pos] = make_int2(-1, -1);
    return;
  }
  const int64_t j = a.perm ? (int64_t)a.perm[pos] : pos;
  const double x = a.sl * (double)a.l[j];
  const double y = a.sm * (double)a.m[j];
  const double z = a.sn * ((double)a.n[j] + a.n_offset);
  float b = 0.f;
  if (a.bright) {
    b = a.bright[j];
    if (a.trunc) b = (float)(int)b;  // int addFF = FF[..] (vissGen10M_shade.cu:128)
  }
  const uint32_t A = fix32(x), B = fix32(y), C = fix32(z);
  a.rec0[pos] = make_int4((int)A, (int)B, (int)C, __float_as_int(b));
  if (a.rec1) {
    // coordinates for the fractional part of uvw; z without the n_offset shift (|s*n| <= 1)
    a.rec1[pos] = make_int4(__float_as_int((float)x), __float_as_int((float)y),
                            __float_as_int((float)(a.sn * (double)a.n[j])), (int)j);
  }
  if (a.lo) {
    const double sc = 4294967296.0;
    const double xa = x * sc, ya = y * sc, za = z * sc;
    a.lo[pos] = make_float4((float)((xa - rint(xa)) / sc), (float)((ya - rint(ya)) / sc),
                          (float)((za - rint(za)) / sc), 0.f);
  }
  if (a.geo) {
    const double gx = a.l[j], gy = a.m[j], gz = a.n[j];
    const double nn = sqrt(gx * gx + gy * gy + gz * gz);
    const double inv = nn > 0 ? 1.0 / nn : 0.0;
    a.geo[pos] = make_float4((float)(gx * inv), (float)(gy * inv), (float)(gz * inv), __int_as_float((int)j));
  }
  if (a.qr) {
    const int res = a.res > 0 ? a.res : 1;
    const int64_t i = a.widx ? (int64_t)a.widx[j] : j;
    int64_t q = i / res, r = i - q * res;
    if (r < 0) { r += res; --q; }  // floor division for negative indices
    a.qr[pos] = make_int2((int)q, (int)r);
  }
}

// {min, max} of widx over each run of VIS_P positions (the fine indices a vis
// tile's REF windows test), {1, 0} for a run past J
__global__ void ref_ranges_kernel(const int32_t* widx, int64_t J, int64_t ntiles, int2* rng) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  int lo = 0x7fffffff, hi = -0x7fffffff - 1;
  for (int64_t j = t * VIS_P; j < (t + 1) * VIS_P && j < J; ++j) {
    lo = min(lo, widx[j]);
    hi = max(hi, widx[j]);
  }
  rng[t] = lo <= hi ? make_int2(lo, hi) : make_int2(1, 0);
}

int launch_prep_ref_ranges(const int32_t* widx, int64_t J, int64_t ntiles, int2* rng, cudaStream_t st) {
  if (ntiles <= 0) return VISS_OK;
  ref_ranges_kernel<<<(unsigned)((ntiles + 127) / 128), 128, 0, st>>>(widx, J, ntiles, rng);
  VISS_LAUNCH_CHECK("ref_ranges_kernel");
  return VISS_OK;
}

// ------------------------------------------------------------- pixel order
// Spatial order of the sky for the geometric mask: the direction is projected
// on the face of the cube it points to and the face coordinates (10 bits each)
// are interleaved (Morton), so consecutive positions are neighbouring pixels
// and a warp's pixels see the Moon's limb together.
// 10 bits -> the even bits of 20 (2-D Morton interleave)
__device__ __forceinline__ uint32_t spread10(uint32_t x) {
  x &= 0x3ff;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

__global__ void pixel_keys_kernel(const float* l, const float* m, const float* n, int64_t J, uint32_t* keys,
                                  int32_t* idx) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= J) return;
  const float x = l[j], y = m[j], z = n[j];
  const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  uint32_t face;
  float a, b, d;
  if (ax >= ay && ax >= az) { face = x >= 0 ? 0 : 1; a = y; b = z; d = ax; }
  else if (ay >= az) { face = y >= 0 ? 2 : 3; a = x; b = z; d = ay; }
  else { face = z >= 0 ? 4 : 5; a = x; b = y; d = az; }
  const float inv = d > 0.f ? 1.0f / d : 0.f;
  const uint32_t ia = (uint32_t)fminf(1023.f, fmaxf(0.f, (a * inv + 1.0f) * 511.5f));
  const uint32_t ib = (uint32_t)fminf(1023.f, fmaxf(0.f, (b * inv + 1.0f) * 511.5f));
  keys[j] = (face << 20) | (spread10(ia) << 1) | spread10(ib);
  idx[j] = (int32_t)j;
}

int launch_pixel_keys(const float* l, const float* m, const float* n, int64_t J, uint32_t* keys, int32_t* idx,
                      cudaStream_t st) {
  if (J <= 0) return VISS_OK;
  pixel_keys_kernel<<<(unsigned)((J + 255) / 256), 256, 0, st>>>(l, m, n, J, keys, idx);
  VISS_LAUNCH_CHECK("pixel_keys_kernel");
  return VISS_OK;
}

int launch_prep_pixels(const PixPrepArgs& a, cudaStream_t st) {
  if (a.Jpad <= 0) return VISS_OK;
  const int bs = 256;
  prep_pixels_kernel<<<(unsigned)((a.Jpad + bs - 1) / bs), bs, 0, st>>>(a);
  VISS_LAUNCH_CHECK("prep_pixels_kernel");
  return VISS_OK;
}

// ------------------------------------------------------------- rows
// Reference recon mask (vissGen10M_shade.cu:166): skip iff
//   fabsf(r1 - thetaP) < r1 && fabsf(r2 - phiP) < r2,  r = (float)Ma / (float)Mb
// with thetaP, phiP non-negative integers.  The set of integers t passing the
// first test is {1..tmax} (empty when r1 <= 0 or NaN); tmax is found from the
// exact float predicate.
__device__ int recon_ratio_tmax(float r) {
  if (!(r > 0.f) || isinf(r)) return 0;
  // candidates t < 2r; find the largest t >= 1 with fabsf(r - t) < r
  double lim = 2.0 * (double)r;
  long long t = (long long)ceil(lim) - 1;
  if (t > 2147483000LL) t = 2147483000LL;
  for (long long c = t + 1; c >= t - 1 && c >= 1; --c) {
    if (fabsf(r - (float)c) < r) return (int)c;
  }
  return 0;
}

// Input row of padded row pr, or -1 for a padding row.
__device__ __forceinline__ int64_t padded_row_source(const ChannelRows& ch, int64_t pr) {
  const int64_t b = pr / VIS_ROWS;
  int lo = 0, hi = ch.nch - 1;  // channel c with rb_off[c] <= b < rb_off[c+1]
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (ch.rb_off[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  const int64_t k = ch.row_off[lo] + (pr - ch.rb_off[lo] * VIS_ROWS);
  return k < ch.row_off[lo + 1] ? k : -1;
}

__global__ void prep_rows_kernel(RowPrepArgs a, bool recon) {
  const int64_t pr = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pr >= a.Kpad) return;
  const int64_t k = a.padded ? padded_row_source(a.ch, pr) : (pr < a.K ? pr : -1);
  if (k < 0) {
    a.rows0[pr] = make_int4(0, 0, 0, PHASE_BIAS);
    a.rows1[pr] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.rowsat) a.rowsat[pr] = PAD_PACKED;
    if (a.uf) a.uf[pr] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.win) a.win[pr] = recon ? make_int4(0, 0, 0, 0) : make_int4(1, 0, 0, 0);
    return;
  }
  const double uu = a.u[k], vv = a.v[k], ww = a.w[k];
  const double Uu = floor(uu + 0.5), Uv = floor(vv + 0.5), Uw = floor(ww + 0.5);
  const double lim = 1073741824.0;  // |U| < 2^30
  if (!(fabs(Uu) < lim && fabs(Uv) < lim && fabs(Uw) < lim)) atomicOr(a.flags + FLAG_ERR, 1);
  const double fu = uu - Uu, fv = vv - Uv, fw = ww - Uw;  // exact, in [-1/2, 1/2)
  if (fu != 0.0 || fv != 0.0 || fw != 0.0) atomicOr(a.flags + FLAG_FRAC, 1);
  if (a.rowsat) {
    int packed = PAD_PACKED;
    const int s = a.snap[k];
    const int pr2 = a.pair[k];
    const int pm = pr2 & 0xffff, pn = (pr2 >> 16) & 0xffff;
    if (s < 0 || s >= a.S || pm >= a.nsat || pn >= a.nsat) atomicOr(a.flags + FLAG_ERR, 2);
    else packed = (s * a.nsat + pm) | ((pn - pm + 32) << 26);
    a.rowsat[pr] = packed;
  }
  // PHASE_BIAS plus the per-row part of f_w * z: f_w * sn * n_offset; the
  // reconstruction folds the visibility's phase in too: y e^{ix} = |y| e^{i(x + arg y)}
  uint32_t bias = (uint32_t)PHASE_BIAS + fix32(fw * a.sn * a.n_offset);
  float c = 0.f;
  if (recon) {
    const double wg = a.wgt ? (double)a.wgt[k] : 1.0;
    const double yr = wg * (double)a.V[2 * k], yi = wg * (double)a.V[2 * k + 1];
    c = (float)sqrt(yr * yr + yi * yi);
    if (c > 0.f) bias += fix32(atan2(yi, yr) * (0.5 / kPi));
    // every other row: half a turn more and -|y| (the same term), so that a
    // systematic error of the SFU's sin/cos cancels over the rows instead of
    // adding up with the all-positive weights |y|
    if (k & 1) {
      bias += 0x80000000u;
      c = -c;
    }
  }
  a.rows0[pr] = make_int4((int)(long long)Uu, (int)(long long)Uv, (int)(long long)Uw, (int)bias);
  // the FP32 parts of the phase are summed in radians: coefficients times 2 pi
  a.rows1[pr] = make_float4((float)(fu * (double)K2PI), (float)(fv * (double)K2PI), (float)(fw * (double)K2PI), c);
  if (a.uf) a.uf[pr] = make_float4((float)(Uu * (double)K2PI), (float)(Uv * (double)K2PI), (float)(Uw * (double)K2PI), 0.f);
  if (a.win) {
    int4 wv = recon ? make_int4(0, 0, 0, 0) : make_int4(1, 0, 0, 0);  // empty
    if (a.shade) {
      const int M1 = a.shade[4 * k], M2 = a.shade[4 * k + 1], M3 = a.shade[4 * k + 2],
                M4 = a.shade[4 * k + 3];
      if (!recon) {
        if (a.mask_mode == VISS_MASK_REF_QUIRK) {
          if (M3 <= 0 && M4 >= 0) wv = make_int4(0, M4, M1, M2);
        } else if (a.mask_mode == VISS_MASK_REF_INTENDED) {
          if (M3 <= M4) wv = make_int4(M3, M4, M1, M2);
        }
      } else if (a.recon_mask == VISS_RECON_MASK_REF) {
        const float r1 = (float)M1 / (float)M2, r2 = (float)M3 / (float)M4;
        wv = make_int4(recon_ratio_tmax(r1), recon_ratio_tmax(r2), 0, 0);
      }
    }
    a.win[pr] = wv;
  }
}

int launch_prep_rows(const RowPrepArgs& a, bool recon, cudaStream_t st) {
  if (a.Kpad <= 0) return VISS_OK;
  const int bs = 256;
  prep_rows_kernel<<<(unsigned)((a.Kpad + bs - 1) / bs), bs, 0, st>>>(a, recon);
  VISS_LAUNCH_CHECK("prep_rows_kernel");
  return VISS_OK;
}

// Reference recon ratio arrays given directly (viss_imagerecon): same tmax rule.
__global__ void prep_recon_ratios_kernel(const float* thetaP0, const float* phiP0, const float* dtheta,
                                         const float* dphi, int64_t K, int64_t Kpad, int4* win,
                                         int* flags) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= Kpad) return;
  if (k >= K) { win[k] = make_int4(0, 0, 0, 0); return; }
  // skip iff fabsf(t0 - thetaP) < dt && fabsf(p0 - phiP) < dp.  The reference
  // passes the same ratio array twice (t0 == dt, p0 == dp, :514-517); rows
  // of another form set flag bit 4 and the call is rejected.
  const float t0 = thetaP0[k], dt = dtheta[k], p0 = phiP0[k], dp = dphi[k];
  const bool same_t = (t0 == dt) || (t0 != t0 && dt != dt);
  const bool same_p = (p0 == dp) || (p0 != p0 && dp != dp);
  if (!same_t || !same_p) atomicOr(flags + 1, 4);
  win[k] = make_int4(recon_ratio_tmax(t0), recon_ratio_tmax(p0), 0, 0);
}

// ------------------------------------------------------------- satellites
// satdir[i] = {p/|p|, cos(alpha)}, alpha = asin(R/|p|) the Moon's angular radius
// seen from the satellite.  Occluded <=> s_hat . p_hat < -cos(alpha).  A
// satellite inside the sphere (|p| <= R) gets cos(alpha) = 0 (occluded <=> s.p < 0),
// which is what the exact predicate gives there.
__global__ void prep_satdir_kernel(const float* pos, int64_t nsd, double R, float4* satdir) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsd) return;
  const double px = pos[3 * i], py = pos[3 * i + 1], pz = pos[3 * i + 2];
  const double r = sqrt(px * px + py * py + pz * pz);
  if (!(r > 0.0)) {
    satdir[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  const double ca = r > R ? sqrt(1.0 - (R / r) * (R / r)) : 0.0;
  satdir[i] = make_float4((float)(px / r), (float)(py / r), (float)(pz / r), (float)ca);
}

int launch_prep_satdir(const float* sat_pos, int64_t nsd, double R, float4* satdir, cudaStream_t st) {
  if (nsd <= 0) return VISS_OK;
  prep_satdir_kernel<<<(unsigned)((nsd + 255) / 256), 256, 0, st>>>(sat_pos, nsd, R, satdir);
  VISS_LAUNCH_CHECK("prep_satdir_kernel");
  return VISS_OK;
}

// ------------------------------------------------------------- cones
// For a set of satellites {p_i} with shadow cones (axis -p_hat_i, half angle
// alpha_i): axis c = normalise(sum -p_hat_i), rho = max angle(c, -p_hat_i).
// A pixel s_hat with s_hat.c > cos(alpha_min - rho - eps) is occluded for every
// satellite of the set; with s_hat.c < cos(alpha_max + rho + eps) it is visible
// from every one.  cone[0] = {c, cos_occ}, cone[1] = {cos_vis, sin_occ, sin_vis, -}
// (the sines of the two angles, 0 where the cosine is the 2 / -2 of "never").
// Degenerate sets (a satellite at the origin) get cos_occ = 2, cos_vis = -2.
// From the axis, the smallest cosine to it (mc) and the cone-angle range [a0, a1].
__device__ void cone_write(const double* axis, double mc, double a0, double a1, bool degen, int64_t count,
                           float4* out) {
  const double eps = 1e-5;
  float cos_occ = 2.f, cos_vis = -2.f, sin_occ = 0.f, sin_vis = 0.f;
  if (!degen && count > 0) {
    const double rho = acos(fmin(1.0, fmax(-1.0, mc)));
    const double lo = a0 - rho - eps, hi = a1 + rho + eps;
    if (lo > 0) { cos_occ = (float)cos(lo); sin_occ = (float)sin(lo); }
    if (hi < kPi) { cos_vis = (float)cos(hi); sin_vis = (float)sin(hi); }
    // widen by float rounding of the test s_hat . c
    if (cos_occ <= 1.f) cos_occ = fminf(2.f, cos_occ + 1e-6f);
    if (cos_vis >= -1.f) cos_vis = cos_vis - 1e-6f;
  }
  out[0] = make_float4((float)axis[0], (float)axis[1], (float)axis[2], cos_occ);
  out[1] = make_float4(cos_vis, sin_occ, sin_vis, 0.f);
}

// Block-wide: one block per cone; members enumerated by `member(i)` -> satdir index.
template <class Member>
__device__ void cone_block(const float4* satdir, int64_t count, Member member, float4* out) {
  __shared__ double red[4][32];
  __shared__ double axis[3];
  __shared__ int degen_s;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  if (tid == 0) degen_s = 0;
  __syncthreads();
  double sx = 0, sy = 0, sz = 0;
  for (int64_t i = tid; i < count; i += blockDim.x) {
    const float4 d = satdir[member(i)];
    if (d.x == 0.f && d.y == 0.f && d.z == 0.f) { atomicOr(&degen_s, 1); continue; }
    if (d.w == 0.f) atomicOr(&degen_s, 1);  // inside the sphere: no cone
    sx -= d.x; sy -= d.y; sz -= d.z;
  }
  for (int o = 16; o; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
    sz += __shfl_xor_sync(0xffffffffu, sz, o);
  }
  if (lane == 0) { red[0][wid] = sx; red[1][wid] = sy; red[2][wid] = sz; }
  __syncthreads();
  if (tid == 0) {
    double a = 0, b = 0, c = 0;
    for (int w = 0; w < nw; ++w) { a += red[0][w]; b += red[1][w]; c += red[2][w]; }
    const double nn = sqrt(a * a + b * b + c * c);
    axis[0] = nn > 0 ? a / nn : 0; axis[1] = nn > 0 ? b / nn : 0; axis[2] = nn > 0 ? c / nn : 1;
    if (!(nn > 0)) degen_s = 1;
  }
  __syncthreads();
  // rho (as min cos), alpha range
  double mincos = 2.0, amin = 10.0, amax = -1.0;
  for (int64_t i = tid; i < count; i += blockDim.x) {
    const float4 d = satdir[member(i)];
    const double c = -(axis[0] * d.x + axis[1] * d.y + axis[2] * d.z);
    mincos = fmin(mincos, c);
    const double al = acos(fmin(1.0, fmax(-1.0, (double)d.w)));
    amin = fmin(amin, al);
    amax = fmax(amax, al);
  }
  for (int o = 16; o; o >>= 1) {
    mincos = fmin(mincos, __shfl_xor_sync(0xffffffffu, mincos, o));
    amin = fmin(amin, __shfl_xor_sync(0xffffffffu, amin, o));
    amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  }
  __syncthreads();
  if (lane == 0) { red[0][wid] = mincos; red[1][wid] = amin; red[2][wid] = amax; }
  __syncthreads();
  if (tid == 0) {
    double mc = 2.0, a0 = 10.0, a1 = -1.0;
    for (int w = 0; w < nw; ++w) { mc = fmin(mc, red[0][w]); a0 = fmin(a0, red[1][w]); a1 = fmax(a1, red[2][w]); }
    cone_write(axis, mc, a0, a1, degen_s != 0, count, out);
  }
}

struct RowMember {
  const int* rowsat;
  int64_t base;
  __device__ int operator()(int64_t i) const {
    const int p = rowsat[base + (i >> 1)];
    return (i & 1) ? sat_gn(p) : sat_gm(p);
  }
};

// One cone per padded block of VIS_ROWS rows, over the block's real rows; the
// sines in cone[1] (which the vis kernel does not use) are replaced by the range
// of satellite indices those rows use (y: the first, z: how many, as int bits;
// z = 0 for an empty block).
__global__ void rowblock_cones_kernel(const int* rowsat, const float4* satdir, const ChannelRows ch, float4* cones) {
  const int64_t b = blockIdx.x;
  int c = 0;
  while (c + 1 < ch.nch && b >= ch.rb_off[c + 1]) ++c;
  int64_t cnt = (ch.row_off[c + 1] - ch.row_off[c]) - (b - ch.rb_off[c]) * VIS_ROWS;
  if (cnt > VIS_ROWS) cnt = VIS_ROWS;
  if (cnt < 0) cnt = 0;
  cone_block(satdir, 2 * cnt, RowMember{rowsat, b * VIS_ROWS}, cones + 2 * b);
  __shared__ int rlo[32], rhi[32];
  int lo = 0x7fffffff, hi = -1;
  for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) {
    const int pk = rowsat[b * VIS_ROWS + i];
    lo = min(lo, min(sat_gm(pk), sat_gn(pk)));
    hi = max(hi, max(sat_gm(pk), sat_gn(pk)));
  }
  for (int o = 16; o; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) { rlo[threadIdx.x >> 5] = lo; rhi[threadIdx.x >> 5] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { lo = min(lo, rlo[w]); hi = max(hi, rhi[w]); }
    cones[2 * b + 1].y = __int_as_float(hi >= lo ? lo : 0);
    cones[2 * b + 1].z = __int_as_float(hi >= lo ? hi - lo + 1 : 0);
  }
}

int launch_prep_rowblock_cones(const int* rowsat, const float4* satdir, const ChannelRows& ch, int64_t nblocks,
                               float4* cones, cudaStream_t st) {
  if (nblocks <= 0) return VISS_OK;
  rowblock_cones_kernel<<<(unsigned)nblocks, 256, 0, st>>>(rowsat, satdir, ch, cones);
  VISS_LAUNCH_CHECK("rowblock_cones_kernel");
  return VISS_OK;
}

// Bounding cone of each block of `block` consecutive sky positions (unit
// directions in pgeo): axis = normalised mean, radius r = largest angle from it,
// widened by 1e-6.  {axis, cos r}, {sin r}; cos r = -2 when the block has no axis.
__global__ void block_cones_kernel(const float4* pgeo, int64_t J, int block, float4* cones) {
  __shared__ double red[3][32];
  __shared__ double axis[3];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int64_t j0 = (int64_t)blockIdx.x * block;
  int64_t j1 = j0 + block;
  if (j1 > J) j1 = J;
  double sx = 0, sy = 0, sz = 0;
  for (int64_t j = j0 + tid; j < j1; j += blockDim.x) {
    const float4 g = pgeo[j];
    sx += g.x; sy += g.y; sz += g.z;
  }
  for (int o = 16; o; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
    sz += __shfl_xor_sync(0xffffffffu, sz, o);
  }
  if (lane == 0) { red[0][wid] = sx; red[1][wid] = sy; red[2][wid] = sz; }
  __syncthreads();
  if (tid == 0) {
    double a = 0, b = 0, c = 0;
    for (int w = 0; w < nw; ++w) { a += red[0][w]; b += red[1][w]; c += red[2][w]; }
    const double nn = sqrt(a * a + b * b + c * c);
    axis[0] = nn > 1e-3 ? a / nn : 0.0; axis[1] = nn > 1e-3 ? b / nn : 0.0; axis[2] = nn > 1e-3 ? c / nn : 0.0;
  }
  __syncthreads();
  double mc = 2.0;
  for (int64_t j = j0 + tid; j < j1; j += blockDim.x) {
    const float4 g = pgeo[j];
    mc = fmin(mc, axis[0] * g.x + axis[1] * g.y + axis[2] * g.z);
  }
  for (int o = 16; o; o >>= 1) mc = fmin(mc, __shfl_xor_sync(0xffffffffu, mc, o));
  __syncthreads();
  if (lane == 0) red[0][wid] = mc;
  __syncthreads();
  if (tid == 0) {
    for (int w = 0; w < nw; ++w) mc = fmin(mc, red[0][w]);
    const bool ok = (axis[0] != 0.0 || axis[1] != 0.0 || axis[2] != 0.0) && mc <= 1.0 && mc > -1.0;
    double cr = -2.0, sr = 1.0;
    if (ok) {
      const double r = acos(fmin(1.0, mc)) + 1e-6;
      cr = cos(r);
      sr = sin(r);
    }
    cones[2 * blockIdx.x] = make_float4((float)axis[0], (float)axis[1], (float)axis[2], (float)cr);
    cones[2 * blockIdx.x + 1] = make_float4((float)sr, 0.f, 0.f, 0.f);
  }
}

int launch_prep_block_cones(const float4* pgeo, int64_t J, int block, int64_t nblocks, float4* cones,
                            cudaStream_t st) {
  if (nblocks <= 0) return VISS_OK;
  block_cones_kernel<<<(unsigned)nblocks, 256, 0, st>>>(pgeo, J, block, cones);
  VISS_LAUNCH_CHECK("block_cones_kernel");
  return VISS_OK;
}

// One thread per snapshot (its nsat satellites in a loop): the bounds of
// cone_block, without a block's reductions and serial tail per snapshot.
__global__ void snapshot_cones_kernel(const float4* satdir, int64_t S, int nsat, float4* cones) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const float4* d0 = satdir + s * nsat;
  bool degen = false;
  double sx = 0, sy = 0, sz = 0;
  for (int i = 0; i < nsat; ++i) {
    const float4 d = d0[i];
    if (d.x == 0.f && d.y == 0.f && d.z == 0.f) { degen = true; continue; }
    if (d.w == 0.f) degen = true;  // inside the sphere: no cone
    sx -= d.x; sy -= d.y; sz -= d.z;
  }
  const double nn = sqrt(sx * sx + sy * sy + sz * sz);
  double axis[3] = {nn > 0 ? sx / nn : 0, nn > 0 ? sy / nn : 0, nn > 0 ? sz / nn : 1};
  if (!(nn > 0)) degen = true;
  double mc = 2.0, a0 = 10.0, a1 = -1.0;
  for (int i = 0; i < nsat; ++i) {
    const float4 d = d0[i];
    mc = fmin(mc, -(axis[0] * d.x + axis[1] * d.y + axis[2] * d.z));
    const double al = acos(fmin(1.0, fmax(-1.0, (double)d.w)));
    a0 = fmin(a0, al);
    a1 = fmax(a1, al);
  }
  cone_write(axis, mc, a0, a1, degen, nsat, cones + 2 * s);
}

int launch_prep_snapshot_cones(const float4* satdir, int64_t S, int nsat, float4* cones, cudaStream_t st) {
  if (S <= 0) return VISS_OK;
  snapshot_cones_kernel<<<(unsigned)((S + 127) / 128), 128, 0, st>>>(satdir, S, nsat, cones);
  VISS_LAUNCH_CHECK("snapshot_cones_kernel");
  return VISS_OK;
}

int launch_prep_recon_ratios(const float* thetaP0, const float* phiP0, const float* dtheta, const float* dphi,
                             int64_t K, int64_t Kpad, int4* win, int* flags, cudaStream_t st) {
  if (Kpad <= 0) return VISS_OK;
  prep_recon_ratios_kernel<<<(unsigned)((Kpad + 255) / 256), 256, 0, st>>>(thetaP0, phiP0, dtheta, dphi, K,
                                                                          Kpad, win, flags);
  VISS_LAUNCH_CHECK("prep_recon_ratios_kernel");
  return VISS_OK;
}

}  // namespace viss
