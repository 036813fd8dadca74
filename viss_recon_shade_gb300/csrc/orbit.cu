// orbit.cu -- satellite positions at the windowed snapshots and baseline uvw
// (MIncline_generate_uvw_float.cu:83-160, 343-397).
//
// The reference materialises 8 x 140 x 864000 positions per coordinate
// (calculateOrbit, 11.6 GB), copies a window of each orbit (uvwPosition) and
// then forms uvw per ordered pair.  Here one thread computes the position of
// one satellite at one windowed snapshot directly -- only the S = counts*res/3
// snapshots that are used are evaluated -- and a second kernel forms every
// baseline of a snapshot.  The FP32 mode evaluates the reference's float
// formulas operation by operation (including its double-precision pieces), so
// it reproduces the reference kernels' positions; the FP64 mode gives
// continuous positions for the continuous-uvw (geometric-mask) configurations.
#include <cub/cub.cuh>

#include <vector>

#include "viss_internal.cuh"

namespace viss {

// x / d for 0 <= x < 2^31 by a multiply-high with magic = ceil(2^32 / d)
// (the estimate is floor(x / d) or one above it), corrected by one step either way
struct FastDiv {
  int d = 1;
  uint32_t magic = 0;
  void set(int dd) { d = dd; magic = dd > 1 ? 0xFFFFFFFFu / (uint32_t)dd + 1 : 0; }
  __device__ __forceinline__ int div(int x) const {
    if (d == 1) return x;
    int q = (int)__umulhi((uint32_t)x, magic);
    const int r = x - q * d;
    if (r < 0) --q;
    else if (r >= d) ++q;
    return q;
  }
};

// Every index below is a 32-bit int: the launcher admits only
// orbit_res * orbit_counts * (nsat + 1) < 2^31 (the reference's own int indices),
// so sample indices, snapshots, threads and 3 x threads all stay below 2^31.
struct OrbitDev {
  int nsat, orbit_res, orbit_counts, index;
  int span, interval;
  int total, S, half, reset_index;
  FastDiv by_span, by_res, by_nsat;
  float a, e, incl, argp, d2r;
  double dm_den;                 // (double)(2a) * 1e3, the divisor of calculate_dM
  float dm_hi, dm_lo, dm_inv;    // dm_den = dm_hi + dm_lo exactly; dm_inv = fl(1 / dm_den)
  double a64, e64, incl64, argp64, raan_step;
  float step_mt;
  int fp64;
  float r1[32], r2[32];
  float s1[32], s2[32];  // linspace steps of the separation ramps
};

// uvwPosition (:113-151) index arithmetic for snapshot g: the global sample
// `circle` of the satellite's array, or zero-fill (kind 1), or the reference's
// read of one element past the satellite's array (kind 2): that is the next
// satellite's slot, not yet computed when uvwPosition runs for this satellite
// (:224-308), so it reads zero as well.
__device__ __forceinline__ int window_index(const OrbitDev& o, int g, int* circle) {
  const int k = o.by_span.div(g) + 1;
  const int offset = (k - 1) * o.interval;
  int endIdx = (k - 1) * o.orbit_res + offset + o.span;
  int startIdx = (k - 1) * o.orbit_res + offset;
  if ((k - 1) * (o.orbit_res + o.interval) > o.total) {
    const int reset_index = o.reset_index;  // total / (orbit_res + interval) + 1
    startIdx = (k - 1 - reset_index) * o.orbit_res + offset;
    endIdx = (k - 1 - reset_index) * o.orbit_res + offset + o.span;
  }
  const int c = startIdx + (g - (k - 1) * o.span);
  *circle = c;
  if (endIdx > o.total) {
    if (c > o.total) return 1;
    if (c == o.total) return 2;
  }
  return 0;
}

// calculate_dM (:51-58): (float)(asin((double)d / ((double)(2a) * 1e3)) * 2)
__device__ __noinline__ float dm_exact(float d, double den) { return (float)(asin((double)d / den) * 2); }

// The same value without FP64 for |x| = |d / den| <= 0.05.  x = xh + xl to
// 2^-44 |x| (the FMA residual d - xh * dm_hi is exact); asin(x) = x + c,
// c = x^3 (1/6 + 3x^2/40 + 15x^4/336 + 105x^6/3456) + x^2 xl / 2 evaluated in
// FP32 (series tail < 2^-48 |x|; rounding < 2^-21 |c| <= 2^-23.6 x^2 |x|), and
// hi + lo = xh + (xl + c) by Fast2Sum.  The reference rounds 2 asin(x) (double,
// within 2^-50 |x|) to float: 2 hi is that float unless x could lie within
// E = |hi| (x^2 2^-23 + 2^-42) of a rounding boundary, i.e. unless |lo| + E reaches
// half the spacing to hi's nearer neighbour.  Those values, a few in 10^4, divide
// and take asin in double.
__device__ __forceinline__ float dm_value(const OrbitDev& o, float d) {
  if (d == 0.f) return d;  // asin(+-0) * 2 = +-0
  const float xh = __fmul_rn(d, o.dm_inv);
  const float r = __fmaf_rn(-xh, o.dm_hi, d);
  const float r2 = __fmaf_rn(-xh, o.dm_lo, r);
  const float xl = __fmul_rn(r2, o.dm_inv);
  const float x2 = __fmul_rn(xh, xh);
  float P = __fmaf_rn(105.f / 3456.f, x2, 15.f / 336.f);
  P = __fmaf_rn(P, x2, 3.f / 40.f);
  P = __fmaf_rn(P, x2, 1.f / 6.f);
  const float c = __fmul_rn(__fmul_rn(x2, xh), P);
  const float S = __fadd_rn(__fadd_rn(xl, c), __fmul_rn(__fmul_rn(0.5f, x2), xl));
  const float hi = __fadd_rn(xh, S);
  const float lo = __fsub_rn(S, __fsub_rn(hi, xh));
  const float ah = fabsf(hi);
  const int bits = __float_as_int(ah);
  const float half_gap = 0.5f * fminf(__int_as_float(bits + 1) - ah, ah - __int_as_float(bits - 1));
  const float E = ah * __fmaf_rn(x2, 0x1p-23f, 0x1p-42f);
  if (fabsf(xh) <= 0.05f && __fadd_rn(fabsf(lo), E) < half_gap) return 2.f * hi;
  return dm_exact(d, o.dm_den);
}

// RAAN of orbit k (:88-89) in the reference's mixed float/double arithmetic;
// base = (index - 1) * orbit_counts.  One compiled copy serves the per-block
// table and the positions outside it.
__device__ __noinline__ float raan_of(int k, int base, float d2r, double step) {
  return (float)((double)((float)k * d2r) * step + 0.0 + (double)((float)base * d2r) * step);
}

constexpr int RAAN_TAB = 4;  // orbits per block with a precomputed RAAN

// calculateOrbit (:83-110) in the reference's arithmetic.  raan_tab holds the
// RAAN of orbits k_base .. k_base + RAAN_TAB - 1.  The final rotation keeps the
// reference's expression shape: written with cosf/sinf values computed elsewhere
// the compiler fuses its products differently, and about half of the positions
// move by an ulp.
__device__ void position_f32(const OrbitDev& o, int sat, int idx, const float* raan_tab, int k_base,
                             float* out) {
  const int half = o.half;
  const int k = o.by_res.div(idx), po = idx - k * o.orbit_res;
  float d;
  if (idx < half) d = fmaf(o.s1[sat], (float)idx, o.r1[sat]);   // linspace r1 -> r2 (:42-49)
  else d = fmaf(o.s2[sat], (float)(idx - half), o.r2[sat]);     // linspace r2 -> r1
  const float dM = dm_value(o, d);  // calculate_dM (:51-58)
  const int dk = k - k_base;
  const float raan = (dk >= 0 && dk < RAAN_TAB) ? raan_tab[dk]
                                                : raan_of(k, (o.index - 1) * o.orbit_counts, o.d2r, o.raan_step);
  // Mt[po] is rounded on its own (thrust linspace with a = 0), then dM is added
  const float M = __fmul_rn(o.step_mt, (float)po) + dM;
  // Newton on Kepler's equation, at most 99 updates (:95-102).  An update is a
  // function of E0 alone, so once E0 repeats it cycles to the last update: a
  // fixed point stays, a 2-cycle ends on the value the parity of the updates
  // left selects.  In FP32 a few percent of samples end in such a cycle without
  // meeting the exit test; they leave at the repeat with the same result.
  // With e = 0 the first test already sees err = M - (M - 0 * sinf(M)) = 0 and
  // leaves E0 = M.  The exit test is the reference's double comparison: a float
  // is below 1e-15 exactly when it is below 1e-15f (no float lies between).
  float E0 = M, Ep = M;
  for (int i = 1; i < 100 && o.e != 0.f; ++i) {
    const float M0 = E0 - o.e * sinf(E0);
    const float err = M - M0;
    if (fabsf(err) < 1e-15f) break;
    const float En = E0 + err / (1 - o.e * cosf(E0));
    if (__float_as_int(En) == __float_as_int(E0)) break;
    if (i >= 2 && __float_as_int(En) == __float_as_int(Ep)) {
      if (((99 - i) & 1) == 0) E0 = En;
      break;
    }
    Ep = E0;
    E0 = En;
  }
  // e = 0: the divisor is sqrtf(1 / 1) = 1 and the quotient tanf(E0 / 2) itself
  const float tan_half = tanf(E0 / 2);
  const float temp = o.e != 0.f ? tan_half / sqrtf((1 - o.e) / (1 + o.e)) : tan_half;
  const float theta = atanf(temp) * 2;
  // e = 0: a * 1 / 1 = a exactly, without evaluating cosf(theta)
  const float r = o.e != 0.f ? o.a * (1 - o.e * o.e) / (1 + o.e * cosf(theta)) : o.a;
  const float w = theta + o.argp;
  out[0] = r * (cosf(w) * cosf(raan) - sinf(w) * cosf(o.incl) * sinf(raan));
  out[1] = r * (cosf(w) * sinf(raan) + sinf(w) * cosf(o.incl) * cosf(raan));
  out[2] = r * (sinf(w) * sinf(o.incl));
}

__device__ void position_f64(const OrbitDev& o, int sat, int idx, double* out) {
  const int half = o.total / 2;
  const int k = idx / o.orbit_res, po = idx % o.orbit_res;
  const double d2r = kPi / 180.0;
  const double r1 = o.r1[sat], r2 = o.r2[sat];
  double d;
  if (idx < half) d = r1 + (r2 - r1) / (double)(half - 1) * (double)idx;
  else d = r2 + (r1 - r2) / (double)(half - 1) * (double)(idx - half);
  const double dM = 2.0 * asin(d / (2.0 * o.a64 * 1e3));
  const double raan = (double)k * d2r * o.raan_step + (double)(o.index - 1) * (double)o.orbit_counts * d2r * o.raan_step;
  const double M = 2.0 * kPi / (double)(o.orbit_res - 1) * (double)po + dM;
  double E = M, Ep = M;  // the same cycle exits as the FP32 loop
  for (int i = 1; i < 100 && o.e64 != 0.0; ++i) {
    const double err = M - (E - o.e64 * sin(E));
    if (fabs(err) < 1e-15) break;
    const double En = E + err / (1.0 - o.e64 * cos(E));
    if (__double_as_longlong(En) == __double_as_longlong(E)) break;
    if (i >= 2 && __double_as_longlong(En) == __double_as_longlong(Ep)) {
      if (((99 - i) & 1) == 0) E = En;
      break;
    }
    Ep = E;
    E = En;
  }
  const double theta = 2.0 * atan(tan(E / 2.0) / sqrt((1.0 - o.e64) / (1.0 + o.e64)));
  const double r = o.a64 * (1.0 - o.e64 * o.e64) / (1.0 + o.e64 * cos(theta));
  const double w = theta + o.argp64;
  out[0] = r * (cos(w) * cos(raan) - sin(w) * cos(o.incl64) * sin(raan));
  out[1] = r * (cos(w) * sin(raan) + sin(w) * cos(o.incl64) * cos(raan));
  out[2] = r * (sin(w) * sin(o.incl64));
}

__global__ void orbit_positions_kernel(const OrbitDev o, float* pos, double* pos64) {
  // The block's snapshots lie on one or two orbits: their RAAN (FP64 work) is
  // computed once per block, from the orbit of the block's first snapshot on.
  __shared__ float raan_tab[RAAN_TAB];
  __shared__ int k_base_s;
  if (!o.fp64 && threadIdx.x < RAAN_TAB) {
    int c0;
    const int kind0 = window_index(o, o.by_nsat.div((int)(blockIdx.x * blockDim.x)), &c0);
    const int k0 = kind0 == 0 ? o.by_res.div(c0) : 0;
    raan_tab[threadIdx.x] = raan_of(k0 + (int)threadIdx.x, (o.index - 1) * o.orbit_counts, o.d2r, o.raan_step);
    if (threadIdx.x == 0) k_base_s = k0;
  }
  __syncthreads();
  const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (t >= o.S * o.nsat) return;
  const int g = o.by_nsat.div(t);
  const int sat = t - g * o.nsat;
  int circle;
  const int kind = window_index(o, g, &circle);
  const bool zero = kind != 0;
  if (o.fp64) {
    double p[3] = {0.0, 0.0, 0.0};
    if (!zero) position_f64(o, sat, circle, p);
    pos[3 * t] = (float)p[0]; pos[3 * t + 1] = (float)p[1]; pos[3 * t + 2] = (float)p[2];
    if (pos64) { pos64[3 * t] = p[0]; pos64[3 * t + 1] = p[1]; pos64[3 * t + 2] = p[2]; }
  } else {
    float p[3] = {0.f, 0.f, 0.f};
    if (!zero) position_f32(o, sat, circle, raan_tab, k_base_s, p);
    pos[3 * t] = p[0]; pos[3 * t + 1] = p[1]; pos[3 * t + 2] = p[2];
    if (pos64) { pos64[3 * t] = p[0]; pos64[3 * t + 1] = p[1]; pos64[3 * t + 2] = p[2]; }
  }
}

// pair q -> (m, n): ordered pairs m != n m-major (:350-353), unordered m < n.
__device__ __forceinline__ void pair_of(int q, int nsat, int ordered, int* m, int* n) {
  if (ordered) {
    const int mm = q / (nsat - 1), r = q % (nsat - 1);
    *m = mm;
    *n = r < mm ? r : r + 1;
  } else {
    int mm = 0, base = 0;
    while (q >= base + (nsat - 1 - mm)) { base += nsat - 1 - mm; ++mm; }
    *m = mm;
    *n = mm + 1 + (q - base);
  }
}

// ceil((double)diff * 1e3 / lambda) rounded to float, as computeUVW evaluates it
__device__ __noinline__ float ceil_quotient_exact(float diff, double lambda) {
  return (float)ceil((double)diff * 1e3 / lambda);
}

// The reference's ceil((double)diff * 1e3 / lambda) (computeUVW, :156-158) from
// FP32 arithmetic where that is certain.  scale = {hi, lo} holds 1e3 / lambda to
// 2^-48; x = diff * scale is carried as xh + xl to 2^-45 |x| (xh rounded, xl its
// FMA residual plus diff * lo).  floor(xh) comes from the round-down sum
// xh + 1.5 * 2^23 (exact for |xh| < 2^22), and f2 = (xh - floor(xh)) + xl is the
// quotient's distance above that integer to within 2^-24 + 2^-45 |x|.  Where f2
// keeps T = 2^-23 + 2^-44 |x| from both ends, the quotient and its double
// rounding lie strictly inside (floor, floor + 1): the ceil is floor + 1, the
// floor of the negated quotient -(floor + 1) + 1.  Elsewhere (a few in 10^7 for
// orbit baselines, and |x| >= 2^22) the quotient is taken in double.
// Returns whether the fast path holds; *y = floor(xh) + 1.5 * 2^23.
__device__ __forceinline__ bool ceil_is_floor_plus_one(float diff, float2 scale, float* y) {
  const float xh = __fmul_rn(diff, scale.x);
  const float xl = __fmaf_rn(diff, scale.y, __fmaf_rn(diff, scale.x, -xh));
  const float yy = __fadd_rd(xh, 12582912.f);
  const float f2 = __fadd_rn(__fsub_rn(xh, __fsub_rn(yy, 12582912.f)), xl);
  const float T = __fmaf_rn(fabsf(xh), 0x1p-44f, 0x1p-23f);
  *y = yy;
  return fabsf(xh) < 4194304.f && f2 > T && f2 < 1.f - T;
}

// computeUVW (:156-158) for one coordinate: ceil((double)diff * 1e3 / lambda) as
// float (the sign of zero included: (-1, 0) gives -0), or without the ceil.
__device__ __forceinline__ float baseline_coord(float diff, double lambda, float2 scale, int rounding) {
  if (diff == 0.f) return diff;  // +-0 * 1e3 / lambda and its ceil keep the sign of zero
  if (!rounding) return (float)((double)diff * 1e3 / lambda);
  float y;
  // floor + 1 rounded down: an exact sum, -0 for floor = -1 as ceil gives
  if (ceil_is_floor_plus_one(diff, scale, &y)) return __fadd_rd(__fsub_rn(y, 12582912.f), 1.f);
  return ceil_quotient_exact(diff, lambda);
}

__global__ void baseline_uvw_kernel(const float* pos, const double* pos64, int64_t S, int nsat, int ordered, int npairs,
                                    uint64_t pair_magic, double lambda, float2 scale, int rounding, float* u,
                                    float* v, float* w, int32_t* snap, int32_t* pair) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S * npairs) return;
  // k / npairs by a multiply-high (magic = ceil(2^64 / npairs)), corrected once
  int64_t g = (int64_t)__umul64hi((uint64_t)k, pair_magic);
  int q = (int)(k - g * npairs);
  if (q < 0) { --g; q += npairs; }
  if (q >= npairs) { ++g; q -= npairs; }
  int m, n;
  pair_of(q, nsat, ordered, &m, &n);
  float out[3];
  for (int c = 0; c < 3; ++c) {
    if (pos64) {
      const double x = (pos64[(g * nsat + n) * 3 + c] - pos64[(g * nsat + m) * 3 + c]) * 1e3 / lambda;
      out[c] = rounding ? (float)ceil(x) : (float)x;
      continue;
    }
    out[c] = baseline_coord(pos[(g * nsat + n) * 3 + c] - pos[(g * nsat + m) * 3 + c], lambda, scale, rounding);
  }
  u[k] = out[0]; v[k] = out[1]; w[k] = out[2];
  if (snap) snap[k] = (int32_t)g;
  if (pair) pair[k] = m | (n << 16);
}

// ---------------------------------------------------------------- dedup
// Integer-valued uvw -> 63-bit key preserving the lexicographic (u, v, w)
// order of SortCompare (:60-71); -0 and +0 share a key as they compare equal.
__device__ __forceinline__ uint64_t uvw_key(float a, float b, float c, int* bad) {
  const float x3[3] = {a, b, c};
  uint64_t key = 0;
  for (int i = 0; i < 3; ++i) {
    const float x = x3[i];
    if (!(x == rintf(x)) || !(fabsf(x) < 1048576.f)) { atomicOr(bad, 1); }
    const int64_t q = (int64_t)x + 1048576;
    key = (key << 21) | ((uint64_t)q & 0x1fffff);
  }
  return key;
}

__global__ void dedup_keys_kernel(const float* u, const float* v, const float* w, int64_t K, uint64_t* keys,
                                  uint32_t* idx, int* bad) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  keys[k] = uvw_key(u[k], v[k], w[k], bad);
  idx[k] = (uint32_t)k;
}

__global__ void dedup_gather_kernel(const uint64_t* keys, const uint32_t* idx, int64_t K, const float* u,
                                    const float* v, const float* w, float* ou, float* ov, float* ow, int* flag) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  flag[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
  const uint32_t s = idx[k];
  ou[k] = u[s]; ov[k] = v[s]; ow[k] = w[s];
}

// Hash pass: the unique keys of the input with the first row index of each, in
// an open-addressing table (linear probing, at most DEDUP_PROBES slots per key;
// a key that finds no slot sets overflow and the caller falls back to sorting
// every row).  Most rows repeat a key already present: they cost a read and,
// when they come earlier than the recorded row, an atomicMin.
constexpr uint64_t DEDUP_EMPTY = ~0ull;
constexpr int DEDUP_PROBES = 256;

__device__ __forceinline__ uint64_t dedup_hash(uint64_t k) {  // splitmix64 finaliser
  k ^= k >> 30; k *= 0xbf58476d1ce4e5b9ull;
  k ^= k >> 27; k *= 0x94d049bb133111ebull;
  return k ^ (k >> 31);
}

// key -> its slot (claimed if new), the slot's row index lowered to k
__device__ __forceinline__ void dedup_insert(uint64_t* tkeys, uint32_t* tidx, uint64_t mask, uint64_t key,
                                             uint32_t k, int* overflow) {
  uint64_t h = dedup_hash(key) & mask;
  for (int probe = 0; probe < DEDUP_PROBES; ++probe, h = (h + 1) & mask) {
    uint64_t cur = *((volatile uint64_t*)(tkeys + h));
    if (cur == DEDUP_EMPTY) {
      cur = atomicCAS((unsigned long long*)(tkeys + h), (unsigned long long)DEDUP_EMPTY, (unsigned long long)key);
      if (cur == DEDUP_EMPTY) cur = key;
    }
    if (cur == key) {
      if (*((volatile uint32_t*)(tidx + h)) > k) atomicMin(tidx + h, k);
      return;
    }
  }
  atomicOr(overflow, 1);
}

// The same for rows that mostly bring a new key or one last seen long ago (the
// fused pass): the row index is lowered by a reduction that does not wait for
// its result, one dependent trip fewer per insert.
__device__ __forceinline__ void dedup_insert_red(uint64_t* tkeys, uint32_t* tidx, uint64_t mask, uint64_t key,
                                                 uint32_t k, int* overflow) {
  uint64_t h = dedup_hash(key) & mask;
  for (int probe = 0; probe < DEDUP_PROBES; ++probe, h = (h + 1) & mask) {
    uint64_t cur = *((volatile uint64_t*)(tkeys + h));
    if (cur == DEDUP_EMPTY) {
      cur = atomicCAS((unsigned long long*)(tkeys + h), (unsigned long long)DEDUP_EMPTY, (unsigned long long)key);
      if (cur == DEDUP_EMPTY) cur = key;
    }
    if (cur == key) {
      atomicMin(tidx + h, k);
      return;
    }
  }
  atomicOr(overflow, 1);
}

__global__ void dedup_hash_kernel(const float* u, const float* v, const float* w, int64_t K, uint64_t* tkeys,
                                  uint32_t* tidx, uint64_t mask, int* bad, int* overflow) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  dedup_insert(tkeys, tidx, mask, uvw_key(u[k], v[k], w[k], bad), (uint32_t)k, overflow);
}

// Fused baselines + hash pass over the rows (snapshot g, pair q) of float
// positions [S][nsat][3], ranked pair-major (row q * S + g) as the reference
// concatenates its per-pair lists before the global sort + unique
// (MIncline_generate_uvw_float.cu:370-397): the first occurrence of a key is its
// lowest pair, then its earliest snapshot.  A thread walks one satellite pair
// m < n over consecutive snapshots, for ordered pairs both rows (m, n) and (n, m),
// and inserts a row only where its key differs from the previous snapshot's: an
// equal key there has the smaller row index already.  Baselines move by far
// less than a wavelength between snapshots, so most rows touch no table slot.
constexpr int UNIQUE_RUN = 256;
constexpr int UNIQUE_BATCH = 2;

// Key fields of row (m, n) and row (n, m) for one coordinate: F = ceil(q) + 2^20
// with q = (double)(+-diff) * 1e3 / lambda, the integers baseline_coord gives
// (without their sign of zero).  Where ceil(q) = floor + 1 is certain,
// ceil(-q) = -floor: F(n, m) = 2^21 + 1 - F(m, n).  With |x| < 2^20 - 2 as well,
// both fields lie in [2, 2^21 - 2] and the three fields of (n, m) are one 64-bit
// subtraction from those of (m, n).  Returns false where the fields are set
// otherwise: diff = 0 (both 0), or the slow path (exact, or 0 with *oor set when
// out of |c| < 2^20).
__device__ __forceinline__ bool coord_fields(float diff, double lambda, float2 scale, uint32_t* ff, uint32_t* fr,
                                             bool* oor) {
  if (diff == 0.f) {  // equal positions (the reference's zero-filled samples): 0 both ways
    *ff = *fr = 1048576u;
    return false;
  }
  float y;
  if (ceil_is_floor_plus_one(diff, scale, &y) && fabsf(y - 12582912.f) < 1048573.f) {
    *ff = (uint32_t)(__float_as_int(y) - 0x4b400000 + 1 + 1048576);
    return true;
  }
  const float a = ceil_quotient_exact(diff, lambda), b = ceil_quotient_exact(-diff, lambda);
  const bool ok = fabsf(a) < 1048576.f && fabsf(b) < 1048576.f;
  *oor |= !ok;
  *ff = ok ? (uint32_t)((int)a + 1048576) : 0u;
  *fr = ok ? (uint32_t)((int)b + 1048576) : 0u;
  return false;
}

// sum over the three fields of (2^21 + 1) * 2^(21 i): KEY_MIRROR - key mirrors every field
constexpr uint64_t KEY_MIRROR = 2097153ull * ((1ull << 42) + (1ull << 21) + 1ull);

// Keys of row (m, n) and, ordered, of row (n, m) from the baseline diffs d.
__device__ __forceinline__ void row_keys(const float* d, double lambda, float2 scale, int ordered, uint64_t* kf,
                                         uint64_t* kr, bool* oor) {
  uint32_t ff[3], fr[3];
  bool fc[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) fc[c] = coord_fields(d[c], lambda, scale, &ff[c], &fr[c], oor);
  *kf = ((uint64_t)ff[0] << 42) | ((uint64_t)ff[1] << 21) | (uint64_t)ff[2];
  if (!ordered) return;
  if (fc[0] && fc[1] && fc[2]) {
    *kr = KEY_MIRROR - *kf;
    return;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)  // fields of the slow coordinates are exact already
    if (fc[c]) fr[c] = 2097153u - ff[c];
  *kr = ((uint64_t)fr[0] << 42) | ((uint64_t)fr[1] << 21) | (uint64_t)fr[2];
}

__global__ void __launch_bounds__(256, 6) unique_insert_kernel(const float* __restrict__ pos, int64_t S, int nsat,
                                                            int ordered, int npairs, double lambda, float2 scale,
                                                            uint64_t* tkeys, uint32_t* tidx, uint64_t mask, int* bad,
                                                            int* overflow) {
  const int nup = nsat * (nsat - 1) / 2;  // satellite pairs m < n
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t chunk = t / nup;
  const int up = (int)(t - chunk * nup);
  const int64_t g0 = chunk * UNIQUE_RUN;
  if (g0 >= S) return;
  const int cnt = (int)(g0 + UNIQUE_RUN < S ? UNIQUE_RUN : S - g0);
  int m, n;
  pair_of(up, nsat, 0, &m, &n);
  // row offsets within a snapshot: (m, n) and, ordered, (n, m) (pair_of's order)
  const int qf = ordered ? m * (nsat - 1) + (n - 1) : up;
  const int qr = n * (nsat - 1) + m;
  const int stride = nsat * 3;
  const float* pm = pos + (g0 * nsat + m) * 3;
  const float* pn = pos + (g0 * nsat + n) * 3;
  const float* pend = pos + (g0 + cnt) * nsat * 3;  // prefetches stay inside the chunk
  // keys of the snapshot before the chunk: a row equal to it is no first occurrence
  uint64_t prevf = DEDUP_EMPTY, prevr = DEDUP_EMPTY;  // no key equals it (bit 63 is never set)
  bool oor = false;
  if (g0 > 0) {
    const float dp[3] = {__ldg(pn - stride) - __ldg(pm - stride), __ldg(pn - stride + 1) - __ldg(pm - stride + 1),
                         __ldg(pn - stride + 2) - __ldg(pm - stride + 2)};
    row_keys(dp, lambda, scale, ordered, &prevf, &prevr, &oor);
  }
  uint32_t rowf = (uint32_t)(qf * S + g0), rowr = (uint32_t)(qr * S + g0);
  // UNIQUE_BATCH snapshots' positions are loaded together.  The kernel runs at
  // 6 CTAs per SM (40 registers; 4 CTAs without spills measured 11% slower): a
  // batch of 4 spilled ~1.5x as much and took 10.2 ms on the MIncline campaign
  // against 9.8 ms for 1 or 2.
  for (int j0 = 0; j0 < cnt; j0 += UNIQUE_BATCH) {
    const float* ahead = pn + (j0 + 32) * stride;
    if (ahead < pend) asm volatile("prefetch.global.L2 [%0];" ::"l"(ahead));
    float d[UNIQUE_BATCH][3];
#pragma unroll
    for (int j = 0; j < UNIQUE_BATCH; ++j) {
      const int o = (j0 + j < cnt ? j0 + j : cnt - 1) * stride;
#pragma unroll
      for (int c = 0; c < 3; ++c) d[j][c] = __ldg(pn + o + c) - __ldg(pm + o + c);
    }
#pragma unroll
    for (int j = 0; j < UNIQUE_BATCH; ++j) {
      if (j0 + j >= cnt) break;
      uint64_t kf, kr;
      row_keys(d[j], lambda, scale, ordered, &kf, &kr, &oor);
      if (kf != prevf) dedup_insert_red(tkeys, tidx, mask, kf, rowf, overflow);
      prevf = kf;
      ++rowf;
      if (ordered) {
        if (kr != prevr) dedup_insert_red(tkeys, tidx, mask, kr, rowr, overflow);
        prevr = kr;
        ++rowr;
      }
    }
  }
  if (oor) atomicOr(bad, 1);
}

// occupied slots -> (key, first row) pairs, in any order (they are sorted next).
// A block takes COMPACT_SLOTS slots and one atomic on the counter.
constexpr int COMPACT_PER_THREAD = 16;
constexpr int COMPACT_SLOTS = 256 * COMPACT_PER_THREAD;

__global__ void __launch_bounds__(256) unique_compact_kernel(const uint64_t* tkeys, const uint32_t* tidx, int64_t T,
                                                             uint64_t* k1, uint32_t* i1,
                                                             unsigned long long* count) {
  __shared__ unsigned warp_sum[8];
  __shared__ unsigned long long block_base;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int64_t base = (int64_t)blockIdx.x * COMPACT_SLOTS + tid;
  uint64_t keys[COMPACT_PER_THREAD];
  unsigned mine = 0;
#pragma unroll
  for (int i = 0; i < COMPACT_PER_THREAD; ++i) {
    const int64_t sl = base + (int64_t)i * 256;
    keys[i] = sl < T ? tkeys[sl] : DEDUP_EMPTY;
    mine += keys[i] != DEDUP_EMPTY;
  }
  unsigned incl = mine;  // inclusive warp scan
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_sum[wid] = incl;
  __syncthreads();
  unsigned before = 0, total = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    before += w < wid ? warp_sum[w] : 0;
    total += warp_sum[w];
  }
  if (tid == 0) block_base = total ? atomicAdd(count, (unsigned long long)total) : 0ull;
  __syncthreads();
  unsigned long long at = block_base + before + incl - mine;
#pragma unroll
  for (int i = 0; i < COMPACT_PER_THREAD; ++i) {
    if (keys[i] != DEDUP_EMPTY) {
      k1[at] = keys[i];
      i1[at] = tidx[base + (int64_t)i * 256];
      ++at;
    }
  }
}

// sorted unique row indices -> their uvw, recomputed as the baselines kernel does
__global__ void unique_emit_kernel(const uint32_t* idx, const int64_t* n, const float* pos, int64_t S, int nsat,
                                   int ordered, double lambda, float2 scale, float* u, float* v, float* w) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *n) return;
  const int64_t r = idx[k];  // pair-major row q * S + g
  const int64_t q = r / S;
  const int64_t g = r - q * S;
  int m, nn;
  pair_of((int)q, nsat, ordered, &m, &nn);
  const float* pm = pos + (g * nsat + m) * 3;
  const float* pn = pos + (g * nsat + nn) * 3;
  u[k] = baseline_coord(pn[0] - pm[0], lambda, scale, 1);
  v[k] = baseline_coord(pn[1] - pm[1], lambda, scale, 1);
  w[k] = baseline_coord(pn[2] - pm[2], lambda, scale, 1);
}

__global__ void dedup_table_init_kernel(uint64_t* tkeys, uint32_t* tidx, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) { tkeys[t] = DEDUP_EMPTY; tidx[t] = 0xffffffffu; }
}

// sorted unique rows -> u, v, w (the first occurrence's values)
__global__ void dedup_emit_kernel(const uint32_t* idx, const int64_t* n, const float* u, const float* v,
                                  const float* w, float* ou, float* ov, float* ow) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= *n) return;
  const uint32_t s = idx[k];
  ou[k] = u[s]; ov[k] = v[s]; ow[k] = w[s];
}

struct DedupPlan {
  uint64_t *k0 = nullptr, *k1 = nullptr;
  uint32_t *i0 = nullptr, *i1 = nullptr;
  float *tu = nullptr, *tv = nullptr, *tw = nullptr;
  int* flag = nullptr;
  int* bad = nullptr;
  int64_t* nsel = nullptr;
  void* cub = nullptr;
  size_t cub_bytes = 0, bytes = 0;
  void layout(void* ws, int64_t K) {
    Carver c(ws);
    k0 = c.take<uint64_t>(K); k1 = c.take<uint64_t>(K);
    i0 = c.take<uint32_t>(K); i1 = c.take<uint32_t>(K);
    tu = c.take<float>(K); tv = c.take<float>(K); tw = c.take<float>(K);
    flag = c.take<int>(K);
    bad = c.take<int>(4);
    nsel = c.take<int64_t>(4);
    size_t a = 0, b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (uint64_t*)nullptr, (uint64_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, (int64_t)K, 0, 63);
    cub::DeviceSelect::Flagged(nullptr, b, (float*)nullptr, (int*)nullptr, (float*)nullptr, (int64_t*)nullptr,
                               (int64_t)K);
    cub_bytes = a > b ? a : b;
    cub = c.take<char>(cub_bytes);
    bytes = c.size();
  }
};

// 1e3 / lambda as a float pair hi + lo (to 2^-48)
inline float2 scale_pair(double lambda) {
  const double s = 1e3 / lambda;
  const float hi = (float)s;
  return make_float2(hi, (float)(s - (double)hi));
}

// Workspace of viss_unique_uvw: a table of up to T = 2K slots (pow2, 2^10 ..
// 2^28), the compacted (key, first row) pairs and the CUB scratch.
struct UniquePlan {
  int64_t T = 0;
  uint64_t *tkeys = nullptr, *k1 = nullptr;
  uint32_t *tidx = nullptr, *i1 = nullptr;
  int* bad = nullptr;
  int64_t* nsel = nullptr;
  void* cub = nullptr;
  size_t cub_bytes = 0, bytes = 0;
  void layout(void* ws, int64_t K) {
    T = 1024;
    while (T < 2 * K && T < ((int64_t)1 << 28)) T <<= 1;
    Carver c(ws);
    tkeys = c.take<uint64_t>(T); k1 = c.take<uint64_t>(T);
    tidx = c.take<uint32_t>(T); i1 = c.take<uint32_t>(T);
    bad = c.take<int>(4);
    nsel = c.take<int64_t>(4);
    cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, (uint64_t*)nullptr, (uint64_t*)nullptr, (uint32_t*)nullptr,
                                    (uint32_t*)nullptr, T, 0, 63);
    cub = c.take<char>(cub_bytes);
    bytes = c.size();
  }
};

}  // namespace viss

using namespace viss;

extern "C" {

int64_t viss_orbit_snapshots(const viss_orbit_cfg* cfg) {
  if (!cfg || cfg->orbit_res < 3 || cfg->orbit_counts < 1) return 0;
  return (int64_t)cfg->orbit_counts * (cfg->orbit_res / 3);
}

int viss_orbit_positions(const viss_orbit_cfg* cfg, float* pos, double* pos64, void* stream) {
  if (!cfg || !pos) return fail(VISS_ERR_INVALID, "cfg or pos NULL");
  if (cfg->nsat < 2 || cfg->nsat > 32) return fail(VISS_ERR_RANGE, "nsat must be in [2, 32]");
  if (cfg->orbit_res < 360 || cfg->orbit_counts < 1) return fail(VISS_ERR_RANGE, "orbit_res >= 360, orbit_counts >= 1");
  if ((int64_t)cfg->orbit_res * cfg->orbit_counts * (cfg->nsat + 1) >= ((int64_t)1 << 31))
    return fail(VISS_ERR_RANGE, "orbit_res * orbit_counts * nsat must fit the reference's int indices");
  if (!cfg->r1_m || !cfg->r2_m) return fail(VISS_ERR_INVALID, "r1_m / r2_m NULL");
  if (cfg->index < 1) return fail(VISS_ERR_RANGE, "index >= 1");
  OrbitDev o{};
  o.nsat = cfg->nsat; o.orbit_res = cfg->orbit_res; o.orbit_counts = cfg->orbit_counts; o.index = cfg->index;
  o.span = cfg->orbit_res / 3;
  o.interval = cfg->orbit_res / 360 * 10;
  o.total = cfg->orbit_res * cfg->orbit_counts;  // below 2^31 by the check above
  o.S = cfg->orbit_counts * o.span;
  o.half = o.total / 2;
  o.reset_index = o.total / (o.orbit_res + o.interval) + 1;
  o.by_span.set(o.span);
  o.by_res.set(o.orbit_res);
  o.by_nsat.set(o.nsat);
  o.d2r = (float)(kPi / 180);
  o.a = (float)cfg->a_km; o.e = (float)cfg->e;
  o.dm_den = (double)(2.0f * o.a) * 1e3;  // exact: 24-bit x 10-bit
  o.dm_hi = (float)o.dm_den;
  o.dm_lo = (float)(o.dm_den - (double)o.dm_hi);
  o.dm_inv = (float)(1.0 / o.dm_den);
  o.incl = (float)cfg->incl_deg * o.d2r;
  o.argp = (float)cfg->argp_deg * o.d2r;
  o.a64 = cfg->a_km; o.e64 = cfg->e; o.incl64 = cfg->incl_deg * kPi / 180.0; o.argp64 = cfg->argp_deg * kPi / 180.0;
  o.raan_step = cfg->raan_step_deg;
  o.step_mt = (float)(2 * kPi) / float(cfg->orbit_res - 1);
  o.fp64 = cfg->fp64;
  const int half = o.total / 2;
  if (half < 2) return fail(VISS_ERR_RANGE, "orbit too short");
  for (int s = 0; s < o.nsat; ++s) {
    o.r1[s] = cfg->r1_m[s];
    o.r2[s] = cfg->r2_m[s];
    o.s1[s] = (o.r2[s] - o.r1[s]) / float(half - 1);
    o.s2[s] = (o.r1[s] - o.r2[s]) / float(half - 1);
  }
  const int64_t n = (int64_t)o.S * o.nsat;
  if (n == 0) return VISS_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  orbit_positions_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(o, pos, pos64);
  VISS_LAUNCH_CHECK("orbit_positions_kernel");
  return VISS_OK;
}

int viss_baseline_uvw(const float* pos, const double* pos64, int64_t S, int32_t nsat, int ordered, double lambda_m,
                      int rounding, float* u, float* v, float* w, int32_t* snap, int32_t* pair, void* stream) {
  if ((!pos && !pos64) || !u || !v || !w) return fail(VISS_ERR_INVALID, "NULL argument");
  if (nsat < 2 || nsat > 32) return fail(VISS_ERR_RANGE, "nsat must be in [2, 32]");
  if (!(lambda_m > 0)) return fail(VISS_ERR_RANGE, "lambda must be > 0");
  if (S < 0) return fail(VISS_ERR_RANGE, "S < 0");
  const int npairs = ordered ? nsat * (nsat - 1) : nsat * (nsat - 1) / 2;
  const int64_t K = S * npairs;
  if (K == 0) return VISS_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t magic = ~0ull / (uint64_t)npairs + 1;
  baseline_uvw_kernel<<<(unsigned)((K + 255) / 256), 256, 0, st>>>(
      pos, pos64, S, nsat, ordered, npairs, magic, lambda_m, scale_pair(lambda_m), rounding, u, v, w, snap, pair);
  VISS_LAUNCH_CHECK("baseline_uvw_kernel");
  return VISS_OK;
}

size_t viss_dedup_uvw_workspace(int64_t K) {
  if (K <= 0) return 0;
  DedupPlan p;
  p.layout(nullptr, K);
  return p.bytes;
}

int viss_dedup_uvw(float* u, float* v, float* w, int64_t K, int64_t* count_out, void* workspace,
                   size_t workspace_bytes, void* stream) {
  if (!count_out) return fail(VISS_ERR_INVALID, "count_out NULL");
  if (K <= 0) { *count_out = 0; return VISS_OK; }
  if (K >= ((int64_t)1 << 32)) return fail(VISS_ERR_RANGE, "K too large");
  if (!u || !v || !w) return fail(VISS_ERR_INVALID, "u/v/w NULL");
  DedupPlan p;
  p.layout(nullptr, K);
  if (!workspace || workspace_bytes < p.bytes) return fail(VISS_ERR_WORKSPACE, "dedup workspace too small");
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return fail(VISS_ERR_WORKSPACE, "workspace misaligned");
  p.layout(workspace, K);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  VISS_CUDA(cudaMemsetAsync(p.bad, 0, 4 * sizeof(int), st));
  const unsigned nb = (unsigned)((K + 255) / 256);
  // Hash pass first, in the sort path's buffers: a table of T slots (keys in k0,
  // first indices in i0; T <= K, the buffers' length), from 2^25 slots up to 2^28
  // while it fills up.  The occupied slots (unique keys and their first rows) are
  // compacted into k1/i1, sorted by key back into k0/i0 and emitted.  A table that
  // stays full leaves the work to the sort over every row below.
  for (int64_t T = (int64_t)1 << 25, prev = 0; K >= 4096; prev = T, T <<= 3) {
    while (T > K) T >>= 1;
    if (T <= prev) break;
    dedup_table_init_kernel<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(p.k0, p.i0, T);
    VISS_LAUNCH_CHECK("dedup_table_init_kernel");
    dedup_hash_kernel<<<nb, 256, 0, st>>>(u, v, w, K, p.k0, p.i0, (uint64_t)(T - 1), p.bad, p.bad + 1);
    VISS_LAUNCH_CHECK("dedup_hash_kernel");
    int hb[2] = {0, 0};
    VISS_CUDA(cudaMemcpyAsync(hb, p.bad, sizeof(hb), cudaMemcpyDeviceToHost, st));
    VISS_CUDA(cudaStreamSynchronize(st));
    if (hb[0]) return fail(VISS_ERR_RANGE, "dedup needs integer-valued uvw with |x| < 2^20");
    if (!hb[1]) {
      VISS_CUDA(cudaMemsetAsync(p.nsel, 0, sizeof(int64_t), st));
      unique_compact_kernel<<<(unsigned)((T + COMPACT_SLOTS - 1) / COMPACT_SLOTS), 256, 0, st>>>(
          p.k0, p.i0, T, p.k1, p.i1, (unsigned long long*)p.nsel);
      VISS_LAUNCH_CHECK("unique_compact_kernel");
      int64_t n = 0;
      VISS_CUDA(cudaMemcpyAsync(&n, p.nsel, sizeof(n), cudaMemcpyDeviceToHost, st));
      VISS_CUDA(cudaStreamSynchronize(st));
      // unique keys: the sort's stability does not matter
      size_t cb = p.cub_bytes;
      VISS_CUDA(cub::DeviceRadixSort::SortPairs(p.cub, cb, p.k1, p.k0, p.i1, p.i0, n, 0, 63, st));
      if (n > 0) {
        dedup_emit_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p.i0, p.nsel, u, v, w, p.tu, p.tv, p.tw);
        VISS_LAUNCH_CHECK("dedup_emit_kernel");
        VISS_CUDA(cudaMemcpyAsync(u, p.tu, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
        VISS_CUDA(cudaMemcpyAsync(v, p.tv, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
        VISS_CUDA(cudaMemcpyAsync(w, p.tw, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
      }
      VISS_CUDA(cudaStreamSynchronize(st));
      *count_out = n;
      return VISS_OK;
    }
    VISS_CUDA(cudaMemsetAsync(p.bad, 0, 4 * sizeof(int), st));
    if (T >= ((int64_t)1 << 28)) break;
  }
  dedup_keys_kernel<<<nb, 256, 0, st>>>(u, v, w, K, p.k0, p.i0, p.bad);
  VISS_LAUNCH_CHECK("dedup_keys_kernel");
  // stable radix sort: among equal keys the first input occurrence stays first
  size_t cb = p.cub_bytes;
  VISS_CUDA(cub::DeviceRadixSort::SortPairs(p.cub, cb, p.k0, p.k1, p.i0, p.i1, K, 0, 63, st));
  dedup_gather_kernel<<<nb, 256, 0, st>>>(p.k1, p.i1, K, u, v, w, p.tu, p.tv, p.tw, p.flag);
  VISS_LAUNCH_CHECK("dedup_gather_kernel");
  float* src[3] = {p.tu, p.tv, p.tw};
  float* dst[3] = {u, v, w};
  for (int c = 0; c < 3; ++c) {
    cb = p.cub_bytes;
    VISS_CUDA(cub::DeviceSelect::Flagged(p.cub, cb, src[c], p.flag, dst[c], p.nsel, K, st));
  }
  int bad = 0;
  int64_t cnt = 0;
  VISS_CUDA(cudaMemcpyAsync(&bad, p.bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  VISS_CUDA(cudaMemcpyAsync(&cnt, p.nsel, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  VISS_CUDA(cudaStreamSynchronize(st));
  if (bad) return fail(VISS_ERR_RANGE, "dedup needs integer-valued uvw with |x| < 2^20");
  *count_out = cnt;
  return VISS_OK;
}

size_t viss_unique_uvw_workspace(int64_t S, int32_t nsat, int ordered) {
  if (S <= 0 || nsat < 2 || nsat > 32) return 0;
  UniquePlan p;
  p.layout(nullptr, S * (ordered ? nsat * (nsat - 1) : nsat * (nsat - 1) / 2));
  return p.bytes;
}

int viss_unique_uvw(const float* pos, int64_t S, int32_t nsat, int ordered, double lambda_m, float* u, float* v,
                    float* w, int64_t capacity, int64_t* count_out, void* workspace, size_t workspace_bytes,
                    void* stream) {
  if (!count_out) return fail(VISS_ERR_INVALID, "count_out NULL");
  *count_out = 0;
  if (nsat < 2 || nsat > 32) return fail(VISS_ERR_RANGE, "nsat must be in [2, 32]");
  if (!(lambda_m > 0)) return fail(VISS_ERR_RANGE, "lambda must be > 0");
  if (S < 0 || capacity < 0) return fail(VISS_ERR_RANGE, "S < 0 or capacity < 0");
  if (S == 0) return VISS_OK;
  if (!pos) return fail(VISS_ERR_INVALID, "pos NULL");
  if (capacity > 0 && (!u || !v || !w)) return fail(VISS_ERR_INVALID, "u/v/w NULL");
  const int npairs = ordered ? nsat * (nsat - 1) : nsat * (nsat - 1) / 2;
  const int64_t K = S * npairs;
  if (K >= ((int64_t)1 << 32)) return fail(VISS_ERR_RANGE, "S x pairs must be < 2^32");
  UniquePlan p;
  p.layout(nullptr, K);
  if (!workspace || workspace_bytes < p.bytes) return fail(VISS_ERR_WORKSPACE, "unique_uvw workspace too small");
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return fail(VISS_ERR_WORKSPACE, "workspace misaligned");
  p.layout(workspace, K);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const float2 scale = scale_pair(lambda_m);
  const int64_t threads = (S + UNIQUE_RUN - 1) / UNIQUE_RUN * (nsat * (nsat - 1) / 2);
  // a table of 2^25 slots first (the few tens of millions of unique rows of an
  // orbit campaign), the workspace's full table if that one fills
  int64_t n = 0;
  for (int64_t T = p.T < ((int64_t)1 << 25) ? p.T : ((int64_t)1 << 25);; T = p.T) {
    VISS_CUDA(cudaMemsetAsync(p.bad, 0, 4 * sizeof(int), st));
    VISS_CUDA(cudaMemsetAsync(p.nsel, 0, sizeof(int64_t), st));
    dedup_table_init_kernel<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(p.tkeys, p.tidx, T);
    VISS_LAUNCH_CHECK("dedup_table_init_kernel");
    unique_insert_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
        pos, S, nsat, ordered, npairs, lambda_m, scale, p.tkeys, p.tidx, (uint64_t)(T - 1), p.bad, p.bad + 1);
    VISS_LAUNCH_CHECK("unique_insert_kernel");
    unique_compact_kernel<<<(unsigned)((T + COMPACT_SLOTS - 1) / COMPACT_SLOTS), 256, 0, st>>>(
        p.tkeys, p.tidx, T, p.k1, p.i1, (unsigned long long*)p.nsel);
    VISS_LAUNCH_CHECK("unique_compact_kernel");
    int hb[2] = {0, 0};
    VISS_CUDA(cudaMemcpyAsync(hb, p.bad, sizeof(hb), cudaMemcpyDeviceToHost, st));
    VISS_CUDA(cudaMemcpyAsync(&n, p.nsel, sizeof(n), cudaMemcpyDeviceToHost, st));
    VISS_CUDA(cudaStreamSynchronize(st));
    if (hb[0]) return fail(VISS_ERR_RANGE, "uvw beyond |x| < 2^20 cannot be keyed");
    if (!hb[1]) break;
    if (T == p.T)
      return fail(VISS_ERR_RANGE, "more unique uvw than the table holds: use viss_baseline_uvw + viss_dedup_uvw");
  }
  *count_out = n;
  if (n > capacity) {
    if (capacity == 0) return VISS_OK;  // count only
    return fail(VISS_ERR_RANGE, "capacity below the unique count (in *count_out)");
  }
  // unique keys, sorted with their first rows back into the table's buffers
  size_t cb = p.cub_bytes;
  VISS_CUDA(cub::DeviceRadixSort::SortPairs(p.cub, cb, p.k1, p.tkeys, p.i1, p.tidx, n, 0, 63, st));
  if (n > 0) {
    unique_emit_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(p.tidx, p.nsel, pos, S, nsat, ordered,
                                                                    lambda_m, scale, u, v, w);
    VISS_LAUNCH_CHECK("unique_emit_kernel");
  }
  return VISS_OK;
}

}  // extern "C"
