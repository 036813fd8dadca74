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

struct OrbitDev {
  int nsat, orbit_res, orbit_counts, index;
  int span, interval;
  int64_t total, S;
  float a, e, incl, argp, d2r;
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
__device__ __forceinline__ int window_index(const OrbitDev& o, int64_t g, int64_t* circle) {
  const int64_t k = g / o.span + 1;
  const int64_t offset = (k - 1) * o.interval;
  int64_t endIdx = (k - 1) * o.orbit_res + offset + o.span;
  int64_t startIdx = (k - 1) * o.orbit_res + offset;
  if ((k - 1) * (int64_t)(o.orbit_res + o.interval) > o.total) {
    const int64_t reset_index = o.total / (o.orbit_res + o.interval) + 1;
    startIdx = (k - 1 - reset_index) * o.orbit_res + offset;
    endIdx = (k - 1 - reset_index) * o.orbit_res + offset + o.span;
  }
  const int64_t c = startIdx + (g - (k - 1) * o.span);
  *circle = c;
  if (endIdx > o.total) {
    if (c > o.total) return 1;
    if (c == o.total) return 2;
  }
  return 0;
}

// calculateOrbit (:83-110) in the reference's arithmetic.
__device__ void position_f32(const OrbitDev& o, int sat, int64_t idx, float* out) {
  const int64_t half = o.total / 2;
  const int k = (int)(idx / o.orbit_res), po = (int)(idx % o.orbit_res);
  float d;
  if (idx < half) d = fmaf(o.s1[sat], (float)idx, o.r1[sat]);   // linspace r1 -> r2 (:42-49)
  else d = fmaf(o.s2[sat], (float)(idx - half), o.r2[sat]);     // linspace r2 -> r1
  const float dM = (float)(asin((double)d / ((double)(2 * o.a) * 1e3)) * 2);  // calculate_dM (:51-58)
  const float raan = (float)((double)((float)k * o.d2r) * o.raan_step + 0.0 +
                             (double)((float)((o.index - 1) * o.orbit_counts) * o.d2r) * o.raan_step);
  // Mt[po] is rounded on its own (thrust linspace with a = 0), then dM is added
  const float M = __fmul_rn(o.step_mt, (float)po) + dM;
  float E0 = M;
  for (int i = 1; i < 100; ++i) {
    const float M0 = E0 - o.e * sinf(E0);
    const float err = M - M0;
    if (fabsf(err) < 1e-15) break;
    E0 = E0 + err / (1 - o.e * cosf(E0));
  }
  const float temp = tanf(E0 / 2) / sqrtf((1 - o.e) / (1 + o.e));
  const float theta = atanf(temp) * 2;
  const float r = o.a * (1 - o.e * o.e) / (1 + o.e * cosf(theta));
  const float w = theta + o.argp;
  out[0] = r * (cosf(w) * cosf(raan) - sinf(w) * cosf(o.incl) * sinf(raan));
  out[1] = r * (cosf(w) * sinf(raan) + sinf(w) * cosf(o.incl) * cosf(raan));
  out[2] = r * (sinf(w) * sinf(o.incl));
}

__device__ void position_f64(const OrbitDev& o, int sat, int64_t idx, double* out) {
  const int64_t half = o.total / 2;
  const int64_t k = idx / o.orbit_res, po = idx % o.orbit_res;
  const double d2r = kPi / 180.0;
  const double r1 = o.r1[sat], r2 = o.r2[sat];
  double d;
  if (idx < half) d = r1 + (r2 - r1) / (double)(half - 1) * (double)idx;
  else d = r2 + (r1 - r2) / (double)(half - 1) * (double)(idx - half);
  const double dM = 2.0 * asin(d / (2.0 * o.a64 * 1e3));
  const double raan = (double)k * d2r * o.raan_step + (double)(o.index - 1) * (double)o.orbit_counts * d2r * o.raan_step;
  const double M = 2.0 * kPi / (double)(o.orbit_res - 1) * (double)po + dM;
  double E = M;
  for (int i = 1; i < 100 && o.e64 != 0.0; ++i) {
    const double err = M - (E - o.e64 * sin(E));
    if (fabs(err) < 1e-15) break;
    E = E + err / (1.0 - o.e64 * cos(E));
  }
  const double theta = 2.0 * atan(tan(E / 2.0) / sqrt((1.0 - o.e64) / (1.0 + o.e64)));
  const double r = o.a64 * (1.0 - o.e64 * o.e64) / (1.0 + o.e64 * cos(theta));
  const double w = theta + o.argp64;
  out[0] = r * (cos(w) * cos(raan) - sin(w) * cos(o.incl64) * sin(raan));
  out[1] = r * (cos(w) * sin(raan) + sin(w) * cos(o.incl64) * cos(raan));
  out[2] = r * (sin(w) * sin(o.incl64));
}

__global__ void orbit_positions_kernel(const OrbitDev o, float* pos, double* pos64) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= o.S * o.nsat) return;
  const int64_t g = t / o.nsat;
  const int sat = (int)(t % o.nsat);
  int64_t circle;
  const int kind = window_index(o, g, &circle);
  const bool zero = kind != 0;
  if (o.fp64) {
    double p[3] = {0.0, 0.0, 0.0};
    if (!zero) position_f64(o, sat, circle, p);
    pos[3 * t] = (float)p[0]; pos[3 * t + 1] = (float)p[1]; pos[3 * t + 2] = (float)p[2];
    if (pos64) { pos64[3 * t] = p[0]; pos64[3 * t + 1] = p[1]; pos64[3 * t + 2] = p[2]; }
  } else {
    float p[3] = {0.f, 0.f, 0.f};
    if (!zero) position_f32(o, sat, circle, p);
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

__global__ void baseline_uvw_kernel(const float* pos, const double* pos64, int64_t S, int nsat, int ordered, int npairs,
                                    uint64_t pair_magic, double lambda, float scale32, int rounding, float* u,
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
    const float diff = pos[(g * nsat + n) * 3 + c] - pos[(g * nsat + m) * 3 + c];
    if (!rounding) {
      out[c] = (float)((double)diff * 1e3 / lambda);  // computeUVW without the ceil
      continue;
    }
    // computeUVW (:156-158): ceil((double)diff * 1e3 / lambda).  The FP32 product
    // x = diff * fl(1e3 / lambda) is within 2^-23 |x| of the quotient; where x lies
    // more than 2^-21 |x| inside (n, n + 1) the quotient and its double rounding
    // do too, so ceilf(x) is the same integer (and sign of zero).  Elsewhere, and
    // for |x| >= 2^22 where x - floor(x) stops being exact, divide in double.
    const float x = diff * scale32;
    const float f = x - floorf(x);
    const float tol = fabsf(x) * 4.76837158203125e-7f + 1e-30f;
    out[c] = (fabsf(x) < 4194304.f && f > tol && 1.f - f > tol) ? ceilf(x) : ceil_quotient_exact(diff, lambda);
  }
  u[k] = out[0]; v[k] = out[1]; w[k] = out[2];
  if (snap) snap[k] = (int32_t)g;
  if (pair) pair[k] = m | (n << 16);
}

// ---------------------------------------------------------------- dedup
// Integer-valued uvw -> 63-bit key preserving the lexicographic (u, v, w)
// order of SortCompare (:60-71); -0 and +0 share a key as they compare equal.
__global__ void dedup_keys_kernel(const float* u, const float* v, const float* w, int64_t K, uint64_t* keys,
                                  uint32_t* idx, int* bad) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const float c[3] = {u[k], v[k], w[k]};
  uint64_t key = 0;
  for (int i = 0; i < 3; ++i) {
    const float x = c[i];
    if (!(x == rintf(x)) || !(fabsf(x) < 1048576.f)) { atomicOr(bad, 1); }
    const int64_t q = (int64_t)x + 1048576;
    key = (key << 21) | ((uint64_t)q & 0x1fffff);
  }
  keys[k] = key;
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

__global__ void dedup_hash_kernel(const float* u, const float* v, const float* w, int64_t K, uint64_t* tkeys,
                                  uint32_t* tidx, uint64_t mask, int* bad, int* overflow) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const float c[3] = {u[k], v[k], w[k]};
  uint64_t key = 0;
  for (int i = 0; i < 3; ++i) {
    const float x = c[i];
    if (!(x == rintf(x)) || !(fabsf(x) < 1048576.f)) { atomicOr(bad, 1); }
    const int64_t q = (int64_t)x + 1048576;
    key = (key << 21) | ((uint64_t)q & 0x1fffff);
  }
  uint64_t h = dedup_hash(key) & mask;
  for (int probe = 0; probe < DEDUP_PROBES; ++probe, h = (h + 1) & mask) {
    uint64_t cur = *((volatile uint64_t*)(tkeys + h));
    if (cur == DEDUP_EMPTY) {
      cur = atomicCAS((unsigned long long*)(tkeys + h), (unsigned long long)DEDUP_EMPTY, (unsigned long long)key);
      if (cur == DEDUP_EMPTY) cur = key;
    }
    if (cur == key) {
      if (*((volatile uint32_t*)(tidx + h)) > (uint32_t)k) atomicMin(tidx + h, (uint32_t)k);
      return;
    }
  }
  atomicOr(overflow, 1);
}

__global__ void dedup_table_init_kernel(uint64_t* tkeys, uint32_t* tidx, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) { tkeys[t] = DEDUP_EMPTY; tidx[t] = 0xffffffffu; }
}

__global__ void dedup_occupied_kernel(const uint64_t* tkeys, int64_t n, int* flag) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) flag[t] = tkeys[t] != DEDUP_EMPTY;
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
    size_t c2 = 0, c3 = 0;
    cub::DeviceSelect::Flagged(nullptr, c2, (uint64_t*)nullptr, (int*)nullptr, (uint64_t*)nullptr,
                               (int64_t*)nullptr, (int64_t)K);
    cub::DeviceSelect::Flagged(nullptr, c3, (uint32_t*)nullptr, (int*)nullptr, (uint32_t*)nullptr,
                               (int64_t*)nullptr, (int64_t)K);
    cub_bytes = a > b ? a : b;
    if (c2 > cub_bytes) cub_bytes = c2;
    if (c3 > cub_bytes) cub_bytes = c3;
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
  o.total = (int64_t)cfg->orbit_res * cfg->orbit_counts;
  o.S = (int64_t)cfg->orbit_counts * o.span;
  o.d2r = (float)(kPi / 180);
  o.a = (float)cfg->a_km; o.e = (float)cfg->e;
  o.incl = (float)cfg->incl_deg * o.d2r;
  o.argp = (float)cfg->argp_deg * o.d2r;
  o.a64 = cfg->a_km; o.e64 = cfg->e; o.incl64 = cfg->incl_deg * kPi / 180.0; o.argp64 = cfg->argp_deg * kPi / 180.0;
  o.raan_step = cfg->raan_step_deg;
  o.step_mt = (float)(2 * kPi) / float(cfg->orbit_res - 1);
  o.fp64 = cfg->fp64;
  const int64_t half = o.total / 2;
  if (half < 2) return fail(VISS_ERR_RANGE, "orbit too short");
  for (int s = 0; s < o.nsat; ++s) {
    o.r1[s] = cfg->r1_m[s];
    o.r2[s] = cfg->r2_m[s];
    o.s1[s] = (o.r2[s] - o.r1[s]) / float(half - 1);
    o.s2[s] = (o.r1[s] - o.r2[s]) / float(half - 1);
  }
  const int64_t n = o.S * o.nsat;
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
      pos, pos64, S, nsat, ordered, npairs, magic, lambda_m, (float)(1e3 / lambda_m), rounding, u, v, w, snap, pair);
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
      dedup_occupied_kernel<<<(unsigned)((T + 255) / 256), 256, 0, st>>>(p.k0, T, p.flag);
      VISS_LAUNCH_CHECK("dedup_occupied_kernel");
      size_t cb = p.cub_bytes;
      VISS_CUDA(cub::DeviceSelect::Flagged(p.cub, cb, p.k0, p.flag, p.k1, p.nsel, T, st));
      cb = p.cub_bytes;
      VISS_CUDA(cub::DeviceSelect::Flagged(p.cub, cb, p.i0, p.flag, p.i1, p.nsel, T, st));
      int64_t n = 0;
      VISS_CUDA(cudaMemcpyAsync(&n, p.nsel, sizeof(n), cudaMemcpyDeviceToHost, st));
      VISS_CUDA(cudaStreamSynchronize(st));
      // unique keys: the sort's stability does not matter
      cb = p.cub_bytes;
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

}  // extern "C"
