// viss_internal.cuh -- shared definitions of the libvissgb.so kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>

#include "viss_gb300.h"

namespace viss {

// ------------------------------------------------------------------ errors
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
void count_launch();

#define VISS_CUDA(call)                                      \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ::viss::cuda_fail(e_, #call); \
  } while (0)

#define VISS_LAUNCH_CHECK(what)                              \
  do {                                                       \
    cudaError_t e_ = cudaGetLastError();                     \
    if (e_ != cudaSuccess) return ::viss::cuda_fail(e_, what); \
    ::viss::count_launch();                                  \
  } while (0)

// --------------------------------------------------------------- workspace
// Carves 256-byte aligned sub-buffers out of one caller workspace.  With
// base == nullptr it only measures.
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base(static_cast<char*>(b)) {}
  template <class T>
  T* take(size_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += count * sizeof(T);
    return p;
  }
  size_t size() const { return (off + 255) & ~size_t(255); }
};

// ------------------------------------------------------------- constants
constexpr double kPi = 3.14159265358979323846;
// fmaf(f, K2PI, KM3PI) maps f in [1,2) to [-pi, pi) with one rounding.  KM3PI
// is -1.5*K2PI rounded to float; its rounding (a constant rotation) is removed
// in the integer phase: PHASE_BIAS = 2^8 (rounds the 9 bits dropped by
// turns_to_angle to nearest) minus that rotation in units of 2^-32 turns.
constexpr float K2PI = 6.28318548f;
constexpr float KM3PI = -1.5f * K2PI;
constexpr double kRotTurns = ((double)KM3PI + 1.5 * (double)K2PI) / (double)K2PI;
constexpr int32_t PHASE_BIAS =
    256 - (int32_t)(kRotTurns * 4294967296.0 + (kRotTurns >= 0 ? 0.5 : -0.5));

// Sizes of the tiled kernels.
constexpr int VIS_THREADS = 256;
constexpr int VIS_TK = 4;                 // visibilities per thread
constexpr int VIS_ROWS = VIS_THREADS * VIS_TK;
constexpr int VIS_P = 512;                // pixels per shared-memory tile
constexpr int REC_THREADS = 256;
constexpr int REC_TJ = 4;                 // pixels per thread
constexpr int REC_PIX = REC_THREADS * REC_TJ;
constexpr int REC_Q = 256;                // visibilities per shared-memory tile

// Resident CTAs per SM the tiled kernels are compiled for (register budget
// 65536 / (256 * n)).
#ifndef VISS_VIS_MINB
#define VISS_VIS_MINB 3
#endif
#ifndef VISS_REC_MINB
#define VISS_REC_MINB 3
#endif

// Geometric test: |e| below this margin is re-decided in double.
constexpr float GEO_EPS = 2e-6f;

enum PixClass : int { CLS_VIS = 0, CLS_OCC = 1, CLS_MIX = 2 };

// ----------------------------------------------------- fixed-point phase
// A pixel coordinate x (turns per wavelength) is held as
//   A  = round(x * 2^32) mod 2^32  -- the integer part of u multiplies it exactly mod 1 turn
//   A' = round(x * 2^30)           -- for the fractional part of u (|x| < 2)
//   lo = x - A*2^-32 (float)       -- compensation of the rounding of A
// A visibility coordinate u is split u = U + f, U = floor(u + 1/2), f in [-1/2, 1/2).
// Phase (turns * 2^32, mod 2^32) = U*A + V*B + W*C + bias_k + frac, where the
// fractional part delta = f_u*x + f_v*y + f_w*z' (FP32, |delta| < 2, z' = s*n) is
// folded in with one FADD: the bits of (delta + 6.0f) hold delta in units of
// 2^-21 turns above the constant 0x40C00000, whose shift by 11 vanishes mod 2^32,
// so frac = bits(delta + 6) << 11.  bias_k carries f_w*s*n_offset.
__device__ __forceinline__ uint32_t fix32(double x) {
  return (uint32_t)(unsigned long long)llrint(x * 4294967296.0);
}

// Turns (as uint32 mod 2^32, PHASE_BIAS already added) -> angle in [-pi, pi)
// shifted by half a turn: returns x = 2 pi (t - 1/2), so cos/sin come out negated.
__device__ __forceinline__ float turns_to_angle(uint32_t q) {
  const float f = __uint_as_float((q >> 9) | 0x3f800000u);
  return fmaf(f, K2PI, KM3PI);
}

// delta (turns, |delta| < 2) -> its fixed-point phase contribution (units 2^-32, resolution 2^-21)
__device__ __forceinline__ uint32_t frac_phase(float delta) {
  return __float_as_uint(delta + 6.0f) << 11;
}

// Satellite indices of a visibility (geometric mask): gm = snapshot*nsat + m in the
// low 26 bits, n - m + 32 in the top 6.
__device__ __forceinline__ int sat_gm(int packed) { return packed & 0x3ffffff; }
__device__ __forceinline__ int sat_gn(int packed) { return (packed & 0x3ffffff) + (int)((uint32_t)packed >> 26) - 32; }

// s += x with the rounding error of the sum carried in c (Kahan).
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// Exact geometric predicate in double, same operation order as the oracle.
__device__ __forceinline__ bool geo_occluded_exact(float sx_, float sy_, float sz_, const float* p,
                                                   double R) {
  const double sx = sx_, sy = sy_, sz = sz_;
  const double px = p[0], py = p[1], pz = p[2];
  const double b = __dadd_rn(__dadd_rn(__dmul_rn(sx, px), __dmul_rn(sy, py)), __dmul_rn(sz, pz));
  const double a = __dadd_rn(__dadd_rn(__dmul_rn(sx, sx), __dmul_rn(sy, sy)), __dmul_rn(sz, sz));
  const double pp = __dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz));
  const double c = __dsub_rn(pp, __dmul_rn(R, R));
  const double disc = __dsub_rn(__dmul_rn(b, b), __dmul_rn(a, c));
  return (b < 0.0) && (disc > 0.0);
}

// -------------------------------------------------------- kernel params
struct PixPrepArgs {
  const int32_t* perm;  // position -> pixel (NULL: identity)
  const float* l;
  const float* m;
  const float* n;
  const float* bright;
  int64_t J, Jpad;
  double sl, sm, sn, n_offset;
  int res;
  int trunc;
  int4* rec0;     // {A, B, C, bright bits}
  int4* rec1;     // {x, y, s*n (float bits), j}
  float4* lo;     // {a_lo, b_lo, c_lo, 0}
  float4* geo;    // {unit s, j bits}
  int2* qr;       // {j / res, j % res}
};

struct RowPrepArgs {
  double sn, n_offset;   // z = sn * (n + n_offset): the f_w * sn * n_offset part goes to the row bias
  const float* u;
  const float* v;
  const float* w;
  const float* wgt;
  const float* V;        // recon: K x 2
  const int32_t* shade;  // K x 4
  const int32_t* snap;
  const int32_t* pair;
  int nsat;
  int64_t S;
  int64_t K, Kpad;
  int mask_mode;
  int recon_mask;
  int4* rec0;   // {U, V, W, packed satellite indices}
  int4* rec1;   // {f_u, f_v, f_w (float bits), phase bias}
  float4* uf;   // {U, V, W as float, 0}   (compensation)
  int4* win;    // vis REF: {lo_a, lo_b, M1, M2}; recon REF: {tmax, pmax, 0, 0}
  float2* y;    // recon: wgt * V
  int* flags;   // [0] |= any fractional uvw, [1] |= |U| out of range
};

struct VisParams {
  const int4* pix0;
  const int4* pix1;
  const float4* plo;
  const float4* pgeo;
  const int2* pqr;
  const int4* rows0;
  const int4* rows1;
  const float4* rowsf;
  const int4* win;
  const float4* satdir;   // [S*nsat] {p_hat, cos_alpha}
  const float4* cones;    // [nrb*2]
  const float* l;
  const float* m;
  const float* n;
  const float* sat_pos;
  const int* flags;
  float2* out;            // partial [nsplit][K] or final [K]
  int64_t K, J;
  int64_t jchunk;
  int nsplit;
  int res;
  float occ_val;
  double R;
  int mask;               // VISS_MASK_*
};

struct ReconParams {
  const int4* pix0;
  const int4* pix1;
  const float4* plo;
  const float4* pgeo;
  const int2* pqr;
  const int4* rows0;
  const int4* rows1;
  const float4* rowsf;
  const int4* win;
  const float2* y;
  const float4* satdir;
  const float4* scones;   // [S*2] per-snapshot cones
  const float* l;
  const float* m;
  const float* n;
  const float* sat_pos;
  const int* flags;
  const int32_t* perm;    // position -> pixel (NULL: identity)
  float2* out;            // partial [nsplit][J] by position, or final F by pixel
  int64_t K, J;
  int64_t kchunk;
  int nsplit;
  int res;
  int nsat;
  double R;
  float norm;
  int recon_mask;
};

// ------------------------------------------------------------- launchers
int launch_prep_pixels(const PixPrepArgs& a, cudaStream_t st);
int launch_pixel_keys(const float* l, const float* m, const float* n, int64_t J, uint32_t* keys, int32_t* idx,
                      cudaStream_t st);
// Spatial permutation of the sky (keys, then a stable radix sort); scratch from
// the caller's workspace.  perm[pos] = pixel.
size_t pixel_order_scratch(int64_t J);
int pixel_order(const float* l, const float* m, const float* n, int64_t J, void* scratch, size_t scratch_bytes,
                int32_t* perm, cudaStream_t st);
int launch_prep_rows(const RowPrepArgs& a, bool recon, cudaStream_t st);
int launch_prep_satdir(const float* sat_pos, int64_t nsd, double R, float4* satdir, cudaStream_t st);
int launch_prep_rowblock_cones(const int4* rows0, const int4* rows1, const float4* satdir, int64_t K,
                               int rows_per_block, int64_t nblocks, float4* cones, cudaStream_t st);
int launch_prep_snapshot_cones(const float4* satdir, int64_t S, int nsat, float4* cones, cudaStream_t st);

int launch_vis_fast(const VisParams& p, int64_t nrb, bool compensated, cudaStream_t st);
int launch_vis_reduce(const float2* partial, int nsplit, int64_t K, float2* out, cudaStream_t st);
int launch_vis_plain(const viss_dft_cfg& cfg, const viss_sky& sky, const viss_vis_set& vis,
                     const viss_geometry* geo, const float4* satdir, const float* dlmn, float2* out, cudaStream_t st);

int launch_recon_fast(const ReconParams& p, int64_t npb, bool compensated, cudaStream_t st);
int launch_recon_reduce(const float2* partial, int nsplit, int64_t J, float norm, const int32_t* perm, float2* out,
                        cudaStream_t st);
int launch_recon_plain(const viss_dft_cfg& cfg, const viss_sky& sky, const viss_vis_set& vis,
                       const viss_geometry* geo, const float* V, const float* ratios, const float4* satdir,
                       const float* dlmn, float2* out, cudaStream_t st);

// Fast geometric test of direction s (need not be unit) against satellite
// direction d = {p_hat, cos alpha}: s_hat.p_hat + cos(alpha) < 0, decided in
// double (from the original inputs) within GEO_EPS of the limb.
__device__ __forceinline__ bool geo_test_plain(float sx, float sy, float sz, const float4& d, const float* pos,
                                               double R) {
  const float inv = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
  const float e = fmaf(sx * inv, d.x, fmaf(sy * inv, d.y, fmaf(sz * inv, d.z, d.w)));
  if (fabsf(e) >= 4.0f * GEO_EPS) return e < 0.f;
  return geo_occluded_exact(sx, sy, sz, pos, R);
}

int device_sm_count();

}  // namespace viss
