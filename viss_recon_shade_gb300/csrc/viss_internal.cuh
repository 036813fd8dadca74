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
// Geometric mask: occlusion bits of a tile's straddling pixels against every
// satellite its rowblock uses, in shared memory (satellites x 32-pixel words).
constexpr int VIS_SAT_WORDS = 5120;
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

// Channels of one batched pass, and visibility segments of its reconstruction
// (their tables travel in the kernel parameters).
constexpr int VISS_MAX_CH = VISS_MAX_CHANNELS;
constexpr int VISS_MAX_SEG = 256;

// Precisions served by the one-thread-per-item kernels (the reference's plain
// method, and the FP64-phase arm of precision sweeps).
inline bool plain_precision(int p) { return p == VISS_PREC_PLAIN || p == VISS_PREC_F64_PHASE; }

// Geometric test: |e| below this margin is re-decided in double.
constexpr float GEO_EPS = 2e-6f;

enum PixClass : int { CLS_VIS = 0, CLS_OCC = 1, CLS_MIX = 2 };

// ----------------------------------------------------- fixed-point phase
// A pixel coordinate x (turns per wavelength) is held as
//   A  = round(x * 2^32) mod 2^32  -- the integer part of u multiplies it exactly mod 1 turn
//   A' = round(x * 2^30)           -- for the fractional part of u (|x| < 2)
//   lo = x - A*2^-32 (float)       -- compensation of the rounding of A
// A visibility coordinate u is split u = U + f, U = floor(u + 1/2), f in [-1/2, 1/2).
// Phase (turns * 2^32, mod 2^32) = U*A + V*B + W*C + bias_k; bias_k carries
// PHASE_BIAS, f_w*s*n_offset and (reconstruction) the phase of the row's
// visibility.  The fractional part delta = f_u*x + f_v*y + f_w*z' (FP32, z' = s*n,
// |delta| <= 0.87 turn) and the compensation terms are evaluated in radians (the
// row coefficients carry the 2 pi) on top of the angle's constant, and enter with
// the FFMA that converts the fixed-point turn.
__device__ __forceinline__ uint32_t fix32(double x) {
  return (uint32_t)(unsigned long long)llrint(x * 4294967296.0);
}

// Turns (as uint32 mod 2^32, PHASE_BIAS already added) -> angle shifted by half a
// turn, x = 2 pi (t - 1/2) + (e - KM3PI), so cos/sin come out negated.  e is
// KM3PI plus the FP32 parts of the phase in radians (fractional uvw, compensation),
// summed onto the constant so the conversion and the addition share one FFMA.
__device__ __forceinline__ float turns_to_angle(uint32_t q, float e) {
  const float f = __uint_as_float((q >> 9) | 0x3f800000u);
  return fmaf(f, K2PI, e);
}

// Satellite indices of a visibility (geometric mask): gm = snapshot*nsat + m in the
// low 26 bits, n - m + 32 in the top 6.  Padding rows carry PAD_PACKED (both
// indices 0, always in range).
constexpr int PAD_PACKED = 32 << 26;
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
  int2* qr;       // {i / res, i % res} of the fine index i the REF windows test
  const int32_t* widx;  // i = widx[j] (NULL: i = j)
};

// Visibility rows of a (batched) pass: channel c owns input rows
// [row_off[c], row_off[c+1]).  The vis pass pads every channel to whole blocks
// of VIS_ROWS rows: its padded blocks are [rb_off[c], rb_off[c+1]).
struct ChannelRows {
  int nch;
  int64_t rb_off[VISS_MAX_CH + 1];
  int64_t row_off[VISS_MAX_CH + 1];
};

// Row records (both passes):
//   rows0 {U, V, W, bias}            integer uvw and the fixed-point phase bias
//   rows1 {f_u, f_v, f_w, c}         fractional uvw; c = |wgt V| (recon) or 0 (vis)
//   rowsat packed satellite indices  (geometric mask)
//   rowsf {U, V, W as float, 0}      (compensation)
//   win                              vis REF: {lo_a, lo_b, M1, M2}; recon REF: {tmax, pmax, 0, 0}
struct RowPrepArgs {
  double sn, n_offset;   // z = sn * (n + n_offset): the f_w * sn * n_offset part goes to the row bias
  ChannelRows ch;        // padded (vis): row pr of block b of channel c is input row
  bool padded;           //   row_off[c] + pr - rb_off[c]*VIS_ROWS when below row_off[c+1]
  const float* u;
  const float* v;
  const float* w;
  const float* wgt;
  const float* V;        // recon: K x 2, folded into bias and c
  const int32_t* shade;  // K x 4
  const int32_t* snap;
  const int32_t* pair;
  int nsat;
  int64_t S;
  int64_t K, Kpad;
  int mask_mode;
  int recon_mask;
  int4* rows0;
  float4* rows1;
  int* rowsat;
  float4* uf;
  int4* win;
  int* flags;   // [0] |= any fractional uvw, [1] |= |U| out of range, |= 2 bad satellite index
};

// flags words of a pass
// flag words at the start of every pass's workspace; FLAG_LIMB (words 2-3) counts,
// as one 64-bit integer, the geometric decisions settled in double near the limb
constexpr int FLAG_FRAC = 0, FLAG_ERR = 1, FLAG_LIMB = 2, FLAG_VIS_COUNTER = 8, FLAG_REC_COUNTER = 9,
              FLAG_WORDS = 64;

__device__ __forceinline__ void count_limb(int* flags) {
  if (flags) atomicAdd(reinterpret_cast<unsigned long long*>(flags + FLAG_LIMB), 1ull);
}

// A fine sky grid mapped onto the coarse pixels: pixel (position) j has
// members[start_j .. start_j + cnt_j), fine indices as the reference reads them
// (NXq[c] truncated to an integer).
struct FineMapDev {
  const int4* box;        // [Jpad] {qmin, qmax, rmin, rmax}: rows/columns (i / res, i % res) of the members
  const int2* mem;        // [Jpad] {start, cnt}
  const int* members;     // [X]
  const float* FF;        // [X] fine brightness
  const int2* tile_rng;   // [Jpad / VIS_P] {min, max} member fine index of each pixel tile
  int trunc;              // int truncation of FF (the plain reference variant)
};

struct VisParams {
  const int4* pix0;
  const int4* pix1;
  const float4* plo;
  const float4* pgeo;
  const int2* pqr;
  const int4* rows0;
  const float4* rows1;
  const int* rowsat;
  const float4* rowsf;
  const int4* win;
  const float4* satdir;   // [S*nsat] {p_hat, cos_alpha}
  const float4* cones;    // [nrb*2]; cones[2b+1].y/.z: the block's first satellite and span (int bits)
  const float* l;
  const float* m;
  const float* n;
  const float* sat_pos;
  const float* bright;    // [nch][J] per-channel brightness, or NULL (pixel records carry it)
  int* flags;             // flags[FLAG_VIS_COUNTER]: next work item
  float2* out;            // partial [nsplit][K] or final [K] (K = all channels' visibilities)
  int64_t K, J;
  int64_t jchunk;
  int nsplit;
  int nitems;             // work items (rowblock, pixel chunk) = nrb * nsplit
  int res;
  int nsat;               // satellites per snapshot (geometric)
  float occ_val;
  double R;
  int mask;               // VISS_MASK_*
  ChannelRows ch;
  // non-identity fine->coarse map (REF masks): a pixel's brightness for row k is
  // the mean over its fine members, each replaced by the occluded value inside
  // k's window (vissGen10M_shade.cu:120-136)
  FineMapDev map;
  const int2* ref_rng;    // per VIS_P positions: {min, max} fine index the REF windows test (NULL: the positions)
  int use_map;            // 0: identity map
  int small_tile;         // sky tiles of VIS_P / 2 pixels
};

struct ReconParams {
  const int4* pix0;
  const int4* pix1;
  const float4* plo;
  const float4* pgeo;
  const int2* pqr;
  const int4* rows0;
  const float4* rows1;
  const int* rowsat;
  const float4* rowsf;
  const int4* win;
  const float4* satdir;
  const float4* scones;   // [S*2] per-snapshot cones
  const float4* bcones;   // [npb*2] bounding cone of each pixel block: {axis, cos r}, {sin r}
  const float4* wcones;   // [npb*2*REC_THREADS/32] the same per warp's patch of 32*REC_TJ positions
  const float* l;
  const float* m;
  const float* n;
  const float* sat_pos;
  int* flags;             // flags[FLAG_REC_COUNTER]: next work item
  const int32_t* perm;    // position -> pixel (NULL: identity)
  float2* out;            // F [nch][J] by pixel
  float2* partial;        // [nslot][J] by position (segments that share a channel)
  int64_t K, J;
  int res;
  int nsat;
  double R;
  int recon_mask;
  // work items (segment, pixel block): segments are row ranges of one channel,
  // longest first; item i is segment i / npb, pixel block i % npb
  int nitems;
  int npb;
  int nseg;
  int64_t seg_lo[VISS_MAX_SEG], seg_hi[VISS_MAX_SEG];
  int seg_ch[VISS_MAX_SEG], seg_slot[VISS_MAX_SEG];   // slot -1: the segment writes F directly
  float ch_norm[VISS_MAX_CH];
  int row_tile;           // visibility rows per tile: 0 REC_Q, 1 REC_Q / 2, 2 2 * REC_Q (geometric, not compensated: 4 * REC_Q)
};

// Per-channel sum of partial slots (channels split into several segments).
struct RecReduceParams {
  const float2* partial;
  const int32_t* perm;
  float2* out;            // F [nch][J]
  int64_t J;
  int nch;
  int slot0[VISS_MAX_CH], nslot[VISS_MAX_CH];
  float norm[VISS_MAX_CH];
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
int launch_prep_rowblock_cones(const int* rowsat, const float4* satdir, const ChannelRows& ch, int64_t nblocks,
                               float4* cones, cudaStream_t st);
int launch_prep_snapshot_cones(const float4* satdir, int64_t S, int nsat, float4* cones, cudaStream_t st);
int launch_prep_block_cones(const float4* pgeo, int64_t J, int block, int64_t nblocks, float4* cones, cudaStream_t st);

// Persistent launches: ctas_per_sm 0 = as many as fit.
int launch_vis_fast(const VisParams& p, int ctas_per_sm, bool compensated, cudaStream_t st);
// Fine->coarse map records for the vis pass: per-pixel base brightness (mean of
// FF over the members), member boxes and ranges, per-tile fine-index ranges.
size_t fine_map_scratch(int64_t J);
int prep_fine_map(const float* NXq_f, const int32_t* NXq_i, const int32_t* countLoc, const float* FF, int64_t J,
                  int64_t X, int res, int trunc, int64_t Jpad, float* base, int4* box, int2* mem, int* members,
                  int2* tile_rng, void* scratch, size_t scratch_bytes, int* flags, cudaStream_t st);
int launch_vis_reduce(const float2* partial, int nsplit, int64_t K, float2* out, cudaStream_t st);
int launch_vis_plain(const viss_dft_cfg& cfg, const viss_sky& sky, const viss_vis_set& vis,
                     const viss_geometry* geo, const float4* satdir, const float* dlmn, float2* out, cudaStream_t st,
                     const viss_fine_map* map = nullptr, int* flags = nullptr, const int32_t* widx = nullptr);
int launch_prep_ref_ranges(const int32_t* widx, int64_t J, int64_t ntiles, int2* rng, cudaStream_t st);

int launch_recon_fast(const ReconParams& p, int ctas_per_sm, bool compensated, cudaStream_t st);
int launch_recon_reduce(const RecReduceParams& p, cudaStream_t st);
int launch_recon_plain(const viss_dft_cfg& cfg, const viss_sky& sky, const viss_vis_set& vis,
                       const viss_geometry* geo, const float* V, const float* ratios, const float4* satdir,
                       const float* dlmn, float2* out, cudaStream_t st, int* flags = nullptr);

// Fast geometric test of direction s (need not be unit) against satellite
// direction d = {p_hat, cos alpha}: s_hat.p_hat + cos(alpha) < 0, decided in
// double (from the original inputs) within GEO_EPS of the limb.
__device__ __forceinline__ bool geo_test_plain(float sx, float sy, float sz, const float4& d, const float* pos,
                                               double R, int* flags) {
  const float inv = rsqrtf(fmaf(sx, sx, fmaf(sy, sy, sz * sz)));
  const float e = fmaf(sx * inv, d.x, fmaf(sy * inv, d.y, fmaf(sz * inv, d.z, d.w)));
  if (fabsf(e) >= 4.0f * GEO_EPS) return e < 0.f;
  count_limb(flags);
  return geo_occluded_exact(sx, sy, sz, pos, R);
}

int device_sm_count();

// Grid of a persistent kernel: its resident CTAs per SM (capped by
// ctas_per_sm when > 0) on every SM, no more than the work items.
template <class Kernel>
inline int persistent_grid(Kernel k, int threads, int ctas_per_sm, int nitems) {
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, threads, 0) != cudaSuccess || occ < 1) occ = 1;
  if (ctas_per_sm > 0 && ctas_per_sm < occ) occ = ctas_per_sm;
  const int64_t g = (int64_t)occ * device_sm_count();
  return (int)(g < nitems ? g : nitems);
}

}  // namespace viss
