/*
 * viss_gb300.h -- C ABI of libvissgb.so, the GB300-native (sm_103a) hot path of
 * the SSshuishui/viss_recon_shade lunar-orbit interferometry simulator:
 *
 *   orbit positions + baseline uvw   (MIncline_generate_uvw_float.cu:83-160, 350-397)
 *   Moon shade windows               (shade1M.cu:62-105, 218-225)
 *   shaded visibility DFT            (visscal, vissGen10M_shade.cu:108-145)
 *   direct-DFT reconstruction        (imagerecon, vissGen10M_shade.cu:149-175)
 *
 * Conventions
 *   - Every entry point returns VISS_OK (0) or a negative status; it never
 *     exits the process.  viss_last_error() gives a message for the calling
 *     thread's last failure.
 *   - All array arguments are DEVICE pointers owned by the caller, unless a
 *     comment says "host".  Complex values are interleaved float pairs
 *     (re, im), i.e. the layout of thrust::complex<float> / complex64.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *     Work is enqueued on it; calls return without synchronising unless noted.
 *   - Scratch memory comes from a caller workspace whose size the matching
 *     *_workspace() query returns (256-byte aligned).  The reference-shaped
 *     entry points viss_visscal / viss_imagerecon allocate their workspace
 *     stream-ordered (cudaMallocAsync) instead.
 *   - Thread-safe: no global mutable state besides the thread-local error text.
 */
#ifndef VISS_GB300_H
#define VISS_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define VISS_API __attribute__((visibility("default")))
#else
#define VISS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  VISS_OK = 0,
  VISS_ERR_INVALID = -1,     /* null pointer, negative size, unknown mode */
  VISS_ERR_WORKSPACE = -2,   /* workspace missing, too small or misaligned */
  VISS_ERR_CUDA = -3,        /* a CUDA runtime call failed */
  VISS_ERR_RANGE = -4,       /* input outside the supported range */
  VISS_ERR_TIMEOUT = -5,     /* a bounded device-side wait gave up */
  VISS_ERR_UNSUPPORTED = -6, /* combination not implemented */
  VISS_ERR_IO = -7,          /* file could not be opened / written */
  VISS_ERR_FORMAT = -8       /* file content does not parse */
};

/* Replaces the reference's CHECK() macro (error.cuh:3-18), which exits. */
VISS_API const char* viss_status_str(int status);
VISS_API const char* viss_last_error(void);
VISS_API int viss_version(void);
/* Number of kernels the calling thread's viss_* calls have launched so far
 * (library-internal CUB kernels of viss_dedup_uvw not included). */
VISS_API uint64_t viss_launch_count(void);

/* ------------------------------------------------------------------ modes */
enum {                         /* which (visibility, pixel) terms are occluded */
  VISS_MASK_NONE = 0,
  VISS_MASK_REF_QUIRK = 1,     /* vissGen10M_shade.cu:130 as written: window rows run only
                                  when M3 <= 0, then rows 0..M4; cols M1 < c < M2           */
  VISS_MASK_REF_INTENDED = 2,  /* rows M3..M4, cols M1 < c < M2                              */
  VISS_MASK_GEOMETRIC = 3      /* ray from either satellite of the baseline hits the Moon   */
};
enum {                         /* recon-side mask */
  VISS_RECON_MASK_NONE = 0,
  VISS_RECON_MASK_REF = 1,     /* |M1/M2-thetaP|<M1/M2 && |M3/M4-phiP|<M3/M4 (vissGen10M_shade.cu:166) */
  VISS_RECON_MASK_GEOMETRIC = 2
};
enum {                         /* phase + sincos arithmetic */
  VISS_PREC_PLAIN = 0,         /* the reference's FP32 formula, precise sinf/cosf, 1 thread per item */
  VISS_PREC_FAST = 1,          /* 32-bit fixed-point phase (exact mod 1 for integer uvw), SFU sincos */
  VISS_PREC_COMPENSATED = 2,   /* FAST + FP32 correction of the pixel fixed-point rounding */
  VISS_PREC_F64_PHASE = 3      /* precision sweeps (no counterpart in the reference): the phase in FP64,
                                  range-reduced in FP64, FP32 sincosf, Kahan-compensated FP32 sums;
                                  one thread per item like PLAIN, and slow (GB300's FP64 rate) */
};

/* One DFT pass.  Phase in turns: t = phase_scale * (u l + v m + w (n + n_offset)).
 * vis:   V_k = sum_j C_kj exp(-2 pi i t_kj),  C_kj = occluded_value inside the mask else bright_j
 * recon: F_j = norm * sum_k [not masked] wgt_k V_k exp(+2 pi i t_kj)
 * The reference uses phase_scale = 1/d with d = 2*RES/(RES-1) in integer arithmetic (= 2),
 * n_offset = 0 (its w(n-1) term and trailing e^{-2 pi i w/d} combine to w n), occluded_value 240,
 * norm = 1/K.  The geometric-mask convention is phase_scale = 1, n_offset = -1, occluded_value 0. */
typedef struct viss_dft_cfg {
  int32_t mask_mode;         /* VISS_MASK_* (vis) */
  int32_t recon_mask;        /* VISS_RECON_MASK_* (recon) */
  int32_t precision;         /* VISS_PREC_* */
  int32_t res;               /* fine-grid row width for the REF masks */
  int32_t trunc_brightness;  /* 1: brightness truncated to int first (plain visscal, :128) */
  float occluded_value;      /* brightness inside the vis mask */
  double phase_scale;
  double n_offset;
  double moon_radius_km;     /* GEOMETRIC */
  double norm;               /* recon output scale */
} viss_dft_cfg;

typedef struct viss_sky {    /* J sky pixels: direction cosines and brightness */
  const float* l;
  const float* m;
  const float* n;
  const float* bright;       /* vis only; may be NULL for recon */
  int64_t J;
} viss_sky;

typedef struct viss_vis_set { /* K visibilities */
  const float* u;            /* in wavelengths */
  const float* v;
  const float* w;
  const float* wgt;          /* recon weight per visibility (reference: 1/freq or 1/count); NULL = 1 */
  const int32_t* shade;      /* K x 4 normalised windows (M1<=M2, M3<=M4, 0-based); REF masks */
  const int32_t* snap;       /* K snapshot index; GEOMETRIC */
  const int32_t* pair;       /* K satellite pair, m | (n << 16); GEOMETRIC */
  int64_t K;
} viss_vis_set;

typedef struct viss_geometry { /* satellite positions per snapshot; GEOMETRIC */
  const float* sat_pos;      /* S x nsat x 3, km, Moon-centred */
  int64_t S;
  int32_t nsat;
  int32_t reserved;
} viss_geometry;

/* Shaded visibility DFT (replaces visscal, vissGen10M_shade.cu:108-145 and its
 * launchers, vissGen10M_shade_optim2.cu:150-215).  V: K x 2 float. */
VISS_API size_t viss_vis_dft_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J, const viss_geometry* geo);
VISS_API int viss_vis_dft(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
                 const viss_geometry* geo, float* V, void* workspace, size_t workspace_bytes,
                 void* stream);

/* Shaded visibility DFT without any allocation (no counterpart in the reference).
 * For callers that must not have a library allocate device memory -- hosts
 * that own a fixed memory budget or pool, or latency-bound loops that cannot
 * take cudaMalloc's synchronisation -- and that do not want to pass a
 * workspace either.  Same arguments and result as viss_vis_dft; the scratch is
 * a VISS_NOALLOC_SCRATCH_BYTES array inside the library, resident on every GPU
 * that loads it.  It splits the sky into fewer chunks than viss_vis_dft (its
 * partial sums are the largest part of the scratch); passes that still need more
 * than the scratch are rejected with VISS_ERR_RANGE (131,072 visibilities x
 * 196,608 pixels with the geometric mask fit; the full 1,835,008 x 196,608
 * workload does not).  Every call looks up the array's device address on the
 * current device (so a device reset does not leave a stale address); the first
 * call on a device, or after a reset, loads the library's device code: make it
 * before any stream capture.  The caller cannot reach the scratch to read the
 * pass's input checks (viss_workspace_flags), so the call waits for the pass
 * (synchronises `stream`) and returns them: VISS_ERR_RANGE for |uvw| >= 2^30,
 * VISS_ERR_INVALID for a snapshot or satellite index outside the geometry.
 * Calls share the array: calls that overlap on the GPU race. */
#define VISS_NOALLOC_SCRATCH_BYTES (32u << 20)
VISS_API int viss_vis_dft_noalloc(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
                                  const viss_geometry* geo, float* V, void* stream);

/* Direct-DFT reconstruction (replaces imagerecon, vissGen10M_shade.cu:149-175,
 * and launch_imagerecon, vissGen10M_shade_optim2.cu:320-389).  V: K x 2, F: J x 2.
 * With norm = 1, wgt = NULL and the vis mask this is the adjoint of viss_vis_dft
 * with respect to the brightness. */
VISS_API size_t viss_recon_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J, const viss_geometry* geo);
VISS_API int viss_recon(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
               const viss_geometry* geo, const float* V, float* F, void* workspace,
               size_t workspace_bytes, void* stream);

/* Non-identity fine->coarse sky map (vissGen10M_shade.cu:120-136, 261-286;
 * vissGen1M_shade_optim1.cu:54-115, 134-171): coarse pixel j's brightness for
 * visibility k is the mean of its countLoc[j] fine pixels, listed in NXq (in
 * pixel order, ascending within a pixel), each replaced by the occluded value
 * inside k's REF window.  NXq as floats (the 10M text files; values are
 * truncated to integers as the reference does) or as int32 (viss_nxq, the 1M
 * in-program form): exactly one of NXq_f / NXq_i is set.  Indices outside
 * [0, X) make the pixel NaN instead of being read. */
typedef struct viss_fine_map {
  const float* FF;           /* X fine brightness */
  const float* NXq_f;
  const int32_t* NXq_i;
  const int32_t* countLoc;   /* J */
  int64_t X;                 /* fine pixels (entries of FF and NXq) */
} viss_fine_map;

/* Shaded visibility DFT over a fine->coarse map (visscal with NXq/countLoc,
 * vissGen10M_shade.cu:120-136); sky->bright is unused (the coarse brightness comes from FF).  Same configuration and result layout as
 * viss_vis_dft. */
VISS_API size_t viss_vis_dft_map_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J, const viss_fine_map* map,
                                           const viss_geometry* geo);
VISS_API int viss_vis_dft_map(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_fine_map* map,
                              const viss_vis_set* vis, const viss_geometry* geo, float* V, void* workspace,
                              size_t workspace_bytes, void* stream);

/* NX -> (countLoc, NXq) (replaces computeLocCount / computeLocViss,
 * vissGen1M_shade_optim1.cu:54-115): NX holds the 1-based coarse pixel of each
 * of X fine pixels as floats; countLoc[q] counts the fine pixels with
 * NX[i] - 1 == q, NXq lists them grouped by q, ascending (the first
 * sum(countLoc) entries; fine pixels that match no coarse pixel follow). */
VISS_API size_t viss_nxq_workspace(int64_t X, int64_t J);
VISS_API int viss_nxq(const float* NX, int64_t X, int64_t J, int32_t* countLoc, int32_t* NXq, void* workspace,
                      size_t workspace_bytes, void* stream);

/* viss_vis_dft with a REF mask whose window tests win_index[j] (J int32, may be negative
 * or beyond the grid) for pixel j instead of j itself.  vissGen1M_shade_appro.cu:113-118
 * tests NX[j] - 1, the fine-array entry read at the coarse index; its write of 240 into
 * the shared brightness array is a race between threads and is not reproduced: the
 * occluded value replaces the brightness for that (visibility, pixel) term only. */
VISS_API size_t viss_vis_dft_windowed_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J);
VISS_API int viss_vis_dft_windowed(const viss_dft_cfg* cfg, const viss_sky* sky, const int32_t* win_index,
                                   const viss_vis_set* vis, float* V, void* workspace, size_t workspace_bytes,
                                   void* stream);

/* Input problems a pass records instead of reading out of bounds (a pass never
 * synchronises to look): after the pass has completed, reads the flag word at
 * the start of its workspace (synchronises `stream`).  Bits: 1 = |uvw| >= 2^30,
 * 2 = a snapshot or satellite index outside the geometry (that visibility's
 * occlusion test used satellite 0 of snapshot 0), 4 = recon ratio arrays not of
 * the reference's form, 8 = a fine-map index outside [0, X) (that pixel is NaN).
 * No counterpart in the reference, which reads such inputs unchecked. */
VISS_API int viss_workspace_flags(const void* workspace, int32_t* flags, void* stream);
/* No counterpart in the reference (its masks are the REF windows of shade1M.cu:73-105).
 * GEOMETRIC mask: how many occlusion tests of the completed pass fell within 2e-6 (in the
 * cosine of the angle to the limb) of the Moon's limb and were decided in double from the
 * original inputs instead (count of occlusion tests; the plain kernels test every
 * (visibility, pixel, satellite), the fast ones drop blocks the cones decide and the fast
 * vis kernel tests a (pixel, satellite) pair once per block of 1,024 visibilities).  Reads the
 * workspace like viss_workspace_flags (synchronises `stream`). */
VISS_API int viss_workspace_limb_count(const void* workspace, int64_t* count, void* stream);

/* Batched passes: many frequency channels (or periods) in one persistent
 * launch.  The reference runs one channel per program run or per OpenMP
 * iteration (vissGen10M_shade.cu:298-545, one visscal + imagerecon launch pair
 * per period); here the visibility set holds all channels' rows back to back and
 * persistent CTAs pull (rows x pixels) work items of every channel from one
 * queue, so uneven channels (row counts, occluded fractions) share the GPU
 * without per-channel tails.  The passes enqueue no host synchronisation and
 * take their scratch from the workspace, so they can be captured in a CUDA graph
 * once the workspace exists.
 *   channel c owns visibility rows [row_off[c], row_off[c+1]), row_off[0] = 0,
 *   row_off[nch] = K; V is K x 2 as for one channel; F is nch x J x 2.
 * batch = NULL is one channel (exactly viss_vis_dft / viss_recon). */
#define VISS_MAX_CHANNELS 64
typedef struct viss_batch {
  int32_t nch;               /* 1 .. VISS_MAX_CHANNELS */
  int32_t reserved;
  const int64_t* row_off;    /* HOST, nch + 1 entries */
  const float* bright;       /* DEVICE nch x J per-channel brightness (vis); NULL: sky->bright for every channel */
  const double* norm;        /* HOST nch recon normalisation per channel; NULL: cfg->norm for every channel */
} viss_batch;

/* Launch choices of the persistent passes (all zero: defaults).  Any values give
 * the same results up to the order of float additions; viss_recon_shade_gb300's
 * autotuner times candidates on the caller's own data and picks one. */
typedef struct viss_tuning {
  int32_t ctas_per_sm;       /* persistent CTAs per SM (0: as many as fit) */
  int32_t vis_split;         /* sky chunks per visibility block, each a work item (0: enough for ~32 items per CTA) */
  int32_t rec_items;         /* recon work items per persistent CTA the row segments aim at (0: 64) */
  int32_t tile;              /* tile shapes: bit 0 vis sky tiles of 256 pixels (else 512),
                                bit 1 recon row tiles of 128 visibilities, bit 3 of 256
                                (else 512, 1,024 with the geometric mask at FAST precision;
                                bit 2 asks for that default explicitly) */
} viss_tuning;

VISS_API size_t viss_vis_dft_batch_workspace(const viss_dft_cfg* cfg, const viss_batch* batch, int64_t K, int64_t J,
                                             const viss_geometry* geo, const viss_tuning* tuning);
VISS_API int viss_vis_dft_batch(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
                                const viss_batch* batch, const viss_geometry* geo, const viss_tuning* tuning,
                                float* V, void* workspace, size_t workspace_bytes, void* stream);
VISS_API size_t viss_recon_batch_workspace(const viss_dft_cfg* cfg, const viss_batch* batch, int64_t K, int64_t J,
                                           const viss_geometry* geo, const viss_tuning* tuning);
VISS_API int viss_recon_batch(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
                              const viss_batch* batch, const viss_geometry* geo, const viss_tuning* tuning,
                              const float* V, float* F, void* workspace, size_t workspace_bytes, void* stream);

/* Reference-shaped operators: the argument lists of the reference kernels
 * (the complex constants I1, CPI, zero, two are implied).  variant selects the
 * brightness arithmetic: VISS_VARIANT_PLAIN truncates FF to int (vissGen10M_shade.cu:128),
 * VISS_VARIANT_OPTIM keeps it float (vissGen10M_shade_optim1.cu:180).
 * NXq/countLoc may both be NULL for the identity fine->coarse map (countLoc = 1,
 * NXq[j] = j); otherwise NXq holds float indices as in the 10M files and FF
 * the fine brightness (the fine pixel count is taken as sum(countLoc)).
 * mask_mode is VISS_MASK_REF_QUIRK for the reference's behaviour. */
enum { VISS_VARIANT_PLAIN = 0, VISS_VARIANT_OPTIM = 1 };
VISS_API int viss_visscal(int uvws_index, int lmnC_index, int res, const float* FF, float* viss,
                 const float* u, const float* v, const float* w, const float* l, const float* m,
                 const float* n, const int* shadeM1, const int* shadeM2, const int* shadeM3,
                 const int* shadeM4, const float* NXq, const int* countLoc, float dl, float dm,
                 float dn, int variant, int mask_mode, int precision, void* stream);
VISS_API int viss_imagerecon(int uvw_index, int lmnC_index, int res, float* F, const float* viss,
                    const float* u, const float* v, const float* w, const float* l, const float* m,
                    const float* n, const float* uvwFrequencyMap, const float* thetaP0,
                    const float* phiP0, const float* dtheta, const float* dphi, float dl, float dm,
                    float dn, int precision, void* stream);

/* ---------------------------------------------------------- orbit + uvw */
typedef struct viss_orbit_cfg {  /* MIncline_generate_uvw_float.cu:22-30, 184-190 */
  int32_t nsat;
  int32_t orbit_res;      /* samples per orbit (reference 864000 = 2.4*3600/0.01) */
  int32_t orbit_counts;   /* orbits (reference 140) */
  int32_t index;          /* observation period, >= 1 */
  double a_km;            /* orbit radius (reference 2038.14) */
  double e;               /* eccentricity (reference 0) */
  double incl_deg;        /* reference 30 */
  double argp_deg;        /* reference 0 */
  double raan_step_deg;   /* node advance per orbit (reference 0.08) */
  const float* r1_m;      /* HOST [nsat] separation ramp ends (reference r1) */
  const float* r2_m;      /* HOST [nsat] separation ramp middle (reference r2) */
  int32_t fp64;           /* 0: reference FP32 arithmetic; 1: FP64 positions */
  int32_t reserved;
} viss_orbit_cfg;

/* Number of windowed snapshots: orbit_counts * (orbit_res / 3). */
VISS_API int64_t viss_orbit_snapshots(const viss_orbit_cfg* cfg);
/* Satellite positions at every snapshot (calculateOrbit + uvwPosition,
 * MIncline_generate_uvw_float.cu:83-151):
 * pos: S x nsat x 3 float (km); pos64 (optional, may be NULL): the same in double. */
VISS_API int viss_orbit_positions(const viss_orbit_cfg* cfg, float* pos, double* pos64, void* stream);
/* Baseline uvw (computeUVW, MIncline_generate_uvw_float.cu:153-160), snapshot-major then pair.  pairs: 1 = ordered
 * (m != n, the reference's 56 for 8 satellites), 0 = unordered (m < n).  rounding: 1 = the
 * reference's ceil(), 0 = none.  From pos64 when given (no rounding to float first).
 * snap/pair outputs may be NULL.  K = S * npairs entries are written. */
VISS_API int viss_baseline_uvw(const float* pos, const double* pos64, int64_t S, int32_t nsat, int ordered,
                      double lambda_m, int rounding, float* u, float* v, float* w, int32_t* snap,
                      int32_t* pair, void* stream);
/* Global lexicographic sort + unique of integer-valued uvw (the reference's per-pair and
 * global thrust sort/unique, MIncline_generate_uvw_float.cu:370-397).  In place on u, v, w; *count_out (HOST) receives
 * the unique count (the call synchronises the stream).  |u|,|v|,|w| must be < 2^20. */
VISS_API size_t viss_dedup_uvw_workspace(int64_t K);
VISS_API int viss_dedup_uvw(float* u, float* v, float* w, int64_t K, int64_t* count_out, void* workspace,
                   size_t workspace_bytes, void* stream);
/* The uvw generation of MIncline_generate_uvw_float.cu:341-397 in one pass that never
 * materialises the S x pairs rows: viss_baseline_uvw (float positions, ceil), the rows
 * concatenated pair-major as the reference does, then viss_dedup_uvw.  The unique rows in
 * SortCompare order, each with the values of its first occurrence (lowest pair, then
 * earliest snapshot: the sign of a zero coordinate).  Rows repeated from the previous
 * snapshot of the same pair skip the hash table.  u, v, w receive up to `capacity` rows; *count_out (HOST) the unique
 * count (the call synchronises the stream).  capacity 0 only counts; a smaller nonzero
 * capacity than the count returns VISS_ERR_RANGE with the count set.  More unique rows
 * than the internal table holds (~2^28) return VISS_ERR_RANGE: use the two calls then. */
VISS_API size_t viss_unique_uvw_workspace(int64_t S, int32_t nsat, int ordered);
VISS_API int viss_unique_uvw(const float* pos, int64_t S, int32_t nsat, int ordered, double lambda_m, float* u,
                    float* v, float* w, int64_t capacity, int64_t* count_out, void* workspace,
                    size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------- shade windows */
/* Cart2SphKernel + mean radius + ShadeMatrix (shade1M.cu:62-105, 218-225).
 * out: K x 4 int32 (thetaIndS, thetaIndE, phiIndS, phiIndE), 1-based as in the shadeM files.
 * mean_r_km > 0 uses that mean radius (rounded to float); otherwise it is computed as the
 * reference computes it -- the FP32 sum of r by thrust::transform_reduce (shade1M.cu:219,
 * same CUB reduction, same order) divided by K -- and read back to the host, so the call
 * synchronises `stream` once.  r0 = atanf(1737.74f / (mean_r + 1737.74f)), dtheta and dphi
 * are computed on the host as there (:222-224); the windows equal the reference's bit for
 * bit.  mean_r_out (HOST, may be NULL) receives the mean radius used. */
VISS_API size_t viss_shade_windows_workspace(int64_t K);
VISS_API int viss_shade_windows(const float* u, const float* v, const float* w, int64_t K, int RES,
                       double mean_r_km, int32_t* out, double* mean_r_out, void* workspace,
                       size_t workspace_bytes, void* stream);
/* shadeM normalisation on load (vissGen10M_shade.cu:383-399): (min-1, max-1) per pair. */
VISS_API int viss_normalise_shade(const int32_t* raw, int64_t K, int32_t* M, void* stream);

/* ------------------------------------------------------------- text files */
/* The reference's whitespace-separated text files (HOST buffers).  Reading is
 * chunk-parallel and stops at the first token that does not parse, as the
 * reference's `while (file >> ...)` loops do; writing formats every value as
 * std::ostream formats a float by default ("%g", 6 significant digits).
 *   l.txt / FF.txt carry a count header (vissGen10M_shade.cu:237-238): header = 1.
 *   uvw files: 3 columns (u v w, MIncline:425) or 4 (u v w freq, vissGen10M_shade.cu:359).
 *   shadeM files: 4 integer columns (shade1M.cu:118-121).
 * viss_text_read_floats stores column c of row r at out[c*cap + r]; with out == NULL it only
 * counts rows.  viss_text_write_floats reads column c of row r at cols[c*stride + r]. */
VISS_API int viss_text_read_floats(const char* path, int header, int ncols, float* out, int64_t cap,
                                   int64_t* nrows, int64_t* header_value);
VISS_API int viss_text_read_ints(const char* path, int ncols, int32_t* out, int64_t cap, int64_t* nrows);
VISS_API int viss_text_write_floats(const char* path, int ncols, const float* cols, int64_t stride,
                                    int64_t nrows);
VISS_API int viss_text_write_ints(const char* path, int ncols, const int32_t* rows, int64_t nrows);

/* ------------------------------------------------------------- measurement */
/* SFU throughput probe (no counterpart in the reference): launches
 * blocks_per_sm * SMs blocks of 256 threads, each thread running `iters` rounds of
 * 8 independent __sincosf; *sfu_ops (HOST) receives the number of SFU operations
 * (2 per sincos).  The caller times the launch on `stream`. */
VISS_API int viss_sfu_probe(int iters, int blocks_per_sm, float* out, int64_t* sfu_ops, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VISS_GB300_H */
