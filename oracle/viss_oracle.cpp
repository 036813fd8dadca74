// viss_oracle.cpp -- CPU oracle for the shaded visibility DFT hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, the smoke test
// and bench.py's CPU-baseline leg load it; the product (libvissgb.so) never
// links or calls it.
//
// It restates, in plain C++ with OpenMP, the arithmetic of the reference
// programs of SSshuishui/viss_recon_shade:
//   * orbit propagation and snapshot windowing  MIncline_generate_uvw_float.cu:83-151
//   * baseline uvw                               MIncline_generate_uvw_float.cu:153-160
//   * uvw dedup (per-pair + global sort/unique)  MIncline_generate_uvw_float.cu:350-397
//   * Cart2Sph + mean radius + ShadeMatrix       shade1M.cu:62-105, 218-225
//   * shadeM normalisation on load               vissGen10M_shade.cu:383-399
//   * visscal (plain / optim)                    vissGen10M_shade.cu:108-145,
//                                                vissGen10M_shade_optim1.cu:154-205
//   * recon-mask ratios                          vissGen10M_shade.cu:511-517
//   * imagerecon                                 vissGen10M_shade.cu:149-175
//   * NX -> (countLoc, NXq) inversion            vissGen1M_shade_optim1.cu:54-115
// plus the geometric Moon-occlusion predicate that the new build adds.
//
// Two arithmetic modes exist where the reference's float rounding matters:
//   FP64   -- everything in double; the accuracy yardstick.
//   MIMIC  -- the reference's FP32 operation order, using the host libm float
//             functions; it bounds how far the reference's own FP32 result sits
//             from FP64 and pins the formulas against the reference's outputs.
//
// Parity of this oracle is pinned against outputs of the reference's own CUDA
// kernels (compiled from the reference sources and run on the GPU); the
// generating script and the fixtures live in tests/golden/.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <tuple>
#include <vector>
#include <omp.h>

#define ORACLE_API extern "C" __attribute__((visibility("default")))

namespace {

constexpr double kPi = 3.14159265358979323846;

enum MaskMode { MASK_NONE = 0, MASK_REF_QUIRK = 1, MASK_REF_INTENDED = 2, MASK_GEOMETRIC = 3 };

int nthreads_or_default(int n) { return n > 0 ? n : omp_get_max_threads(); }

// ---------------------------------------------------------------------------
// Geometric occlusion: the ray from satellite position p (km, Moon-centred)
// along direction s hits the Moon sphere of radius R.  s need not be unit.
//   b = s.p, a = |s|^2, c = |p|^2 - R^2 ;  occluded  <=>  b < 0  and  b^2 - a c > 0
// Evaluated in double with an explicit operation order (no contraction, the
// file is built with -ffp-contract=off); the GPU fallback uses the same order.
// margin = alpha - angle(s, -p), alpha = asin(R/|p|): > 0 inside the shadow cone.
// ---------------------------------------------------------------------------
inline int geo_occluded(const float* s, const float* p, double R, double* margin) {
  const double sx = s[0], sy = s[1], sz = s[2];
  const double px = p[0], py = p[1], pz = p[2];
  const double b = (sx * px + sy * py) + sz * pz;
  const double a = (sx * sx + sy * sy) + sz * sz;
  const double pp = (px * px + py * py) + pz * pz;
  const double c = pp - R * R;
  const double disc = b * b - a * c;
  const int occ = (b < 0.0) && (disc > 0.0);
  if (margin) {
    double ca = -b / std::sqrt(a * pp);
    ca = std::max(-1.0, std::min(1.0, ca));
    const double ang = std::acos(ca);
    const double r = std::min(1.0, R / std::sqrt(pp));
    *margin = std::asin(r) - ang;
  }
  return occ;
}

// REF window membership of fine pixel index i for normalised window
// (M1, M2, M3, M4) -- vissGen10M_shade.cu:130-134.  The reference loop is
//   for (lo = 0; lo >= M3 && lo <= M4; ++lo) if (i >= lo*res+M1+1 && i < lo*res+M2) hit
// so it only runs when M3 <= 0 and then covers rows 0..M4 (REF_QUIRK).
// REF_INTENDED runs rows M3..M4.
inline bool ref_window_hit(int64_t i, int res, int M1, int M2, int M3, int M4, int mode) {
  int64_t lo_a, lo_b;
  if (mode == MASK_REF_QUIRK) {
    if (M3 > 0 || M4 < 0) return false;
    lo_a = 0; lo_b = M4;
  } else {
    lo_a = M3; lo_b = M4;
    if (lo_a > lo_b) return false;
  }
  // exists lo in [lo_a, lo_b] with lo*res + M1 + 1 <= i < lo*res + M2
  for (int64_t lo = lo_a; lo <= lo_b; ++lo) {
    const int64_t base = lo * (int64_t)res;
    if (i >= base + M1 + 1 && i < base + M2) return true;
  }
  return false;
}

// Faster equivalent used on large cases; falls back to the literal loop when the
// column range is not inside one row.
inline bool ref_window_hit_fast(int64_t i, int res, int M1, int M2, int M3, int M4, int mode) {
  if (M1 + 1 >= 0 && M2 <= res) {
    int64_t lo_a, lo_b;
    if (mode == MASK_REF_QUIRK) {
      if (M3 > 0 || M4 < 0) return false;
      lo_a = 0; lo_b = M4;
    } else {
      lo_a = M3; lo_b = M4;
    }
    if (i < 0) return false;
    const int64_t q = i / res, r = i % res;
    return q >= lo_a && q <= lo_b && r > M1 && r < M2;
  }
  return ref_window_hit(i, res, M1, M2, M3, M4, mode);
}

inline double frac_turns(double t) { return t - std::nearbyint(t); }

// float -> int as CUDA's cvt.rzi.s32.f32 does it: NaN -> 0, saturating.
inline int f2i_cuda(float x) {
  if (std::isnan(x)) return 0;
  if (x >= 2147483647.0f) return 2147483647;
  if (x <= -2147483648.0f) return (-2147483647 - 1);
  return (int)x;
}

}  // namespace

extern "C" {

// Configuration of one DFT pass (vis or recon); field meaning matches the
// product's viss_dft_cfg.
typedef struct oracle_dft_cfg {
  int32_t mask_mode;         // MaskMode
  int32_t res;               // fine-grid row width (REF masks, recon mask)
  int32_t trunc_brightness;  // plain vissGen: int addFF = FF[..]
  int32_t recon_ref_mask;    // recon: 1 = reference ratio mask, 0 = same predicate as mask_mode
  float occluded_value;      // 240 in the reference
  float pad0;
  double phase_scale;        // s : phase turns = s*(u l + v m + w (n + n_offset))
  double n_offset;           // 0 (reference net phase) or -1
  double moon_radius_km;     // geometric mask
  double norm;               // recon scale (1/K in the reference)
} oracle_dft_cfg;

typedef struct oracle_geo {
  const float* sat_pos;  // [S][nsat][3] km
  const int32_t* snap;   // [K]
  const int32_t* pair;   // [K] m | (n << 16)
  int32_t nsat;
  int32_t pad;
  int64_t S;
} oracle_geo;

}  // extern "C"

namespace {

// widx: the fine index the REF window tests for pixel j (NULL: j itself)
inline bool term_masked(const oracle_dft_cfg* cfg, const int32_t* shade, const oracle_geo* geo,
                        const float* l, const float* m, const float* n, int64_t k, int64_t j,
                        const int32_t* widx = nullptr) {
  switch (cfg->mask_mode) {
    case MASK_REF_QUIRK:
    case MASK_REF_INTENDED: {
      const int32_t* M = shade + 4 * k;
      return ref_window_hit(widx ? (int64_t)widx[j] : j, cfg->res, M[0], M[1], M[2], M[3], cfg->mask_mode);
    }
    case MASK_GEOMETRIC: {
      const int32_t s = geo->snap[k];
      const int32_t pm = geo->pair[k] & 0xffff, pn = (geo->pair[k] >> 16) & 0xffff;
      const float sv[3] = {l[j], m[j], n[j]};
      const float* p1 = geo->sat_pos + ((int64_t)s * geo->nsat + pm) * 3;
      const float* p2 = geo->sat_pos + ((int64_t)s * geo->nsat + pn) * 3;
      return geo_occluded(sv, p1, cfg->moon_radius_km, nullptr) ||
             geo_occluded(sv, p2, cfg->moon_radius_km, nullptr);
    }
    default:
      return false;
  }
}

}  // namespace

// ===========================================================================
// Shaded visibility DFT, FP64.
// V_k = sum_j C_kj exp(-2 pi i s (u_k l_j + v_k m_j + w_k (n_j + n_offset)))
// With s = 1/d and n_offset = 0 this is the reference's
//   e^{-2 pi i w/d} * sum_j C_kj e^{-2 pi i (u l + v m + w (n-1))/d}
// (vissGen10M_shade.cu:137-143): the trailing factor cancels the -1.
// C_kj = occluded_value inside the mask, else FF_j (truncated to int in the
// plain variant, vissGen10M_shade.cu:128).  Identity fine->coarse mapping.
// ===========================================================================
ORACLE_API int oracle_vis_dft(const oracle_dft_cfg* cfg, const float* u, const float* v, const float* w,
                              int64_t K, const int32_t* shade, const oracle_geo* geo, const float* l,
                              const float* m, const float* n, const float* bright, int64_t J,
                              double* V, int nthreads) {
  const double s = cfg->phase_scale, noff = cfg->n_offset;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t k = 0; k < K; ++k) {
    const double uk = u[k], vk = v[k], wk = w[k];
    double re = 0.0, im = 0.0;
    for (int64_t j = 0; j < J; ++j) {
      double c = bright[j];
      if (cfg->trunc_brightness) c = (double)(int)bright[j];
      if (cfg->mask_mode != MASK_NONE && term_masked(cfg, shade, geo, l, m, n, k, j))
        c = cfg->occluded_value;
      if (c == 0.0) continue;
      const double t = s * (uk * (double)l[j] + vk * (double)m[j] + wk * ((double)n[j] + noff));
      const double x = 2.0 * kPi * frac_turns(t);
      re += c * std::cos(x);
      im -= c * std::sin(x);
    }
    V[2 * k] = re;
    V[2 * k + 1] = im;
  }
  return 0;
}

// The same with the REF window tested on widx[j] instead of the pixel index j: the
// appro program's visscal (vissGen1M_shade_appro.cu:113-118) tests NX[j] - 1, the
// fine-array entry at the coarse index, against the window of row k (its write of
// 240 into the shared brightness is a race and is not followed: the occluded
// value replaces C_j for that term only).
ORACLE_API int oracle_vis_dft_windex(const oracle_dft_cfg* cfg, const float* u, const float* v, const float* w,
                                     int64_t K, const int32_t* shade, const int32_t* widx, const float* l,
                                     const float* m, const float* n, const float* bright, int64_t J, double* V,
                                     int nthreads) {
  const double s = cfg->phase_scale, noff = cfg->n_offset;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t k = 0; k < K; ++k) {
    const double uk = u[k], vk = v[k], wk = w[k];
    double re = 0.0, im = 0.0;
    for (int64_t j = 0; j < J; ++j) {
      double c = bright[j];
      if (cfg->trunc_brightness) c = (double)(int)bright[j];
      if (cfg->mask_mode != MASK_NONE && term_masked(cfg, shade, nullptr, l, m, n, k, j, widx))
        c = cfg->occluded_value;
      if (c == 0.0) continue;
      const double t = s * (uk * (double)l[j] + vk * (double)m[j] + wk * ((double)n[j] + noff));
      const double x = 2.0 * kPi * frac_turns(t);
      re += c * std::cos(x);
      im -= c * std::sin(x);
    }
    V[2 * k] = re;
    V[2 * k + 1] = im;
  }
  return 0;
}

// General fine->coarse form of visscal (vissGen10M_shade.cu:120-136): coarse
// pixel j averages its countLoc[j] fine pixels NXq[start..start+cnt) (float
// indices, truncated to int64 as the reference does), each replaced by the
// occluded value inside the window of row k.
ORACLE_API int oracle_vis_dft_nxq(const oracle_dft_cfg* cfg, const float* u, const float* v,
                                  const float* w, int64_t K, const int32_t* shade, const float* l,
                                  const float* m, const float* n, int64_t J, const float* FF,
                                  const float* NXq, const int32_t* countLoc, double* V, int nthreads) {
  const double s = cfg->phase_scale, noff = cfg->n_offset;
  std::vector<int64_t> start(J + 1, 0);
  for (int64_t j = 0; j < J; ++j) start[j + 1] = start[j] + countLoc[j];
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t k = 0; k < K; ++k) {
    const int32_t* M = shade ? shade + 4 * k : nullptr;
    double re = 0.0, im = 0.0;
    for (int64_t j = 0; j < J; ++j) {
      double sum = 0.0;
      for (int64_t c = start[j]; c < start[j + 1]; ++c) {
        const int64_t loc = (int64_t)NXq[c];
        double ff = FF[loc];
        if (cfg->trunc_brightness) ff = (double)(int)FF[loc];
        if (M && cfg->mask_mode != MASK_NONE &&
            ref_window_hit(loc, cfg->res, M[0], M[1], M[2], M[3], cfg->mask_mode))
          ff = cfg->occluded_value;
        sum += ff;
      }
      const double cj = sum / (double)countLoc[j];
      const double t = s * ((double)u[k] * l[j] + (double)v[k] * m[j] + (double)w[k] * ((double)n[j] + noff));
      const double x = 2.0 * kPi * frac_turns(t);
      re += cj * std::cos(x);
      im -= cj * std::sin(x);
    }
    V[2 * k] = re;
    V[2 * k + 1] = im;
  }
  return 0;
}

// ===========================================================================
// Direct-DFT reconstruction, FP64 (vissGen10M_shade.cu:149-175).
// F_j = norm * sum_k [not skipped] wgt_k V_k exp(+2 pi i s (u l + v m + w (n + n_offset)))
// Reference recon mask (recon_ref_mask=1): skip iff
//   |M1/M2 - thetaP| < M1/M2  and  |M3/M4 - phiP| < M3/M4
// with float ratios (thrust::divides<float>, :514-517), phiP = floorf(j/res)
// (integer division), thetaP = j - phiP*res.  Otherwise the geometric mask.
// ===========================================================================
ORACLE_API int oracle_recon(const oracle_dft_cfg* cfg, const float* u, const float* v, const float* w,
                            const float* wgt, const float* Vin /* K x 2 float */, int64_t K,
                            const int32_t* shade, const oracle_geo* geo, const float* l, const float* m,
                            const float* n, int64_t J, double* F, int nthreads) {
  const double s = cfg->phase_scale, noff = cfg->n_offset;
  std::vector<float> r1, r2;
  if (cfg->recon_ref_mask && shade) {
    r1.resize(K);
    r2.resize(K);
    for (int64_t k = 0; k < K; ++k) {
      r1[k] = (float)shade[4 * k] / (float)shade[4 * k + 1];
      r2[k] = (float)shade[4 * k + 2] / (float)shade[4 * k + 3];
    }
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t j = 0; j < J; ++j) {
    const float phiP = std::floor((float)(j / cfg->res));
    const float thetaP = (float)j - phiP * (float)cfg->res;
    const double lj = l[j], mj = m[j], nj = (double)n[j] + noff;
    double re = 0.0, im = 0.0;
    for (int64_t k = 0; k < K; ++k) {
      bool skip = false;
      if (cfg->recon_ref_mask && shade) {
        skip = std::fabs(r1[k] - thetaP) < r1[k] && std::fabs(r2[k] - phiP) < r2[k];
      } else if (cfg->mask_mode == MASK_GEOMETRIC) {
        skip = term_masked(cfg, shade, geo, l, m, n, k, j);
      }
      if (skip) continue;
      const double wk = wgt ? (double)wgt[k] : 1.0;
      const double yr = wk * Vin[2 * k], yi = wk * Vin[2 * k + 1];
      const double t = s * ((double)u[k] * lj + (double)v[k] * mj + (double)w[k] * nj);
      const double x = 2.0 * kPi * frac_turns(t);
      const double cs = std::cos(x), sn = std::sin(x);
      re += yr * cs - yi * sn;
      im += yr * sn + yi * cs;
    }
    F[2 * j] = re * cfg->norm;
    F[2 * j + 1] = im * cfg->norm;
  }
  return 0;
}

// ===========================================================================
// FP32 mimic of the reference plain kernels, operation by operation
// (vissGen10M_shade.cu:108-175), to bound the reference's FP32 error and to
// pin the formulas against the reference's own outputs.
// dl = dm = dn = d (float).  Identity mapping (countLoc = 1).
// ===========================================================================
ORACLE_API int oracle_vis_plain_f32(const oracle_dft_cfg* cfg, const float* u, const float* v,
                                    const float* w, int64_t K, const int32_t* shade, const float* l,
                                    const float* m, const float* n, const float* FF, int64_t J,
                                    float d, float* V, int nthreads, int optim) {
  const float two_pi_f = -2.0f * (float)kPi;  // (0 - i) * 2 * pi, imaginary part
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t k = 0; k < K; ++k) {
    float ar = 0.f, ai = 0.f;
    for (int64_t j = 0; j < J; ++j) {
      float c = cfg->trunc_brightness ? (float)(int)FF[j] : FF[j];
      if (cfg->mask_mode != MASK_NONE && shade) {
        const int32_t* M = shade + 4 * k;
        if (ref_window_hit_fast(j, cfg->res, M[0], M[1], M[2], M[3], cfg->mask_mode)) c = cfg->occluded_value;
      }
      // plain: u*l/dl + ... (:137); optim: u/dl hoisted, sum contracted to FMAs
      // (vissGen10M_shade_optim1.cu:161-163, 193)
      const float ph = optim ? std::fmaf(w[k] * (1.0f / d), n[j] - 1.0f, std::fmaf(v[k] * (1.0f / d), m[j], (u[k] * (1.0f / d)) * l[j]))
                             : u[k] * l[j] / d + v[k] * m[j] / d + w[k] * (n[j] - 1.0f) / d;
      const float x = two_pi_f * ph;
      ar = ar + c * cosf(x);
      ai = ai + c * sinf(x);
    }
    const float xw = two_pi_f * (w[k] / d);
    const float cr = cosf(xw), ci = sinf(xw);
    V[2 * k] = ar * cr - ai * ci;
    V[2 * k + 1] = ar * ci + ai * cr;
  }
  return 0;
}

ORACLE_API int oracle_recon_plain_f32(const oracle_dft_cfg* cfg, const float* u, const float* v,
                                      const float* w, const float* wgt, const float* Vin, int64_t K,
                                      const int32_t* shade, const float* l, const float* m,
                                      const float* n, int64_t J, float d, float* F, int nthreads, int optim) {
  const float two_pi_f = 2.0f * (float)kPi;
  std::vector<float> r1(K, 0.f), r2(K, 0.f);
  if (shade) {
    for (int64_t k = 0; k < K; ++k) {
      r1[k] = (float)shade[4 * k] / (float)shade[4 * k + 1];
      r2[k] = (float)shade[4 * k + 2] / (float)shade[4 * k + 3];
    }
  }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads_or_default(nthreads))
  for (int64_t j = 0; j < J; ++j) {
    const float phiP = std::floor((float)(j / cfg->res));
    const float thetaP = (float)j - phiP * (float)cfg->res;
    float fr = 0.f, fi = 0.f;
    for (int64_t k = 0; k < K; ++k) {
      if (shade && std::fabs(r1[k] - thetaP) < r1[k] && std::fabs(r2[k] - phiP) < r2[k]) continue;
      const float ph = optim ? std::fmaf(w[k], n[j] * (1.0f / d), std::fmaf(v[k], m[j] * (1.0f / d), u[k] * (l[j] * (1.0f / d))))
                             : u[k] * l[j] / d + v[k] * m[j] / d + w[k] * n[j] / d;
      const float x = two_pi_f * ph;
      const float cs = cosf(x), sn = sinf(x);
      const float yr = wgt[k] * Vin[2 * k], yi = wgt[k] * Vin[2 * k + 1];
      fr = fr + (yr * cs - yi * sn);
      fi = fi + (yr * sn + yi * cs);
    }
    F[2 * j] = fr / (float)K;
    F[2 * j + 1] = fi / (float)K;
  }
  return 0;
}

// ===========================================================================
// Geometric mask of a (K x J) block: mask[k*J+j] = occluded; margin in rad.
// ===========================================================================
ORACLE_API int oracle_geo_mask(const oracle_geo* geo, double R, const float* l, const float* m,
                               const float* n, int64_t K, int64_t J, uint8_t* mask, double* margin,
                               int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (int64_t k = 0; k < K; ++k) {
    const int32_t s = geo->snap[k];
    const int32_t pm = geo->pair[k] & 0xffff, pn = (geo->pair[k] >> 16) & 0xffff;
    const float* p1 = geo->sat_pos + ((int64_t)s * geo->nsat + pm) * 3;
    const float* p2 = geo->sat_pos + ((int64_t)s * geo->nsat + pn) * 3;
    for (int64_t j = 0; j < J; ++j) {
      const float sv[3] = {l[j], m[j], n[j]};
      double m1, m2;
      const int o1 = geo_occluded(sv, p1, R, &m1);
      const int o2 = geo_occluded(sv, p2, R, &m2);
      mask[k * J + j] = (uint8_t)(o1 | o2);
      // distance of the decision to the nearer limb that matters
      if (margin) margin[k * J + j] = std::min(std::fabs(m1), std::fabs(m2));
    }
  }
  return 0;
}

// ===========================================================================
// Orbit positions at the windowed snapshots (MIncline_generate_uvw_float.cu).
// ===========================================================================
typedef struct oracle_orbit_cfg {
  int32_t nsat;
  int32_t orbit_res;     // samples per orbit (reference 864000)
  int32_t orbit_counts;  // orbits (reference 140)
  int32_t index;         // period index (>= 1)
  double a_km;           // semi-major axis (reference 2038.14)
  double e;              // eccentricity (reference 0)
  double incl_deg;       // inclination (reference 30)
  double argp_deg;       // argument of perigee (reference 0)
  double raan_step_deg;  // node step per orbit (reference 0.08)
  const float* r1_m;     // [nsat] separation ramp start (m)
  const float* r2_m;     // [nsat] separation ramp middle (m)
} oracle_orbit_cfg;

namespace {

// Window of uvwPosition (:113-151): snapshot g of satellite `sat` reads global
// sample `circle` of the satellite's (OrbitCounts*OrbitRes) array.  Returns
// 0 normally, 1 when the reference zero-fills, 2 when circle == total: the
// reference then reads x[(sat+1)*total], the next satellite's slot, which its
// loop (:224-308) has not filled yet -- the zero of the initialised vector.
inline int window_index(int64_t g, int orbit_res, int orbit_counts, int64_t* circle) {
  const int span = orbit_res / 3;
  const int interval = orbit_res / 360 * 10;
  const int64_t total = (int64_t)orbit_res * orbit_counts;
  const int64_t k = g / span + 1;
  const int64_t offset = (k - 1) * interval;
  int64_t endIdx = (k - 1) * orbit_res + offset + span;
  int64_t startIdx = (k - 1) * orbit_res + offset;
  if ((k - 1) * (int64_t)(orbit_res + interval) > total) {
    const int64_t reset_index = total / (orbit_res + interval) + 1;
    startIdx = (k - 1 - reset_index) * orbit_res + offset;
    endIdx = (k - 1 - reset_index) * orbit_res + offset + span;
  }
  const int64_t c = startIdx + (g - (k - 1) * span);
  *circle = c;
  if (endIdx > total) {
    if (c > total) return 1;
    if (c == total) return 2;
  }
  return 0;
}

// Position of satellite `sat` at global sample `idx` (k = idx / OrbitRes,
// po = idx % OrbitRes), calculateOrbit (:83-110).
void orbit_position_f64(const oracle_orbit_cfg* cfg, int sat, int64_t idx, double out[3]) {
  const int64_t N = (int64_t)cfg->orbit_res * cfg->orbit_counts;
  const int64_t half = N / 2;
  const int64_t k = idx / cfg->orbit_res, po = idx % cfg->orbit_res;
  const double d2r = kPi / 180.0;
  double d;
  const double r1 = cfg->r1_m[sat], r2 = cfg->r2_m[sat];
  if (idx < half) d = r1 + (r2 - r1) / (double)(half - 1) * (double)idx;
  else d = r2 + (r1 - r2) / (double)(half - 1) * (double)(idx - half);
  const double dM = 2.0 * std::asin(d / (2.0 * cfg->a_km * 1e3));
  const double raan = (double)k * d2r * cfg->raan_step_deg +
                      (double)(cfg->index - 1) * (double)cfg->orbit_counts * d2r * cfg->raan_step_deg;
  const double M = 2.0 * kPi / (double)(cfg->orbit_res - 1) * (double)po + dM;
  // e = 0: Kepler's equation gives E = M; theta = 2 atan(tan(E/2)) wraps E to (-pi, pi]
  double E = M;
  for (int i = 1; i < 100 && cfg->e != 0.0; ++i) {
    const double err = M - (E - cfg->e * std::sin(E));
    if (std::fabs(err) < 1e-15) break;
    E = E + err / (1.0 - cfg->e * std::cos(E));
  }
  const double theta = 2.0 * std::atan(std::tan(E / 2.0) / std::sqrt((1.0 - cfg->e) / (1.0 + cfg->e)));
  const double r = cfg->a_km * (1.0 - cfg->e * cfg->e) / (1.0 + cfg->e * std::cos(theta));
  const double wv = theta + cfg->argp_deg * d2r;
  const double incl = cfg->incl_deg * d2r;
  out[0] = r * (std::cos(wv) * std::cos(raan) - std::sin(wv) * std::cos(incl) * std::sin(raan));
  out[1] = r * (std::cos(wv) * std::sin(raan) + std::sin(wv) * std::cos(incl) * std::cos(raan));
  out[2] = r * (std::sin(wv) * std::sin(incl));
}

// The same in the reference's FP32 arithmetic (host libm float functions).
void orbit_position_f32(const oracle_orbit_cfg* cfg, int sat, int64_t idx, float out[3]) {
  const int N = cfg->orbit_res * cfg->orbit_counts;
  const int half = N / 2;
  const int k = (int)(idx / cfg->orbit_res), po = (int)(idx % cfg->orbit_res);
  const float d2r = (float)(kPi / 180);
  const float a = (float)cfg->a_km;
  const float e = (float)cfg->e;
  const float incl = (float)cfg->incl_deg * d2r;
  const float argp = (float)cfg->argp_deg * d2r;
  float d;
  if (idx < half) {
    const float step = (cfg->r2_m[sat] - cfg->r1_m[sat]) / float(half - 1);
    d = std::fmaf(step, (float)idx, cfg->r1_m[sat]);
  } else {
    const float step = (cfg->r1_m[sat] - cfg->r2_m[sat]) / float(half - 1);
    d = std::fmaf(step, (float)(idx - half), cfg->r2_m[sat]);
  }
  const float dM = (float)(std::asin((double)d / ((double)(2 * a) * 1e3)) * 2);
  const float raan = (float)((double)((float)k * d2r) * (cfg->raan_step_deg) + 0.0 +
                             (double)((float)((cfg->index - 1) * cfg->orbit_counts) * d2r) * cfg->raan_step_deg);
  const float step_mt = (float)(2 * kPi) / float(cfg->orbit_res - 1);
  const float Mt = std::fmaf(step_mt, (float)po, 0.0f);
  const float M = Mt + dM;
  float E0 = M;
  for (int i = 1; i < 100; ++i) {
    const float M0 = E0 - e * sinf(E0);
    const float err = M - M0;
    if (std::fabs(err) < 1e-15) break;
    E0 = E0 + err / (1 - e * cosf(E0));
  }
  const float temp = tanf(E0 / 2) / sqrtf((1 - e) / (1 + e));
  const float theta = atanf(temp) * 2;
  const float r = a * (1 - e * e) / (1 + e * cosf(theta));
  const float wv = theta + argp;
  out[0] = r * (cosf(wv) * cosf(raan) - sinf(wv) * cosf(incl) * sinf(raan));
  out[1] = r * (cosf(wv) * sinf(raan) + sinf(wv) * cosf(incl) * cosf(raan));
  out[2] = r * (sinf(wv) * sinf(incl));
}

}  // namespace

// Satellite positions at every windowed snapshot: pos[g][sat][3] (km).
// mode 0 = FP64 (rounded to float on output), 1 = FP32 mimic.
ORACLE_API int oracle_orbit_positions(const oracle_orbit_cfg* cfg, int mode, float* pos, int nthreads) {
  const int span = cfg->orbit_res / 3;
  const int64_t S = (int64_t)cfg->orbit_counts * span;
  const int64_t total = (int64_t)cfg->orbit_res * cfg->orbit_counts;
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (int64_t g = 0; g < S; ++g) {
    int64_t circle;
    const int kind = window_index(g, cfg->orbit_res, cfg->orbit_counts, &circle);
    for (int sat = 0; sat < cfg->nsat; ++sat) {
      float* o = pos + (g * cfg->nsat + sat) * 3;
      if (kind != 0) {
        o[0] = o[1] = o[2] = 0.f;
        continue;
      }
      (void)total;
      if (mode == 0) {
        double p[3];
        orbit_position_f64(cfg, sat, circle, p);
        o[0] = (float)p[0]; o[1] = (float)p[1]; o[2] = (float)p[2];
      } else {
        orbit_position_f32(cfg, sat, circle, o);
      }
    }
  }
  return 0;
}

// FP64 positions without rounding (for the continuous-uvw mode).
ORACLE_API int oracle_orbit_positions_f64(const oracle_orbit_cfg* cfg, double* pos, int nthreads) {
  const int span = cfg->orbit_res / 3;
  const int64_t S = (int64_t)cfg->orbit_counts * span;
#pragma omp parallel for schedule(static) num_threads(nthreads_or_default(nthreads))
  for (int64_t g = 0; g < S; ++g) {
    int64_t circle;
    const int kind = window_index(g, cfg->orbit_res, cfg->orbit_counts, &circle);
    for (int sat = 0; sat < cfg->nsat; ++sat) {
      double* o = pos + (g * cfg->nsat + sat) * 3;
      if (kind != 0) { o[0] = o[1] = o[2] = 0.0; continue; }
      orbit_position_f64(cfg, sat, circle, o);
    }
  }
  return 0;
}

// Baseline uvw for every snapshot (snapshot-major, then pair).
// pairs: ordered (m != n, m-major, :350-353) or unordered (m < n).
// rounding: 1 = reference ceil((x_n - x_m) * 1e3 / lambda) with the difference
// in float and the scaling in double (:156-158); 0 = no rounding.
ORACLE_API int64_t oracle_uvw(const float* pos, int64_t S, int32_t nsat, int ordered, double lambda_m,
                              int rounding, float* u, float* v, float* w, int32_t* snap, int32_t* pair) {
  std::vector<std::pair<int, int>> pairs;
  for (int a = 0; a < nsat; ++a)
    for (int b = 0; b < nsat; ++b)
      if (ordered ? a != b : a < b) pairs.emplace_back(a, b);
  const int64_t P = (int64_t)pairs.size();
#pragma omp parallel for schedule(static)
  for (int64_t g = 0; g < S; ++g) {
    for (int64_t q = 0; q < P; ++q) {
      const int a = pairs[q].first, b = pairs[q].second;
      const float* pa = pos + (g * nsat + a) * 3;
      const float* pb = pos + (g * nsat + b) * 3;
      const int64_t k = g * P + q;
      float out[3];
      for (int c = 0; c < 3; ++c) {
        const float diff = pb[c] - pa[c];
        const double x = (double)diff * 1e3 / lambda_m;
        out[c] = rounding ? (float)std::ceil(x) : (float)x;
      }
      u[k] = out[0]; v[k] = out[1]; w[k] = out[2];
      if (snap) snap[k] = (int32_t)g;
      if (pair) pair[k] = a | (b << 16);
    }
  }
  return S * P;
}

// Continuous uvw from FP64 positions: (p_n - p_m) * 1e3 / lambda in double.
ORACLE_API int64_t oracle_uvw_f64(const double* pos, int64_t S, int32_t nsat, int ordered, double lambda_m,
                                  float* u, float* v, float* w) {
  int64_t k = 0;
  std::vector<std::pair<int, int>> pairs;
  for (int a = 0; a < nsat; ++a)
    for (int b = 0; b < nsat; ++b)
      if (ordered ? a != b : a < b) pairs.emplace_back(a, b);
  for (int64_t g = 0; g < S; ++g)
    for (auto& pr : pairs) {
      const double* pa = pos + (g * nsat + pr.first) * 3;
      const double* pb = pos + (g * nsat + pr.second) * 3;
      u[k] = (float)((pb[0] - pa[0]) * 1e3 / lambda_m);
      v[k] = (float)((pb[1] - pa[1]) * 1e3 / lambda_m);
      w[k] = (float)((pb[2] - pa[2]) * 1e3 / lambda_m);
      ++k;
    }
  return k;
}

// Reference dedup (:350-397): per ordered pair sort + unique, concatenate,
// then global sort + unique, lexicographic on (u, v, w).  The two-level
// procedure equals one global sort + unique.  In place; returns the count.
ORACLE_API int64_t oracle_dedup_uvw(float* u, float* v, float* w, int64_t K) {
  std::vector<std::tuple<float, float, float>> t((size_t)K);
  for (int64_t k = 0; k < K; ++k) t[k] = std::make_tuple(u[k], v[k], w[k]);
  std::sort(t.begin(), t.end());
  auto end = std::unique(t.begin(), t.end());
  int64_t n = end - t.begin();
  for (int64_t k = 0; k < n; ++k) {
    u[k] = std::get<0>(t[k]); v[k] = std::get<1>(t[k]); w[k] = std::get<2>(t[k]);
  }
  return n;
}

// ===========================================================================
// Shade windows (shade1M.cu:62-105, 218-225).  Output: 4 ints per uvw
// (thetaIndS, thetaIndE, phiIndS, phiIndE), 1-based as in the shadeM files.
// mode 1 mimics the FP32 ops; mode 0 evaluates angles in double.  mean_r is
// passed in (the reference sums in FP32 with thrust; order unknown), or
// computed here in double when mean_r_in <= 0.
// ===========================================================================
ORACLE_API double oracle_shade_windows(const float* u, const float* v, const float* w, int64_t K, int RES,
                                       double mean_r_in, int mode, int32_t* out) {
  double mean_r = mean_r_in;
  if (mean_r <= 0) {
    double acc = 0.0;
    for (int64_t k = 0; k < K; ++k) acc += std::sqrt((double)u[k] * u[k] + (double)v[k] * v[k] + (double)w[k] * w[k]);
    mean_r = acc / (double)K;
  }
  const float mean_rf = (float)mean_r;
  const float r0 = atanf(1737.74f / (mean_rf + 1737.74f));
  const float dtheta = (float)(2 * kPi / RES);
  const float dphi = (float)(kPi / RES);
  const int thetaR = (int)roundf(r0 / dtheta);
  const int phiR = (int)roundf((float)(thetaR / 2));
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < K; ++k) {
    int thetaInd, phiInd;
    if (mode == 1) {
      const float r = sqrtf(u[k] * u[k] + v[k] * v[k] + w[k] * w[k]);
      float th = atan2f(v[k], u[k]);
      float ph = asinf(w[k] / r);
      th = th + (float)kPi;
      ph = ph + (float)(kPi / 2);
      th = (float)(2 * kPi) - th;
      ph = (float)kPi - ph;
      thetaInd = f2i_cuda(roundf(th / dtheta));
      phiInd = f2i_cuda(roundf(ph / dphi));
    } else {
      const double r = std::sqrt((double)u[k] * u[k] + (double)v[k] * v[k] + (double)w[k] * w[k]);
      const double th = kPi - std::atan2((double)v[k], (double)u[k]);
      const double ph = kPi / 2 - std::asin((double)w[k] / r);
      thetaInd = f2i_cuda((float)std::round(th / (2 * kPi / RES)));
      phiInd = f2i_cuda((float)std::round(ph / (kPi / RES)));
    }
    int tS = thetaInd - thetaR, tE = thetaInd + thetaR, pS = phiInd - phiR, pE = phiInd + phiR;
    if (tS <= 0) tS += RES;
    if (tE > RES) tE -= RES;
    if (pS <= 0) pS += RES;
    if (pE > RES) pE -= RES;
    out[4 * k] = tS; out[4 * k + 1] = tE; out[4 * k + 2] = pS; out[4 * k + 3] = pE;
  }
  return mean_r;
}

// shadeM normalisation on load (vissGen10M_shade.cu:383-399): (min-1, max-1).
ORACLE_API void oracle_normalise_shade(const int32_t* raw, int64_t K, int32_t* M) {
  for (int64_t k = 0; k < K; ++k) {
    const int32_t a = raw[4 * k], b = raw[4 * k + 1], c = raw[4 * k + 2], d = raw[4 * k + 3];
    M[4 * k] = std::min(a, b) - 1;
    M[4 * k + 1] = std::max(a, b) - 1;
    M[4 * k + 2] = std::min(c, d) - 1;
    M[4 * k + 3] = std::max(c, d) - 1;
  }
}

// NX -> (countLoc, NXq) (vissGen1M_shade_optim1.cu:54-115): NX holds 1-based
// coarse ids as floats; NXq lists fine indices grouped by coarse id, ascending.
ORACLE_API void oracle_nxq(const float* NX, int64_t X, int64_t J, int32_t* countLoc, int32_t* NXq) {
  std::fill(countLoc, countLoc + J, 0);
  for (int64_t i = 0; i < X; ++i) {
    const int64_t q = (int64_t)(NX[i] - 1.0f);
    if (q >= 0 && q < J) countLoc[q]++;
  }
  std::vector<int64_t> start(J + 1, 0);
  for (int64_t q = 0; q < J; ++q) start[q + 1] = start[q] + countLoc[q];
  for (int64_t i = 0; i < X; ++i) {
    const int64_t q = (int64_t)(NX[i] - 1.0f);
    if (q >= 0 && q < J) NXq[start[q]++] = (int32_t)i;
  }
}

ORACLE_API int oracle_max_threads(void) { return omp_get_max_threads(); }

// ===========================================================================
// The reference's text I/O, restated as the CPU baseline of the text I/O path:
// one thread, formatted stream extraction of `ncols` floats per line until it
// fails (vissGen10M_shade.cu:354-365, `uvwFile >> u >> v >> w >> freq`), and one
// `file << value << std::endl` per value (:573-578).  Column c of row r lives at
// cols[c * cap + r].  Returns the rows read / written, -1 if the file does not open.
// ===========================================================================
ORACLE_API int64_t oracle_text_read_stream(const char* path, int ncols, float* cols, int64_t cap) {
  std::ifstream f(path);
  if (!f.is_open() || ncols < 1 || ncols > 8) return -1;
  float x[8];
  int64_t r = 0;
  for (;;) {
    int c = 0;
    while (c < ncols && (f >> x[c])) ++c;
    if (c < ncols) break;
    if (r < cap)
      for (int k = 0; k < ncols; ++k) cols[k * cap + r] = x[k];
    ++r;
  }
  return r;
}

ORACLE_API int64_t oracle_text_write_stream(const char* path, const float* values, int64_t n) {
  std::ofstream f(path);
  if (!f.is_open()) return -1;
  for (int64_t i = 0; i < n; ++i) f << values[i] << std::endl;
  return n;
}
