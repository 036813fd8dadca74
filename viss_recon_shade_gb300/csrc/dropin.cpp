// dropin.cpp -- drop-in replacements for the reference's programs, driving
// libvissgb.so through its C ABI with the reference's directory layout and
// text formats.  One binary; the program is chosen by the name it is run as
// (bin/ holds links) or by the first argument:
//
//   vissGen10M_shade   vissGen10M_shade.cu:178-611 (+ _optim1/_optim2 file names)
//   vissGen1M_shade    vissGen1M_shade_optim1.cu:265-726 (uvwMap130 weights, NX expansion)
//   vissGen1M_shade_appro     vissGen1M_shade_appro.cu:153-605 (coarse mean brightness,
//                      window on NX[j] - 1, d = 2.000955, F_recon_1M_appro/Ex...)
//   vissGen1M_shade_accurate  vissGen1M_shade_accurate.cu:95-620 (int-truncated
//                      brightness, F_recon_1M_accu/Ex{p}frequency1M.txt; the reference
//                      file itself does not compile: `totalnode` is undeclared at :300)
//   shade1M/10M/30M    shade1M.cu:130-280, shade10M.cu, shade30M.cu
//   MIncline_generate_uvw_float   MIncline_generate_uvw_float.cu:184-484
//
// Every constant the reference hard-codes is a flag with the reference's value
// as default.  Non-identity fine->coarse sky maps average the fine pixels of
// every coarse pixel, as the reference's visscal does.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <sys/stat.h>
#include <unordered_map>
#include <vector>

#include "viss_gb300.h"

namespace {

struct Args {
  std::map<std::string, std::string> kv;
  std::string get(const std::string& k, const std::string& d) const {
    auto it = kv.find(k);
    return it == kv.end() ? d : it->second;
  }
  long geti(const std::string& k, long d) const { return std::stol(get(k, std::to_string(d))); }
  double getd(const std::string& k, double d) const { return std::stod(get(k, std::to_string(d))); }
};

Args parse(int argc, char** argv, int first) {
  Args a;
  for (int i = first; i < argc; ++i) {
    std::string s = argv[i];
    if (s.rfind("--", 0) == 0) {
      auto eq = s.find('=');
      if (eq != std::string::npos) a.kv[s.substr(2, eq - 2)] = s.substr(eq + 1);
      else if (i + 1 < argc && std::string(argv[i + 1]).rfind("--", 0) != 0) a.kv[s.substr(2)] = argv[++i];
      else a.kv[s.substr(2)] = "1";
    }
  }
  return a;
}

#define CHECKV(call)                                                                       \
  do {                                                                                     \
    int rc_ = (call);                                                                      \
    if (rc_ != VISS_OK) {                                                                  \
      std::fprintf(stderr, "%s failed: %s (%s)\n", #call, viss_status_str(rc_), viss_last_error()); \
      return 1;                                                                            \
    }                                                                                      \
  } while (0)

#define CHECKC(call)                                                                       \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      std::fprintf(stderr, "%s failed: %s\n", #call, cudaGetErrorString(e_));              \
      return 1;                                                                            \
    }                                                                                      \
  } while (0)

template <class T>
struct Dev {
  T* p = nullptr;
  size_t n = 0;
  ~Dev() { if (p) cudaFree(p); }
  int alloc(size_t count) {
    n = count;
    return cudaMalloc(&p, sizeof(T) * (count ? count : 1)) == cudaSuccess ? 0 : 1;
  }
  int up(const T* h, size_t count) {
    if (alloc(count)) return 1;
    return count && cudaMemcpy(p, h, sizeof(T) * count, cudaMemcpyHostToDevice) != cudaSuccess;
  }
};

// Binary sidecar (--sidecar): full-precision copies of the outputs the text files
// round to 6 digits.  Little-endian: "VISS" magic, uint32 version 1, uint32 type
// (1 = complex64 pairs, 2 = float32), uint32 reserved, int64 count, then the data.
int write_sidecar(const std::string& path, const float* data, int64_t count, uint32_t type) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return 1;
  const uint32_t hdr[4] = {0x53534956u /* "VISS" */, 1u, type, 0u};
  const size_t per = type == 1 ? 2 : 1;
  bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(&count, sizeof(count), 1, f) == 1 &&
            (count == 0 || std::fwrite(data, sizeof(float) * per, (size_t)count, f) == (size_t)count);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? 0 : 1;
}

double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void mkdir_p(const std::string& d) { ::mkdir(d.c_str(), 0755); }

// Resume (--resume 1): the reference resumes a campaign by editing start_period by
// hand (vissGen10M_shade_optim2.cu:795); here a period whose output file already
// holds all of its lines is skipped.  Outputs are written under a temporary name
// and renamed when complete, so an interrupted run never leaves a partial file
// under the final name (a partial file from elsewhere fails the line count).
bool output_complete(const std::string& path, int ncols, int64_t rows, bool ints = false) {
  int64_t n = -1;
  const int rc = ints ? viss_text_read_ints(path.c_str(), ncols, nullptr, 0, &n)
                      : viss_text_read_floats(path.c_str(), 0, ncols, nullptr, 0, &n, nullptr);
  return rc == VISS_OK && n == rows;
}

int finish_output(const std::string& tmp, const std::string& path, int rc) {
  if (rc != VISS_OK) {
    std::remove(tmp.c_str());
    return rc;
  }
  return std::rename(tmp.c_str(), path.c_str()) == 0 ? VISS_OK : VISS_ERR_IO;
}

int write_floats_atomic(const std::string& path, int ncols, const float* cols, int64_t stride, int64_t rows) {
  const std::string tmp = path + ".part";
  return finish_output(tmp, path, viss_text_write_floats(tmp.c_str(), ncols, cols, stride, rows));
}

int write_ints_atomic(const std::string& path, int ncols, const int32_t* rows_data, int64_t rows) {
  const std::string tmp = path + ".part";
  return finish_output(tmp, path, viss_text_write_ints(tmp.c_str(), ncols, rows_data, rows));
}

int read_col(const std::string& path, bool header, std::vector<float>& out, int64_t* hv = nullptr) {
  int64_t rows = 0, h = 0;
  int rc = viss_text_read_floats(path.c_str(), header, 1, nullptr, 0, &rows, &h);
  if (rc) return rc;
  if (header && hv) *hv = h;
  out.resize(rows);
  return viss_text_read_floats(path.c_str(), header, 1, out.data(), rows, &rows, &h);
}

int read_cols(const std::string& path, int ncols, std::vector<float>& out, int64_t* rows) {
  int rc = viss_text_read_floats(path.c_str(), 0, ncols, nullptr, 0, rows, nullptr);
  if (rc) return rc;
  out.resize((size_t)*rows * ncols);
  return viss_text_read_floats(path.c_str(), 0, ncols, out.data(), *rows, rows, nullptr);
}

// ------------------------------------------------------------------ vissGen
// Shared by the 10M and 1M programs: per period, read uvw (+weights) and
// shadeM, run the vis DFT and the reconstruction, write Re(F).
int vissgen(const Args& a, bool tenM) {
  const std::string root = a.get("root", ".");
  const int RES = (int)a.geti("res", tenM ? 20940 : 2094);
  const std::string variant = a.get("variant", tenM ? "plain" : "optim1");
  const int start_period = (int)a.geti("start-period", tenM && variant == "optim2" ? 1 : 0);
  const int days = (int)a.geti("days", tenM && variant == "optim2" ? 34 : 1);
  const std::string prec_s = a.get("precision", "fast");
  const int precision = prec_s == "plain" ? VISS_PREC_PLAIN : prec_s == "comp" ? VISS_PREC_COMPENSATED : VISS_PREC_FAST;
  const std::string mask_s = a.get("mask", "quirk");
  const int mask = mask_s == "none" ? VISS_MASK_NONE : mask_s == "intended" ? VISS_MASK_REF_INTENDED : VISS_MASK_REF_QUIRK;
  const float d = (float)(2 * RES / (RES - 1));  // integer division, vissGen10M_shade.cu:183-185
  const std::string lmn = tenM ? root + "/lmn10M/" : root + "/frequency_1M/";
  const std::string freq_dir = tenM ? root + "/frequency_10M/" : root + "/frequency_1M/";
  const std::string dur = tenM ? "frequency10M" : "frequency1M";

  std::vector<float> l, m, n, C, NX, FF, NXq;
  int64_t J = 0, X = 0;
  if (read_col(lmn + "l.txt", true, l, &J) || read_col(lmn + "m.txt", false, m) || read_col(lmn + "n.txt", false, n) ||
      read_col(lmn + "C.txt", false, C) || read_col(lmn + "NX.txt", false, NX) || read_col(lmn + "FF.txt", true, FF, &X)) {
    std::fprintf(stderr, "cannot read the sky files under %s: %s\n", lmn.c_str(), viss_last_error());
    return 1;
  }
  if ((int64_t)l.size() < J || (int64_t)m.size() < J || (int64_t)n.size() < J || (int64_t)FF.size() < X) {
    std::fprintf(stderr, "sky files shorter than their headers\n");
    return 1;
  }
  l.resize(J); m.resize(J); n.resize(J); FF.resize(X); NX.resize(std::min<size_t>(NX.size(), (size_t)X));
  if ((int64_t)NX.size() < X) NX.resize(X, 0.0f);
  // fine->coarse map: the identity (X == J, NX[i] = i + 1, countLoc = 1) runs on the
  // coarse brightness directly; any other map averages the fine pixels per coarse
  // pixel (10M: countLoc.txt / NXq.txt as read, :261-286; 1M: inverted from NX,
  // vissGen1M_shade_optim1.cu:54-115)
  std::vector<float> cl;
  bool identity = X == J;
  for (int64_t i = 0; identity && i < X; ++i) identity = (int64_t)NX[i] == i + 1;
  if (tenM) {
    if (read_col(lmn + "countLoc.txt", false, cl) || read_col(lmn + "NXq.txt", false, NXq)) {
      std::fprintf(stderr, "cannot read countLoc.txt / NXq.txt under %s: %s\n", lmn.c_str(), viss_last_error());
      return 1;
    }
    if ((int64_t)cl.size() < J || (int64_t)NXq.size() < X) {
      std::fprintf(stderr, "countLoc.txt / NXq.txt shorter than the sky\n");
      return 1;
    }
    cl.resize(J); NXq.resize(X);
    for (int64_t j = 0; identity && j < J; ++j) identity = cl[j] == 1.0f;
    for (int64_t i = 0; identity && i < X; ++i) identity = (int64_t)NXq[i] == i;
  }
  if (tenM)  // clip_functor (vissGen10M_shade.cu:308); the 1M programs do not clip
    for (auto& x : n) x = std::fmax(-1.0f, std::fmin(1.0f, x));

  std::unordered_map<long long, float> uvwmap;  // 1M: uvwMap130.txt weights
  if (!tenM) {
    std::vector<float> mp;
    int64_t rows = 0;
    // header line = count, then "u v w count"
    if (viss_text_read_floats((freq_dir + "uvwMap130.txt").c_str(), 1, 4, nullptr, 0, &rows, nullptr) == VISS_OK) {
      mp.resize((size_t)rows * 4);
      int64_t hv;
      viss_text_read_floats((freq_dir + "uvwMap130.txt").c_str(), 1, 4, mp.data(), rows, &rows, &hv);
      for (int64_t r = 0; r < rows; ++r) {
        const long long key = ((long long)(int)mp[r] * 1000003LL + (long long)(int)mp[rows + r]) * 1000003LL +
                              (long long)(int)mp[2 * rows + r];
        uvwmap[key] = mp[3 * rows + r];
      }
    }
  }

  Dev<float> dl_, dm_, dn_, dFF, dNXqf;
  Dev<int32_t> dcl, dNXqi;
  if (dl_.up(l.data(), J) || dm_.up(m.data(), J) || dn_.up(n.data(), J) || dFF.up(FF.data(), identity ? J : X)) {
    std::fprintf(stderr, "device allocation failed\n");
    return 1;
  }
  if (!identity) {
    if (tenM) {
      std::vector<int32_t> cli(J);
      for (int64_t j = 0; j < J; ++j) cli[j] = (int32_t)cl[j];
      if (dcl.up(cli.data(), J) || dNXqf.up(NXq.data(), X)) {
        std::fprintf(stderr, "device allocation failed\n");
        return 1;
      }
    } else {
      Dev<float> dNX;
      Dev<char> ws;
      const size_t nb = viss_nxq_workspace(X, J);
      if (dNX.up(NX.data(), X) || dcl.alloc(J) || dNXqi.alloc(X) || ws.alloc(nb)) {
        std::fprintf(stderr, "device allocation failed\n");
        return 1;
      }
      CHECKV(viss_nxq(dNX.p, X, J, dcl.p, dNXqi.p, ws.p, nb, nullptr));
      CHECKC(cudaDeviceSynchronize());
    }
  }
  const bool accurate = variant == "accurate";
  const std::string outdir = tenM ? root + "/F_recon_10M/" : root + (accurate ? "/F_recon_1M_accu/" : "/F_recon_1M/");
  mkdir_p(outdir);
  const bool resume = a.get("resume", "0") != "0";
  for (int p = start_period; p < days; ++p) {
    const double t0 = now();
    std::string out;
    if (tenM) {
      const std::string suf = variant == "optim1" ? "_optim1" : variant == "optim2" ? "_optim2" : "";
      out = outdir + "F" + std::to_string(p + 1) + "period10M" + suf + ".txt";
    } else {
      out = accurate ? outdir + "Ex" + std::to_string(p + 1) + dur + ".txt"
                     : outdir + "F" + std::to_string(p + 1) + "_" + variant + ".txt";
    }
    if (resume && output_complete(out, 1, tenM ? J : X)) {
      std::printf("Period %d: %s complete, skipped\n", p + 1, out.c_str());
      continue;
    }
    std::vector<float> uvw;
    int64_t K = 0;
    const std::string uvw_path = freq_dir + (tenM ? "updated_uvw" : "uvw") + std::to_string(p + 1) + dur + ".txt";
    if (read_cols(uvw_path, tenM ? 4 : 3, uvw, &K)) {
      std::fprintf(stderr, "cannot read %s\n", uvw_path.c_str());
      return 1;
    }
    std::vector<float> wgt(K, 1.0f);
    for (int64_t k = 0; k < K; ++k) {
      if (tenM) {
        wgt[k] = 1.0f / uvw[3 * K + k];  // uvwFrequencyMap = 1/freq (:364)
      } else {
        const long long key = ((long long)(int)uvw[k] * 1000003LL + (long long)(int)uvw[K + k]) * 1000003LL +
                              (long long)(int)uvw[2 * K + k];
        auto it = uvwmap.find(key);
        wgt[k] = it != uvwmap.end() ? 1.0f / it->second : 1.0f;  // :458-470
      }
    }
    const std::string sh_path = freq_dir + "shadeM" + std::to_string(p + 1) + dur + ".txt";
    int64_t Ks = 0;
    std::vector<int32_t> raw;
    if (viss_text_read_ints(sh_path.c_str(), 4, nullptr, 0, &Ks) == VISS_OK) {
      raw.resize((size_t)Ks * 4);
      viss_text_read_ints(sh_path.c_str(), 4, raw.data(), Ks, &Ks);
    }
    if (Ks != K) std::printf("load wrong! uvw shape must be equal to shadeM shape\n");  // :402-406
    std::vector<int32_t> M1(K, 0), M2(K, 0), M3(K, 0), M4(K, 0);
    for (int64_t k = 0; k < K && k < Ks; ++k) {
      const int32_t* r = &raw[4 * k];
      M1[k] = std::min(r[0], r[1]) - 1; M2[k] = std::max(r[0], r[1]) - 1;
      M3[k] = std::min(r[2], r[3]) - 1; M4[k] = std::max(r[2], r[3]) - 1;
    }
    std::vector<float> r1(K), r2(K);
    for (int64_t k = 0; k < K; ++k) {
      r1[k] = (float)M1[k] / (float)M2[k];
      r2[k] = (float)M3[k] / (float)M4[k];
    }
    Dev<float> du, dv, dw, dwgt, dr1, dr2, dV, dF;
    Dev<int32_t> dM1, dM2, dM3, dM4;
    if (du.up(uvw.data(), K) || dv.up(uvw.data() + K, K) || dw.up(uvw.data() + 2 * K, K) || dwgt.up(wgt.data(), K) ||
        dM1.up(M1.data(), K) || dM2.up(M2.data(), K) || dM3.up(M3.data(), K) || dM4.up(M4.data(), K) ||
        dr1.up(r1.data(), K) || dr2.up(r2.data(), K) || dV.alloc(2 * K) || dF.alloc(2 * J)) {
      std::fprintf(stderr, "device allocation failed\n");
      return 1;
    }
    const double t1 = now();
    // plain and accurate truncate the fine brightness to int (vissGen1M_shade_accurate.cu:115)
    const int var = variant == "plain" || accurate ? VISS_VARIANT_PLAIN : VISS_VARIANT_OPTIM;
    if (identity || tenM) {
      CHECKV(viss_visscal((int)K, (int)J, RES, dFF.p, dV.p, du.p, dv.p, dw.p, dl_.p, dm_.p, dn_.p, dM1.p, dM2.p,
                          dM3.p, dM4.p, identity ? nullptr : dNXqf.p, identity ? nullptr : dcl.p, d, d, d, var, mask,
                          precision, nullptr));
    } else {
      // 1M with the in-program int NXq: the general map entry point with visscal's conventions
      viss_dft_cfg cfg{};
      cfg.mask_mode = mask; cfg.recon_mask = VISS_RECON_MASK_NONE; cfg.precision = precision; cfg.res = RES;
      cfg.trunc_brightness = var == VISS_VARIANT_PLAIN; cfg.occluded_value = 240.0f; cfg.phase_scale = 1.0 / d;
      cfg.n_offset = 0.0; cfg.moon_radius_km = 1737.4; cfg.norm = 1.0;
      std::vector<int32_t> sh(4 * (size_t)K);
      for (int64_t k = 0; k < K; ++k) {
        sh[4 * k] = M1[k]; sh[4 * k + 1] = M2[k]; sh[4 * k + 2] = M3[k]; sh[4 * k + 3] = M4[k];
      }
      Dev<int32_t> dsh;
      Dev<char> ws;
      viss_sky sky{dl_.p, dm_.p, dn_.p, nullptr, J};
      viss_fine_map fm{dFF.p, nullptr, dNXqi.p, dcl.p, X};
      viss_vis_set vs{du.p, dv.p, dw.p, nullptr, nullptr, nullptr, nullptr, K};
      const size_t nb = viss_vis_dft_map_workspace(&cfg, K, J, &fm, nullptr);
      if (dsh.up(sh.data(), 4 * K) || ws.alloc(nb)) {
        std::fprintf(stderr, "device allocation failed\n");
        return 1;
      }
      vs.shade = dsh.p;
      CHECKV(viss_vis_dft_map(&cfg, &sky, &fm, &vs, nullptr, dV.p, ws.p, nb, nullptr));
    }
    CHECKC(cudaDeviceSynchronize());
    const double t2 = now();
    CHECKV(viss_imagerecon((int)K, (int)J, RES, dF.p, dV.p, du.p, dv.p, dw.p, dl_.p, dm_.p, dn_.p, dwgt.p, dr1.p,
                           dr2.p, dr1.p, dr2.p, d, d, d, precision, nullptr));
    CHECKC(cudaDeviceSynchronize());
    const double t3 = now();
    std::vector<float> F(2 * J);
    CHECKC(cudaMemcpy(F.data(), dF.p, sizeof(float) * 2 * J, cudaMemcpyDeviceToHost));
    if (tenM) {
      std::vector<float> re(J);
      for (int64_t j = 0; j < J; ++j) re[j] = F[2 * j];
      CHECKV(write_floats_atomic(out, 1, re.data(), J, J));
    } else {
      // expanded to the fine grid: F[NX[c]-1] (vissGen1M_shade_optim1.cu:680-684,
      // vissGen1M_shade_accurate.cu:571-585 as Ex{p}frequency1M.txt)
      std::vector<float> re(X);
      for (int64_t c = 0; c < X; ++c) re[c] = F[2 * ((int64_t)NX[c] - 1)];
      CHECKV(write_floats_atomic(out, 1, re.data(), X, X));
    }
    if (a.get("sidecar", "0") != "0") {
      // V (which the reference never writes) and complex F at full precision, next to the text file
      std::vector<float> Vh(2 * K);
      CHECKC(cudaMemcpy(Vh.data(), dV.p, sizeof(float) * 2 * K, cudaMemcpyDeviceToHost));
      const std::string stem = out.substr(0, out.size() - 4);
      if (write_sidecar(stem + ".V.c64", Vh.data(), K, 1) || write_sidecar(stem + ".F.c64", F.data(), J, 1)) {
        std::fprintf(stderr, "cannot write the sidecar files %s.{V,F}.c64\n", stem.c_str());
        return 1;
      }
    }
    const double t4 = now();
    std::printf("Period %d Load UWV Cost Time is: %f s\n", p + 1, t1 - t0);
    std::printf("Period %d Compute Viss Cost Time is: %f s\n", p + 1, t2 - t1);
    std::printf("Period %d Image Reconstruction Cost Time is: %f s\n", p + 1, t3 - t2);
    std::printf("Period %d Save Image Cost Time is: %f s (%s)\n", p + 1, t4 - t3, out.c_str());
  }
  return 0;
}

// ------------------------------------------------------------------ appro
// vissGen1M_shade_appro.cu:153-605: C_j = mean of FF over the fine pixels with
// NX == j + 1 (computeC, :72-90; 0 without members), the window of row k tested
// on NX[j] - 1 (:113-118; the 240 replaces C_j for that term only: the
// reference's write into the shared C is a race), d = (float)2 * RES / (RES - 1)
// (:155-157), reconstruction without a mask (its masked value is overwritten,
// :142-144), uvwMap130 weights, F / K, written expanded to the fine grid as
// F_recon_1M_appro/Ex{p}frequency1M.txt (:553-568).
int appro(const Args& a) {
  const std::string root = a.get("root", ".");
  const int RES = (int)a.geti("res", 2094);
  const int start_period = (int)a.geti("start-period", 0);
  const int days = (int)a.geti("days", 1);
  const std::string prec_s = a.get("precision", "fast");
  const int precision = prec_s == "plain" ? VISS_PREC_PLAIN : prec_s == "comp" ? VISS_PREC_COMPENSATED : VISS_PREC_FAST;
  const std::string mask_s = a.get("mask", "quirk");
  const int mask = mask_s == "intended" ? VISS_MASK_REF_INTENDED : VISS_MASK_REF_QUIRK;
  const float d = (float)2 * RES / (RES - 1);
  const std::string dir = root + "/frequency_1M/";
  std::vector<float> l, m, n, NX, FF;
  int64_t J = 0, X = 0;
  if (read_col(dir + "l.txt", true, l, &J) || read_col(dir + "m.txt", false, m) || read_col(dir + "n.txt", false, n) ||
      read_col(dir + "NX.txt", false, NX) || read_col(dir + "FF.txt", true, FF, &X)) {
    std::fprintf(stderr, "cannot read the sky files under %s: %s\n", dir.c_str(), viss_last_error());
    return 1;
  }
  if ((int64_t)l.size() < J || (int64_t)m.size() < J || (int64_t)n.size() < J || (int64_t)FF.size() < X) {
    std::fprintf(stderr, "sky files shorter than their headers\n");
    return 1;
  }
  l.resize(J); m.resize(J); n.resize(J); FF.resize(X);
  NX.resize((size_t)X, 0.0f);
  // computeC: float sums in fine-index order
  std::vector<float> Csum(J, 0.0f), C(J, 0.0f);
  std::vector<int> cnt(J, 0);
  for (int64_t i = 0; i < X; ++i) {
    const int64_t q = (int64_t)NX[i] - 1;
    if (q >= 0 && q < J && (float)(q + 1) == NX[i]) { Csum[q] += FF[i]; ++cnt[q]; }
  }
  for (int64_t j = 0; j < J; ++j) C[j] = cnt[j] > 0 ? Csum[j] / (float)cnt[j] : 0.0f;
  std::vector<int32_t> widx(J);
  for (int64_t j = 0; j < J; ++j) widx[j] = j < X ? (int32_t)NX[j] - 1 : -1;
  std::unordered_map<long long, float> uvwmap;
  {
    int64_t rows = 0;
    const std::string mp_path = dir + "uvwMap130.txt";
    if (viss_text_read_floats(mp_path.c_str(), 1, 4, nullptr, 0, &rows, nullptr) == VISS_OK) {
      std::vector<float> mp((size_t)rows * 4);
      int64_t hv;
      viss_text_read_floats(mp_path.c_str(), 1, 4, mp.data(), rows, &rows, &hv);
      for (int64_t r = 0; r < rows; ++r) {
        const long long key = ((long long)(int)mp[r] * 1000003LL + (long long)(int)mp[rows + r]) * 1000003LL +
                              (long long)(int)mp[2 * rows + r];
        uvwmap[key] = mp[3 * rows + r];
      }
    }
  }
  Dev<float> dl_, dm_, dn_, dC;
  Dev<int32_t> dwidx;
  if (dl_.up(l.data(), J) || dm_.up(m.data(), J) || dn_.up(n.data(), J) || dC.up(C.data(), J) ||
      dwidx.up(widx.data(), J)) {
    std::fprintf(stderr, "device allocation failed\n");
    return 1;
  }
  const std::string outdir = root + "/F_recon_1M_appro/";
  mkdir_p(outdir);
  const bool resume = a.get("resume", "0") != "0";
  for (int p = start_period; p < days; ++p) {
    const std::string out = outdir + "Ex" + std::to_string(p + 1) + "frequency1M.txt";
    if (resume && output_complete(out, 1, X)) {
      std::printf("Period %d: %s complete, skipped\n", p + 1, out.c_str());
      continue;
    }
    std::vector<float> uvw;
    int64_t K = 0;
    const std::string uvw_path = dir + "uvw" + std::to_string(p + 1) + "frequency1M.txt";
    if (read_cols(uvw_path, 3, uvw, &K)) {
      std::fprintf(stderr, "cannot read %s\n", uvw_path.c_str());
      return 1;
    }
    std::vector<float> wgt(K, 1.0f);
    for (int64_t k = 0; k < K; ++k) {
      const long long key = ((long long)(int)uvw[k] * 1000003LL + (long long)(int)uvw[K + k]) * 1000003LL +
                            (long long)(int)uvw[2 * K + k];
      auto it = uvwmap.find(key);
      wgt[k] = it != uvwmap.end() ? 1.0f / it->second : 1.0f;
    }
    const std::string sh_path = dir + "shadeM" + std::to_string(p + 1) + "frequency1M.txt";
    int64_t Ks = 0;
    std::vector<int32_t> raw;
    if (viss_text_read_ints(sh_path.c_str(), 4, nullptr, 0, &Ks) == VISS_OK) {
      raw.resize((size_t)Ks * 4);
      viss_text_read_ints(sh_path.c_str(), 4, raw.data(), Ks, &Ks);
    }
    std::vector<int32_t> sh(4 * (size_t)K, 0);
    for (int64_t k = 0; k < K && k < Ks; ++k) {
      const int32_t* r = &raw[4 * k];
      sh[4 * k] = std::min(r[0], r[1]) - 1; sh[4 * k + 1] = std::max(r[0], r[1]) - 1;
      sh[4 * k + 2] = std::min(r[2], r[3]) - 1; sh[4 * k + 3] = std::max(r[2], r[3]) - 1;
    }
    Dev<float> du, dv, dw, dwgt, dV, dF;
    Dev<int32_t> dsh;
    Dev<char> ws;
    if (du.up(uvw.data(), K) || dv.up(uvw.data() + K, K) || dw.up(uvw.data() + 2 * K, K) || dwgt.up(wgt.data(), K) ||
        dsh.up(sh.data(), 4 * K) || dV.alloc(2 * K) || dF.alloc(2 * J)) {
      std::fprintf(stderr, "device allocation failed\n");
      return 1;
    }
    viss_dft_cfg cfg{};
    cfg.mask_mode = mask; cfg.recon_mask = VISS_RECON_MASK_NONE; cfg.precision = precision; cfg.res = RES;
    cfg.trunc_brightness = 0; cfg.occluded_value = 240.0f; cfg.phase_scale = 1.0 / (double)d; cfg.n_offset = 0.0;
    cfg.moon_radius_km = 1737.4; cfg.norm = K > 0 ? 1.0 / (double)K : 1.0;
    viss_sky sky{dl_.p, dm_.p, dn_.p, dC.p, J};
    viss_vis_set vs{du.p, dv.p, dw.p, dwgt.p, dsh.p, nullptr, nullptr, K};
    const size_t nb = std::max(viss_vis_dft_windowed_workspace(&cfg, K, J), viss_recon_workspace(&cfg, K, J, nullptr));
    if (ws.alloc(nb)) return 1;
    CHECKV(viss_vis_dft_windowed(&cfg, &sky, dwidx.p, &vs, dV.p, ws.p, nb, nullptr));
    CHECKV(viss_recon(&cfg, &sky, &vs, nullptr, dV.p, dF.p, ws.p, nb, nullptr));
    std::vector<float> F(2 * J);
    CHECKC(cudaMemcpy(F.data(), dF.p, sizeof(float) * 2 * J, cudaMemcpyDeviceToHost));
    std::vector<float> re(X);
    for (int64_t c = 0; c < X; ++c) {
      const int64_t q = (int64_t)NX[c] - 1;
      re[c] = q >= 0 && q < J ? F[2 * q] : 0.0f;
    }
    CHECKV(write_floats_atomic(out, 1, re.data(), X, X));
    std::printf("Period %d: %lld uvw -> %s\n", p + 1, (long long)K, out.c_str());
  }
  return 0;
}

// ------------------------------------------------------------------ shade
int shade(const Args& a, const std::string& which) {
  const std::string root = a.get("root", ".");
  int RES = which == "shade1M" ? 2094 : which == "shade10M" ? 20940 : 62820;
  RES = (int)a.geti("res", RES);
  const std::string dir = root + (which == "shade1M" ? "/frequency_1M/" : which == "shade10M" ? "/frequency_10M/"
                                                                                               : "/frequency_30M/");
  const std::string dur = which == "shade1M" ? "frequency1M" : which == "shade10M" ? "frequency10M" : "frequency30M";
  // shade1M: periods 1..130 of uvw{p}; shade10M: updated_uvw{p}, p = 2..34 (its loop starts at
  // tid+1, so period 1 is skipped, shade10M.cu:152); shade30M: one file uvw1 -> ./shade30Mperiod1.txt
  const int first = (int)a.geti("first", which == "shade10M" ? 2 : 1);
  const int last = (int)a.geti("last", which == "shade1M" ? 130 : which == "shade10M" ? 34 : 1);
  const bool resume = a.get("resume", "0") != "0";
  for (int p = first; p <= last; ++p) {
    const std::string in = dir + (which == "shade10M" ? "updated_uvw" : "uvw") + std::to_string(p) + dur + ".txt";
    const std::string op = which == "shade30M" ? root + "/shade30Mperiod1.txt"
                                               : dir + "shadeM" + std::to_string(p) + dur + ".txt";
    std::vector<float> uvw;
    int64_t K = 0;
    if (read_cols(in, which == "shade10M" ? 4 : 3, uvw, &K)) {
      std::printf("address_uvw: %s (missing, skipped)\n", in.c_str());
      continue;
    }
    if (resume && output_complete(op, 4, K, true)) {
      std::printf("period %d: %s complete, skipped\n", p, op.c_str());
      continue;
    }
    Dev<float> du, dv, dw;
    Dev<int32_t> dout;
    Dev<char> ws;
    const size_t wsb = viss_shade_windows_workspace(K);
    if (du.up(uvw.data(), K) || dv.up(uvw.data() + K, K) || dw.up(uvw.data() + 2 * K, K) || dout.alloc(4 * K) ||
        ws.alloc(wsb)) {
      std::fprintf(stderr, "device allocation failed\n");
      return 1;
    }
    double mean_r = 0;
    CHECKV(viss_shade_windows(du.p, dv.p, dw.p, K, RES, a.getd("mean-r", 0.0), dout.p, &mean_r, ws.p, wsb, nullptr));
    std::vector<int32_t> out(4 * K);
    CHECKC(cudaMemcpy(out.data(), dout.p, sizeof(int32_t) * 4 * K, cudaMemcpyDeviceToHost));
    CHECKV(write_ints_atomic(op, 4, out.data(), K));
    std::printf("period %d: %lld uvw, mean r %.6g, wrote %s\n", p, (long long)K, mean_r, op.c_str());
  }
  return 0;
}

// ------------------------------------------------------------------ MIncline
int mincline(const Args& a) {
  const std::string root = a.get("root", ".");
  const int periods = (int)a.geti("periods", 34);
  const int first = (int)a.geti("first", 1);
  const double frequency = a.getd("frequency", 1e7);
  const double stride = a.getd("stride", 0.01);
  viss_orbit_cfg cfg{};
  cfg.nsat = 8;
  cfg.orbit_res = (int)(2.4 * 3600 * (int)(1.0 / stride));  // :185
  cfg.orbit_res = (int)a.geti("orbit-res", cfg.orbit_res);
  cfg.orbit_counts = (int)a.geti("orbit-counts", 140);
  cfg.a_km = 2038.14; cfg.e = 0; cfg.incl_deg = 30; cfg.argp_deg = 0; cfg.raan_step_deg = 0.08;
  static const float r1[8] = {0, 1e3, 4.45e3, 6e3, 9.1e3, 16.2e3, 35.3e3, 100e3};
  static const float r2[8] = {0, 0.1e3, 0.445e3, 0.6e3, 0.91e3, 1.62e3, 3.53e3, 10e3};
  cfg.r1_m = r1; cfg.r2_m = r2;
  cfg.fp64 = 0;
  const int lambda = (int)(3e8 / frequency);  // int lambda (:190)
  const std::string dir = root + "/frequency_10M/";
  mkdir_p(dir);
  for (int index = first; index <= periods; ++index) {
    cfg.index = index;
    const int64_t S = viss_orbit_snapshots(&cfg);
    const int P = 56;
    const int64_t K = S * P;
    Dev<float> pos, u, v, w;
    Dev<char> ws;
    if (pos.alloc(S * 8 * 3)) {
      std::fprintf(stderr, "device allocation failed\n");
      return 1;
    }
    CHECKV(viss_orbit_positions(&cfg, pos.p, nullptr, nullptr));
    // baselines, the pairs' lists concatenated pair-major, global sort + unique, in one pass
    const size_t wsb = viss_unique_uvw_workspace(S, 8, 1);
    if (ws.alloc(wsb)) return 1;
    int64_t cnt = 0;
    CHECKV(viss_unique_uvw(pos.p, S, 8, 1, (double)lambda, nullptr, nullptr, nullptr, 0, &cnt, ws.p, wsb, nullptr));
    if (u.alloc(cnt > 0 ? cnt : 1) || v.alloc(cnt > 0 ? cnt : 1) || w.alloc(cnt > 0 ? cnt : 1)) return 1;
    CHECKV(viss_unique_uvw(pos.p, S, 8, 1, (double)lambda, u.p, v.p, w.p, cnt, &cnt, ws.p, wsb, nullptr));
    std::vector<float> h(3 * cnt);
    CHECKC(cudaMemcpy(h.data(), u.p, sizeof(float) * cnt, cudaMemcpyDeviceToHost));
    CHECKC(cudaMemcpy(h.data() + cnt, v.p, sizeof(float) * cnt, cudaMemcpyDeviceToHost));
    CHECKC(cudaMemcpy(h.data() + 2 * cnt, w.p, sizeof(float) * cnt, cudaMemcpyDeviceToHost));
    const std::string out = dir + "uvw" + std::to_string(index) + "frequency10M.txt";
    CHECKV(viss_text_write_floats(out.c_str(), 3, h.data(), cnt, cnt));
    std::printf("period %d: %lld unique uvw of %lld -> %s\n", index, (long long)cnt, (long long)K, out.c_str());
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  std::string prog = argv[0];
  auto slash = prog.find_last_of('/');
  if (slash != std::string::npos) prog = prog.substr(slash + 1);
  int first = 1;
  if (prog == "viss_dropin" && argc > 1) {
    prog = argv[1];
    first = 2;
  }
  const Args a = parse(argc, argv, first);
  if (prog.rfind("vissGen10M", 0) == 0) {
    Args b = a;
    if (prog.find("optim1") != std::string::npos && !a.kv.count("variant")) b.kv["variant"] = "optim1";
    if (prog.find("optim2") != std::string::npos && !a.kv.count("variant")) b.kv["variant"] = "optim2";
    return vissgen(b, true);
  }
  if (prog.rfind("vissGen1M", 0) == 0) {
    Args b = a;
    if (prog.find("optim2") != std::string::npos && !a.kv.count("variant")) b.kv["variant"] = "optim2";
    if (prog.find("accurate") != std::string::npos && !a.kv.count("variant")) b.kv["variant"] = "accurate";
    if (prog.find("appro") != std::string::npos) return appro(a);
    return vissgen(b, false);
  }
  if (prog == "shade1M" || prog == "shade10M" || prog == "shade30M") return shade(a, prog);
  if (prog.rfind("MIncline", 0) == 0) return mincline(a);
  std::fprintf(stderr,
               "usage: viss_dropin {vissGen10M_shade|vissGen10M_shade_optim1|vissGen10M_shade_optim2|"
               "vissGen1M_shade_optim1|vissGen1M_shade_optim2|vissGen1M_shade_accurate|vissGen1M_shade_appro|"
               "shade1M|shade10M|shade30M|"
               "MIncline_generate_uvw_float} [--root DIR] [--flag value ...]\n");
  return 2;
}
