// capi.cu -- the extern "C" entry points of libvissgb.so for the DFT passes:
// argument checks, workspace layout, launch planning and kernel dispatch.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "viss_internal.cuh"

namespace viss {

thread_local std::string g_last_error;
thread_local uint64_t g_launches = 0;

void count_launch() { ++g_launches; }

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}
int cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return VISS_ERR_CUDA;
}

int device_sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 148;
  return n;
}

int launch_prep_recon_ratios(const float* thetaP0, const float* phiP0, const float* dtheta, const float* dphi,
                             int64_t K, int64_t Kpad, int4* win, int* flags, cudaStream_t st);

static inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// ------------------------------------------------------------------ plans
// Channels of a pass (a single-channel call is a batch of one).
struct Batch {
  ChannelRows ch{};
  const float* bright = nullptr;   // [nch][J] or NULL
  float norm[VISS_MAX_CH] = {};
};

// Runtime launch choices (viss_tuning); zeros pick the defaults.
struct Tuning {
  int ctas_per_sm = 0;
  int vis_split = 0;
  int rec_items = 0;
  int tile = 0;  // bit 0: vis sky tiles of VIS_P / 2; recon row tiles: bit 1 REC_Q / 2, bit 3 REC_Q, else 2 REC_Q
};

static int make_batch(const viss_batch* b, int64_t K, const viss_dft_cfg& cfg, Batch& out) {
  const int nch = b ? b->nch : 1;
  if (nch < 1 || nch > VISS_MAX_CH) return fail(VISS_ERR_RANGE, "nch must be in [1, 64]");
  out.ch.nch = nch;
  out.ch.row_off[0] = 0;
  for (int c = 0; c < nch; ++c) {
    const int64_t e = b ? (b->row_off ? b->row_off[c + 1] : -1) : K;
    if (b && (!b->row_off || b->row_off[0] != 0)) return fail(VISS_ERR_INVALID, "batch row_off must start at 0");
    if (e < out.ch.row_off[c]) return fail(VISS_ERR_INVALID, "batch row_off must be non-decreasing");
    out.ch.row_off[c + 1] = e;
    out.norm[c] = (float)((b && b->norm) ? b->norm[c] : cfg.norm);
  }
  if (out.ch.row_off[nch] != K) return fail(VISS_ERR_INVALID, "batch row_off[nch] must equal the visibility count");
  out.ch.rb_off[0] = 0;
  for (int c = 0; c < nch; ++c) {
    const int64_t kc = out.ch.row_off[c + 1] - out.ch.row_off[c];
    out.ch.rb_off[c + 1] = out.ch.rb_off[c] + (kc + VIS_ROWS - 1) / VIS_ROWS;
  }
  out.bright = b ? b->bright : nullptr;
  return VISS_OK;
}

static Tuning make_tuning(const viss_tuning* t) {
  Tuning r;
  if (t) {
    r.ctas_per_sm = t->ctas_per_sm > 0 ? t->ctas_per_sm : 0;
    r.vis_split = t->vis_split > 0 ? t->vis_split : 0;
    r.rec_items = t->rec_items > 0 ? t->rec_items : 0;
    r.tile = t->tile & 15;
  }
  return r;
}

// Resident CTAs the persistent kernels are planned for.
static int64_t planned_ctas(const Tuning& t, int minb) {
  const int per_sm = (t.ctas_per_sm > 0 && t.ctas_per_sm < minb) ? t.ctas_per_sm : minb;
  return (int64_t)device_sm_count() * per_sm;
}

// Layout of the workspace of one vis pass.  Chosen from (rows per channel, J,
// mode, tuning) only, so the size query and the call agree.
struct VisPlan {
  int64_t K = 0, J = 0, Jpad = 0, Kpad = 0, nrb = 0, jchunk = 0, nsd = 0, X = 0;
  int nsplit = 1;
  bool geo = false, ref = false, comp = false, plain = false, map = false;
  bool windexed = false;  // REF windows test a per-pixel index (viss_vis_dft_windowed)
  int2* rrng = nullptr;
  float* mbase = nullptr;
  int4* mbox = nullptr;
  int2 *mmem = nullptr, *mtile = nullptr;
  int* members = nullptr;
  char* mscratch = nullptr;
  size_t mscratch_bytes = 0;
  int4 *pix0 = nullptr, *pix1 = nullptr, *rows0 = nullptr, *win = nullptr;
  float4 *rows1 = nullptr, *plo = nullptr, *pgeo = nullptr, *rowsf = nullptr, *satdir = nullptr, *cones = nullptr;
  int* rowsat = nullptr;
  int2* pqr = nullptr;
  float2* partial = nullptr;
  int* flags = nullptr;
  size_t bytes = 0;

  void layout(void* ws) {
    Carver c(ws);
    flags = c.take<int>(FLAG_WORDS);
    if (plain && geo) satdir = c.take<float4>(nsd);
    if (!plain) {
      pix0 = c.take<int4>(Jpad);
      pix1 = c.take<int4>(Jpad);
      if (comp) plo = c.take<float4>(Jpad);
      if (geo) pgeo = c.take<float4>(Jpad);
      if (ref) pqr = c.take<int2>(Jpad);
      rows0 = c.take<int4>(Kpad);
      rows1 = c.take<float4>(Kpad);
      if (geo) rowsat = c.take<int>(Kpad);
      if (comp) rowsf = c.take<float4>(Kpad);
      if (ref) win = c.take<int4>(Kpad);
      if (geo) { satdir = c.take<float4>(nsd); cones = c.take<float4>(2 * nrb); }
      if (nsplit > 1) partial = c.take<float2>((size_t)nsplit * K);
      if (map) {
        mbase = c.take<float>(Jpad);
        mbox = c.take<int4>(Jpad);
        mmem = c.take<int2>(Jpad);
        mtile = c.take<int2>(Jpad / VIS_P);
        members = c.take<int>(X > 0 ? X : 1);
        mscratch_bytes = fine_map_scratch(J);
        mscratch = c.take<char>(mscratch_bytes);
      }
      if (windexed && ref) rrng = c.take<int2>(Jpad / VIS_P);
    }
    bytes = c.size();
  }
};

static void plan_vis(VisPlan& p, const viss_dft_cfg& cfg, const Batch& bt, int64_t J, const viss_geometry* geo,
                     const Tuning& tn, const viss_fine_map* map = nullptr, bool windexed = false) {
  p.K = bt.ch.row_off[bt.ch.nch]; p.J = J;
  p.windexed = windexed;
  p.map = map != nullptr;
  p.X = map ? map->X : 0;
  p.plain = plain_precision(cfg.precision);
  p.geo = cfg.mask_mode == VISS_MASK_GEOMETRIC;
  p.ref = cfg.mask_mode == VISS_MASK_REF_QUIRK || cfg.mask_mode == VISS_MASK_REF_INTENDED;
  p.comp = cfg.precision == VISS_PREC_COMPENSATED;
  p.Jpad = round_up(J > 0 ? J : 1, REC_PIX);
  p.nrb = bt.ch.rb_off[bt.ch.nch];
  p.Kpad = (p.nrb > 0 ? p.nrb : 1) * VIS_ROWS;
  p.nsd = (geo && p.geo) ? geo->S * (int64_t)geo->nsat : 0;
  // Split the sky into chunks until there are ~64 work items (visibility block x
  // sky chunk) per resident CTA: blocks see different occluded fractions of the sky,
  // and short items balance them (10 MHz vis: 1 chunk 158 ms, 2 149 ms, 9 143.3 ms,
  // 16 142.6 ms, 24 142.5 ms).
  const int64_t slots = planned_ctas(tn, VISS_VIS_MINB);
  int64_t nsplit = 1;
  if (tn.vis_split > 0) nsplit = tn.vis_split;
  else if (p.nrb > 0 && p.nrb < 64 * slots) nsplit = (64 * slots + p.nrb - 1) / p.nrb;
  const int64_t maxsplit = (J + VIS_P - 1) / VIS_P;
  if (nsplit > maxsplit) nsplit = maxsplit;
  if (nsplit < 1) nsplit = 1;
  p.jchunk = round_up((J + nsplit - 1) / nsplit, VIS_P);
  if (p.jchunk <= 0) p.jchunk = VIS_P;
  p.nsplit = (int)((J + p.jchunk - 1) / p.jchunk);
  if (p.nsplit < 1) p.nsplit = 1;
  p.layout(nullptr);
}

struct RecPlan {
  int64_t K = 0, J = 0, Jpad = 0, Kpad = 0, npb = 0, nsd = 0, S = 0;
  int nseg = 0, nslot = 0;
  int64_t seg_lo[VISS_MAX_SEG] = {}, seg_hi[VISS_MAX_SEG] = {};
  int seg_ch[VISS_MAX_SEG] = {}, seg_slot[VISS_MAX_SEG] = {};
  int slot0[VISS_MAX_CH] = {}, nslot_ch[VISS_MAX_CH] = {};
  bool geo = false, ref = false, comp = false, plain = false;
  int4 *pix0 = nullptr, *pix1 = nullptr, *rows0 = nullptr, *win = nullptr;
  float4 *rows1 = nullptr, *plo = nullptr, *pgeo = nullptr, *rowsf = nullptr, *satdir = nullptr, *scones = nullptr;
  float4 *bcones = nullptr, *wcones = nullptr;
  int* rowsat = nullptr;
  int2* pqr = nullptr;
  float2* partial = nullptr;
  float* ratios = nullptr;
  int* flags = nullptr;
  int32_t* perm = nullptr;
  char* order_scratch = nullptr;
  size_t order_bytes = 0;
  size_t bytes = 0;

  void layout(void* ws) {
    Carver c(ws);
    flags = c.take<int>(FLAG_WORDS);
    if (plain) {
      if (ref) ratios = c.take<float>(2 * (size_t)Kpad);
      if (geo) satdir = c.take<float4>(nsd);
    } else {
      if (geo) {
        perm = c.take<int32_t>(J > 0 ? J : 1);
        order_bytes = pixel_order_scratch(J);
        order_scratch = c.take<char>(order_bytes);
      }
      pix0 = c.take<int4>(Jpad);
      pix1 = c.take<int4>(Jpad);
      if (comp) plo = c.take<float4>(Jpad);
      if (geo) pgeo = c.take<float4>(Jpad);
      if (ref) pqr = c.take<int2>(Jpad);
      rows0 = c.take<int4>(Kpad);
      rows1 = c.take<float4>(Kpad);
      if (geo) rowsat = c.take<int>(Kpad);
      if (comp) rowsf = c.take<float4>(Kpad);
      if (ref) win = c.take<int4>(Kpad);
      if (geo) {
        satdir = c.take<float4>(nsd);
        scones = c.take<float4>(2 * S);
        bcones = c.take<float4>(2 * npb);
        wcones = c.take<float4>(2 * npb * (REC_THREADS / 32));
      }
      if (nslot > 0) partial = c.take<float2>((size_t)nslot * J);
    }
    bytes = c.size();
  }
};

// Recon work: every channel's rows cut into segments of about L rows, L chosen
// for ~rec_items work items (segment x pixel block) per resident CTA; at most
// VISS_MAX_SEG segments.  Segments are ordered longest first.
static void plan_segments(RecPlan& p, const Batch& bt, const Tuning& tn) {
  constexpr int64_t unit = REC_Q;
  const int nch = bt.ch.nch;
  // items per CTA: many short segments balance blocks whose pixels the Moon hides for
  // different parts of the orbit (10 MHz recon: 4 items 191 ms, 8 176 ms, 32 167 ms, 64 165 ms)
  // resident CTAs: VISS_REC_MINB for the geometric kernel, one more for the others (recon.cu)
  const int64_t target = (tn.rec_items > 0 ? tn.rec_items : 64) * planned_ctas(tn, p.geo ? VISS_REC_MINB : VISS_REC_MINB + 1);
  int64_t L = p.npb > 0 ? (p.K * p.npb + target - 1) / target : p.K;
  L = round_up(L > unit ? L : unit, unit);
  auto count = [&](int64_t len) {
    int64_t n = 0;
    for (int c = 0; c < nch; ++c) {
      const int64_t kc = bt.ch.row_off[c + 1] - bt.ch.row_off[c];
      n += (kc + len - 1) / len;
    }
    return n;
  };
  while (count(L) > VISS_MAX_SEG) L = round_up(L + L / 4 + 1, unit);
  struct Seg { int64_t lo, hi; int ch, idx; };
  Seg segs[VISS_MAX_SEG];
  int ns = 0, slots = 0;
  for (int c = 0; c < nch; ++c) {
    const int64_t r0 = bt.ch.row_off[c], kc = bt.ch.row_off[c + 1] - r0;
    const int64_t n = (kc + L - 1) / L;
    p.slot0[c] = slots;
    p.nslot_ch[c] = n > 1 ? (int)n : 0;
    for (int64_t i = 0; i < n; ++i) {
      segs[ns] = Seg{r0 + kc * i / n, r0 + kc * (i + 1) / n, c, n > 1 ? slots + (int)i : -1};
      ++ns;
    }
    if (n > 1) slots += (int)n;
  }
  // longest first (stable)
  for (int i = 1; i < ns; ++i) {
    const Seg s = segs[i];
    int j = i - 1;
    while (j >= 0 && segs[j].hi - segs[j].lo < s.hi - s.lo) { segs[j + 1] = segs[j]; --j; }
    segs[j + 1] = s;
  }
  p.nseg = ns;
  p.nslot = slots;
  for (int i = 0; i < ns; ++i) {
    p.seg_lo[i] = segs[i].lo; p.seg_hi[i] = segs[i].hi; p.seg_ch[i] = segs[i].ch; p.seg_slot[i] = segs[i].idx;
  }
}

static void plan_recon(RecPlan& p, const viss_dft_cfg& cfg, const Batch& bt, int64_t J, const viss_geometry* geo,
                       const Tuning& tn) {
  p.K = bt.ch.row_off[bt.ch.nch]; p.J = J;
  p.plain = plain_precision(cfg.precision);
  p.geo = cfg.recon_mask == VISS_RECON_MASK_GEOMETRIC;
  p.ref = cfg.recon_mask == VISS_RECON_MASK_REF;
  p.comp = cfg.precision == VISS_PREC_COMPENSATED;
  p.Jpad = round_up(J > 0 ? J : 1, REC_PIX);
  p.Kpad = p.K > 0 ? p.K : 1;
  p.npb = p.Jpad / REC_PIX;
  p.S = (geo && p.geo) ? geo->S : 0;
  p.nsd = (geo && p.geo) ? geo->S * (int64_t)geo->nsat : 0;
  if (!p.plain) plan_segments(p, bt, tn);
  p.layout(nullptr);
}

// ------------------------------------------------------------------ checks
static int check_cfg(const viss_dft_cfg* cfg) {
  if (!cfg) return fail(VISS_ERR_INVALID, "cfg is NULL");
  if (cfg->mask_mode < VISS_MASK_NONE || cfg->mask_mode > VISS_MASK_GEOMETRIC)
    return fail(VISS_ERR_INVALID, "mask_mode out of range");
  if (cfg->recon_mask < VISS_RECON_MASK_NONE || cfg->recon_mask > VISS_RECON_MASK_GEOMETRIC)
    return fail(VISS_ERR_INVALID, "recon_mask out of range");
  if (cfg->precision < VISS_PREC_PLAIN || cfg->precision > VISS_PREC_F64_PHASE)
    return fail(VISS_ERR_INVALID, "precision out of range");
  if (!(cfg->phase_scale > 0.0) || !(cfg->phase_scale <= 1.0))
    return fail(VISS_ERR_RANGE, "phase_scale must be in (0, 1]");
  if (!(cfg->n_offset >= -1.0 && cfg->n_offset <= 0.0)) return fail(VISS_ERR_RANGE, "n_offset must be in [-1, 0]");
  return VISS_OK;
}

static int check_geo(const viss_geometry* geo, const viss_vis_set* vis, const viss_dft_cfg* cfg) {
  if (!geo || !geo->sat_pos) return fail(VISS_ERR_INVALID, "GEOMETRIC mask needs satellite positions");
  if (geo->nsat < 1 || geo->nsat > 32) return fail(VISS_ERR_RANGE, "nsat must be in [1, 32]");
  if (geo->S < 1) return fail(VISS_ERR_INVALID, "geometry has no snapshots");
  if (geo->S * (int64_t)geo->nsat >= ((int64_t)1 << 26)) return fail(VISS_ERR_RANGE, "S * nsat must be < 2^26");
  if (!vis->snap || !vis->pair) return fail(VISS_ERR_INVALID, "GEOMETRIC mask needs snap and pair per visibility");
  if (!(cfg->moon_radius_km > 0.0)) return fail(VISS_ERR_RANGE, "moon_radius_km must be > 0");
  return VISS_OK;
}

static int check_sky(const viss_sky* sky, bool need_bright) {
  if (!sky) return fail(VISS_ERR_INVALID, "sky is NULL");
  if (sky->J < 0 || sky->J > (int64_t)1 << 30) return fail(VISS_ERR_RANGE, "J out of range");
  if (sky->J > 0 && (!sky->l || !sky->m || !sky->n)) return fail(VISS_ERR_INVALID, "sky l/m/n NULL");
  if (need_bright && sky->J > 0 && !sky->bright) return fail(VISS_ERR_INVALID, "sky brightness NULL");
  return VISS_OK;
}

static int check_vis(const viss_vis_set* vis) {
  if (!vis) return fail(VISS_ERR_INVALID, "vis set is NULL");
  if (vis->K < 0 || vis->K > (int64_t)1 << 31) return fail(VISS_ERR_RANGE, "K out of range");
  if (vis->K > 0 && (!vis->u || !vis->v || !vis->w)) return fail(VISS_ERR_INVALID, "u/v/w NULL");
  return VISS_OK;
}

static int check_ws(void* ws, size_t have, size_t need) {
  if (need == 0) return VISS_OK;
  if (!ws) return fail(VISS_ERR_WORKSPACE, "workspace is NULL");
  if (reinterpret_cast<uintptr_t>(ws) & 255) return fail(VISS_ERR_WORKSPACE, "workspace not 256-byte aligned");
  if (have < need)
    return fail(VISS_ERR_WORKSPACE, "workspace too small: need " + std::to_string(need) + " bytes");
  return VISS_OK;
}

// ------------------------------------------------------------------ passes
static viss_vis_set channel_rows(const viss_vis_set& vis, int64_t r0, int64_t r1) {
  viss_vis_set c = vis;
  c.u = vis.u + r0; c.v = vis.v + r0; c.w = vis.w + r0;
  if (vis.wgt) c.wgt = vis.wgt + r0;
  if (vis.shade) c.shade = vis.shade + 4 * r0;
  if (vis.snap) c.snap = vis.snap + r0;
  if (vis.pair) c.pair = vis.pair + r0;
  c.K = r1 - r0;
  return c;
}

int vis_dft_impl(const viss_dft_cfg& cfg, const double scale[3], const float dlmn[3], const viss_sky& sky,
                 const viss_vis_set& vis, const Batch& bt, const viss_geometry* geo, const Tuning& tn, float* V,
                 void* ws, size_t ws_bytes, cudaStream_t st, const viss_fine_map* map = nullptr,
                 const int32_t* widx = nullptr) {
  VisPlan p;
  plan_vis(p, cfg, bt, sky.J, geo, tn, map, widx != nullptr);
  // work items are counted in int (a caller's vis_split can ask for more)
  if (!p.plain && p.nrb * (int64_t)p.nsplit > (int64_t)INT32_MAX)
    return fail(VISS_ERR_RANGE, "visibility blocks x sky chunks must be < 2^31: lower vis_split");
  int rc = check_ws(ws, ws_bytes, p.bytes);
  if (rc) return rc;
  if (vis.K == 0) return VISS_OK;
  if (sky.J == 0) {
    VISS_CUDA(cudaMemsetAsync(V, 0, sizeof(float2) * (size_t)vis.K, st));
    return VISS_OK;
  }
  p.layout(ws);
  VISS_CUDA(cudaMemsetAsync(p.flags, 0, FLAG_WORDS * sizeof(int), st));
  if (p.plain) {
    // the reference's form: one launch per channel
    if (p.geo && (rc = launch_prep_satdir(geo->sat_pos, p.nsd, cfg.moon_radius_km, p.satdir, st))) return rc;
    for (int c = 0; c < bt.ch.nch; ++c) {
      const int64_t r0 = bt.ch.row_off[c], r1 = bt.ch.row_off[c + 1];
      if (r1 == r0) continue;
      viss_sky sc = sky;
      if (bt.bright) sc.bright = bt.bright + (int64_t)c * sky.J;
      if ((rc = launch_vis_plain(cfg, sc, channel_rows(vis, r0, r1), geo, p.satdir, dlmn,
                                 reinterpret_cast<float2*>(V) + r0, st, map, p.flags, widx)))
        return rc;
    }
    return VISS_OK;
  }
  if (map && (rc = prep_fine_map(map->NXq_f, map->NXq_i, map->countLoc, map->FF, sky.J, map->X, cfg.res,
                                 cfg.trunc_brightness, p.Jpad, p.mbase, p.mbox, p.mmem, p.members, p.mtile,
                                 p.mscratch, p.mscratch_bytes, p.flags, st)))
    return rc;
  PixPrepArgs pa{};
  pa.l = sky.l; pa.m = sky.m; pa.n = sky.n; pa.bright = bt.bright ? nullptr : (map ? p.mbase : sky.bright);
  pa.J = sky.J; pa.Jpad = p.Jpad;
  pa.sl = scale[0]; pa.sm = scale[1]; pa.sn = scale[2]; pa.n_offset = cfg.n_offset;
  pa.res = cfg.res; pa.trunc = map ? 0 : cfg.trunc_brightness;  // the map's base brightness is truncated per member
  pa.rec0 = p.pix0; pa.rec1 = p.pix1; pa.lo = p.plo; pa.geo = p.pgeo; pa.qr = p.pqr;
  pa.widx = p.ref ? widx : nullptr;
  if ((rc = launch_prep_pixels(pa, st))) return rc;
  if (p.rrng && (rc = launch_prep_ref_ranges(widx, sky.J, p.Jpad / VIS_P, p.rrng, st))) return rc;
  RowPrepArgs ra{};
  ra.u = vis.u; ra.v = vis.v; ra.w = vis.w; ra.shade = vis.shade;
  ra.snap = p.geo ? vis.snap : nullptr; ra.pair = p.geo ? vis.pair : nullptr;
  ra.nsat = geo ? geo->nsat : 0; ra.S = geo ? geo->S : 0;
  ra.sn = scale[2]; ra.n_offset = cfg.n_offset;
  ra.ch = bt.ch; ra.padded = true;
  ra.K = vis.K; ra.Kpad = p.Kpad; ra.mask_mode = cfg.mask_mode; ra.recon_mask = VISS_RECON_MASK_NONE;
  ra.rows0 = p.rows0; ra.rows1 = p.rows1; ra.rowsat = p.rowsat; ra.uf = p.rowsf; ra.win = p.win;
  ra.flags = p.flags;
  if ((rc = launch_prep_rows(ra, false, st))) return rc;
  if (p.geo) {
    if ((rc = launch_prep_satdir(geo->sat_pos, p.nsd, cfg.moon_radius_km, p.satdir, st))) return rc;
    if ((rc = launch_prep_rowblock_cones(p.rowsat, p.satdir, bt.ch, p.nrb, p.cones, st))) return rc;
  }
  VisParams vp{};
  vp.pix0 = p.pix0; vp.pix1 = p.pix1; vp.plo = p.plo; vp.pgeo = p.pgeo; vp.pqr = p.pqr;
  vp.rows0 = p.rows0; vp.rows1 = p.rows1; vp.rowsat = p.rowsat; vp.rowsf = p.rowsf; vp.win = p.win;
  vp.satdir = p.satdir; vp.cones = p.cones;
  vp.l = sky.l; vp.m = sky.m; vp.n = sky.n; vp.sat_pos = geo ? geo->sat_pos : nullptr;
  vp.bright = bt.bright;
  vp.flags = p.flags;
  vp.out = p.nsplit > 1 ? p.partial : reinterpret_cast<float2*>(V);
  vp.K = vis.K; vp.J = sky.J; vp.jchunk = p.jchunk; vp.nsplit = p.nsplit;
  vp.nitems = (int)(p.nrb * p.nsplit);
  vp.res = cfg.res > 0 ? cfg.res : 1; vp.occ_val = cfg.occluded_value; vp.R = cfg.moon_radius_km;
  vp.nsat = geo ? geo->nsat : 1;
  vp.mask = cfg.mask_mode;
  vp.ch = bt.ch;
  vp.small_tile = tn.tile & 1;
  vp.ref_rng = p.rrng;
  if (map) {
    vp.use_map = 1;
    vp.map.box = p.mbox; vp.map.mem = p.mmem; vp.map.members = p.members; vp.map.FF = map->FF;
    vp.map.tile_rng = p.mtile; vp.map.trunc = cfg.trunc_brightness;
  }
  if ((rc = launch_vis_fast(vp, tn.ctas_per_sm, p.comp, st))) return rc;
  if (p.nsplit > 1) return launch_vis_reduce(p.partial, p.nsplit, vis.K, reinterpret_cast<float2*>(V), st);
  return VISS_OK;
}

int recon_impl(const viss_dft_cfg& cfg, const double scale[3], const float dlmn[3], const viss_sky& sky,
               const viss_vis_set& vis, const Batch& bt, const viss_geometry* geo, const Tuning& tn, const float* V,
               float* F, void* ws, size_t ws_bytes, cudaStream_t st, const float* ratio_arrays[4]) {
  RecPlan p;
  plan_recon(p, cfg, bt, sky.J, geo, tn);
  int rc = check_ws(ws, ws_bytes, p.bytes);
  if (rc) return rc;
  if (sky.J == 0) return VISS_OK;
  if (vis.K == 0) {
    VISS_CUDA(cudaMemsetAsync(F, 0, sizeof(float2) * (size_t)sky.J * bt.ch.nch, st));
    return VISS_OK;
  }
  p.layout(ws);
  VISS_CUDA(cudaMemsetAsync(p.flags, 0, FLAG_WORDS * sizeof(int), st));
  float2* const F2 = reinterpret_cast<float2*>(F);
  // channels without visibilities reconstruct to zero
  for (int c = 0; c < bt.ch.nch; ++c)
    if (bt.ch.row_off[c + 1] == bt.ch.row_off[c])
      VISS_CUDA(cudaMemsetAsync(F2 + (int64_t)c * sky.J, 0, sizeof(float2) * (size_t)sky.J, st));
  if (p.plain) {
    // the reference's form: one launch per channel
    if (p.geo && (rc = launch_prep_satdir(geo->sat_pos, p.nsd, cfg.moon_radius_km, p.satdir, st))) return rc;
    for (int c = 0; c < bt.ch.nch; ++c) {
      const int64_t r0 = bt.ch.row_off[c], r1 = bt.ch.row_off[c + 1];
      if (r1 == r0) continue;
      const viss_vis_set vc = channel_rows(vis, r0, r1);
      const float* ratios = nullptr;
      if (p.ref) {
        float* rc_ratios = p.ratios + 2 * r0;  // [r1 (K_c), r2 (K_c)]
        if (ratio_arrays) {
          VISS_CUDA(cudaMemcpyAsync(rc_ratios, ratio_arrays[0] + r0, sizeof(float) * vc.K, cudaMemcpyDeviceToDevice,
                                    st));
          VISS_CUDA(cudaMemcpyAsync(rc_ratios + vc.K, ratio_arrays[1] + r0, sizeof(float) * vc.K,
                                    cudaMemcpyDeviceToDevice, st));
        } else {
          extern int launch_shade_ratios(const int32_t* shade, int64_t K, float* r, cudaStream_t st);
          if ((rc = launch_shade_ratios(vc.shade, vc.K, rc_ratios, st))) return rc;
        }
        ratios = rc_ratios;
      }
      viss_dft_cfg cc = cfg;
      cc.norm = bt.norm[c];
      if ((rc = launch_recon_plain(cc, sky, vc, geo, V + 2 * r0, ratios, p.satdir, dlmn, F2 + (int64_t)c * sky.J,
                                   st, p.flags)))
        return rc;
    }
    return VISS_OK;
  }
  if (p.geo) {
    if ((rc = pixel_order(sky.l, sky.m, sky.n, sky.J, p.order_scratch, p.order_bytes, p.perm, st))) return rc;
  }
  PixPrepArgs pa{};
  pa.perm = p.perm;
  pa.l = sky.l; pa.m = sky.m; pa.n = sky.n; pa.bright = nullptr;
  pa.J = sky.J; pa.Jpad = p.Jpad;
  pa.sl = scale[0]; pa.sm = scale[1]; pa.sn = scale[2]; pa.n_offset = cfg.n_offset;
  pa.res = cfg.res; pa.trunc = 0;
  pa.rec0 = p.pix0; pa.rec1 = p.pix1; pa.lo = p.plo; pa.geo = p.pgeo; pa.qr = p.pqr;
  if ((rc = launch_prep_pixels(pa, st))) return rc;
  RowPrepArgs ra{};
  ra.u = vis.u; ra.v = vis.v; ra.w = vis.w; ra.wgt = vis.wgt; ra.V = V;
  ra.shade = ratio_arrays ? nullptr : vis.shade;
  ra.snap = p.geo ? vis.snap : nullptr; ra.pair = p.geo ? vis.pair : nullptr;
  ra.nsat = geo ? geo->nsat : 0; ra.S = geo ? geo->S : 0;
  ra.sn = scale[2]; ra.n_offset = cfg.n_offset;
  ra.ch = bt.ch; ra.padded = false;
  ra.K = vis.K; ra.Kpad = p.Kpad; ra.mask_mode = VISS_MASK_NONE; ra.recon_mask = cfg.recon_mask;
  ra.rows0 = p.rows0; ra.rows1 = p.rows1; ra.rowsat = p.rowsat; ra.uf = p.rowsf; ra.win = p.win;
  ra.flags = p.flags;
  if ((rc = launch_prep_rows(ra, true, st))) return rc;
  if (p.ref && ratio_arrays) {
    if ((rc = launch_prep_recon_ratios(ratio_arrays[0], ratio_arrays[1], ratio_arrays[2], ratio_arrays[3], vis.K,
                                       p.Kpad, p.win, p.flags, st)))
      return rc;
  }
  if (p.geo) {
    if ((rc = launch_prep_satdir(geo->sat_pos, p.nsd, cfg.moon_radius_km, p.satdir, st))) return rc;
    if ((rc = launch_prep_snapshot_cones(p.satdir, geo->S, geo->nsat, p.scones, st))) return rc;
    if ((rc = launch_prep_block_cones(p.pgeo, sky.J, REC_PIX, p.npb, p.bcones, st))) return rc;
    if ((rc = launch_prep_block_cones(p.pgeo, sky.J, 32 * REC_TJ, p.npb * (REC_THREADS / 32), p.wcones, st)))
      return rc;
  }
  ReconParams rp{};
  rp.pix0 = p.pix0; rp.pix1 = p.pix1; rp.plo = p.plo; rp.pgeo = p.pgeo; rp.pqr = p.pqr;
  rp.rows0 = p.rows0; rp.rows1 = p.rows1; rp.rowsat = p.rowsat; rp.rowsf = p.rowsf; rp.win = p.win;
  rp.satdir = p.satdir; rp.scones = p.scones; rp.bcones = p.bcones; rp.wcones = p.wcones;
  rp.l = sky.l; rp.m = sky.m; rp.n = sky.n; rp.sat_pos = geo ? geo->sat_pos : nullptr;
  rp.flags = p.flags;
  rp.perm = p.perm;
  rp.out = F2;
  rp.partial = p.partial;
  rp.K = vis.K; rp.J = sky.J;
  rp.res = cfg.res > 0 ? cfg.res : 1; rp.nsat = geo ? geo->nsat : 1; rp.R = cfg.moon_radius_km;
  rp.recon_mask = cfg.recon_mask;
  // Row tiles: as asked, else 512 rows (1,024 with the geometric mask, recon.cu).
  // Geometric recon, 512 against 256 rows: 10 MHz 167.8 / 169.9 ms, its 49,152-pixel
  // case 12.38 / 12.58 ms, 30 MHz 2,541 / 2,579 ms (longer tiles drop hidden rows and
  // meet at barriers less often); unmasked 168.3 / 168.2 ms.
  if ((tn.tile >> 1) & 1) rp.row_tile = 1;
  else if ((tn.tile >> 3) & 1) rp.row_tile = 0;
  else rp.row_tile = 2;
  rp.npb = (int)p.npb;
  rp.nseg = p.nseg;
  rp.nitems = (int)(p.nseg * p.npb);
  for (int i = 0; i < p.nseg; ++i) {
    rp.seg_lo[i] = p.seg_lo[i]; rp.seg_hi[i] = p.seg_hi[i]; rp.seg_ch[i] = p.seg_ch[i]; rp.seg_slot[i] = p.seg_slot[i];
  }
  for (int c = 0; c < bt.ch.nch; ++c) rp.ch_norm[c] = bt.norm[c];
  if ((rc = launch_recon_fast(rp, tn.ctas_per_sm, p.comp, st))) return rc;
  if (p.nslot > 0) {
    RecReduceParams rr{};
    rr.partial = p.partial; rr.perm = p.perm; rr.out = F2; rr.J = sky.J; rr.nch = bt.ch.nch;
    for (int c = 0; c < bt.ch.nch; ++c) { rr.slot0[c] = p.slot0[c]; rr.nslot[c] = p.nslot_ch[c]; rr.norm[c] = bt.norm[c]; }
    return launch_recon_reduce(rr, st);
  }
  return VISS_OK;
}

__global__ void sum_counts_kernel(const int32_t* c, int64_t n, unsigned long long* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  long long v = i < n ? (long long)c[i] : 0;
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v != 0) atomicAdd(out, (unsigned long long)v);
}

// sum of n device ints, read back to the host (synchronises the stream)
int sum_counts(const int32_t* c, int64_t n, int64_t* total, cudaStream_t st) {
  unsigned long long* d = nullptr;
  VISS_CUDA(cudaMallocAsync(&d, sizeof(unsigned long long), st));
  unsigned long long h = 0;
  cudaError_t e = cudaMemsetAsync(d, 0, sizeof(h), st);
  if (e == cudaSuccess && n > 0) {
    sum_counts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(c, n, d);
    e = cudaGetLastError();
    if (e == cudaSuccess) count_launch();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st);
  cudaError_t e2 = cudaFreeAsync(d, st);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "sum of countLoc");
  *total = (int64_t)(long long)h;
  return VISS_OK;
}

// SoA shade columns -> K x 4
__global__ void pack_shade_kernel(const int* M1, const int* M2, const int* M3, const int* M4, int64_t K, int4* out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < K) out[k] = make_int4(M1[k], M2[k], M3[k], M4[k]);
}

__global__ void shade_ratios_kernel(const int32_t* shade, int64_t K, float* r) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  r[k] = (float)shade[4 * k] / (float)shade[4 * k + 1];
  r[K + k] = (float)shade[4 * k + 2] / (float)shade[4 * k + 3];
}

int launch_shade_ratios(const int32_t* shade, int64_t K, float* r, cudaStream_t st) {
  if (K <= 0) return VISS_OK;
  shade_ratios_kernel<<<(unsigned)((K + 255) / 256), 256, 0, st>>>(shade, K, r);
  VISS_LAUNCH_CHECK("shade_ratios_kernel");
  return VISS_OK;
}

}  // namespace viss

using namespace viss;

// ====================================================================== C ABI
extern "C" {

const char* viss_status_str(int status) {
  switch (status) {
    case VISS_OK: return "ok";
    case VISS_ERR_INVALID: return "invalid argument";
    case VISS_ERR_WORKSPACE: return "workspace missing, misaligned or too small";
    case VISS_ERR_CUDA: return "CUDA runtime error";
    case VISS_ERR_RANGE: return "input out of supported range";
    case VISS_ERR_TIMEOUT: return "device-side wait timed out";
    case VISS_ERR_UNSUPPORTED: return "unsupported combination";
    case VISS_ERR_IO: return "file I/O error";
    case VISS_ERR_FORMAT: return "file format error";
    default: return "unknown status";
  }
}

const char* viss_last_error(void) { return g_last_error.c_str(); }

int viss_version(void) { return 10000; }

uint64_t viss_launch_count(void) { return g_launches; }

size_t viss_vis_dft_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J, const viss_geometry* geo) {
  return viss_vis_dft_batch_workspace(cfg, nullptr, K, J, geo, nullptr);
}

size_t viss_vis_dft_batch_workspace(const viss_dft_cfg* cfg, const viss_batch* batch, int64_t K, int64_t J,
                                    const viss_geometry* geo, const viss_tuning* tuning) {
  if (!cfg || K < 0 || J < 0) return 0;
  Batch bt;
  if (make_batch(batch, K, *cfg, bt)) return 0;
  VisPlan p;
  plan_vis(p, *cfg, bt, J, geo, make_tuning(tuning));
  return p.bytes;
}

static int check_vis_call(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
                          const viss_geometry* geo, const viss_batch* batch, const float* V) {
  int rc;
  const bool own_bright = batch && batch->bright;
  if ((rc = check_cfg(cfg)) || (rc = check_sky(sky, !own_bright)) || (rc = check_vis(vis))) return rc;
  if (vis->K > 0 && !V) return fail(VISS_ERR_INVALID, "V is NULL");
  if ((cfg->mask_mode == VISS_MASK_REF_QUIRK || cfg->mask_mode == VISS_MASK_REF_INTENDED)) {
    if (!vis->shade) return fail(VISS_ERR_INVALID, "REF mask needs shade windows");
    if (cfg->res < 1) return fail(VISS_ERR_RANGE, "REF mask needs res >= 1");
  }
  if (own_bright && cfg->trunc_brightness && !plain_precision(cfg->precision))
    return fail(VISS_ERR_UNSUPPORTED, "trunc_brightness with per-channel brightness");
  if (cfg->mask_mode == VISS_MASK_GEOMETRIC && (rc = check_geo(geo, vis, cfg))) return rc;
  return VISS_OK;
}

int viss_workspace_flags(const void* workspace, int32_t* flags, void* stream) {
  if (!workspace || !flags) return fail(VISS_ERR_INVALID, "workspace or flags is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the flag words are the first carve of every pass's workspace
  VISS_CUDA(cudaMemcpyAsync(flags, static_cast<const int*>(workspace) + FLAG_ERR, sizeof(int32_t),
                            cudaMemcpyDeviceToHost, st));
  VISS_CUDA(cudaStreamSynchronize(st));
  return VISS_OK;
}

int viss_workspace_limb_count(const void* workspace, int64_t* count, void* stream) {
  if (!workspace || !count) return fail(VISS_ERR_INVALID, "workspace or count is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  VISS_CUDA(cudaMemcpyAsync(count, static_cast<const int*>(workspace) + FLAG_LIMB, sizeof(int64_t),
                            cudaMemcpyDeviceToHost, st));
  VISS_CUDA(cudaStreamSynchronize(st));
  return VISS_OK;
}

int viss_vis_dft(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis, const viss_geometry* geo,
                 float* V, void* workspace, size_t workspace_bytes, void* stream) {
  return viss_vis_dft_batch(cfg, sky, vis, nullptr, geo, nullptr, V, workspace, workspace_bytes, stream);
}

int viss_vis_dft_batch(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
                       const viss_batch* batch, const viss_geometry* geo, const viss_tuning* tuning, float* V,
                       void* workspace, size_t workspace_bytes, void* stream) {
  int rc;
  if ((rc = check_vis_call(cfg, sky, vis, geo, batch, V))) return rc;
  Batch bt;
  if ((rc = make_batch(batch, vis->K, *cfg, bt))) return rc;
  const double s = cfg->phase_scale;
  const double scale[3] = {s, s, s};
  const float d = (float)(1.0 / s);
  const float dlmn[3] = {d, d, d};
  return vis_dft_impl(*cfg, scale, dlmn, *sky, *vis, bt, geo, make_tuning(tuning), V, workspace, workspace_bytes,
                      static_cast<cudaStream_t>(stream));
}

size_t viss_vis_dft_windowed_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J) {
  if (!cfg || K < 0 || J < 0) return 0;
  Batch bt;
  if (make_batch(nullptr, K, *cfg, bt)) return 0;
  VisPlan p;
  plan_vis(p, *cfg, bt, J, nullptr, Tuning{}, nullptr, true);
  return p.bytes;
}

int viss_vis_dft_windowed(const viss_dft_cfg* cfg, const viss_sky* sky, const int32_t* win_index,
                          const viss_vis_set* vis, float* V, void* workspace, size_t workspace_bytes, void* stream) {
  int rc;
  if ((rc = check_vis_call(cfg, sky, vis, nullptr, nullptr, V))) return rc;
  if (cfg->mask_mode != VISS_MASK_REF_QUIRK && cfg->mask_mode != VISS_MASK_REF_INTENDED)
    return fail(VISS_ERR_INVALID, "viss_vis_dft_windowed needs a REF mask mode");
  if (sky->J > 0 && !win_index) return fail(VISS_ERR_INVALID, "win_index is NULL");
  Batch bt;
  if ((rc = make_batch(nullptr, vis->K, *cfg, bt))) return rc;
  const double s = cfg->phase_scale;
  const double scale[3] = {s, s, s};
  const float d = (float)(1.0 / s);
  const float dlmn[3] = {d, d, d};
  return vis_dft_impl(*cfg, scale, dlmn, *sky, *vis, bt, nullptr, Tuning{}, V, workspace, workspace_bytes,
                      static_cast<cudaStream_t>(stream), nullptr, win_index);
}

static int check_map(const viss_fine_map* map, int64_t J) {
  if (!map) return fail(VISS_ERR_INVALID, "fine map is NULL");
  if (map->X < 0 || map->X > ((int64_t)1 << 31) - 1) return fail(VISS_ERR_RANGE, "fine map X out of range");
  if (J > 0 && !map->countLoc) return fail(VISS_ERR_INVALID, "fine map countLoc is NULL");
  if (map->X > 0 && (!map->FF || (!map->NXq_f == !map->NXq_i)))
    return fail(VISS_ERR_INVALID, "fine map needs FF and exactly one of NXq_f / NXq_i");
  return VISS_OK;
}

size_t viss_vis_dft_map_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J, const viss_fine_map* map,
                                  const viss_geometry* geo) {
  if (!cfg || !map || K < 0 || J < 0) return 0;
  Batch bt;
  if (make_batch(nullptr, K, *cfg, bt)) return 0;
  VisPlan p;
  plan_vis(p, *cfg, bt, J, geo, Tuning{}, map);
  return p.bytes;
}

int viss_vis_dft_map(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_fine_map* map, const viss_vis_set* vis,
                     const viss_geometry* geo, float* V, void* workspace, size_t workspace_bytes, void* stream) {
  int rc;
  if ((rc = check_cfg(cfg)) || (rc = check_sky(sky, false)) || (rc = check_vis(vis))) return rc;
  if ((rc = check_map(map, sky->J))) return rc;
  if (vis->K > 0 && !V) return fail(VISS_ERR_INVALID, "V is NULL");
  if ((cfg->mask_mode == VISS_MASK_REF_QUIRK || cfg->mask_mode == VISS_MASK_REF_INTENDED)) {
    if (!vis->shade) return fail(VISS_ERR_INVALID, "REF mask needs shade windows");
    if (cfg->res < 1) return fail(VISS_ERR_RANGE, "REF mask needs res >= 1");
  }
  if (cfg->mask_mode == VISS_MASK_GEOMETRIC && (rc = check_geo(geo, vis, cfg))) return rc;
  Batch bt;
  if ((rc = make_batch(nullptr, vis->K, *cfg, bt))) return rc;
  const double s = cfg->phase_scale;
  const double scale[3] = {s, s, s};
  const float d = (float)(1.0 / s);
  const float dlmn[3] = {d, d, d};
  return vis_dft_impl(*cfg, scale, dlmn, *sky, *vis, bt, geo, Tuning{}, V, workspace, workspace_bytes,
                      static_cast<cudaStream_t>(stream), map);
}

size_t viss_recon_workspace(const viss_dft_cfg* cfg, int64_t K, int64_t J, const viss_geometry* geo) {
  return viss_recon_batch_workspace(cfg, nullptr, K, J, geo, nullptr);
}

size_t viss_recon_batch_workspace(const viss_dft_cfg* cfg, const viss_batch* batch, int64_t K, int64_t J,
                                  const viss_geometry* geo, const viss_tuning* tuning) {
  if (!cfg || K < 0 || J < 0) return 0;
  Batch bt;
  if (make_batch(batch, K, *cfg, bt)) return 0;
  RecPlan p;
  plan_recon(p, *cfg, bt, J, geo, make_tuning(tuning));
  return p.bytes;
}

int viss_recon(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis, const viss_geometry* geo,
               const float* V, float* F, void* workspace, size_t workspace_bytes, void* stream) {
  return viss_recon_batch(cfg, sky, vis, nullptr, geo, nullptr, V, F, workspace, workspace_bytes, stream);
}

int viss_recon_batch(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis, const viss_batch* batch,
                     const viss_geometry* geo, const viss_tuning* tuning, const float* V, float* F,
                     void* workspace, size_t workspace_bytes, void* stream) {
  int rc;
  if ((rc = check_cfg(cfg)) || (rc = check_sky(sky, false)) || (rc = check_vis(vis))) return rc;
  if (sky->J > 0 && !F) return fail(VISS_ERR_INVALID, "F is NULL");
  if (vis->K > 0 && !V) return fail(VISS_ERR_INVALID, "V is NULL");
  if (cfg->recon_mask == VISS_RECON_MASK_REF) {
    if (!vis->shade) return fail(VISS_ERR_INVALID, "REF recon mask needs shade windows");
    if (cfg->res < 1) return fail(VISS_ERR_RANGE, "REF recon mask needs res >= 1");
  }
  if (cfg->recon_mask == VISS_RECON_MASK_GEOMETRIC && (rc = check_geo(geo, vis, cfg))) return rc;
  Batch bt;
  if ((rc = make_batch(batch, vis->K, *cfg, bt))) return rc;
  const double s = cfg->phase_scale;
  const double scale[3] = {s, s, s};
  const float d = (float)(1.0 / s);
  const float dlmn[3] = {d, d, d};
  return recon_impl(*cfg, scale, dlmn, *sky, *vis, bt, geo, make_tuning(tuning), V, F, workspace, workspace_bytes,
                    static_cast<cudaStream_t>(stream), nullptr);
}

int viss_visscal(int uvws_index, int lmnC_index, int res, const float* FF, float* viss, const float* u,
                 const float* v, const float* w, const float* l, const float* m, const float* n, const int* shadeM1,
                 const int* shadeM2, const int* shadeM3, const int* shadeM4, const float* NXq, const int* countLoc,
                 float dl, float dm, float dn, int variant, int mask_mode, int precision, void* stream) {
  if (uvws_index < 0 || lmnC_index < 0) return fail(VISS_ERR_RANGE, "negative size");
  if (!NXq != !countLoc) return fail(VISS_ERR_INVALID, "NXq and countLoc go together (both NULL: identity map)");
  if (!(dl > 0.f && dm > 0.f && dn > 0.f)) return fail(VISS_ERR_RANGE, "dl, dm, dn must be > 0");
  if (mask_mode != VISS_MASK_NONE && mask_mode != VISS_MASK_REF_QUIRK && mask_mode != VISS_MASK_REF_INTENDED)
    return fail(VISS_ERR_INVALID, "viss_visscal takes NONE or a REF mask");
  if (mask_mode != VISS_MASK_NONE && (!shadeM1 || !shadeM2 || !shadeM3 || !shadeM4))
    return fail(VISS_ERR_INVALID, "shadeM arrays NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  viss_dft_cfg cfg{};
  cfg.mask_mode = mask_mode;
  cfg.recon_mask = VISS_RECON_MASK_NONE;
  cfg.precision = precision;
  cfg.res = res;
  cfg.trunc_brightness = variant == VISS_VARIANT_PLAIN ? 1 : 0;
  cfg.occluded_value = 240.0f;  // vissGen10M_shade.cu:132
  cfg.phase_scale = 1.0 / dl;
  cfg.n_offset = 0.0;           // w(n-1) inside, e^{-2 pi i w/dn} outside (:137-143)
  cfg.moon_radius_km = 1737.4;
  cfg.norm = 1.0;
  int rc = check_cfg(&cfg);
  if (rc) return rc;
  viss_sky sky{l, m, n, FF, lmnC_index};
  viss_vis_set vis{u, v, w, nullptr, nullptr, nullptr, nullptr, uvws_index};
  const double scale[3] = {1.0 / dl, 1.0 / dm, 1.0 / dn};
  const float dlmn[3] = {dl, dm, dn};
  viss_fine_map map{FF, NXq, nullptr, countLoc, 0};
  if (countLoc) {
    // the fine pixel count is not among the reference's arguments: sum(countLoc)
    if ((rc = sum_counts(countLoc, lmnC_index, &map.X, st))) return rc;
    sky.bright = nullptr;
  }
  Batch bt;
  if ((rc = make_batch(nullptr, uvws_index, cfg, bt))) return rc;
  VisPlan p;
  plan_vis(p, cfg, bt, lmnC_index, nullptr, Tuning{}, countLoc ? &map : nullptr);
  const size_t shade_bytes = mask_mode != VISS_MASK_NONE ? ((sizeof(int4) * (size_t)uvws_index + 255) & ~size_t(255)) : 0;
  void* ws = nullptr;
  const size_t total = p.bytes + shade_bytes;
  if (total) VISS_CUDA(cudaMallocAsync(&ws, total, st));
  if (shade_bytes && uvws_index > 0) {
    int4* packed = reinterpret_cast<int4*>(static_cast<char*>(ws) + p.bytes);
    pack_shade_kernel<<<(unsigned)((uvws_index + 255) / 256), 256, 0, st>>>(shadeM1, shadeM2, shadeM3, shadeM4,
                                                                            uvws_index, packed);
    VISS_LAUNCH_CHECK("pack_shade_kernel");
    vis.shade = reinterpret_cast<const int32_t*>(packed);
  }
  rc = vis_dft_impl(cfg, scale, dlmn, sky, vis, bt, nullptr, Tuning{}, viss, ws, p.bytes, st,
                    countLoc ? &map : nullptr);
  if (ws) {
    cudaError_t e = cudaFreeAsync(ws, st);
    if (rc == VISS_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaFreeAsync");
  }
  return rc;
}

int viss_imagerecon(int uvw_index, int lmnC_index, int res, float* F, const float* viss, const float* u,
                    const float* v, const float* w, const float* l, const float* m, const float* n,
                    const float* uvwFrequencyMap, const float* thetaP0, const float* phiP0, const float* dtheta,
                    const float* dphi, float dl, float dm, float dn, int precision, void* stream) {
  if (uvw_index < 0 || lmnC_index < 0) return fail(VISS_ERR_RANGE, "negative size");
  if (!(dl > 0.f && dm > 0.f && dn > 0.f)) return fail(VISS_ERR_RANGE, "dl, dm, dn must be > 0");
  const bool masked = thetaP0 && phiP0 && dtheta && dphi;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  viss_dft_cfg cfg{};
  cfg.mask_mode = VISS_MASK_NONE;
  cfg.recon_mask = masked ? VISS_RECON_MASK_REF : VISS_RECON_MASK_NONE;
  cfg.precision = precision;
  cfg.res = res;
  cfg.occluded_value = 0.f;
  cfg.phase_scale = 1.0 / dl;
  cfg.n_offset = 0.0;  // w*n/dn (:169)
  cfg.moon_radius_km = 1737.4;
  cfg.norm = uvw_index > 0 ? 1.0 / (double)uvw_index : 1.0;  // F / amount (:174)
  int rc = check_cfg(&cfg);
  if (rc) return rc;
  if (masked && res < 1) return fail(VISS_ERR_RANGE, "res must be >= 1");
  viss_sky sky{l, m, n, nullptr, lmnC_index};
  viss_vis_set vis{u, v, w, uvwFrequencyMap, nullptr, nullptr, nullptr, uvw_index};
  const double scale[3] = {1.0 / dl, 1.0 / dm, 1.0 / dn};
  const float dlmn[3] = {dl, dm, dn};
  Batch bt;
  if ((rc = make_batch(nullptr, uvw_index, cfg, bt))) return rc;
  RecPlan p;
  plan_recon(p, cfg, bt, lmnC_index, nullptr, Tuning{});
  void* ws = nullptr;
  if (p.bytes) VISS_CUDA(cudaMallocAsync(&ws, p.bytes, st));
  const float* ratios[4] = {thetaP0, phiP0, dtheta, dphi};
  rc = recon_impl(cfg, scale, dlmn, sky, vis, bt, nullptr, Tuning{}, viss, F, ws, p.bytes, st,
                  masked ? ratios : nullptr);
  if (rc == VISS_OK && masked && !plain_precision(precision)) {
    // rows whose ratio arrays are not of the reference's form are rejected
    int flags[2] = {0, 0};
    p.layout(ws);
    cudaError_t e = cudaMemcpyAsync(flags, p.flags, sizeof(flags), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "flag readback");
    else if (flags[FLAG_ERR] & 4) rc = fail(VISS_ERR_UNSUPPORTED, "thetaP0 != dtheta or phiP0 != dphi");
  }
  if (ws) {
    cudaError_t e = cudaFreeAsync(ws, st);
    if (rc == VISS_OK && e != cudaSuccess) rc = cuda_fail(e, "cudaFreeAsync");
  }
  return rc;
}

}  // extern "C"
