// C ABI of libfsgb300.so: argument validation, launch configuration, workspace layout and
// launches of the sweep kernels.  See include/fsgb300.h for the contract of each entry point.

#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>

#include "../../include/fsgb300.h"
#include "fsg_common.cuh"
#include "fsg_internal.h"

namespace fsg {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int check_cuda(cudaError_t err, const char* what) {
  if (err == cudaSuccess) return FSG_OK;
  return set_error(FSG_ECUDA, "%s: %s", what, cudaGetErrorString(err));
}

int device_sm_count(int* out) {
  static std::mutex mu;
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return set_error(FSG_ECUDA, "cudaGetDevice failed");
  std::lock_guard<std::mutex> lock(mu);
  if (cache[dev] == 0) {
    int n = 0;
    cudaError_t e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return check_cuda(e, "cudaDeviceGetAttribute(MultiProcessorCount)");
    cache[dev] = n;
  }
  *out = cache[dev];
  return FSG_OK;
}

static int next_pow2(int v) {
  int p = 1;
  while (p < v) p <<= 1;
  return p;
}

int validate_common(const FsgProbe* probe, const FsgMedium* medium, const FsgFreqPlan* plan, int ffd) {
  if (!probe || !medium || !plan) return set_error(FSG_EINVAL, "probe, medium and plan must be non-NULL");
  if (probe->n_elements < 1) return set_error(FSG_EINVAL, "n_elements must be >= 1 (got %d)", probe->n_elements);
  if (probe->n_sub < 1) return set_error(FSG_EINVAL, "n_sub must be >= 1 (got %d)", probe->n_sub);
  if (!(probe->pitch > 0) || !(probe->element_width > 0) || !(probe->freq_center > 0) || !(probe->radius > 0))
    return set_error(FSG_EINVAL, "pitch, element_width, freq_center and radius must be > 0");
  if (probe->baffle < FSG_BAFFLE_SOFT || probe->baffle > FSG_BAFFLE_IMPEDANCE)
    return set_error(FSG_EINVAL, "unknown baffle %d", probe->baffle);
  if (probe->baffle == FSG_BAFFLE_IMPEDANCE && !(probe->baffle_impedance >= 0))
    return set_error(FSG_EINVAL, "baffle impedance must be >= 0");
  if (!(medium->speed_of_sound > 0) || !(medium->attenuation >= 0))
    return set_error(FSG_EINVAL, "speed_of_sound must be > 0 and attenuation >= 0");
  if (plan->n_freq < 1) return set_error(FSG_EINVAL, "plan has no frequencies");
  if (!plan->pulse_spectrum || !plan->probe_spectrum)
    return set_error(FSG_EINVAL, "plan pulse/probe spectrum pointers must be non-NULL");
  if (!isfinite(plan->freq_start) || !isfinite(plan->freq_step) || !isfinite(plan->seg_length))
    return set_error(FSG_EINVAL, "plan freq_start/freq_step/seg_length must be finite");
  if (probe->n_elements > kThreads)
    return set_error(FSG_EUNSUPPORTED, "n_elements %d > %d is not supported by this library", probe->n_elements, kThreads);
  if (probe->n_elements * probe->n_sub > 32 * kSrcPerThread)
    return set_error(FSG_EUNSUPPORTED, "n_elements * n_sub = %d > %d is not supported by this library",
                     probe->n_elements * probe->n_sub, 32 * kSrcPerThread);
  if (ffd) {
    // the per-frequency directivity is evaluated as a polynomial valid for |k_f seg / 2| <= 2 pi,
    // i.e. sub-elements up to two wavelengths of the highest selected frequency wide (the
    // automatic sub-element count keeps them within about one)
    const double f_max = plan->freq_start + (plan->n_freq - 1) * plan->freq_step;
    const double x_max = 2.0 * kPi * f_max / medium->speed_of_sound * plan->seg_length / 2.0;
    if (x_max > 2.0 * kPi)
      return set_error(FSG_EUNSUPPORTED,
                       "full_frequency_directivity with sub-elements wider than two wavelengths "
                       "(k_max seg / 2 = %.3f > 2 pi) is not supported by this library",
                       x_max);
  }
  return FSG_OK;
}

SweepConst make_sweep_const(const FsgProbe* p, const FsgMedium* m, const FsgFreqPlan* plan, int ffd) {
  SweepConst C;
  const double c = m->speed_of_sound;
  dfl dk = split_double(2.0 * kPi * plan->freq_step / c);
  C.dk = make_float2(dk.hi, dk.lo);
  C.dalpha = (float)(m->attenuation / 8.685889638065035 * plan->freq_step / 1e6 * 1e2);
  C.inv_nsub = (float)(1.0 / p->n_sub);
  dfl md = split_double(c / p->freq_center / 2.0);
  C.min_dist = make_float2(md.hi, md.lo);
  C.dir_coef = (float)(2.0 * kPi * p->freq_center / c * plan->seg_length / 2.0);
  C.baffle_val = (float)p->baffle_impedance;
  C.baffle = p->baffle;
  C.ffd = ffd;
  C.half_seg = (float)(plan->seg_length / 2.0);
  return C;
}

static size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

size_t tables_bytes(int E, int U, int F) {
  const int n_src = E * U;
  const int n_anchor = (F + kAnchor - 1) / kAnchor;
  size_t b = 0;
  b += align256((size_t)n_src * 16);
  b += align256((size_t)E * 8);
  b += align256((size_t)F * 8);
  b += align256((size_t)F * 4);
  b += align256((size_t)F * 8);
  b += align256((size_t)F * 4);
  b += align256((size_t)n_anchor * E * 8);
  b += align256((size_t)E * 8);
  b += align256((size_t)n_anchor * E * 8);
  b += align256((size_t)E * 4);
  return b;
}

Tables carve_tables(unsigned char* base, int E, int U, int F) {
  const int n_src = E * U;
  const int n_anchor = (F + kAnchor - 1) / kAnchor;
  Tables t;
  size_t o = 0;
  t.src_pos = reinterpret_cast<float4*>(base + o); o += align256((size_t)n_src * 16);
  t.rot_e = reinterpret_cast<float2*>(base + o); o += align256((size_t)E * 8);
  t.kf = reinterpret_cast<float2*>(base + o); o += align256((size_t)F * 8);
  t.af = reinterpret_cast<float*>(base + o); o += align256((size_t)F * 4);
  t.pp = reinterpret_cast<float2*>(base + o); o += align256((size_t)F * 8);
  t.probe = reinterpret_cast<float*>(base + o); o += align256((size_t)F * 4);
  t.da = reinterpret_cast<float2*>(base + o); o += align256((size_t)n_anchor * E * 8);
  t.dstep = reinterpret_cast<float2*>(base + o); o += align256((size_t)E * 8);
  t.dph = reinterpret_cast<float2*>(base + o); o += align256((size_t)n_anchor * E * 8);
  t.wtx = reinterpret_cast<float*>(base + o);
  return t;
}

int launch_setup(const FsgProbe* p, const FsgMedium* m, const FsgFreqPlan* plan, const double* delays,
                 const double* apod, const Tables& t, cudaStream_t stream) {
  SetupArgs a;
  a.E = p->n_elements;
  a.U = p->n_sub;
  a.F = plan->n_freq;
  a.n_anchor = (plan->n_freq + kAnchor - 1) / kAnchor;
  a.pitch = p->pitch;
  a.width = p->element_width;
  a.radius = p->radius;
  a.c = m->speed_of_sound;
  a.att = m->attenuation;
  a.f0 = plan->freq_start;
  a.df = plan->freq_step;
  a.seg = plan->seg_length;
  a.delays = delays;
  a.apod = apod;
  a.pulse = plan->pulse_spectrum;
  a.probe = plan->probe_spectrum;
  a.t = t;
  int n = a.E * a.U;
  if (a.F > n) n = a.F;
  if (a.n_anchor * a.E > n) n = a.n_anchor * a.E;
  setup_tables<<<(n + 127) / 128, 128, 0, stream>>>(a);
  return check_cuda(cudaGetLastError(), "setup_tables launch");
}

void convex_geometry(const FsgProbe* p, int* convex, double* apex, double* radius2) {
  *convex = isinf(p->radius) ? 0 : 1;
  *apex = 0.0;
  *radius2 = 0.0;
  if (*convex) {
    const int E = p->n_elements;
    double half = asin(p->pitch / 2.0 / p->radius);
    double chord = 2.0 * p->radius * sin(half * (E - 1));
    *apex = sqrt(p->radius * p->radius - (chord / 2.0) * (chord / 2.0));
    *radius2 = p->radius * p->radius;
  }
}

// Padding between the sub-element planes of the geometry arrays that minimises shared-memory
// bank conflicts of the transmit accesses: lane l of a warp touches source g + GN i of tile
// point l / GN (g = l % GN), i.e. word u * plane + e * pitch + point.  Ties go to the smaller
// pad; the receive reads (consecutive elements, stride pitch) are conflict-free for any pad.
static int choose_plane_pad(int E, int U, int gn, int st) {
  const int pitch = st + 1;
  int best_pad = 0, best_cost = 1 << 30;
  for (int pad = 0; pad < 32; ++pad) {
    const int plane = E * pitch + pad;
    int cost = 0;
    for (int i = 0; i < kSrcPerThread; ++i) {
      int count[32] = {0};
      int worst = 0;
      for (int l = 0; l < 32; ++l) {
        const int g = l % gn, pt = l / gn, src = g + gn * i;
        if (src >= E * U) continue;
        const int word = (src % U) * plane + (src / U) * pitch + pt;
        const int c = ++count[word % 32];
        if (c > worst) worst = c;
      }
      cost += worst;
    }
    if (cost < best_cost) {
      best_cost = cost;
      best_pad = pad;
    }
  }
  return best_pad;
}

// Geometry cache per chunk: sized to stay resident in L2 while every band's CTAs read it.
constexpr size_t kGeoCacheBudget = size_t(48) << 20;

// Grid of one simus chunk: every (band, tile) unit is one CTA's work at most.
static int simus_grid(int n_bands, int64_t chunk_tiles, int num_sms) {
  const int64_t units = (int64_t)n_bands * chunk_tiles;
  return (int)(units < num_sms ? units : num_sms);
}

// Simus sweep shape.  The scatterers are processed in chunks of chunk_tiles tiles, so that the
// chunk's geometry cache (chunk_tiles * geo_bytes) stays below cache_budget.  A chunk's
// n_bands x chunk_tiles (band, tile) units are split evenly over min(num_sms, units) CTAs in
// band-major order: every SM gets the same work whatever the band count divides into, and a
// CTA whose share crosses a band boundary sweeps two bands one after the other.  n_slices
// bounds the number of CTAs that share a band (the partial-spectrum slots per band) for any
// chunk size: a band's ct units hold fewer than ceil(grid / n_bands) CTA starts besides its
// first unit's CTA.
// simus_stash_kernel shape: the fewest lanes per point (GN) whose element slots cover the probe
// (16 source slots per lane; one, two or four per element for U = 1, 2, 3-4), with bands of
// kTxAnchor frequencies, else of kAnchor, such that the shared memory fits.  False when no
// shape fits (simus_band_kernel takes those probes).
static bool stash_shape(int E, int U, int ffd, SweepConfig* c) {
  if (U < 1 || U > 8) return false;
  const int spe = U == 1 ? 1 : (U == 2 ? 2 : (U <= 4 ? 4 : 8));
  const int epl = kSrcPerThread / spe;
  // the warp-specialised kernel: E = 64, 128 (U <= 4) or 256 (U <= 2); 128 transmit threads
  if ((E == 64 || E == 128 || E == 256) && U <= (E == 256 ? 2 : 4)) {
    int gn = E * spe / kSrcPerThread;
    if (gn < 4) gn = 4;
    const int st = 128 / gn, fb = E > 128 ? 32 : 64;
    const int pad = choose_plane_pad(E, U, gn, st);
    const WsLayout L = ws_layout(st, fb, E, U, pad, ffd != 0);
    if (gn <= 32 && L.total <= kMaxDynSmem - 1024) {
      c->kind = 2;
      c->gn = gn;
      c->st = st;
      c->fb = fb;
      c->plane_pad = pad;
      c->smem = L.total;
      c->geo_bytes = L.g.geo_bytes;
      return true;
    }
  }
  for (int fb = kTxAnchor; fb >= kAnchor; fb /= 2) {
    for (int gn = 4; gn <= 32; gn *= 2) {
      if (gn * epl < E) continue;
      const int st = kThreads / gn;
      const int pad = choose_plane_pad(E, U, gn, st);
      const StashLayout L = stash_layout(st, fb, E, U, pad, ffd != 0);
      if (L.total > kMaxDynSmem - 1024) continue;
      c->kind = 1;
      c->gn = gn;
      c->st = st;
      c->fb = fb;
      c->plane_pad = pad;
      c->smem = L.total;
      c->geo_bytes = L.g.geo_bytes;
      return true;
    }
  }
  return false;
}

SweepConfig simus_config(int E, int U, int F, int64_t n_scat, int num_sms, size_t cache_budget, int ffd) {
  SweepConfig c;
  if (!stash_shape(E, U, ffd, &c)) {
    const int n_src = E * U;
    c.kind = 0;
    c.gn = next_pow2((n_src + kSrcPerThread - 1) / kSrcPerThread);
    if (c.gn < 4) c.gn = 4;
    c.st = kThreads / c.gn;
    int runs = kThreads / E;
    if (runs > 4) runs = 4;
    c.fb = kAnchor * runs;
    c.plane_pad = choose_plane_pad(E, U, c.gn, c.st);
    const SmemLayout L = smem_layout(c.st, c.fb, E, U, c.plane_pad, true, ffd != 0);
    c.smem = L.total;
    c.geo_bytes = L.geo_bytes;
  }
  c.n_bands = (F + c.fb - 1) / c.fb;
  c.per_slice = 0;
  const int64_t tiles = n_scat > 0 ? (n_scat + c.st - 1) / c.st : 1;
  int64_t ct = (int64_t)(cache_budget / c.geo_bytes);
  if (ct < 1) ct = 1;
  if (ct > tiles) ct = tiles;
  c.chunk_tiles = ct;
  c.n_chunks = (tiles + ct - 1) / ct;
  c.n_slices = 1 + (num_sms + c.n_bands - 1) / c.n_bands;
  return c;
}

SweepConfig pfield_config(int E, int U, int F, int64_t n_pts, int num_sms, int ffd) {
  SweepConfig c;
  c.kind = 0;
  const int n_src = E * U;
  c.gn = next_pow2((n_src + kSrcPerThread - 1) / kSrcPerThread);
  if (c.gn < 4) c.gn = 4;
  c.st = kThreads / c.gn;
  const int64_t tiles = n_pts > 0 ? (n_pts + c.st - 1) / c.st : 1;
  // Every band recomputes its points' geometry, so use as few bands as keep the two CTAs per
  // SM busy with at least 8 tiles each (one band for large grids), and at most one band per
  // kAnchor frequencies.
  const int64_t want = (8 * 2 * (int64_t)num_sms + tiles - 1) / tiles;
  const int max_nb = (F + kAnchor - 1) / kAnchor;
  const int nb = want < 1 ? 1 : (want > max_nb ? max_nb : (int)want);
  const int per = (F + nb - 1) / nb;
  c.fb = ((per + kAnchor - 1) / kAnchor) * kAnchor;
  c.n_bands = (F + c.fb - 1) / c.fb;
  int64_t slices = (2 * (int64_t)num_sms) / c.n_bands;
  if (slices < 1) slices = 1;
  if (slices > tiles) slices = tiles;
  const int64_t tps = (tiles + slices - 1) / slices;
  c.per_slice = tps * c.st;
  c.n_slices = (int)((tiles + tps - 1) / tps);
  c.plane_pad = choose_plane_pad(E, U, c.gn, c.st);
  c.smem = smem_layout(c.st, c.fb, E, U, c.plane_pad, false, ffd != 0).total;
  return c;
}

}  // namespace fsg

using namespace fsg;

extern "C" int32_t fsg_abi_version(void) { return FSG_ABI_VERSION; }

extern "C" const char* fsg_last_error_string(void) { return g_last_error.c_str(); }

// Workspace: tables | status word | partial spectra [slots][F][E] | geometry cache.
static size_t simus_ws_size(const SweepConfig& c, int E, int U, int F) {
  return tables_bytes(E, U, F) + 256 + align256((size_t)c.n_slices * F * E * 8) +
         align256((size_t)c.chunk_tiles * c.geo_bytes);
}

// The default workspace, large enough with or without full-frequency directivity (whose
// geometry block carries one more array).
static size_t simus_ws_size(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_scat, int num_sms) {
  size_t need = 0;
  for (int ffd = 0; ffd < 2; ++ffd) {
    SweepConfig c = simus_config(probe->n_elements, probe->n_sub, plan->n_freq, n_scat, num_sms, kGeoCacheBudget, ffd);
    const size_t n = simus_ws_size(c, probe->n_elements, probe->n_sub, plan->n_freq);
    if (n > need) need = n;
  }
  return need;
}

// The smallest workspace fsg_simus runs in for this request: the fixed part (tables, status
// word, partial spectra) plus the geometry cache of one tile, i.e. chunks of one tile each.
// fsg_simus shrinks its chunks to whatever a smaller-than-default workspace holds above this.
size_t fsg::simus_min_workspace(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_scat, int ffd, int num_sms) {
  const int E = probe->n_elements, U = probe->n_sub, F = plan->n_freq;
  SweepConfig c = simus_config(E, U, F, n_scat, num_sms, 0, ffd);  // a zero budget gives one-tile chunks
  return simus_ws_size(c, E, U, F);
}

extern "C" size_t fsg_simus_workspace_size(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_scat) {
  if (!probe || !plan || probe->n_elements < 1 || probe->n_sub < 1 || plan->n_freq < 1 || n_scat < 0) return 0;
  int sms = 0;
  if (device_sm_count(&sms) != FSG_OK) return 0;
  return simus_ws_size(probe, plan, n_scat, sms);
}

extern "C" int32_t fsg_simus_launches(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_scat, int32_t ffd) {
  if (!probe || !plan || probe->n_elements < 1 || probe->n_sub < 1 || plan->n_freq < 1 || n_scat < 0) return -1;
  int sms = 0;
  if (device_sm_count(&sms) != FSG_OK) return -1;
  const SweepConfig c = simus_config(probe->n_elements, probe->n_sub, plan->n_freq, n_scat, sms, kGeoCacheBudget, ffd);
  return 2 + (n_scat > 0 ? (int32_t)(2 * c.n_chunks) : 0);  // setup_tables, per chunk geometry + band, simus_reduce
}

extern "C" int32_t fsg_simus(const FsgProbe* probe, const FsgMedium* medium, const FsgFreqPlan* plan,
                             const double* scat_xz, const double* rc, int64_t n_scat, const double* delays,
                             const double* apod, int32_t ffd, int32_t out_layout, void* out, void* workspace,
                             size_t workspace_bytes, void* stream_ptr) {
  int st = validate_common(probe, medium, plan, ffd);
  if (st != FSG_OK) return st;
  if (probe->n_sub > 8) return set_error(FSG_EUNSUPPORTED, "n_sub = %d > 8 is not supported by this library", probe->n_sub);
  if (n_scat < 0) return set_error(FSG_EINVAL, "n_scat must be >= 0");
  if (n_scat > 0 && (!scat_xz || !rc)) return set_error(FSG_EINVAL, "scatterer and rc pointers must be non-NULL");
  if (!delays) return set_error(FSG_EINVAL, "delays pointer must be non-NULL");
  if (!out) return set_error(FSG_EINVAL, "out pointer must be non-NULL");
  if (out_layout != FSG_OUT_SELECTED_RAW && out_layout != FSG_OUT_FULL_CORRECTED)
    return set_error(FSG_EINVAL, "unknown out_layout %d", out_layout);
  if (out_layout == FSG_OUT_FULL_CORRECTED &&
      (plan->freq_idx_start < 0 || plan->freq_idx_start + plan->n_freq > plan->n_freq_full))
    return set_error(FSG_EINVAL, "selected band [%d, %d) does not fit in n_freq_full = %d", plan->freq_idx_start,
                     plan->freq_idx_start + plan->n_freq, plan->n_freq_full);
  int sms = 0;
  if ((st = device_sm_count(&sms)) != FSG_OK) return st;
  const int E = probe->n_elements, U = probe->n_sub, F = plan->n_freq;
  // the default chunking, or smaller chunks when the caller's workspace is smaller
  SweepConfig c = simus_config(E, U, F, n_scat, sms, kGeoCacheBudget, ffd);
  if (c.kind == 0 && U > 4)
    return set_error(FSG_EUNSUPPORTED,
                     "n_sub = %d > 4 is supported for probes whose 8-slot elements map onto 32 lanes "
                     "(n_elements <= 64); got n_elements = %d",
                     U, E);
  if (workspace && workspace_bytes < simus_ws_size(c, E, U, F)) {
    const size_t fixed = simus_ws_size(c, E, U, F) - align256((size_t)c.chunk_tiles * c.geo_bytes);
    if (workspace_bytes > fixed) c = simus_config(E, U, F, n_scat, sms, workspace_bytes - fixed - 256, ffd);
  }
  const size_t need = simus_ws_size(c, E, U, F);
  if (!workspace || workspace_bytes < need)
    return set_error(FSG_EWORKSPACE, "workspace of %zu bytes is smaller than the %zu bytes required", workspace_bytes,
                     need);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_ptr);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  Tables t = carve_tables(ws, E, U, F);
  int* status = reinterpret_cast<int*>(ws + tables_bytes(E, U, F));
  float2* partial = reinterpret_cast<float2*>(ws + tables_bytes(E, U, F) + 256);
  unsigned char* geo = reinterpret_cast<unsigned char*>(partial) + align256((size_t)c.n_slices * F * E * 8);
  if ((st = check_cuda(cudaMemsetAsync(status, 0, sizeof(int), s), "status reset")) != FSG_OK) return st;
  if ((st = launch_setup(probe, medium, plan, delays, apod, t, s)) != FSG_OK) return st;
  if (n_scat > 0) {
    BandArgs A;
    A.pts = scat_xz;
    A.rc = rc;
    A.n_pts = n_scat;
    A.t = t;
    A.C = make_sweep_const(probe, medium, plan, ffd);
    A.E = E;
    A.U = U;
    A.n_src = E * U;
    A.gn = c.gn;
    A.plane_pad = c.plane_pad;
    A.st = c.st;
    A.fb = c.fb;
    A.F = F;
    A.n_anchor = (F + kAnchor - 1) / kAnchor;
    convex_geometry(probe, &A.convex, &A.apex, &A.radius2);
    A.partial = partial;
    A.geo = geo;
    A.geo_bytes = c.geo_bytes;
    A.status = status;
    A.n_bands = c.n_bands;
    A.n_slots = c.n_slices;
    if ((st = check_cuda(cudaMemsetAsync(partial, 0, (size_t)c.n_slices * F * E * 8, s), "partial reset")) != FSG_OK)
      return st;
    const int64_t tiles = (n_scat + c.st - 1) / c.st;
    for (int64_t k = 0; k < c.n_chunks; ++k) {
      A.chunk_s0 = k * c.chunk_tiles * c.st;
      const int64_t left = tiles - k * c.chunk_tiles;
      const int64_t ct = left < c.chunk_tiles ? left : c.chunk_tiles;
      A.chunk_tiles = ct;
      A.grid = simus_grid(c.n_bands, ct, sms);
      const int64_t cap = (int64_t)sms * 8;
      const int blocks = (int)(ct < cap ? ct : cap);
      geometry_kernel<<<blocks, kThreads, 0, s>>>(A, ct);
      if ((st = check_cuda(cudaGetLastError(), "geometry_kernel launch")) != FSG_OK) return st;
      if ((st = check_cuda(launch_simus_band_any(U, c, A, s), "simus_band_kernel launch")) != FSG_OK) return st;
    }
  }
  const int full = out_layout == FSG_OUT_FULL_CORRECTED;
  const int rows = full ? plan->n_freq_full : F;
  const int64_t n_out = (int64_t)rows * E;
  simus_reduce<<<(unsigned)((n_out + 255) / 256), 256, 0, s>>>(
      partial, n_scat > 0 ? c.n_slices : 0, F, E, t.probe, full ? (float)plan->correction_factor : 1.0f, full, rows,
      plan->freq_idx_start, status, c.kind >= 1 ? delays : nullptr, plan->freq_start, plan->freq_step,
      static_cast<float2*>(out));
  return check_cuda(cudaGetLastError(), "simus_reduce launch");
}

static size_t pfield_ws_size(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_pts, int num_sms) {
  SweepConfig c = pfield_config(probe->n_elements, probe->n_sub, plan->n_freq, n_pts, num_sms, 0);
  return tables_bytes(probe->n_elements, probe->n_sub, plan->n_freq) + align256((size_t)c.n_bands * n_pts * 4);
}

extern "C" size_t fsg_pfield_workspace_size(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_points) {
  if (!probe || !plan || probe->n_elements < 1 || probe->n_sub < 1 || plan->n_freq < 1 || n_points < 0) return 0;
  int sms = 0;
  if (device_sm_count(&sms) != FSG_OK) return 0;
  return pfield_ws_size(probe, plan, n_points, sms);
}

extern "C" int32_t fsg_pfield(const FsgProbe* probe, const FsgMedium* medium, const FsgFreqPlan* plan,
                              const double* points, int64_t n_points, const double* delays, const double* apod,
                              int32_t ffd, float* out, void* workspace, size_t workspace_bytes, void* stream_ptr) {
  int st = validate_common(probe, medium, plan, ffd);
  if (st != FSG_OK) return st;
  if (n_points < 1) return set_error(FSG_EINVAL, "Grid has no points");
  if (!points || !delays || !out) return set_error(FSG_EINVAL, "points, delays and out must be non-NULL");
  int sms = 0;
  if ((st = device_sm_count(&sms)) != FSG_OK) return st;
  const int E = probe->n_elements, U = probe->n_sub, F = plan->n_freq;
  const size_t need = pfield_ws_size(probe, plan, n_points, sms);
  if (!workspace || workspace_bytes < need)
    return set_error(FSG_EWORKSPACE, "workspace of %zu bytes is smaller than the %zu bytes required", workspace_bytes,
                     need);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_ptr);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  Tables t = carve_tables(ws, E, U, F);
  float* partial = reinterpret_cast<float*>(ws + tables_bytes(E, U, F));
  if ((st = launch_setup(probe, medium, plan, delays, apod, t, s)) != FSG_OK) return st;
  SweepConfig c = pfield_config(E, U, F, n_points, sms, ffd);
  BandArgs A;
  A.pts = points;
  A.rc = nullptr;
  A.n_pts = n_points;
  A.per_slice = c.per_slice;
  A.t = t;
  A.C = make_sweep_const(probe, medium, plan, ffd);
  A.E = E;
  A.U = U;
  A.n_src = E * U;
  A.gn = c.gn;
  A.plane_pad = c.plane_pad;
  A.st = c.st;
  A.fb = c.fb;
  A.F = F;
  A.n_anchor = (F + kAnchor - 1) / kAnchor;
  convex_geometry(probe, &A.convex, &A.apex, &A.radius2);
  A.partial = partial;
  if ((st = check_cuda(launch_pfield_band_any(c, A, s), "pfield_band_kernel launch")) != FSG_OK) return st;
  pfield_reduce<<<(unsigned)((n_points + 255) / 256), 256, 0, s>>>(partial, c.n_bands, n_points,
                                                                  (float)plan->correction_factor, out);
  return check_cuda(cudaGetLastError(), "pfield_reduce launch");
}
