// Transmit-field surrogate support: the exact transmit field at arbitrary (x, z, f, theta)
// samples, and the inputs and outputs of the surrogate network.
//
// Exact field (the training target and the check of the network's error).  For a plane wave
// of steering angle theta on a linear array, delays tau_e = x_e sin(theta) / c - min_e(...)
// (tx_delay.py:116-189); the complex transmit pressure at (x, z) and frequency f is
//     p = pulse(f) probe(f) sum_{e,u} apod_e exp(i 2 pi f tau_e) G(x, z, e, u, f)
// with G as in _init_exponentials (_pfield_math.py:202-247) and the 1/n_sub of pfield.py:159-170
// -- the quantity inside _pfield_strategies.py:48 before |.|^2, evaluated in closed form (no
// recurrence: every sample has its own f and theta).
//
// Network inputs and outputs.  The network (trained by fsg_mlp_train.cu, evaluated by
// fsg_mlp_tc.cu) predicts the complex amplitudes of a few analytic carriers whose phases carry
// the fast oscillation of the field: the ideal plane wave of the firing, the waves from the
// two ends of the aperture and the two first grating lobes of the element pitch.  fsg_surrogate_inputs normalises the samples and evaluates the
// carriers (FP64 phases) for training; fsg_surrogate_combine multiplies the predicted
// amplitudes back onto the carriers.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/fsgb300.h"
#include "fsg_common.cuh"
#include "fsg_internal.h"

namespace fsg {

struct TxFieldArgs {
  const double* samples;  // [n][4]: x, z, f (Hz), theta (rad)
  int64_t n;
  float2* out;            // [n] complex transmit pressure
  const float4* src_pos;  // [E*U]
  const float2* rot_e;    // [E]
  float pitch;            // element x = (e - (E-1)/2) * pitch in float32 (utils/geometry.py:33-37)
  int E, U;
  double c, att, fc, bandwidth, n_wavelengths;
  SweepConst C;           // geometry constants (dk/dalpha unused)
};

__device__ double sinc_pi(double x) {  // numpy.sinc: sin(pi x) / (pi x)
  if (x == 0.0) return 1.0;
  const double px = kPi * x;
  return sin(px) / px;
}

__global__ void txfield_kernel(const TxFieldArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double x = a.samples[4 * i], z = a.samples[4 * i + 1], f = a.samples[4 * i + 2], th = a.samples[4 * i + 3];
  // pulse * probe at f (spectrum.py:24-107)
  const double w = 2.0 * kPi * f, wc = 2.0 * kPi * a.fc;
  const double dur = a.n_wavelengths / a.fc;
  const double pulse_im = sinc_pi(dur * (w - wc) / 2.0 / kPi) - sinc_pi(dur * (w + wc) / 2.0 / kPi);  // times i
  const double wb = a.bandwidth * wc;
  const double shape = log(126.0) / log(2.0 * wc / wb);
  const double sigma = wb / 2.0 / pow(log(2.0), 1.0 / shape);
  const double probe = sqrt(exp(-pow(fabs(w - wc) / sigma, shape)));
  // plane-wave delays: tau_e = x_e sin(theta)/c - min_e
  const double st = sin(th);
  double xmin = 1e300;
  for (int e = 0; e < a.E; ++e)
    xmin = fmin(xmin, (double)__fmul_rn(__fsub_rn((float)e, (float)((a.E - 1) * 0.5)), a.pitch) * st);
  const dfl xs = split_double(x), zs = split_double(z);
  const dfl kf = split_double(2.0 * kPi * f / a.c);
  const float alpha = (float)(a.att / 8.685889638065035 * f / 1e6 * 1e2);
  float2 acc = make_float2(0.f, 0.f);
  for (int e = 0; e < a.E; ++e) {
    // delay phase 2 pi f tau in cycles, reduced in double (one per element and sample)
    const double xe = (double)__fmul_rn(__fsub_rn((float)e, (float)((a.E - 1) * 0.5)), a.pitch);
    const double cyc = f * ((xe * st - xmin) / a.c);
    const double fr = cyc - rint(cyc);
    float sd, cd;
    sincospif((float)(2.0 * fr), &sd, &cd);
    float2 es = make_float2(0.f, 0.f);
    for (int u = 0; u < a.U; ++u) {
      const SrcGeo geo = source_geometry(xs, zs, a.src_pos[e * a.U + u], a.rot_e[e], a.C);
      const float2 g = anchor_value(geo.r_hi, geo.r_lo, geo.amp, make_float2(kf.hi, kf.lo), alpha);
      es = cadd(es, g);
    }
    acc = cfma(es, make_float2(cd, sd), acc);
  }
  // times pulse (= i * pulse_im) * probe
  const float s = (float)(pulse_im * probe);
  const bool out_field = z < 0.0;
  a.out[i] = out_field ? make_float2(0.f, 0.f) : make_float2(-acc.y * s, acc.x * s);
}

// ------------------------------------------------------------------------------------------
// Surrogate carriers
// ------------------------------------------------------------------------------------------
constexpr int kMaxCarriers = 5;
constexpr int kAux = 12;  // floats per training row: carriers c_0..c_4, target y (complex)

struct Carriers {
  double2 c[kMaxCarriers];
};

// c_0: the plane wave exp(i k (x sin th + z cos th - xmin)); c_1, c_2: the waves from the two
// ends of the aperture, exp(i k (r_edge + x_edge sin th - xmin)); c_3, c_4: the grating lobes
// m = -1, +1 of the pitch, exp(i k (x sin th_m + z cos th_m - xmin)) with
// sin th_m = sin th + m lambda / pitch, zero where |sin th_m| >= 1 (evanescent).  Phases are
// reduced in cycles in FP64, then sincospi.
__device__ Carriers surrogate_carriers(const FsgSurrogateDomain& d, double x, double z, double f, double th) {
  const double st = sin(th), ct = cos(th);
  const double x0 = -0.5 * (d.n_elements - 1) * d.pitch, x1 = -x0;
  const double xmin = fmin(x0 * st, x1 * st);
  const double kc = f / d.speed_of_sound;  // cycles per metre
  const double lp = d.speed_of_sound / f / d.pitch;  // lambda / pitch
  double path[kMaxCarriers];
  bool on[kMaxCarriers];
  path[0] = x * st + z * ct - xmin;
  const double xl = x0 - 0.5 * d.pitch, xr = x1 + 0.5 * d.pitch;
  path[1] = sqrt((x - xl) * (x - xl) + z * z) + xl * st - xmin;
  path[2] = sqrt((x - xr) * (x - xr) + z * z) + xr * st - xmin;
  on[0] = on[1] = on[2] = true;
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    const double sm = st + (m ? lp : -lp);
    on[3 + m] = fabs(sm) < 1.0;
    path[3 + m] = x * sm + z * sqrt(fmax(0.0, 1.0 - sm * sm)) - xmin;
  }
  Carriers out;
#pragma unroll
  for (int j = 0; j < kMaxCarriers; ++j) {
    const double cyc = kc * path[j];
    const double fr = cyc - rint(cyc);
    double s, c;
    sincospi(2.0 * fr, &s, &c);
    out.c[j] = (on[j] && j < d.n_carriers) ? make_double2(c, s) : make_double2(0.0, 0.0);
  }
  return out;
}

__global__ void surrogate_inputs_kernel(const FsgSurrogateDomain d, const double* __restrict__ samples, int64_t n,
                                        const float2* __restrict__ field, double inv_scale, float4* __restrict__ u,
                                        float* __restrict__ aux) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = samples[4 * i], z = samples[4 * i + 1], f = samples[4 * i + 2], th = samples[4 * i + 3];
  u[i] = make_float4((float)((2.0 * x - (d.x_lo + d.x_hi)) / (d.x_hi - d.x_lo)),
                     (float)((2.0 * z - (d.z_lo + d.z_hi)) / (d.z_hi - d.z_lo)),
                     (float)((2.0 * f - (d.f_lo + d.f_hi)) / (d.f_hi - d.f_lo)), (float)(th / d.max_angle));
  if (!aux) return;
  const Carriers c = surrogate_carriers(d, x, z, f, th);
  float* o = aux + kAux * i;
#pragma unroll
  for (int j = 0; j < kMaxCarriers; ++j) {
    o[2 * j] = (float)c.c[j].x;
    o[2 * j + 1] = (float)c.c[j].y;
  }
  const float2 y = field ? field[i] : make_float2(0.f, 0.f);
  o[kAux - 2] = (float)(y.x * inv_scale);
  o[kAux - 1] = (float)(y.y * inv_scale);
}

__global__ void surrogate_combine_kernel(const FsgSurrogateDomain d, const double* __restrict__ samples, int64_t n,
                                         const float* __restrict__ net, double scale, float2* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Carriers c =
      surrogate_carriers(d, samples[4 * i], samples[4 * i + 1], samples[4 * i + 2], samples[4 * i + 3]);
  const float* o = net + (size_t)i * 2 * d.n_carriers;
  double re = 0.0, im = 0.0;
#pragma unroll
  for (int j = 0; j < kMaxCarriers; ++j) {
    if (j < d.n_carriers) {
      re += (double)o[2 * j] * c.c[j].x - (double)o[2 * j + 1] * c.c[j].y;
      im += (double)o[2 * j] * c.c[j].y + (double)o[2 * j + 1] * c.c[j].x;
    }
  }
  out[i] = make_float2((float)(re * scale), (float)(im * scale));
}

}  // namespace fsg

using namespace fsg;

extern "C" int32_t fsg_txfield(const FsgProbe* probe, const FsgMedium* medium, double tx_n_wavelengths,
                               double bandwidth, const double* samples, int64_t n, void* out, void* workspace,
                               size_t workspace_bytes, void* stream_ptr) {
  if (!probe || !medium || !samples || !out) return set_error(FSG_EINVAL, "NULL argument");
  if (!isinf(probe->radius)) return set_error(FSG_EUNSUPPORTED, "transmit-field samples need a linear array");
  if (probe->n_elements < 1 || probe->n_sub < 1) return set_error(FSG_EINVAL, "bad probe");
  const int E = probe->n_elements, U = probe->n_sub;
  const size_t need = (size_t)E * U * 16 + (size_t)E * 8 + 1024;
  if (!workspace || workspace_bytes < need) return set_error(FSG_EWORKSPACE, "workspace too small (%zu < %zu)",
                                                             workspace_bytes, need);
  if (n <= 0) return FSG_OK;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream_ptr);
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  SetupArgs sa;
  memset(&sa, 0, sizeof(sa));
  sa.E = E;
  sa.U = U;
  sa.pitch = probe->pitch;
  sa.width = probe->element_width;
  sa.radius = probe->radius;
  sa.c = medium->speed_of_sound;
  sa.seg = probe->element_width / U;
  sa.t.src_pos = reinterpret_cast<float4*>(ws);
  sa.t.rot_e = reinterpret_cast<float2*>(ws + (size_t)E * U * 16);
  setup_tables<<<(E * U + 127) / 128, 128, 0, s>>>(sa);
  int st = check_cuda(cudaGetLastError(), "setup_tables launch");
  if (st != FSG_OK) return st;
  TxFieldArgs a;
  a.samples = samples;
  a.n = n;
  a.out = static_cast<float2*>(out);
  a.src_pos = sa.t.src_pos;
  a.rot_e = sa.t.rot_e;
  a.pitch = (float)probe->pitch;
  a.E = E;
  a.U = U;
  a.c = medium->speed_of_sound;
  a.att = medium->attenuation;
  a.fc = probe->freq_center;
  a.bandwidth = bandwidth;
  a.n_wavelengths = tx_n_wavelengths;
  FsgFreqPlan dummy;
  memset(&dummy, 0, sizeof(dummy));
  dummy.seg_length = probe->element_width / U;
  a.C = make_sweep_const(probe, medium, &dummy, 0);
  txfield_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
  return check_cuda(cudaGetLastError(), "txfield_kernel launch");
}

static int validate_domain(const FsgSurrogateDomain* d) {
  if (!d) return set_error(FSG_EINVAL, "NULL domain");
  if (d->n_carriers < 1 || d->n_carriers > kMaxCarriers) return set_error(FSG_EINVAL, "n_carriers must be 1..5");
  if (!(d->x_hi > d->x_lo) || !(d->z_hi > d->z_lo) || !(d->f_hi > d->f_lo) || !(d->max_angle > 0) ||
      !(d->pitch > 0) || !(d->speed_of_sound > 0) || d->n_elements < 1)
    return set_error(FSG_EINVAL, "bad surrogate domain");
  return FSG_OK;
}

extern "C" int32_t fsg_surrogate_inputs(const FsgSurrogateDomain* dom, const double* samples, int64_t n,
                                        const void* field, double inv_scale, float* u, float* aux, void* stream) {
  int st = validate_domain(dom);
  if (st != FSG_OK) return st;
  if (n < 0 || (n > 0 && (!samples || !u))) return set_error(FSG_EINVAL, "bad surrogate input arguments");
  if (n == 0) return FSG_OK;
  surrogate_inputs_kernel<<<(unsigned)((n + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      *dom, samples, n, static_cast<const float2*>(field), inv_scale, reinterpret_cast<float4*>(u), aux);
  return check_cuda(cudaGetLastError(), "surrogate_inputs_kernel launch");
}

extern "C" int32_t fsg_surrogate_combine(const FsgSurrogateDomain* dom, const double* samples, int64_t n,
                                         const float* net, double scale, void* out, void* stream) {
  int st = validate_domain(dom);
  if (st != FSG_OK) return st;
  if (n < 0 || (n > 0 && (!samples || !net || !out))) return set_error(FSG_EINVAL, "bad surrogate combine arguments");
  if (n == 0) return FSG_OK;
  surrogate_combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      *dom, samples, n, net, scale, static_cast<float2*>(out));
  return check_cuda(cudaGetLastError(), "surrogate_combine_kernel launch");
}
