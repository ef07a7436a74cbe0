/*
 * fsgb300.h -- C ABI of libfsgb300.so, the GB300 (sm_103a) implementation of the
 * FastSIMUS simus/pfield frequency sweep.
 *
 * Conventions
 *   - Every array argument is a DEVICE pointer unless stated otherwise; sizes are element
 *     counts.  Complex values are interleaved (re, im).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).  Calls are
 *     asynchronous on that stream; the caller synchronises.
 *   - The library allocates no device memory: the caller passes a workspace of at least the
 *     size reported by the matching *_workspace_size() function.
 *   - Every entry point returns an FsgStatus; fsg_last_error_string() gives a one-line
 *     message for the calling thread's last failure.
 *   - NaN transmit delays are treated as (delay 0, apodization 0), as the reference's
 *     simus_compute/pfield_compute do before their sweep (simus.py:427-429, pfield.py:338-340).
 */
#ifndef FSGB300_H
#define FSGB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSG_ABI_VERSION 4

typedef enum FsgStatus {
  FSG_OK = 0,
  FSG_EINVAL = 1,        /* bad argument (NULL pointer, size out of range, ...) */
  FSG_ECUDA = 2,         /* a CUDA runtime call failed */
  FSG_ETIMEOUT = 3,      /* a bounded device-side wait gave up */
  FSG_EUNSUPPORTED = 4,  /* valid request this library does not implement */
  FSG_EWORKSPACE = 5     /* workspace smaller than *_workspace_size() */
} FsgStatus;

typedef enum FsgBaffle {
  FSG_BAFFLE_SOFT = 0,      /* obliquity cos(theta) */
  FSG_BAFFLE_RIGID = 1,     /* obliquity 1 */
  FSG_BAFFLE_IMPEDANCE = 2  /* obliquity cos(theta) / (cos(theta) + baffle_impedance) */
} FsgBaffle;

typedef enum FsgOutLayout {
  /* (F, E) complex64: selected-band spectrum before the correction factor, the return
   * contract of the reference's simus_cuda (kernels/cuda_simus.py:232-321). */
  FSG_OUT_SELECTED_RAW = 0,
  /* (n_freq_full, E) complex64: selected band times correction_factor placed at rows
   * [freq_idx_start, freq_idx_start + F), zeros elsewhere -- the array the reference's
   * _irfft_and_threshold builds before its irfft (simus.py:336-352). */
  FSG_OUT_FULL_CORRECTED = 1
} FsgOutLayout;

/* Transducer array: the fields of TransducerParams (transducer_params.py:23-160) that the
 * sweep reads.  radius = +INFINITY for a linear array. */
typedef struct FsgProbe {
  int32_t n_elements;
  int32_t n_sub;            /* sub-elements per element (plan.n_sub) */
  double pitch;
  double element_width;
  double radius;
  double freq_center;
  int32_t baffle;           /* FsgBaffle */
  int32_t reserved0;
  double baffle_impedance;  /* used when baffle == FSG_BAFFLE_IMPEDANCE */
} FsgProbe;

/* MediumParams (medium_params.py:6-22). attenuation in dB/cm/MHz. */
typedef struct FsgMedium {
  double speed_of_sound;
  double attenuation;
} FsgMedium;

/* Frequency plan (SimusPlan / PfieldPlan, simus.py:135-162, pfield.py:58-82).
 * The sweep advances from freq_start by freq_step = selected_freqs[1] - selected_freqs[0],
 * as the reference's recurrence does (simus.py:302-308). */
typedef struct FsgFreqPlan {
  int32_t n_freq;                 /* F, number of selected frequencies */
  int32_t n_freq_full;            /* simus only: rows of the full spectrum */
  int32_t freq_idx_start;         /* simus only: row of the first selected frequency */
  int32_t reserved0;
  double freq_start;              /* selected_freqs[0], Hz */
  double freq_step;               /* selected_freqs[1] - selected_freqs[0], Hz (0 if F == 1) */
  double seg_length;              /* element_width / n_sub */
  double correction_factor;       /* df * element_width */
  const double* pulse_spectrum;   /* device, F complex128 (interleaved) */
  const double* probe_spectrum;   /* device, F float64 */
} FsgFreqPlan;

/* ABI version compiled into the library (FSG_ABI_VERSION). */
int32_t fsg_abi_version(void);

/* Message describing the calling thread's most recent failure ("" if none). */
const char* fsg_last_error_string(void);

/* Workspace bytes needed by fsg_simus for this probe / plan / scatterer count. */
size_t fsg_simus_workspace_size(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_scat);

/* Kernel launches one fsg_simus call makes with the default workspace (set-up, a geometry and a
 * band kernel per scatterer chunk, the reduction), or -1 for invalid arguments.  No counterpart
 * in the reference: a measurement aid. */
int32_t fsg_simus_launches(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_scat, int32_t ffd);

/*
 * Plain fused FP32 simus sweep for one transmit.
 * Replaces simus_cuda(scatterers, rc, params, plan, medium, delays_clean, tx_apodization)
 * (kernels/cuda_simus.py:232-321, launched from simus.py:455-469) and the PYTHON-strategy
 * sweep it stands in for (_simus_strategies.py:23-149).
 *
 *   scat_xz [n_scat*2] float64   scatterer (x, z) in metres, interleaved
 *   rc      [n_scat]   float64   reflection coefficients
 *   delays  [E]        float64   transmit delays in seconds (NaN = element off)
 *   apod    [E]        float64   transmit apodization (NULL = all ones)
 *   out     complex64, layout per out_layout (FsgOutLayout)
 * full_frequency_directivity != 0 evaluates the element directivity at every frequency
 * (_simus_strategies.py:59-62) instead of at the centre frequency only.
 * Limits of this library: n_elements * n_sub <= 512; n_sub <= 4, or 5-8 on probes of up to
 * 64 elements (FSG_EUNSUPPORTED otherwise).
 */
int32_t fsg_simus(const FsgProbe* probe, const FsgMedium* medium, const FsgFreqPlan* plan,
                  const double* scat_xz, const double* rc, int64_t n_scat,
                  const double* delays, const double* apod,
                  int32_t full_frequency_directivity, int32_t out_layout, void* out,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Workspace bytes needed by fsg_pfield for this probe / plan / point count. */
size_t fsg_pfield_workspace_size(const FsgProbe* probe, const FsgFreqPlan* plan, int64_t n_points);

/*
 * RMS pressure field sqrt(correction * sum_f |pulse*probe * sum_src G|^2) at n_points points.
 * Replaces pfield_metal (kernels/metal_pfield.py:89-115) plus the final sqrt of
 * pfield_compute (pfield.py:374-378); the sweep it computes is _pfield_strategies.py:21-88.
 *   points  [n_points*2] float64 (x, z) interleaved
 *   out     [n_points]   float32 RMS pressure
 */
int32_t fsg_pfield(const FsgProbe* probe, const FsgMedium* medium, const FsgFreqPlan* plan,
                   const double* points, int64_t n_points, const double* delays, const double* apod,
                   int32_t full_frequency_directivity, float* out,
                   void* workspace, size_t workspace_bytes, void* stream);

/* One phantom of a batched multi-transmit sweep: its scatterers, the plan shared by all of its
 * transmits, and its output, complex64 [n_tx][plan.n_freq_full][n_elements] (selected band times
 * correction_factor, zero-padded: one FSG_OUT_FULL_CORRECTED spectrum per transmit). */
typedef struct FsgPhantom {
  const double* scat_xz;   /* device [n_scat*2] */
  const double* rc;        /* device [n_scat] */
  int64_t n_scat;
  FsgFreqPlan plan;
  void* out;               /* device */
} FsgPhantom;

/* Tile shapes of the batched sweep (chosen by an autotuner; zeros select defaults).  The FP32
 * kernel is compiled for these (freqs_per_item, elements tile, tile_scatterers, packed,
 * CTAs per SM, threads per CTA) shapes, with 256 threads: (2, 64, 64 or 32, 0, 1),
 * (1, 64, 32, 64 or 128, 0, 1), (1, 64, 64 or 32, 1, 1), (1, 64, 32, 0, 2),
 * (1, 128, 64 or 32, 0, 1); with 512 threads: (2, 64, 64, 0, 1), (1, 64, 64 or 128, 0, 1),
 * (1, 128, 64, 0, 1); another combination returns FSG_EUNSUPPORTED.  The tensor-core path
 * reads freqs_per_item and chunk_scatterers only. */
typedef struct FsgBatchTuning {
  int32_t freqs_per_item;    /* 1 or 2 frequencies per work item (Green's tile reuse) */
  int32_t chunk_scatterers;  /* scatterers per work item (rounded up to a multiple of the tile) */
  int32_t ctas_per_sm;       /* persistent CTAs per SM (2: the shape's registers are capped for two) */
  int32_t tile_scatterers;   /* scatterers per tile: 32, 64 or 128 (0 = 64) */
  int32_t packed;            /* 1: complex MACs on the FP32x2 pipe (one frequency, 64-element tile) */
  int32_t threads_per_cta;   /* 256 or 512 (0 = 256): 512 halves each thread's register tile */
  int32_t reserved[2];
} FsgBatchTuning;

/* Workspace bytes needed by fsg_simus_batched (full-frequency directivity adds one float per
 * (scatterer, sub-element) to the geometry cache). */
size_t fsg_simus_batched_workspace_size(const FsgProbe* probe, const FsgPhantom* phantoms, int32_t n_phantoms,
                                        int32_t n_tx, int32_t full_frequency_directivity,
                                        const FsgBatchTuning* tuning);

/*
 * Many transmits x many phantoms in one persistent launch.  Replaces the reference's caller
 * loop of simus_compute over firings with one shared plan per phantom
 * (tests/_picmus_phantom_shared.py:319-367, step body _simus_strategies.py:23-77): the
 * Green's terms of each (scatterer, element, frequency) are generated once and contracted with
 * every transmit.  delays/apod are device [n_tx][n_elements] float64 (apod NULL = ones; NaN
 * delay = element off).  Every probe option of fsg_simus applies (baffle, convex radius,
 * full_frequency_directivity = simus_compute's argument of that name).  Limits of this
 * library: n_elements <= 128 (probes of 65-128 elements use a 128-element tile with one
 * frequency per work item), n_sub <= 8, n_tx <= 80, n_phantoms <= 64.
 * Phantom descriptors travel as a kernel parameter, so the call contains no host-to-device
 * copy and can be captured in a CUDA graph.
 */
int32_t fsg_simus_batched(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* phantoms,
                          int32_t n_phantoms, const double* delays, const double* apod, int32_t n_tx,
                          int32_t full_frequency_directivity, const FsgBatchTuning* tuning, void* workspace,
                          size_t workspace_bytes, void* stream);

/* Workspace bytes needed by fsg_simus_batched_tc. */
size_t fsg_simus_batched_tc_workspace_size(const FsgProbe* probe, const FsgPhantom* phantoms, int32_t n_phantoms,
                                           int32_t n_tx, const FsgBatchTuning* tuning);

/*
 * fsg_simus_batched on the tcgen05 tensor cores.  Same contract and outputs; the transmit
 * contraction over elements and the receive contraction over scatterers run as complex GEMMs
 * on BF16 hi + lo splits of Green's tiles generated on chip in FP32 (three products, FP32
 * accumulation in TMEM).  Accuracy target relative L2 <= 1e-3 against the FP64 reference
 * (measured ~1e-5).  Limits: n_elements <= 64, n_sub <= 2, n_tx <= 96.
 * tuning->freqs_per_item (1..7, default 6) sets how many frequencies share one Green's
 * geometry pass.  Every device-side wait is bounded; a wait that gives up records
 * FSG_ETIMEOUT, readable with fsg_simus_batched_tc_status.
 */
int32_t fsg_simus_batched_tc(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* phantoms,
                             int32_t n_phantoms, const double* delays, const double* apod, int32_t n_tx,
                             const FsgBatchTuning* tuning, void* workspace, size_t workspace_bytes, void* stream);

/* Synchronises `stream` and reads the device-side status word of the last fsg_simus_batched_tc
 * call that used `workspace` (FSG_OK or FSG_ETIMEOUT) into *status_out. */
int32_t fsg_simus_batched_tc_status(const void* workspace, const FsgProbe* probe, const FsgPhantom* phantoms,
                                    int32_t n_phantoms, int32_t n_tx, const FsgBatchTuning* tuning,
                                    int32_t* status_out, void* stream);

/* Verification utility, no counterpart in the reference: one 128 x 64 x 64 tile of the
 * tensor-core GEMM used by fsg_simus_batched_tc.  d[128][64] = a[128][64] * b[64][64]^T with
 * a, b FP32 row-major on the device, split into BF16 hi/lo, placed K-major (0) or MN-major (1)
 * in shared memory.  A bounded wait that gives up writes FSG_ETIMEOUT to *status (device int). */
int32_t fsg_tc_selftest(const float* a, const float* b, float* d, int32_t a_mn_major, int32_t b_mn_major,
                        int32_t* status, void* stream);

/*
 * fsg_simus_batched for one phantom whose transmit field is supplied by the caller instead of
 * computed: tx_field is device complex64 [n_scat][plan.n_freq][n_tx], the pressure
 * pulse*probe*sum_src(...) of each firing at each scatterer and selected frequency (e.g. from a
 * surrogate network).  Only the receive contraction over scatterers runs.  No counterpart in
 * the reference: it is how a learned transmit field drops into the simus sweep
 * (_simus_strategies.py:64-73 with p_k given).
 */
int32_t fsg_simus_batched_rx(const FsgProbe* probe, const FsgMedium* medium, const FsgPhantom* phantom,
                             const double* delays, int32_t n_tx, const void* tx_field, const FsgBatchTuning* tuning,
                             void* workspace, size_t workspace_bytes, void* stream);

/*
 * Exact complex transmit pressure of a plane wave at arbitrary samples (x, z, f, theta)
 * (device float64 [n][4]; metres, Hz, radians; linear arrays, unit apodization), for
 * training and judging a surrogate.  Closed form of the pressure inside
 * _pfield_strategies.py:48 (before |.|^2) with the plane-wave delays of tx_delay.py:116-189.
 * out: device complex64 [n].  workspace >= n_elements*n_sub*16 + n_elements*8 + 1024 bytes.
 */
int32_t fsg_txfield(const FsgProbe* probe, const FsgMedium* medium, double tx_n_wavelengths, double bandwidth,
                    const double* samples, int64_t n, void* out, void* workspace, size_t workspace_bytes,
                    void* stream);

/* Analytic carriers of the transmit-field surrogate (no counterpart in the reference).  For a
 * plane wave of angle theta on a linear array of n_elements at pitch, with k = 2 pi f / c:
 *   c_0 = exp(i k (x sin theta + z cos theta - xmin))          (the plane wave)
 *   c_1 = exp(i k (r_L + x_L sin theta - xmin)),  x_L = x_0 - pitch / 2
 *   c_2 = exp(i k (r_R + x_R sin theta - xmin)),  x_R = x_{E-1} + pitch / 2
 * (the waves of the two aperture edges; r = distance from (x, z) to the edge,
 * xmin = min(x_0 sin theta, x_{E-1} sin theta), x_e = (e - (E-1)/2) pitch), and
 *   c_3, c_4 = exp(i k (x sin theta_m + z cos theta_m - xmin)),  sin theta_m = sin theta + m c / (f pitch)
 * for m = -1, +1 (the grating lobes of the pitch; zero where |sin theta_m| >= 1), phases in FP64.
 * The box normalises u = (2 v - (lo + hi)) / (hi - lo) per input, theta by max_angle. */
typedef struct FsgSurrogateDomain {
  double x_lo, x_hi, z_lo, z_hi, f_lo, f_hi, max_angle;
  double pitch, speed_of_sound;
  int32_t n_elements;
  int32_t n_carriers;             /* 1..5, in the order above */
} FsgSurrogateDomain;

/* samples: device [n][4] float64 (x, z, f, theta).  Writes u: [n][4] float32 (normalised) and,
 * if aux != NULL, aux: [n][12] float32 = c_0 .. c_4 (complex; zero beyond n_carriers),
 * field * inv_scale (complex),
 * with field: device complex64 [n] (the exact transmit field, or NULL for zeros). */
int32_t fsg_surrogate_inputs(const FsgSurrogateDomain* dom, const double* samples, int64_t n, const void* field,
                             double inv_scale, float* u, float* aux, void* stream);
/* out[i] = scale * sum_j (net[i][2j] + i net[i][2j+1]) c_j(samples[i]), complex64 [n];
 * net: [n][2 n_carriers] float32 (the network's outputs). */
int32_t fsg_surrogate_combine(const FsgSurrogateDomain* dom, const double* samples, int64_t n, const float* net,
                              double scale, void* out, void* stream);

/*
 * Tensor-core training of the surrogate network (no counterpart in the reference): features
 * [sin(2 pi B u), cos(2 pi B u)] (B: 64 x 4), hidden layers 128 -> 256 -> 256 -> 256 -> 256
 * with SiLU, head 256 -> n_out (2 per carrier); loss mean_batch |sum_j (o_2j + i o_2j+1) c_j -
 * y|^2 on rows drawn from the training set by a hash of (seed, step, row).  One step is three
 * kernel launches (forward + backward on tcgen05, weight gradients on tcgen05, reduction +
 * Adam); the step counter, the learning-rate schedule (linear warm-up, cosine decay to lr_min)
 * and the loss history live on the device, so a sequence of steps needs no host
 * synchronisation and can be captured in a CUDA graph.  All pointers are device memory owned
 * by the caller.  packed_fwd[l]: fsg_mlp_tc_packed_bytes(K) bytes (the layout of
 * fsg_mlp_tc_pack); packed_bwd[1..3]: 128 KB each; packed_head: 24 KB.  fsg_mlp_train_init
 * writes the packed copies from the FP32 weights and clears the workspace counters.
 */
typedef struct FsgMlpTrain {
  const float* u;                 /* [n_data][4] */
  const float* aux;               /* [n_data][12] (fsg_surrogate_inputs) */
  int64_t n_data;
  uint64_t seed;
  const float* bmat;              /* [64][4] */
  float* w[4];                    /* [256][128] (layer 0), [256][256] */
  float* m_w[4];
  float* v_w[4];
  void* packed_fwd[4];
  void* packed_bwd[4];            /* [0] unused */
  float* b[4];                    /* [256] */
  float* m_b[4];
  float* v_b[4];
  float* w_head;                  /* [n_out][256] */
  float* m_w_head;
  float* v_w_head;
  float* b_head;                  /* [n_out] */
  float* m_b_head;
  float* v_b_head;
  void* packed_head;              /* 24 KB: W_head as BF16 hi + lo (forward) and hi (backward) */
  int32_t n_out;                  /* 2 n_carriers, <= 10 */
  int32_t n_tiles;                /* batch = 128 n_tiles rows */
  int32_t n_split;                /* weight-gradient CTAs per (layer, output half) job; 10 jobs
                                     (15 fills 150 of 152 SMs) */
  int32_t total_steps;
  int32_t warmup_steps;
  float lr, lr_min, beta1, beta2, eps;
  int32_t* step;                  /* device step counter */
  float* loss_hist;               /* device [loss_hist_len]: mean loss of step t at [t] */
  int32_t loss_hist_len;
  int32_t* status;                /* device int: FSG_ETIMEOUT if a bounded wait gave up */
  void* workspace;
  size_t workspace_bytes;
} FsgMlpTrain;

size_t fsg_mlp_train_workspace_size(int32_t n_tiles, int32_t n_split);
int64_t fsg_mlp_train_n_params(int32_t n_out);
int32_t fsg_mlp_train_init(const FsgMlpTrain* t, void* stream);
int32_t fsg_mlp_train_steps(const FsgMlpTrain* t, int32_t n_steps, void* stream);
/* One step's gradients without the update: grads_out [fsg_mlp_train_n_params] in the order
 * W_0, W_1, W_2, W_3 (row-major), b_0..b_3, W_head, b_head; rows_out [128 n_tiles]: the
 * sampled rows of the training set. */
int32_t fsg_mlp_train_gradients(const FsgMlpTrain* t, float* grads_out, int32_t* rows_out, void* stream);

/*
 * fsg_simus without a workspace argument, for callers that cannot allocate device memory
 * (for example a plugin whose host application owns all device memory and passes only input
 * and output buffers).  No counterpart in the reference: it is fsg_simus running on a 16 MiB
 * scratch array held in the library's own device image (see fsg_simus_noalloc_scratch_bytes).
 * The scatterers are processed in chunks sized to the scratch, so any scatterer count runs;
 * a request fails with FSG_EINVAL only when its fixed part (tables, partial spectra of
 * n_freq x n_elements, one tile of geometry) exceeds the scratch.  The first call on a device
 * looks up the array's device address in the device's primary context and caches it for the
 * life of the process; make it before any stream capture.  All calls share the scratch:
 * calls that overlap on the GPU race, so serialise them.
 */
int32_t fsg_simus_noalloc(const FsgProbe* probe, const FsgMedium* medium, const FsgFreqPlan* plan,
                          const double* scat_xz, const double* rc, int64_t n_scat,
                          const double* delays, const double* apod,
                          int32_t full_frequency_directivity, int32_t out_layout, void* out, void* stream);

/* Size in bytes of fsg_simus_noalloc's static scratch (no counterpart in the reference). */
size_t fsg_simus_noalloc_scratch_bytes(void);

/*
 * Tensor-core inference of the transmit-field surrogate network (no counterpart in the
 * reference).  Network: features [sin(2 pi B u), cos(2 pi B u)] (B: 64 x 4, row-major) of the
 * normalised inputs u (n x 4), hidden layers 128 -> 256 -> 256 -> 256 -> 256 with SiLU, head
 * 256 -> n_out (<= 10).  packed[l]: hidden layer l's [256][K] BF16 weights rearranged by
 * fsg_mlp_tc_pack (fsg_mlp_tc_packed_bytes(K) bytes); bias[l]: 256 floats; w_head:
 * [n_out][256] floats; b_head: n_out.  out: n x n_out floats.  status: device int set to
 * FSG_ETIMEOUT if a bounded wait gave up (the caller zeroes it).
 */
typedef struct FsgMlpWeights {
  const void* packed[4];
  const float* bias[4];
  const float* w_head;
  const float* b_head;
  const float* bmat;
  int32_t n_out;
  int32_t reserved0;
} FsgMlpWeights;

size_t fsg_mlp_tc_packed_bytes(int32_t n_in);
int32_t fsg_mlp_tc_pack(const void* w_bf16, int32_t n_out, int32_t n_in, void* packed, void* stream);
int32_t fsg_mlp_tc_forward(const FsgMlpWeights* weights, const float* u, int64_t n, float* out, int32_t* status,
                           void* stream);

/*
 * Spectrum -> RF epilogue.  Replaces _irfft_and_threshold (simus.py:336-367):
 *   rf = irfft(conj(spectrum), n_fft, axis 0)[: (n_fft + 1) / 2]
 *   rf *= 0.5 (1 + tanh((|rf| / max|rf| - 1e-5) / 1e-6))        (when gate != 0)
 * for n_batch frames, each gated with its own peak.  spectrum: n_batch frames of
 * (n_freq_full, n_elements) complex64, frame b at spectrum + b * batch_stride complex
 * elements; only rows [k_first, k_first + k_count) are read (the rest must be zero, as in the
 * zero-padded simus spectrum).  rf_out: (n_batch, (n_fft + 1) / 2, n_elements) float32.
 * workspace: fsg_rf_workspace_size(n_fft, n_batch) bytes.
 */
size_t fsg_rf_workspace_size(int32_t n_fft, int32_t n_batch);
int32_t fsg_irfft_gate(const void* spectrum, int32_t n_batch, int64_t batch_stride, int32_t n_freq_full,
                       int32_t n_elements, int32_t n_fft, int32_t k_first, int32_t k_count, int32_t gate,
                       float* rf_out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Downstream beamforming of the simulated RF.  The reference's validation tests image the RF
 * with PyMUST (tests/_picmus_phantom_shared.py:407-460): pymust.rf2iq(rf, fs, fc), then
 * pymust.dasmtx(1j * iq.shape, x, z, param) times the IQ flattened in Fortran order, summed over
 * firings.  These entry points restate MUST's rf2iq / dasmtx algorithms on the GPU.
 *
 * fsg_rf2iq: I/Q demodulation.  Per column (frame, channel): x[n] = rf[n] exp(-2 pi i fc (n / fs
 * + tau)); then a low-pass IIR filter run forward and backward (zero phase) over x extended at
 * both ends by `pad` odd-reflected samples, each pass started from the filter's steady state for
 * its first input; the result times 2.  (MUST: 5th-order Butterworth, Wn = min(2 fc / fs, 0.5),
 * pad = 3 (order + 1), as scipy.signal.filtfilt.)  The filter is given as n_sections cascaded
 * second-order sections sos[s] = (b0, b1, b2, 1, a1, a2) with steady-state states zi[s] = (z0, z1)
 * for a unit input (scipy.signal.butter(..., output="sos"), scipy.signal.sosfilt_zi): the same
 * transfer function as the (b, a) form, but well conditioned in FP32.  sos and zi are HOST arrays.
 * rf: float32 [n_frames][n_samples][n_channels]; iq_out: complex64 [n_frames][n_channels][n_samples]
 * (channel-major: the Fortran-order columns of each frame's (n_samples, n_channels) IQ).
 * Requires 1 <= n_sections <= FSG_RF2IQ_MAX_SECTIONS and 0 <= pad < n_samples, pad <= FSG_RF2IQ_MAX_PAD.
 */
#define FSG_RF2IQ_MAX_SECTIONS 4
#define FSG_RF2IQ_MAX_PAD 27
int32_t fsg_rf2iq(const float* rf, int32_t n_frames, int32_t n_samples, int32_t n_channels, double fs, double fc,
                  double tau, int32_t n_sections, const double* sos, const double* zi, int32_t pad, void* iq_out,
                  void* stream);

typedef enum FsgDasMethod { FSG_DAS_LINEAR = 0, FSG_DAS_NEAREST = 1 } FsgDasMethod;

/* Delay-and-sum parameters (the fields of MUST's param that dasmtx reads besides the array). */
typedef struct FsgDasParams {
  double speed_of_sound;  /* c, m/s */
  double fs;              /* sampling frequency of the signals, Hz */
  double fc;              /* I/Q rotation frequency, Hz (0 for RF signals) */
  double t0;              /* time of sample 0, s */
  double fnumber;         /* receive f-number; <= 0: every element */
  int32_t method;         /* FsgDasMethod */
  int32_t iq;             /* 1: signals are I/Q (rotate by exp(2 pi i fc t)) */
} FsgDasParams;

/*
 * fsg_das: matrix-free compounded delay-and-sum.  For pixel p and firing f,
 *   d_tx = min over firing elements e of (c tx_delays[f][e] + |p - x_e|)   (NaN delay: not firing)
 *   t_e  = (d_tx + |p - x_e|) / c,  s = (t_e - t0) fs  (fractional 0-based sample)
 *   image[p] += sum over aperture elements e of interp(iq[f][e], s) * exp(2 pi i fc t_e)
 * with linear interpolation between floor(s) and floor(s) + 1 (both inside the record) or the
 * nearest sample; the receive aperture is |lateral| <= axial / (2 fnumber) in the element's frame.
 * Element centres follow the probe (linear: (e - (E - 1) / 2) pitch; convex: radius).
 * iq: complex64 [n_frames][n_elements][n_samples]; tx_delays: float64 [n_frames][n_elements];
 * pixels: float64 [n_pixels][2] (x, z); image_out: complex64 [n_pixels] (overwritten).
 */
int32_t fsg_das(const FsgProbe* probe, const FsgDasParams* params, const void* iq, int32_t n_frames,
                int32_t n_samples, const double* tx_delays, const double* pixels, int64_t n_pixels, void* image_out,
                void* stream);

/* Non-zeros per row of the fsg_dasmtx matrix: 2 n_elements (linear) or n_elements (nearest). */
int32_t fsg_dasmtx_nnz_per_row(int32_t method, int32_t n_elements);

/*
 * fsg_dasmtx: the same delay-and-sum for one firing as a CSR matrix of n_pixels rows and
 * n_samples * n_elements columns (column e * n_samples + i = sample i of element e), the
 * matrix pymust.dasmtx returns.  Every row holds fsg_dasmtx_nnz_per_row entries in increasing
 * column order; entries of elements outside the aperture or the record are explicit zeros.
 * crow: int32 [n_pixels + 1]; col: int32 [n_pixels * nnz_per_row]; val: complex64 (same count).
 */
int32_t fsg_dasmtx(const FsgProbe* probe, const FsgDasParams* params, int32_t n_samples, const double* tx_delays,
                   const double* pixels, int64_t n_pixels, int32_t* crow, int32_t* col, void* val, void* stream);

/* Check of the bounded device-side wait (no counterpart in the reference).  One thread waits,
 * for at most max_tries polls or 2 s, on an mbarrier phase: one it completed itself when arrive
 * != 0, else one that nothing completes.  Writes FSG_OK or FSG_ETIMEOUT to *status (device
 * int); the context stays usable either way. */
int32_t fsg_wait_selftest(int32_t arrive, int32_t max_tries, int32_t* status, void* stream);

/* Measurement utility, no counterpart in the reference: launches `blocks` x 256 threads of
 * independent FP32 FMA chains (`iters` iterations) and reports the FLOPs it performs, so a
 * caller can time it with events and state the device's FP32 FMA roofline.  `out` must hold
 * `blocks` floats (written only in a case that does not occur). */
int32_t fsg_fp32_fma_probe(float* out, int32_t blocks, int32_t iters, double* flops, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FSGB300_H */
