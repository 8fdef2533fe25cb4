/* C ABI of the GB300 excursion-set engine (libes_engine.so).
 *
 * Replaces the GPU half of the reference's Programs/find_HII_bubbles.py and Programs/delta_T.py:
 * plain pointers and sizes, no framework types.  Device pointers are CUDA global-memory
 * addresses on the device that was current when the plan was created; every call is
 * asynchronous on the given stream (a cudaStream_t passed as void*, NULL = legacy default
 * stream).  Return values: 0 on success, a negative ES_E_* code on failure; es_last_error()
 * returns the message of the calling thread's last failure.
 *
 * Layouts: real boxes are C-order float32 [z][y][x] (the reference's INDEX(k,j,i),
 * find_bubbles.cu:6).  A plan owns its workspace (allocated once in es_plan_create); the
 * caller owns every input and output buffer.  A plan serves one stream at a time.
 */
#ifndef ES_ENGINE_H
#define ES_ENGINE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ES_OK 0
#define ES_E_ARG (-1)        /* invalid argument (size, pointer, parameter) */
#define ES_E_CUDA (-2)       /* a CUDA runtime call failed */
#define ES_E_NOMEM (-3)      /* workspace allocation failed */
#define ES_E_UNSUPPORTED (-4) /* box size without compiled kernels */
#define ES_E_DEVICE (-5)     /* a kernel reported a timed-out wait through the plan's error word */

typedef struct es_plan es_plan;

/* One radius of the descending excursion-set schedule (find_HII_bubbles.py:121-128):
 * R [Mpc] and denom = sqrt(2 (sigma_min^2 - sigma^2(R))), both as the reference's float32. */
typedef struct es_radius {
  float R;
  float denom;
} es_radius;

/* Scalars of one ionisation run; the reference pastes DELTAC/ZETA into its kernel source
 * (find_HII_bubbles.py:63-70) and passes R/denom per launch (l.147-175). */
typedef struct es_ionize_params {
  int n_radii;              /* radii in radii[]; the last one is the final radius */
  const es_radius* radii;   /* host array, descending R */
  float delta_c;            /* 1.686 / D(z) */
  float fc_mean_ps;         /* mean collapse fraction erfc(delta_c / (sqrt2 sigma_min)) */
  float zeta;               /* ionising efficiency ZETA */
  float growth_scale;       /* density multiplier before filtering (1/D(z) when LE is false) */
  int normalize_mean;       /* 1: fcoll *= fc_mean_ps / <fcoll> (reference LE == False) */
  int filter_type;          /* 0 real-space top-hat, 1 k-space top-hat, 2 Gaussian */
  int update;               /* 0 centre pixel, 1 sphere painting */
  int ref_compat;           /* 1: reference quirks: filter switch fall-through, sphere radius in
                               Mpc used as cells, spheres clamped at the box edge */
  int output;               /* 0: write x_HI = 1 - ionised; 1: write the ionised fraction */
} es_ionize_params;

/* Replaces the per-box set-up of conv_bubbles (find_HII_bubbles.py:76-91): pyfft Plan, device
 * boxes.  n: HII_DIM (32, 48, 64, 96, 128, 160, 256 or 512); box_len: BOX_LEN [Mpc];
 * max_radii: longest schedule the plan will run. */
int es_plan_create(int n, double box_len, int max_radii, es_plan** plan);
int es_plan_destroy(es_plan* plan);
/* Device bytes es_plan_create allocates for (n, max_radii); 0 for an unsupported n. */
size_t es_plan_workspace_bytes(int n, int max_radii);
/* Box sizes with compiled kernels, written to sizes[0..cap); returns their count. */
int es_supported_sizes(int* sizes, int cap);

/* Plan options.  ES_OPT_COL_VARIANT selects the pass implementation: 1 (default) TMA tiles
 * double-buffered on mbarriers, 0 synchronous tile loads.  ES_OPT_COL_TILE (0..2) and
 * ES_OPT_ROW_TILE (0..3) select the TMA passes' tile shapes; the Python autotuner times them
 * per box size and stores the fastest.  Set options between calls, never while the plan's stream
 * has work of the plan in flight. */
#define ES_OPT_COL_VARIANT 1
#define ES_OPT_COL_TILE 2
#define ES_OPT_ROW_TILE 3
/* ES_OPT_L2_HINTS (default 1): keep the intermediate spectrum in L2 between the passes of a
 * radius when it fits (cache-policy hints on the TMA copies, consumed lines discarded). */
#define ES_OPT_L2_HINTS 4
/* ES_OPT_COL_RADIX / ES_OPT_ROW_RADIX (default 0): radix schedule of the per-radius TMA column
 * passes (z inverse + filter, y inverse) and of the row pass (C2R + ionise): 0 = fewest stages with
 * radices up to 16 (e.g. 16 x 16 for 256 points), 1 = radices up to 8 (8 x 8 x 4).  Chosen by the
 * autotuner with the tile shapes. */
#define ES_OPT_COL_RADIX 5
#define ES_OPT_ROW_RADIX 6
/* ES_OPT_OVERLAP (default 0): with 1, es_ionize alternates two intermediate spectra and runs the
 * column passes (z inverse + filter, y inverse) of radius r + 1 on a stream the plan owns while the
 * row pass of radius r runs on the caller's stream, ordered by events (no device-side waits); the
 * call stays stream-ordered for the caller and can be captured in a CUDA graph.
 * ES_OPT_ROW_CTAS / ES_OPT_COL_CTAS (0..16, default 0 = as many as fit): in overlap mode, caps on
 * the resident CTAs per SM of the row and column passes, leaving room for the other stream's. */
#define ES_OPT_OVERLAP 7
#define ES_OPT_ROW_CTAS 8
#define ES_OPT_COL_CTAS 9
/* ES_OPT_WAIT_LOG2 (0 = default 26, else 8..30): a TMA pass gives up a wait on its tile after
 * 2^value mbarrier polls, records the error word (es_plan_check) and leaves once the copies it
 * issued have landed (a bounded wait too).
 * ES_OPT_DEBUG_STALL (testing the failure path without a GPU fault): while set, CTA 0 of the
 * chosen pass announces 16 bytes more than its first tile brings, so that wait can only time
 * out: ES_STALL_COL_Z_INV (z inverse + filter of es_ionize), ES_STALL_ROW_C2R (row C2R +
 * ionise), ES_STALL_ROW_R2C (row R2C of es_forward); 0 = off.  The results of a stalled call are
 * invalid; the device stays usable. */
#define ES_OPT_WAIT_LOG2 10
#define ES_OPT_DEBUG_STALL 11
#define ES_STALL_COL_Z_INV 1
#define ES_STALL_ROW_C2R 2
#define ES_STALL_ROW_R2C 3
int es_plan_set_option(es_plan* plan, int option, int value);
int es_plan_get_option(es_plan* plan, int option, int* value);
/* Synchronises the stream and reports ES_E_DEVICE if any kernel of the plan gave up a bounded
 * wait since the last check (the word is cleared). */
int es_plan_check(es_plan* plan, void* stream);

/* Forward transform of the density box, once per box (the reference repeats it per radius,
 * find_HII_bubbles.py:141-144).  delta: device float32 n^3. */
int es_forward(es_plan* plan, const float* delta, void* stream);

/* The radius loop of conv_bubbles (find_HII_bubbles.py:121-192) on the spectrum of the last
 * es_forward: filter (HII_filter, find_bubbles.cu:12-42), inverse transform, erfc collapse
 * fraction (fcoll_kernel, cu:43-58), mean normalisation (l.158-160), centre / sphere updates
 * (update_kernel / update_sphere_kernel, cu:59-140) and the final partial ionisation
 * (final_kernel, cu:142-158).  out: device float32 n^3; nf: device float, mean of x_HI
 * (the nf of the output file name, find_HII_bubbles.py:225). */
int es_ionize(es_plan* plan, const es_ionize_params* params, float* out, float* nf, void* stream);

/* delta_T = const_factor * x_HI * (1 + delta) [mK] and its mean (delta_T.py:73-76).
 * xH, delta, dT: device float32 n^3; ave: device float. */
int es_delta_T(es_plan* plan, const float* xH, const float* delta, float const_factor,
               float* dT, float* ave, void* stream);

/* es_delta_T without a plan and without allocating anything: for callers that cannot call
 * cudaMalloc, such as code running inside another runtime's memory pool, host code that is
 * only handed device pointers, or embedders that forbid allocation after start-up.  No
 * counterpart in the reference.  The mean's partial sums live in a static device array of
 * ES_NOALLOC_MAX_CTAS + 64 floats (16.25 KiB) that every GPU loading the library keeps until
 * exit.  The first call on a device looks up that array's device address (cudaGetSymbolAddress)
 * with the device current; make that first call before any stream capture.  Every call shares
 * the array, so calls that overlap on the GPU (other streams, other threads) race: serialise
 * them.  n: even HII_DIM up to ES_NOALLOC_MAX_N; other arguments as es_delta_T, on the
 * current device. */
#define ES_NOALLOC_MAX_CTAS 4096
#define ES_NOALLOC_MAX_N 1024
int es_delta_T_noalloc(int n, const float* xH, const float* delta, float const_factor,
                       float* dT, float* ave, void* stream);

/* Spherically binned power spectrum of g = (dT / ave - 1) V / n^3 (times ave when
 * dimensional), the intended pbox_kernel (delta_T.cu:5-29, delta_T.py:80-98).
 * k2_thresholds: host int[nbins], a mode of integer |k/dk|^2 = m goes to the first bin b
 * with m <= k2_thresholds[b]; the k = 0 mode is excluded.  out: device float[3 * nbins] =
 * per-bin mean of k^3 |g_k|^2 / (2 pi^2 V), mean |k|, and mode count.  nbins <= 128. */
int es_power_spectrum(es_plan* plan, const float* dT, const float* ave, const int* k2_thresholds,
                      int nbins, int dimensional, float* out, void* stream);

/* Plain 3-D transforms in numpy's rfftn layout (n, n, n/2 + 1), for testing the FFT passes:
 * forward unnormalised; inverse unnormalised (numpy irfftn times n^3).  Use the plan's
 * scratch spectrum, so they invalidate the last es_forward. */
int es_fft_r2c(es_plan* plan, const float* in, void* out_half, void* stream);
int es_fft_c2r(es_plan* plan, const void* in_half, float* out, void* stream);

/* Per-launch timing.  es_profile_enable(plan, K) pre-creates event pairs for K launches (0
 * turns timing off); every kernel the plan launches afterwards is bracketed by CUDA events on
 * its stream.  es_profile_read synchronises on the recorded events and writes, per kernel kind
 * (ES_PROF_*), the summed milliseconds and launch counts; it returns the number of launches
 * that found the pool full.  es_profile_reset starts a new window. */
#define ES_PROF_COL_Z_FWD 0
#define ES_PROF_COL_Y_FWD 1
#define ES_PROF_COL_Z_INV_FILTER 2
#define ES_PROF_COL_Y_INV 3
#define ES_PROF_COL_Z_FWD_PK 4
#define ES_PROF_ROW_R2C 5
#define ES_PROF_ROW_R2C_PK 6
#define ES_PROF_ROW_C2R 7
#define ES_PROF_ROW_C2R_IONIZE 8
#define ES_PROF_COL_Z_INV 9
#define ES_PROF_FILTER_TABLE 10
#define ES_PROF_FINAL 11
#define ES_PROF_DELTA_T 12
#define ES_PROF_PAINT 13
#define ES_PROF_COUNT 14
int es_profile_enable(es_plan* plan, int max_launches);
int es_profile_reset(es_plan* plan);
int es_profile_read(es_plan* plan, float* total_ms, int* counts, int nops);

/* Batched form (no counterpart in the reference, whose boxes run one at a time): many boxes of
 * uneven HII_DIM (32..256), each with its own parameters, run in ONE persistent launch.  The
 * host lists every box's passes (forward transform, three passes per radius, final step) and
 * merges them into a work queue: boxes are dealt to lanes balanced by N^3 * N_R, the lanes
 * advance side by side in proportion to work, and CTAs take tickets of `chunk` tiles from a
 * global counter in queue order.  A pass starts once its dependencies (earlier passes of its box)
 * have finished (bounded waits; a timeout aborts the launch and es_batch_check reports
 * ES_E_DEVICE).  Centre-pixel (update 0) and sphere (update 1) modes.  delta / out / nf are
 * device buffers owned by the caller; es_batch_create copies the parameters and allocates the workspace of every box.
 * es_batch_run(use_graph = 1) captures the clear + launch into a CUDA graph on its first call and
 * replays it afterwards. */
typedef struct es_batch es_batch;
typedef struct es_batch_box {
  int n;                      /* HII_DIM */
  double box_len;             /* BOX_LEN [Mpc] */
  const float* delta;         /* device float32 n^3 density */
  float* out;                 /* device float32 n^3 output (x_HI or ionised fraction) */
  float* nf;                  /* device float: mean x_HI */
  es_ionize_params params;    /* as for es_ionize */
  /* Optional 21-cm products of the box (delta_T.py:73-98), as es_delta_T and
   * es_power_spectrum compute them: t_factor = 0 skips both; k2_thresholds = NULL skips P(k). */
  float t_factor;             /* brightness-temperature factor c(z) [mK] */
  float* dT;                  /* device float n^3: delta_T = c x_HI (1 + delta) */
  float* ave;                 /* device float: mean delta_T */
  const int* k2_thresholds;   /* host int[nbins], non-decreasing: P(k) bins as es_power_spectrum */
  int nbins;                  /* 1..128 */
  int dimensional;            /* 1: P(k) of delta_T - ave instead of delta_T / ave - 1 */
  float* pk;                  /* device float[3 * nbins]: mean k^3 |g|^2 / (2 pi^2 V), mean |k|, count */
} es_batch_box;
int es_batch_create(const es_batch_box* boxes, int count, es_batch** batch);
int es_batch_run(es_batch* batch, int use_graph, void* stream);
int es_batch_check(es_batch* batch, void* stream);
int es_batch_info(const es_batch* batch, int* grid, int* passes, unsigned* tiles, int* smem);
/* Queue schedule: `lanes` boxes in flight (0 = every box its own lane, the default), `chunk`
 * tiles per ticket (1..64; by default 16, 8 or 4 as the batch gives each resident CTA at least
 * 4000, 1000 or fewer tiles).  Rebuilds the queue; the next es_batch_run recaptures. */
int es_batch_set_schedule(es_batch* batch, int lanes, int chunk);
int es_batch_get_schedule(const es_batch* batch, int* lanes, int* chunk, unsigned* tickets);
/* Per-op profile of the persistent launch: es_batch_profile(batch, 1) clears and enables
 * counters that every launch afterwards adds to (0 frees them); es_batch_profile_read
 * synchronises the device and writes, per op code (as es_batch_queue's, nops <= 16), four
 * counts: SM clock cycles CTAs spent in the op's tiles, tiles, cycles finding and awaiting the
 * op's tickets, tickets. */
int es_batch_profile(es_batch* batch, int enable);
int es_batch_profile_read(es_batch* batch, unsigned long long* out, int nops);
/* The work queue es_batch_create would build for boxes of HII_DIM n[i] with n_radii[i] radii and
 * update mode update[i] (NULL: all 0) under a schedule, computed on the host (no device needed):
 * per pass 8 ints (box, op, radius, tiles, first ticket, tickets, dependency, second dependency;
 * -1 = none) into out[8 * cap].  op: 0 row r2c, 1 y forward, 2 z forward, 3 z inverse, 4 y
 * inverse, 5 row c2r, 6 final, 7 filter tables, 8 sphere painting, 9 row r2c of delta_T, 10 z
 * forward + P(k) binning.  pk (NULL: none) flags the boxes with delta_T and P(k).  Returns the
 * number of passes, or a negative error code. */
int es_batch_queue(const int* n, const int* n_radii, const int* update, const int* pk, int count, int lanes,
                   int chunk, int* out, int cap);
int es_batch_destroy(es_batch* batch);
/* Failure-detection test hook: pass `pass` waits for one tile more than its dependency
 * completes and every wait gives up after spin_limit polls of ~100 ns.  The launch then aborts
 * cleanly and es_batch_check reports ES_E_DEVICE; the device stays usable. */
int es_batch_debug_stall(es_batch* batch, int pass, long spin_limit);
int es_batch_last_error(char* buf, int len);

/* Learned surrogate (no counterpart in the reference): 3x3x3 circular convolutions of
 * channels-last BF16 boxes on the tensor cores, FP32 accumulation.  Activations [z][y][x][C] bf16,
 * weights [27][cout][cin] bf16 with tap (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1), bias float[cout].
 * mode 0: out = ReLU(conv + bias) bf16; mode 1: out = sigmoid(conv + bias) of channel 0 as float
 * [n^3] (cout = 16, channels 1..15 zero weights); mode 2 (input gradient): out = conv(dZ, W') * 1[mask > 0]
 * bf16, with W'[t][ci][co] = W[26 - t][co][ci] and mask the layer's input activations.
 * n: multiple of 16 up to 128.  Compiled (cin, cout): mode 0 (16, 32), (32, 32); mode 1 (32, 16);
 * mode 2 (32, 32), (16, 32); wgrad (16, 32), (32, 32), (32, 16). */
int sg_conv3d_fwd(int n, int cin, int cout, int mode, const void* in, const void* w, const float* bias,
                  void* out, const void* mask, void* stream);
/* Weight and bias gradients: dw[27][cout][cin] = sum_x dZ[x][co] X[x + tap][ci], db[co] = sum_x
 * dZ[x][co] (float).  ws: caller-owned float workspace of sg_conv3d_wgrad_workspace bytes. */
int sg_conv3d_wgrad(int n, int cin, int cout, const void* x, const void* dz, float* dw, float* db,
                    float* ws, size_t ws_bytes, void* stream);
size_t sg_conv3d_wgrad_workspace(int n, int cin, int cout);
/* Network input for one box: out[n^3][16] bf16 with channel 0 = bf16(delta * scale) (round to
 * nearest even) and channels 1..15 = channels16[1..15] (bf16 bit patterns; channels16[0] unused).
 * delta: float [n^3] on the device; out 16-byte aligned. */
int sg_features(int n, const float* delta, float scale, const uint16_t* channels16, void* out, void* stream);
/* The same with nsm (0..11) smoothed copies of the density in channels 5 .. 4 + nsm:
 * bf16(smoothed[j][voxel] * scale); smoothed holds nsm boxes of n^3 floats one after another.  No
 * counterpart in the reference (network input of the surrogate). */
int sg_features_ms(int n, const float* delta, const float* smoothed, int nsm, float scale, const uint16_t* channels16,
                   void* out, void* stream);
/* Which kernels sg_conv3d_fwd runs (process-wide, no counterpart in the reference):
 * SG_IMPL_AUTO = tcgen05/TMEM kernels for n = 128 (one CTA per SM, TMA-fed, accumulators in tensor
 * memory) and mma.sync kernels for other n; SG_IMPL_MMA_SYNC = mma.sync kernels for every n. */
#define SG_IMPL_AUTO 0
#define SG_IMPL_MMA_SYNC 1
int sg_conv3d_set_impl(int impl);
int sg_conv3d_get_impl(void);
/* Synchronises the device and reports ES_E_DEVICE if a tcgen05 convolution gave up a bounded wait
 * since the last call (the flag is cleared); ES_OK otherwise. */
int sg_check(void);
int sg_last_error(char* buf, int len);

/* Density evolution producing the excursion-set input boxes (perturb_field.py:39-128).
 * pf_plan: device tables for a DIM^3 initial-conditions box and an HII_DIM^3 output grid
 * (pixel_factor = DIM / HII_DIM as float32, INIT_PARAMS.py:7) and the fixed-point accumulator.
 * pf_move_mass replaces move_mass (perturb_field.cu:90-132) with the velocity scaling and
 * normalisation around it (perturb_field.py:91-101): delta [DIM^3], vx, vy, vz [HII_DIM^3]
 * (displacement per unit growth, box-axis order 0, 1, 2), disp_scale = (D(z) - D(z_init)) / BOX_LEN,
 * init_growth = D(z_init); updated [HII_DIM^3] = mass / mass_factor - 1.  Masses are summed exactly
 * in 64-bit fixed point (2^-32), so the result does not depend on the order of the atomics.
 * pf_evolve_linear replaces evolve_linear (perturb_field.py:39-50): out = delta * growth. */
typedef struct pf_plan pf_plan;
int pf_plan_create(int dim, int hii_dim, float pixel_factor, pf_plan** plan);
int pf_plan_destroy(pf_plan* plan);
int pf_move_mass(pf_plan* plan, const float* delta, const float* vx, const float* vy, const float* vz,
                 float init_growth, float disp_scale, float mass_factor, float* updated, void* stream);
int pf_evolve_linear(long long n, const float* delta, float growth, float* out, void* stream);
int pf_last_error(char* buf, int len);

/* Initial conditions around the engine's inverse FFT (initialize.py:33-111).  Boxes and half
 * spectra in numpy rfftn layout ([n][n][n/2+1] complex64), k in units of 2 pi / box_len.
 * ic_spectrum replaces init_kernel (initialize.cu:58-95) with the complex normals of initialize.py:
 * 50-56: H = sqrt(P(|k|) box_len^3) (re + i im) / sqrt(2) off the k_z = 0, n/2 planes (without the
 * 1/sqrt(2) on them), P linear in the table (k_table ascending, k_table[0] below the smallest |k|).
 * ic_shape replaces HII_filter + set_velocity (initialize.cu:12-40, 148-190): out = W(kR) H
 * (filter_type -1: no window) times i k_c / k^2 for component c = 0, 1, 2 (-1: density).
 * ic_subsample replaces subsample (initialize.cu:133-146): small = large[floor(a pf + 0.5)] * scale. */
int ic_spectrum(int n, float box_len, const float* normals_re, const float* normals_im, const float* k_table,
                const float* p_table, int table_n, void* out_half, void* stream);
int ic_shape(int n, float box_len, const void* in_half, int component, int filter_type, float R, int ref_compat,
             void* out_half, void* stream);
int ic_subsample(int dim, int hii_dim, float pixel_factor, float scale, const float* large, float* small,
                 void* stream);
int ic_last_error(char* buf, int len);

/* Self-test of the erfc used for the per-radius sum of fcoll: writes it (fast) and the CUDA
 * library's erfcf (lib) for n device floats x. */
int es_selftest_erfc(const float* x, float* fast, float* lib, int n, void* stream);

/* Message of the calling thread's last failure, copied into buf (NUL-terminated). */
int es_last_error(char* buf, int len);
int es_version(void);

#ifdef __cplusplus
}
#endif
#endif /* ES_ENGINE_H */
