/*
 * pycwb_gb300 — C ABI of the GB300 (sm_103a) coherent sky-scan likelihood.
 *
 * Plain C types only: every array is a DEVICE pointer (CUDA global memory),
 * every size is an integer, `stream` is a cudaStream_t passed as void*
 * (NULL = legacy default stream).  Calls are asynchronous on `stream` and
 * allocate nothing: scratch memory is the caller's `workspace` (size from
 * pgw_workspace_bytes).  Host-side argument errors return a pgw_status at
 * once; errors found by a kernel (a delay index outside the td window, an
 * expired wait) are written as bits (1 << code) into the `status` field of
 * the pgw_scan_result the call fills, which the caller reads back together
 * with l_max.  No call aborts, traps or waits without a time limit.
 *
 * Array layouts are the reference's (pycwb/modules/likelihoodWP):
 *   FP, FX   (n_sky, n_ifo) float32   likelihood_setup.py:162-163
 *   ml       (n_ifo, n_sky) int32     detector.py:1318-1321
 *   rms      (n_pix, n_ifo) float32   likelihood.py:305
 *   td00/90  (n_delay, n_ifo, n_pix) float32, n_delay = 2K+1
 *                                     likelihood.py:303-304
 *   stats    (11, n_sky) float32 in the order of the reference's return
 *            tuple (sky_scan.py:191-192): antenna prior, alignment,
 *            likelihood, null energy, coherent energy, correlation, sky
 *            statistic, disbalance, network index, ellipticity, polarisation.
 */
#ifndef PYCWB_GB300_H
#define PYCWB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGW_MAX_IFO 8
#define PGW_N_STATS 11

typedef enum {
  PGW_OK = 0,
  PGW_ERR_BAD_SHAPE = 1,       /* shape/size argument out of range (reference: ValueError, dpf.py:14-22) */
  PGW_ERR_BAD_ARGUMENT = 2,    /* NULL pointer or misaligned buffer */
  PGW_ERR_CUDA = 3,            /* a CUDA runtime call failed; see pgw_last_error() */
  PGW_ERR_WORKSPACE = 4,       /* workspace smaller than pgw_workspace_bytes() */
  PGW_ERR_DELAY_RANGE = 5,     /* device: ml[i,l] + K outside [0, n_delay) */
  PGW_ERR_TIMEOUT = 6,         /* device: a bounded wait expired */
  PGW_ERR_SKY_INDEX = 7        /* device: a sky_valid_indices entry outside [0, n_sky) */
} pgw_status;

/* Result of one cluster's sky scan, written by the device. */
typedef struct {
  int64_t l_max;        /* selected sky index (sky_scan.py:183-189: >=, last tie wins) */
  float sky_stat_max;   /* statistic at l_max; 0 when no direction qualified */
  int32_t found;        /* 0: no valid direction reached the >= comparison; l_max = valid[0] */
  int32_t status;       /* OR of (1 << pgw_status) for device-detected errors */
  float regulator;      /* REG[1] used by the scan (float32, as stored by likelihood.py:310) */
  int64_t active_pairs; /* (direction, pixel) pairs above the energy threshold: sum over the
                           valid directions of the pixel count NN of sky_stat.py:184 */
} pgw_scan_result;      /* 32 bytes */

/* Library version string. */
const char* pgw_version(void);

/* Message of the last failing call on this host thread ("" when none). */
const char* pgw_last_error(void);

/* Bytes of scratch a call needs for n_clusters clusters holding total_pix
 * pixels in all (plain calls: n_clusters = 1, total_pix = n_pix). */
size_t pgw_workspace_bytes(int n_ifo, int n_delay, int64_t total_pix, int n_clusters);

/* Scan order of the valid directions (host arrays, once per segment):
 * out_order[0..n_valid) = positions of sky_valid_indices sorted by their
 * delay tuple (ml[0, l], ..., ml[n_ifo-1, l]), ties in position order;
 * *out_n_tuples = number of distinct tuples.  Directions with one tuple see
 * the same delayed data and so the same pixel energy mask; passed as
 * `sky_order` to the sky-loop calls, it lets a warp evaluate only the pixels
 * above the energy threshold.  Results do not depend on the order (the sky
 * maximum's tie rule uses the positions in sky_valid_indices).  Counterpart
 * of nothing in the reference (an execution order, not a result). */
int pgw_sky_order(const int32_t* ml, int n_ifo, int64_t n_sky, const int64_t* sky_valid_indices,
                  int64_t n_valid, int32_t* out_order, int64_t* out_n_tuples);

/* Regulator order of the valid directions (host arrays, once per segment):
 * out_order[0..n_valid) = positions of sky_valid_indices sorted by the mean,
 * over fixed draws of normalised detector weights, of the regulator's
 * per-pixel term fx / ni (FP, FX: (n_sky, n_ifo) float32).  The regulator
 * decides most directions after part of the pixels (a running sum already
 * over the threshold, or a bound on the rest already under it); the point
 * depends mainly on that term, so this order gives the 32 directions of a
 * warp similar stopping points.  Passed as `reg_order` to the sky-loop
 * calls; results do not depend on it.  Counterpart of nothing in the
 * reference (an execution order, not a result). */
int pgw_regulator_order(const float* FP, const float* FX, int n_ifo, int64_t n_sky,
                        const int64_t* sky_valid_indices, int64_t n_valid, int32_t* out_order);

/* The same sort, with the sorted directions taken in groups of 32 (one
 * regulator tile, or two) ordered by their distance from the group where
 * the mean term crosses the pass threshold gamma_regulator^2: the
 * directions near it decide last, so their tiles run longest, and taking
 * them first keeps a launch's last tiles short (longest processing time
 * first).  Results do not depend on it either. */
int pgw_regulator_order_lpt(const float* FP, const float* FX, int n_ifo, int64_t n_sky,
                            const int64_t* sky_valid_indices, int64_t n_valid,
                            double gamma_regulator, int32_t* out_order);

/* DPF regulator: REG[1] = (n_valid^2 / (n_pass^2 + 1e-9) - 1) * E_thr, where
 * n_pass counts valid directions whose DPF quality sqrt(NI / (NN + 0.01))
 * exceeds gamma_regulator.
 * Replaces calculate_dpf, pycwb/modules/likelihoodWP/dpf.py:7-34.
 * Writes *out_regulator (float64, device) and, when REG != NULL, REG[1]
 * (float32, device) so the scan can consume it without a host round trip. */
int pgw_calculate_dpf(const float* FP, const float* FX, const float* rms, int64_t n_sky,
                      int n_ifo, int64_t n_pix, double gamma_regulator,
                      double network_energy_threshold, const int64_t* sky_valid_indices,
                      int64_t n_valid, double* out_regulator, float* REG, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Sky scan over the valid directions with a given REG (device, 3 floats).
 * Replaces scan_sky_for_best_fit, pycwb/modules/likelihoodWP/sky_scan.py:17-192.
 * out_stats: (11, n_sky) float32; entries of directions that are masked or
 * rejected are 0, as in the reference.  sky_order: device int32 array from
 * pgw_sky_order (n_valid entries), or NULL to scan in the given order. */
int pgw_scan_sky_for_best_fit(int n_ifo, int64_t n_pix, int64_t n_sky, const float* FP,
                              const float* FX, const float* rms, const float* td00,
                              const float* td90, int n_delay, const int32_t* ml, const float* REG,
                              double netCC, double delta_regulator,
                              double network_energy_threshold,
                              const int64_t* sky_valid_indices, int64_t n_valid,
                              const int32_t* sky_order, float* out_stats,
                              pgw_scan_result* out_result, void* workspace, size_t workspace_bytes,
                              void* stream);

/* Launch shape of the sky-loop kernel (any field 0 = automatic).
 *   threads        CTA size, a multiple of 32 in [64, 256]
 *   lanes_per_sky  1, 2 or 4 lanes share one direction and split its pixels
 *   chunk_pix      pixels per chunk staged in shared memory by one TMA copy
 *   stages         chunks in flight per CTA, 2..4
 *   min_blocks     occupancy target the kernel is compiled for: 3 or 4 CTAs
 *                  per SM for n_ifo <= 4, 2 above
 *   fast_math      0 (automatic) or 1: the scan's two rotation quotients
 *                  are a reciprocal estimate with one correction step
 *                  (Markstein; within one ulp of the correctly rounded
 *                  quotient, no slow-path branch), its other ten quotients
 *                  the estimate's product (about 2 ulp), its square roots
 *                  sqrt.approx.ftz.f32 except the packet-rotation norm,
 *                  refined likewise; -1: IEEE rounding of every division
 *                  and square root.  Both meet the 1e-4 relative parity
 *                  bar; the regulator's decisions are exact either way (its
 *                  fallback always uses IEEE arithmetic). */
typedef struct {
  int threads;
  int lanes_per_sky;
  int chunk_pix;
  int stages;
  int min_blocks;
  int fast_math;
} pgw_tile_shape;

/* Both passes for one cluster in one launch: the regulator, then the scan
 * with REG = {REG0, regulator, 0}.  Replaces the two calls at
 * pycwb/modules/likelihoodWP/likelihood.py:310-325 ("plain" path).  shape
 * may be NULL.  reg_order: device int32 array from pgw_regulator_order, or
 * NULL (the regulator then follows sky_order). */
int pgw_sky_loop(int n_ifo, int64_t n_pix, int64_t n_sky, const float* FP, const float* FX,
                 const float* rms, const float* td00, const float* td90, int n_delay,
                 const int32_t* ml, float REG0, double gamma_regulator, double netCC,
                 double network_energy_threshold, const int64_t* sky_valid_indices,
                 int64_t n_valid, const int32_t* sky_order, const int32_t* reg_order,
                 float* out_stats, pgw_scan_result* out_result, double* out_regulator,
                 const pgw_tile_shape* shape, void* workspace, size_t workspace_bytes,
                 void* stream);

/* Allocation-free form of pgw_sky_loop.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory per call --
 * cudaMalloc/cudaFree may synchronise the device, and a host framework that
 * owns the device memory (its own pool, a fixed budget) may forbid
 * allocations outside it.  Scratch comes from a static device array of
 * pgw_sky_loop_noalloc_max_scratch() bytes (8 MiB, enough for about 7,800
 * pixels at n_ifo = 3 and n_delay = 41) that every GPU loading the library
 * holds until the process exits; a larger cluster is rejected with
 * PGW_ERR_WORKSPACE.  The call allocates nothing (no cudaMalloc/cudaFree, no
 * allocating library routine).  Its first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current:
 * make that first call before any stream capture.  Every call shares the one
 * array and leaves its contents behind (each call clears what must start at
 * zero), so calls that overlap on the GPU -- on different streams or from
 * different host threads -- race: serialise them.  Inputs and outputs as in
 * pgw_sky_loop; the default launch shape is used. */
size_t pgw_sky_loop_noalloc_max_scratch(void);
int pgw_sky_loop_noalloc(int n_ifo, int64_t n_pix, int64_t n_sky, const float* FP,
                         const float* FX, const float* rms, const float* td00, const float* td90,
                         int n_delay, const int32_t* ml, float REG0, double gamma_regulator,
                         double netCC, double network_energy_threshold,
                         const int64_t* sky_valid_indices, int64_t n_valid,
                         const int32_t* sky_order, float* out_stats, pgw_scan_result* out_result,
                         double* out_regulator, void* stream);

/* Regulator and scan for many clusters of one segment in ONE persistent
 * launch driven by a work queue of (cluster, sky tile) items taken in
 * decreasing cluster size.  Replaces the per-cluster loop of
 * evaluate_fragment_clusters, pycwb/modules/likelihoodWP/likelihood.py:58-135
 * (its calls at :310-325).  shape may be NULL.  Clusters are concatenated along the pixel axis:
 * cluster c owns pixels [pix_offsets[c], pix_offsets[c+1]) of rms_all
 * (total_pix, n_ifo) and the float32 block of n_delay*n_ifo*n_pix_c values
 * starting at td_offsets[c] in td00_all/td90_all, laid out (n_delay, n_ifo,
 * n_pix_c) like the plain call.  pix_offsets and td_offsets are device int64
 * arrays of n_clusters+1 entries; total_pix = pix_offsets[n_clusters] (given
 * on the host to size the workspace).  out_stats: (n_clusters, 11, n_sky);
 * out_results and out_regulators: n_clusters entries. */
int pgw_sky_loop_batched(int n_ifo, int n_clusters, const int64_t* pix_offsets,
                         const int64_t* td_offsets, int64_t total_pix, int64_t n_sky, const float* FP, const float* FX, const float* rms_all,
                         const float* td00_all, const float* td90_all, int n_delay,
                         const int32_t* ml, float REG0, double gamma_regulator, double netCC,
                         double network_energy_threshold, const int64_t* sky_valid_indices,
                         int64_t n_valid, const int32_t* sky_order, const int32_t* reg_order,
                         float* out_stats, pgw_scan_result* out_results, double* out_regulators,
                         const pgw_tile_shape* shape, void* workspace, size_t workspace_bytes,
                         void* stream);

/* Regulator only, for every cluster of a batch in one launch: REG[1] of each
 * cluster (pgw_calculate_dpf's value) into out_regulators[n_clusters]
 * (float64).  The batched form of pycwb/modules/likelihoodWP/dpf.py:8-34 as
 * likelihood.py:310-312 calls it per cluster; rms_all and pix_offsets as in
 * pgw_sky_loop_batched, workspace of pgw_workspace_bytes(n_ifo, 1, total_pix,
 * n_clusters) bytes.  sky_order and reg_order (optional, as in pgw_sky_loop)
 * set the order the directions are visited in, which does not change the
 * result. */
int pgw_calculate_dpf_batched(int n_ifo, int n_clusters, const int64_t* pix_offsets,
                              int64_t total_pix, int64_t n_sky, const float* FP, const float* FX,
                              const float* rms_all, double gamma_regulator,
                              double network_energy_threshold, const int64_t* sky_valid_indices,
                              int64_t n_valid, const int32_t* sky_order,
                              const int32_t* reg_order, double* out_regulators,
                              const pgw_tile_shape* shape, void* workspace,
                              size_t workspace_bytes, void* stream);

/* td-amplitude vectors of n_pixels pixels of one (layer, detector) plane:
 * out (n_pixels, 4K+2) float32 = [a00(-K..K), a90(-K..K)] per pixel.
 * Replaces batch_get_td_vecs, pycwb/utils/td_vector_kernels.py:133-199
 * (getTDamp, cwb-core/WDM.cc:1103-1196).  padded00/90: (rows, M+1) float32
 * planes padded by n_coeffs zero rows at both ends; T0, Tx: (2J+1,
 * 2*n_coeffs+1) float64 TD filters; phase: (M+1, 2J+1, 4) float64 factors
 * {cos(same), sin(same), sin(low), sin(high)} (see pycwb_gb300.tdamp).
 * Bit-identical to the reference: float64 accumulation in its order. */
int pgw_batch_get_td_vecs(const int32_t* pixel_indices, int64_t n_pixels, const float* padded00,
                          const float* padded90, int64_t rows, const double* T0, const double* Tx,
                          const double* phase, int M, int n_coeffs, int K, int J, float* out,
                          void* stream);

/* Result of the sub-network-cut sky loop for one cluster: the reference's
 * (l_max, stat, Em, Am, lm, Vm, suball, EE) with lm = l_max
 * (pycwb/modules/super_cluster_native/sub_net_cut.py:517).  `key` is the
 * loop's internal (statistic, direction) maximum; `status` carries
 * device-detected errors as bits 1 << pgw_status. */
typedef struct {
  uint64_t key;
  int64_t l_max;
  float stat, Em, Am, suball, EE;
  int32_t Vm;
  int32_t status;
  int32_t reserved;
} pgw_subnet_result;

/* Sub-network-cut sky loop for a batch of clusters in one launch:
 * optimze_sky_loc_from_td (sub_net_cut.py:404-517) on every cluster, over
 * all n_sky directions (the reference's MIN_SKYRES_HEALPIX grid).  Cluster
 * layout as in pgw_sky_loop_batched (pix_offsets/td_offsets may be NULL for
 * one cluster of total_pix pixels); FP, FX (n_sky, n_ifo); ml (n_ifo, n_sky);
 * network_energy_threshold = float32(2 Acore^2 n_ifo) (:190), e2or and subcut
 * as the reference takes them (subcut < 0 turns the sky gate off).  out:
 * n_clusters results (1 <= n_clusters <= 65535 per call).  Every float32
 * operation is rounded as the reference's (NumPy scalar semantics, no
 * contraction), so the results equal the reference's bit for bit on its own
 * arithmetic. */
int pgw_subnet_sky_batched(int n_ifo, int n_clusters, const int64_t* pix_offsets,
                           const int64_t* td_offsets, int64_t total_pix, int64_t n_sky,
                           const float* FP, const float* FX, const float* rms_all,
                           const float* td00_all, const float* td90_all, int n_delay,
                           const int32_t* ml, float network_energy_threshold, double e2or,
                           double subcut, pgw_subnet_result* out, void* stream);

/* Per-segment sky tables on the device for a HEALPix RING grid of order
 * healpix_order (12 * 4^order directions): FP, FX (n_sky, n_ifo) float32
 * antenna patterns at psi = 0 and ml (n_ifo, n_sky) int32 delay indices
 * clip(rint((n . b_i) / c_light * sample_rate), -td_size, td_size), from each
 * detector's 3x3 response tensor (response, host, n_ifo x 9 float64,
 * row-major) and baseline to the reference detector (baseline, host,
 * n_ifo x 3 float64, metres).  Replaces compute_sky_delay_and_patterns
 * (pycwb/types/detector.py:1243-1329) for HEALPix grids; outputs are device
 * pointers, written asynchronously on `stream`. */
int pgw_sky_tables_healpix(int healpix_order, int n_ifo, const double* response,
                           const double* baseline, double c_light, double sample_rate,
                           int td_size, float* FP, float* FX, int32_t* ml, void* stream);

/* td-amplitude vectors written straight into the batched scan's inputs: the
 * amplitudes of pgw_batch_get_td_vecs for the n_pixels pixels of one
 * (WDM plane, detector `ifo`) go to cluster dst_cluster[p], local pixel
 * dst_pixel[p], of td00_all/td90_all laid out as in pgw_sky_loop_batched
 * (pix_offsets, td_offsets, n_ifo).  Replaces, for the scan's purposes, the
 * per-(layer, detector) calls of pycwb/modules/super_cluster_native/
 * super_cluster.py:545-564 followed by the dense -> CSR -> (D, I, P)
 * rearrangements of pixel_arrays.py:251-258 and likelihood.py:303-304.
 * Destinations outside [0, n_clusters) x [0, P_c) are skipped. */
int pgw_td_vecs_to_clusters(const int32_t* pixel_indices, int64_t n_pixels,
                            const int32_t* dst_cluster, const int32_t* dst_pixel, int n_clusters,
                            const int64_t* pix_offsets, const int64_t* td_offsets, int ifo,
                            int n_ifo, const float* padded00, const float* padded90, int64_t rows,
                            const double* T0, const double* Tx, const double* phase, int M,
                            int n_coeffs, int K, int J, float* td00_all, float* td90_all,
                            void* stream);

/* Sky statistic at continuous directions and its gradient (no counterpart
 * in the reference, which evaluates the statistic only on the grid).  For
 * query q: cluster query_cluster[q] of the concatenated batch (layouts as in
 * pgw_sky_loop_batched), direction (theta[q], phi[q]) in radians (Earth-fixed
 * colatitude and longitude).  F+/Fx come from each detector's response
 * tensor and the delays tau_i = n . b_i are interpolated linearly between td
 * samples.  geometry: (n_ifo, 12) float32 = response tensor (row major, 9)
 * and baseline to the reference detector in TD samples (3).  reg1: REG[1]
 * per cluster.  out: (n_queries, 8) float32 = statistic (likelihood x
 * correlation, sky_scan.py:140), d/dtheta, d/dphi, likelihood, correlation,
 * ellipticity, coherent energy, null energy.  The gradient is exact
 * (dual-number tangents through the whole pipeline), one-sided at kinks. */
int pgw_sky_stat_grad(int n_ifo, int n_queries, const int32_t* query_cluster,
                      const double* theta, const double* phi, const int64_t* pix_offsets,
                      const int64_t* td_offsets, const float* rms_all, const float* td00_all,
                      const float* td90_all, int n_delay, const float* geometry, float REG0,
                      const float* reg1, double network_energy_threshold, float* out,
                      void* stream);

/* Off-grid refinement of sky maxima: for each query, n_steps of gradient
 * ascent on the statistic from (theta0, phi0), steps of step0 radians of arc
 * along the gradient, halved whenever a step would lower the statistic.
 * Writes the final direction (theta_out, phi_out), its 8 outputs as in
 * pgw_sky_stat_grad, and (when trace != NULL) (statistic, theta, phi) after
 * each step: (n_queries, n_steps + 1, 3). */
int pgw_refine_sky(int n_ifo, int n_queries, const int32_t* query_cluster, const double* theta0,
                   const double* phi0, const int64_t* pix_offsets, const int64_t* td_offsets,
                   const float* rms_all, const float* td00_all, const float* td90_all,
                   int n_delay, const float* geometry, float REG0, const float* reg1,
                   double network_energy_threshold, int n_steps, float step0, double* theta_out,
                   double* phi_out, float* out, float* trace, void* stream);

/* Diagnostics (no counterpart in the reference).  Measures the device's
 * FP32 fused-multiply-add throughput (TFLOP/s, 2 flops per FMA) with one
 * timed launch of `iters` x 128 register FMAs per thread; the sky loop's
 * FP32 roofline is reported against this number.  Synchronous. */
int pgw_fp32_fma_peak(int iters, double* out_tflops, double* out_ms, void* stream);

/* Measured float64 multiply + add throughput (G ops/s, a multiply and an add
 * counted as one op each, issued as separate correctly rounded instructions):
 * the denominator of the td-amplitude build's roofline.  Synchronous. */
int pgw_fp64_mul_add_peak(int iters, double* out_gops, double* out_ms, void* stream);

/* WDM forward transform of one series, both quadratures: cWB's
 * WDM::t2w(MM = -1) (cwb-core/WDM.cc:1384-1535), which the reference calls
 * through wdm_wavelet's WDM.t2w (pycwb/utils/td_vector_batch.py:80) and then
 * pads (pycwb/types/time_frequency_map.py:482-521).  ts: n_ts float64
 * samples (device); M: layers, a power of two in [1, 4096]; filter: the
 * basis filter's n_filter float64 coefficients (device; n_filter - 1 a
 * multiple of 2M, n_ts > n_filter).  Outputs (device, either pair may be
 * NULL): map00/map90 (n_time, M+1) float64 with n_time = pgw_wdm_n_time(n_ts,
 * M), row n = time slice n; padded00/padded90 (n_time + 2 n_pad, M+1)
 * float32, the same values between n_pad zero rows on each side (the
 * TDBatchInputs planes of pgw_batch_get_td_vecs).  Asynchronous on `stream`. */
int pgw_wdm_t2w(const double* ts, int64_t n_ts, int M, const double* filter, int64_t n_filter,
                double* map00, double* map90, float* padded00, float* padded90, int n_pad,
                void* stream);

/* Time slices of pgw_wdm_t2w: ceil(n_samples / M) (-1 for M < 1). */
int64_t pgw_wdm_n_time(int64_t n_samples, int M);

/* Statistics at the sky maximum of one cluster (SkyStatistics of
 * sky_statistics.py:246-292, the scalars and the per-detector signal SNR). */
typedef struct {
  double N_pix_effective;
  float Gn, Ec, Dc, Rc, Eh, Es, Np, Em, Lm, norm, cc, rho, xrho, Lo, Eo;
  float S_snr[PGW_MAX_IFO];
  int32_t status;   /* 0, PGW_ERR_DELAY_RANGE, or PGW_ERR_BAD_SHAPE for bad xtalk rows */
  int32_t n_pix;
  int32_t reserved;
} pgw_skystat_result;

/* Bytes of device workspace pgw_skystat_batched needs for total_pix pixels
 * (0 for a bad n_ifo). */
size_t pgw_skystat_workspace_bytes(int n_ifo, int64_t total_pix);

/* compute_statistics_at_sky_position (sky_statistics.py:26-262) for every
 * cluster of a lag in one launch, each at its own direction sky_idx[c]:
 * cluster layout as in pgw_sky_loop_batched (pix_offsets n_clusters+1,
 * td_offsets, rms_all (total_pix, n_ifo), td00_all/td90_all blocks (n_delay,
 * n_ifo, P_c)); regulators[c] = the cluster's REG[1], REG0 = REG[0];
 * xtalk: n_xtalk packed rows of 8 float32 (neighbour index within the
 * cluster, 3 unused, 4 overlap coefficients), xtalk_lookup: per pixel the
 * [start, end) row range (total_pix x 2 int64); ws: at least
 * pgw_skystat_workspace_bytes.  One result per cluster; asynchronous. */
int pgw_skystat_batched(int n_ifo, int n_clusters, const int64_t* pix_offsets,
                        const int64_t* td_offsets, int64_t total_pix, int64_t n_sky,
                        const float* FP, const float* FX, const float* rms_all,
                        const float* td00_all, const float* td90_all, int n_delay,
                        const int32_t* ml, const int64_t* sky_idx, const float* regulators,
                        float REG0, float network_energy_threshold, const float* xtalk,
                        int64_t n_xtalk, const int64_t* xtalk_lookup, int xgb_rho_mode, void* ws,
                        size_t ws_bytes, pgw_skystat_result* out, void* stream);

/* The per-pixel arrays of the reference's SkyStatistics
 * (sky_statistics.py:264-292) for every pixel of the clusters of the last
 * pgw_skystat_batched call that used workspace `ws`, read from it (call on
 * the same stream, after that call).  out32: total_pix records of 9 + 4 n_ifo
 * float32 -- energy_array_plus, energy_array_cross, pixel_mask,
 * gaussian_noise_correction, coherent_energy, p00_POL radius and angle,
 * p90_POL radius and angle, noise_amplitude_00[n_ifo],
 * noise_amplitude_90[n_ifo], f[n_ifo], F[n_ifo] (the dominant-polarisation
 * antenna vectors); out64: total_pix records of 4 n_ifo float64 -- pd, pD,
 * ps, pS (the data and signal packets).  The inputs of the reference's
 * populate_detection_statistics (detection_statistics.py:31-440). */
int pgw_skystat_pixel_arrays(int n_ifo, int64_t total_pix, const void* ws, size_t ws_bytes,
                             float* out32, double* out64, void* stream);

/* Normalised sky probability of selected clusters of a batched sky loop:
 * the reference caller's softmax of the sky-statistic map
 * (pycwb/modules/likelihoodWP/likelihood.py:338-342: p = exp(s - max s) /
 * sum exp(s - max s) over all n_sky entries, float64 arithmetic, float32
 * result), computed where the maps already are, each probability within a
 * few float32 ulp of the reference's (float32-accurate exponentials, a
 * compensated sum carried to float64).  stats: the loop's
 * out_stats, cluster c's (11, n_sky) block at c * stats_stride floats;
 * clusters: n_select cluster indices (device int32), or NULL for clusters
 * 0..n_select-1; out_probability: (n_select, n_sky) float32.  out_summary
 * (may be NULL): per selected cluster 4 float64 -- max s, sum exp(s - max s),
 * and the number of directions, largest probability first, holding 50 % and
 * 90 % of the probability (inputs of an error region; the reference's
 * compute_sky_error_region, detection_statistics.py:520-534, is a
 * placeholder).  A NaN anywhere in a map makes its probabilities NaN, as in
 * NumPy.  Asynchronous on `stream`; allocates nothing. */
int pgw_sky_probability(int n_select, int64_t n_sky, const float* stats, int64_t stats_stride,
                        const int32_t* clusters, float* out_probability, double* out_summary,
                        void* stream);

/* Copy `bytes` from page-locked host memory (cudaHostAlloc'ed or registered)
 * to device memory with a kernel instead of the copy engine, asynchronously
 * on `stream`.  Input staging for the batched loop: the copy engine's first
 * pass over a large host buffer right after a sky-loop launch was measured
 * at 5-11 GB/s on GB300 (210 GB/s on later passes); SM loads keep many host
 * pages in translation at once.  No counterpart in the reference. */
int pgw_copy_from_host(void* dst, const void* host_src, size_t bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PYCWB_GB300_H */
