/*
 * sarbp.h -- C ABI of the GB300-native SAR back-projection imager (libsarbp.so).
 *
 * Drop-in boundary for the reference's back-projection path
 * (wenj-yan/SAR_CambrianAccelerationCard):
 *   launchBackProjection(cufftComplex* Srnm, cufftComplex* Image, const SARParams, int Na, int Nr)
 *     declared code/SAR_BP/CUDA/BPA_CUDA.cpp:8-9, defined BPA_CUDA_kernels.cu:91-98,
 *     called by SAR_Processor::applyBPAlgorithm (BPA_CUDA.cpp:83-90);
 *   launchGenerateEcho(...)  BPA_CUDA.cpp:4-6, BPA_CUDA_kernels.cu:79-89;
 * and of the algorithm those stand for, code/SAR_BP/matlab/BPA_SAR.m
 *   (echo :80-89, range compression :93-100, 8x upsampling :106-111,
 *    back-projection :177-197).
 *
 * Unlike the reference, every entry point
 *   - takes the antenna phase-centre (APC) track and the pixel grid explicitly
 *     (the reference derives them from SARParams only);
 *   - returns a status code instead of calling exit() (CHECK_CUDA, BPA_CUDA.h:11-17);
 *   - works on caller-owned buffers; pointers may be host or device memory
 *     (detected per call).  With host pointers the call is synchronous; with
 *     device pointers it is asynchronous on `stream` (a cudaStream_t, or NULL
 *     for the context's own stream).
 * A context is not thread-safe; use one per host thread.
 *
 * Complex data are interleaved float pairs (layout-compatible with
 * cufftComplex / float2).  Arrays are row-major: echo [np][ns], range-compressed
 * data [np][nbins], APC [np][3] doubles, image [ny][nx].
 */
#ifndef SARBP_H
#define SARBP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Raised when a struct a caller allocates or an entry point changes (2: the
 * serving stats' step and admission device times, the debug switches). */
#define SARBP_ABI_VERSION 2

typedef enum sarbp_status {
    SARBP_OK = 0,
    SARBP_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad enum */
    SARBP_ERR_UNSUPPORTED = 2,      /* valid but outside what this build handles */
    SARBP_ERR_OUT_OF_MEMORY = 3,    /* device or pinned-host allocation failed */
    SARBP_ERR_CUDA = 4,             /* a CUDA runtime call failed; see sarbp_last_error */
    SARBP_ERR_NO_DEVICE = 5,        /* no usable sm_103 device */
    SARBP_ERR_TIMEOUT = 6,          /* a bounded device-side wait ran out */
    SARBP_ERR_DEVICE_CHECK = 7,     /* a kernel's own consistency check tripped */
    SARBP_ERR_NOT_READY = 8,        /* serving: job still running */
    SARBP_ERR_CANCELLED = 9,        /* serving: job cancelled */
    SARBP_ERR_BUDGET = 10,          /* serving: job larger than the HBM budget */
    SARBP_ERR_INTERNAL = 11
} sarbp_status;

/* Back-projection arithmetic. */
typedef enum sarbp_mode {
    SARBP_MODE_FP64 = 0,     /* plain FP64 per pixel and pulse (the comparator) */
    SARBP_MODE_FP32 = 1,     /* plain FP32: absolute ranges and phases in FP32 */
    SARBP_MODE_SPLIT = 2,    /* FP64 per-(tile, pulse) reference range and phase wrap,
                                FP32 per-pixel differential range (a series about
                                the tile centre) and phase */
    SARBP_MODE_FP16STORE = 3 /* SPLIT arithmetic on FP16-stored range-compressed data */
} sarbp_mode;
/* SPLIT and FP16STORE image with tiles of 32 x 64, 32 x 32 or 32 x 16 pixels,
 * the tallest whose differential-range series remainder stays below 5e-7 m
 * (1.1e-4 rad at C band) and whose staging window fits shared memory.  When
 * even 32 x 16 does not, the call returns SARBP_ERR_UNSUPPORTED with the bound
 * that failed: for grids at 45 degrees to the track, pixel spacings above about
 * 1.4 m at 2 km slant range or 2.9 m at 5 km (the series bound, which
 * SARBP_MODE_FP64 does not have), 5 m at 10 km (the staging-window bound,
 * common to every mode: the smallest tile spans more range bins than a
 * 4-pulse chunk stages in 227 KB).  Tiles up to 12 m of
 * half-diagonal use the series form of the phase (about -82 dB against an FP64
 * image); larger ones the linear-term form (per-pixel-step phase increments
 * reduced modulo 2 pi per pulse, FP32 only for the nonlinear remainder: -89 to
 * -113 dB on 0.45-2 m pixels, about 12% more time); sarbp_bp_plan reports the
 * form (linear_phase). */

/* Storage of range-compressed data. */
typedef enum sarbp_storage {
    SARBP_STORE_C64 = 0, /* complex float32 (8 bytes per bin) */
    SARBP_STORE_C32H = 1 /* complex float16 (4 bytes per bin) times a per-pulse float scale */
} sarbp_storage;

typedef struct sarbp_complex64 {
    float re, im;
} sarbp_complex64;

/* Radar constants (replaces SARParams, BPA_CUDA.h:28-50, for this path). */
typedef struct sarbp_radar {
    double c;        /* propagation speed, m/s */
    double fc;       /* carrier frequency, Hz */
    double fs;       /* fast-time sampling rate, Hz */
    double kr;       /* chirp rate, Hz/s */
    double tp;       /* pulse duration, s */
    double tc;       /* time within the pulse where the chirp frequency is 0 (tp/2: centred) */
    double t_rec0;   /* two-way delay of echo sample 0, s */
    int32_t upsample;/* range upsampling factor L: power of two in [1, 16] */
    int32_t reserved;/* must be 0 */
} sarbp_radar;

/* Pixel (x, y) sits at origin + x*ux + y*uy; image is [ny][nx]. */
typedef struct sarbp_grid {
    double origin[3];
    double ux[3];
    double uy[3];
    int32_t nx, ny;
} sarbp_grid;

/* Derived range-compression layout for `ns` echo samples. */
typedef struct sarbp_rc_layout {
    int32_t nc;       /* chirp samples round(tp*fs) */
    int32_t nfft;     /* nextpow2(ns + nc - 1) */
    int32_t shift;    /* output lag shift nc/2 */
    int32_t nbins;    /* upsample * ns bins per pulse */
    double t0_bins;   /* two-way delay of bin 0: t_rec0 - shift/fs */
    double bin_rate;  /* upsample * fs, bins per second of delay */
} sarbp_rc_layout;

/* View of range-compressed data (device or host memory). */
typedef struct sarbp_rc_view {
    const void *data;     /* [np][nbins] complex64 or complex16 */
    const float *scale;   /* [np] per-pulse scale for SARBP_STORE_C32H, else NULL */
    int32_t storage;      /* sarbp_storage */
    int32_t np;
    int32_t nbins;
    int32_t reserved;
    double t0_bins;
    double bin_rate;
} sarbp_rc_view;

/* Point target for the echo synthesiser. */
typedef struct sarbp_target {
    double x, y, z, amp;
} sarbp_target;

typedef struct sarbp_ctx sarbp_ctx;

/* ---------------------------------------------------------------- basics -- */

int sarbp_abi_version(void);
const char *sarbp_status_string(sarbp_status s);

/* Create a context on CUDA device `device` (needs compute capability 10.3).
 * Replaces SAR_Processor's constructor-time allocation (BPA_CUDA.cpp:11-13,51-56). */
sarbp_status sarbp_create(sarbp_ctx **out, int device);
/* Frees every device buffer the context holds (BPA_CUDA.cpp:15-22). */
sarbp_status sarbp_destroy(sarbp_ctx *ctx);
/* Detail message of the last failing call on this context ("" if none). */
const char *sarbp_last_error(const sarbp_ctx *ctx);
/* Waits for all work issued through the context and reports device-side checks. */
sarbp_status sarbp_synchronize(sarbp_ctx *ctx);
/* Releases cached device buffers (they are re-grown on demand). */
sarbp_status sarbp_trim(sarbp_ctx *ctx);
/* Bytes of device memory the context currently holds. */
size_t sarbp_device_bytes(const sarbp_ctx *ctx);

sarbp_status sarbp_rc_layout_get(const sarbp_radar *radar, int32_t ns, sarbp_rc_layout *out);

/* --------------------------------------------------------- imaging path -- */

/* Range compression + upsampling (BPA_SAR.m:93-111; the reference CUDA program
 * declares a cuFFT plan for this, BPA_CUDA.h:65, but never runs it).
 * echo [np][ns] complex64 -> rc_out [np][nbins] (storage), rc_scale_out [np]
 * (required for SARBP_STORE_C32H, ignored otherwise).  nbins = upsample*ns. */
sarbp_status sarbp_range_compress(sarbp_ctx *ctx, const sarbp_radar *radar,
                                  const sarbp_complex64 *echo, int32_t np, int32_t ns,
                                  int32_t storage, void *rc_out, float *rc_scale_out,
                                  void *stream);

/* Range compression that allocates no device memory.  No counterpart in the
 * reference.  For callers that cannot call cudaMalloc while they run -- a host
 * program whose own allocator already reserved the GPU's memory, or a
 * latency-bound loop that must not stall on an allocation.  Same kernels,
 * tables and results as sarbp_range_compress, but all scratch (filter
 * spectrum, FFT phase table for twiddles and upsampling ramp, a batch of pulse
 * spectra) lives in one fixed SARBP_NOALLOC_SCRATCH_BYTES device array that
 * every GPU loading the library holds until exit; every supported layout
 * (range FFT up to 32768 points, upsampling up to 16) fits in it.  Pointers
 * must be device memory; the call is asynchronous on `stream` (NULL: the
 * default stream) except when the radar/layout differs from the previous
 * call's on that device: it then uploads the tables and waits, so such calls
 * must stay outside stream capture.
 * Set-up: the first call on a device (with that device current) looks up the
 * array's address, uploads the tables and loads the kernels; under CUDA's lazy
 * module loading the array and the kernels' code reach the GPU only then.
 * Make that call before the caller's allocator reserves the GPU's memory and
 * before any capture: a call with np = 0 (valid radar and ns, echo and outputs
 * may be NULL) does the set-up and nothing else.  Or run with
 * CUDA_MODULE_LOADING=EAGER.  Calls share the array, which keeps the last
 * call's contents: calls that overlap on the GPU race.
 * SARBP_ERR_UNSUPPORTED: a range FFT beyond 32768 points or upsampling beyond 16. */
#define SARBP_NOALLOC_SCRATCH_BYTES (4u << 20)
sarbp_status sarbp_range_compress_noalloc(const sarbp_radar *radar, const sarbp_complex64 *echo,
                                          int32_t np, int32_t ns, int32_t storage, void *rc_out,
                                          float *rc_scale_out, void *stream);

/* Back-projection of range-compressed data onto the grid (BPA_SAR.m:177-197,
 * with linear interpolation on the upsampled bins; replaces
 * backProjectionKernel / launchBackProjection, BPA_CUDA_kernels.cu:47-77,91-98).
 * apc [np][3]; image [ny][nx].  accumulate != 0 adds into image. */
sarbp_status sarbp_backproject(sarbp_ctx *ctx, const sarbp_radar *radar,
                               const sarbp_rc_view *rc, const double *apc,
                               const sarbp_grid *grid, int32_t mode,
                               sarbp_complex64 *image, int32_t accumulate, void *stream);

/* How sarbp_backproject would run a call with these arguments (no launch of
 * the back-projection itself).  The planner sizes tiles and staging windows from
 * geometry extremes over a 9 x 9 lattice of grid points and every pulse; a
 * squinted or long aperture widens the windows, and windows past the two-CTA
 * shared-memory limit halve the resident CTAs, which this reports so callers can
 * choose sub-aperture sizes.  host_reduction != 0 reduces the extremes on the
 * host (apc must then be host memory), else on the device as sarbp_backproject
 * does; both give identical bits.  No reference counterpart (the reference
 * launches one thread per pixel with no staging, BPA_CUDA_kernels.cu:91-98). */
typedef struct sarbp_bp_plan_info {
    int32_t tile_x, tile_y;  /* pixels per tile (one CTA) */
    int32_t window;          /* staged range bins per (tile, pulse) */
    int32_t series_terms;    /* differential-range series terms (SPLIT / FP16STORE) */
    int32_t segments;        /* pulse segments the launch is split into */
    int32_t ctas_per_sm;     /* resident CTAs per SM of the chosen kernel */
    int32_t pulse_chunk;     /* pulses staged per chunk (16, 8 or 4: two CTAs per SM where it can) */
    int32_t linear_phase;    /* 1: the linear-term phase form (SPLIT / FP16STORE, large tiles) */
    uint64_t smem_bytes;     /* dynamic shared memory per CTA */
    double rmin, rmax;       /* nearest and farthest range, lattice x pulses (m) */
    double cos_x, cos_y;     /* largest |cosine| between line of sight and grid axis x, y */
} sarbp_bp_plan_info;
sarbp_status sarbp_bp_plan(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_rc_view *rc,
                           const double *apc, const sarbp_grid *grid, int32_t mode,
                           int32_t host_reduction, sarbp_bp_plan_info *out);

/* Per-pulse corrections applied inside back-projection: the motion-compensation
 * / autofocus hook on the APC track.  Pulse p's slant range becomes
 * |apc_p - pix| + drange[p] (metres; shifts the range bin and the carrier
 * phase) and its phase gains dphase[p] (radians).  Either pointer may be NULL;
 * host or device memory.  The reference has no counterpart: its APC track is
 * implicit in SARParams (BPA_CUDA.cpp:35-42) and the MATLAB script uses the
 * nominal track (BPA_SAR.m:83,182). */
typedef struct sarbp_pulse_corr {
    const double *drange;  /* [np] or NULL */
    const double *dphase;  /* [np] or NULL */
} sarbp_pulse_corr;

/* sarbp_backproject with per-pulse corrections (corr may be NULL). */
sarbp_status sarbp_backproject_ex(sarbp_ctx *ctx, const sarbp_radar *radar,
                                  const sarbp_rc_view *rc, const double *apc,
                                  const sarbp_grid *grid, int32_t mode,
                                  const sarbp_pulse_corr *corr,
                                  sarbp_complex64 *image, int32_t accumulate, void *stream);

/* Weighted projection, the adjoint of back-projection: for every pulse p,
 * out[p] = sum over pixels of conj(weight[pixel]) * S_p(bin) exp(j phase_p),
 * the pulse's back-projected term with corrections.  With weight = |I|^2 I this
 * is the per-pulse gradient of the image sharpness sum |I|^4:
 * d/d dphase[p] = -4 Im(out[p]).  SPLIT or FP16STORE arithmetic (mode) in the
 * phase form the back-projection takes for the grid, sums over tiles in FP64
 * in a fixed order.  weight [ny][nx] complex64 (host or
 * device); out [np] complex128 as (re, im) pairs (host or device). */
sarbp_status sarbp_project_weighted(sarbp_ctx *ctx, const sarbp_radar *radar,
                                    const sarbp_rc_view *rc, const double *apc,
                                    const sarbp_grid *grid, int32_t mode,
                                    const sarbp_pulse_corr *corr,
                                    const sarbp_complex64 *weight, double *out, void *stream);

/* Autofocus: per-pulse phase errors estimated by maximising the image
 * sharpness sum |I|^4.  Each iteration back-projects with the current phases,
 * forms W = |I|^2 I, projects it onto every pulse (sarbp_project_weighted) and
 * sets dphase[p] -= arg(out[p]), then removes the mean phase.
 * dphase [np] (host) holds the starting phases and receives the estimate;
 * drange [np] (host, may be NULL) is a fixed range correction; image
 * [ny][nx] (host or device, may be NULL) receives the image with the final
 * phases; sharpness [iterations + 1] (host, may be NULL) receives sum |I|^4
 * before each update and for the final image.  Synchronous. */
sarbp_status sarbp_autofocus(sarbp_ctx *ctx, const sarbp_radar *radar,
                             const sarbp_rc_view *rc, const double *apc,
                             const sarbp_grid *grid, int32_t mode, int32_t iterations,
                             const double *drange, double *dphase,
                             sarbp_complex64 *image, double *sharpness, void *stream);

/* The SAR_BP entry point: echo + APC track + radar + grid in, complex image out.
 * Range compression (storage chosen by mode) followed by back-projection
 * (SAR_Processor::processImage + applyBPAlgorithm, BPA_CUDA.cpp:70-90).
 * Each buffer may be host or device memory.  A host echo is uploaded in pulse
 * chunks overlapped with range compression; a pinned host image (cudaHostAlloc,
 * cudaMallocHost) is written by the kernels directly, pageable images are
 * downloaded at the end.  Host buffers make the call synchronous. */
sarbp_status sarbp_image(sarbp_ctx *ctx, const sarbp_radar *radar,
                         const sarbp_complex64 *echo, int32_t np, int32_t ns,
                         const double *apc, const sarbp_grid *grid, int32_t mode,
                         sarbp_complex64 *image, void *stream);

/* ------------------------------------------------------ omega-K imager -- */

/* Parameters of the omega-K (Stolt) imager (WKParams, wk.cc:59-66 and
 * readParams, readfile/read.cc).  kr carries the sign of the reference's
 * parameter file (paras.txt: Kr = -7.2135e11 for the RADARSAT-1 scene), so the
 * reference-function phase is 4 pi r0 / c sqrt((f0 + fr)^2 - c^2 fa^2 / (4 vr^2))
 * + pi fr^2 / kr (task/compression.cc:17-73; mian_wka_sinc.m step 2). */
typedef struct sarbp_wk_params {
    double fr;    /* range sampling rate Fr (Hz) */
    double prf;   /* azimuth sampling rate (Hz) */
    double f0;    /* carrier frequency (Hz) */
    double r0;    /* reference slant range R0 (m) */
    double kr;    /* range FM rate (Hz/s), parameter-file sign */
    double c;     /* propagation speed (m/s) */
    double vr;    /* effective radar velocity (m/s); the reference fixes 7062 */
    double f_nc;  /* Doppler centroid (Hz); the reference fixes -6900 */
    int32_t taps; /* Stolt sinc taps P (the reference uses 6) */
    int32_t reserved;
} sarbp_wk_params;

/* Padded image size of an na x nr echo: na + 2 round(na / 6), nr + 2 round(nr / 3)
 * (preprocess.cc:22-25).  Supported when both sides are powers of two <= 16384
 * or other lengths <= 8192. */
sarbp_status sarbp_wk_padded_size(int32_t na, int32_t nr, int32_t *na_pad, int32_t *nr_pad);

/* The omega-K imager (process_wk, wk.cc:43-343, without its text I/O): zero
 * padding and azimuth down-conversion by exp(-j 2 pi f_nc ta), 2-D FFT,
 * reference-function multiply, Stolt mapping with a taps-point sinc
 * (taps at clip(floor(n - delta + k - taps/2), 0, nr_pad - 1)), 2-D IFFT (1/(na_pad nr_pad)).
 * echo [na][nr], image [na_pad][nr_pad]; host or device pointers. */
sarbp_status sarbp_wk_image(sarbp_ctx *ctx, const sarbp_wk_params *params, const sarbp_complex64 *echo,
                            int32_t na, int32_t nr, sarbp_complex64 *image, void *stream);

/* The omega-K stages one by one, for callers that drive process_wk's steps
 * themselves: sarbp_wk_preprocess, sarbp_dft2d (forward), sarbp_wk_focus,
 * sarbp_dft2d (inverse) give the same bits as sarbp_wk_image.
 * sarbp_wk_preprocess replaces preprocess_wk (task/preprocess.cc:17-167): echo
 * [na][nr] -> out [na_pad][nr_pad] (sarbp_wk_padded_size), zero padding and
 * azimuth down-conversion exp(-j 2 pi f_nc ta).
 * sarbp_wk_focus replaces the reference-function multiply and StoltInterp_sinc
 * (task/compression.cc:17-73, task/stolt.cc:324+) on the 2-D spectrum
 * [na_pad][nr_pad]: out = Stolt-mapped spectrum times exp(j theta); out may
 * equal spectrum. */
sarbp_status sarbp_wk_preprocess(sarbp_ctx *ctx, const sarbp_wk_params *params, const sarbp_complex64 *echo,
                                 int32_t na, int32_t nr, sarbp_complex64 *out, void *stream);
sarbp_status sarbp_wk_focus(sarbp_ctx *ctx, const sarbp_wk_params *params, const sarbp_complex64 *spectrum,
                            int32_t na_pad, int32_t nr_pad, sarbp_complex64 *out, void *stream);

/* Batched 1-D DFT along the rows of data [rows][n], in place: forward
 * (unnormalised) or inverse (times 1/n), any supported n (see above). */
sarbp_status sarbp_dft(sarbp_ctx *ctx, sarbp_complex64 *data, int32_t rows, int32_t n, int32_t inverse,
                       void *stream);

/* 2-D DFT of data [na][nr] (row-major), in place: along the rows (length nr)
 * then down the columns (length na); the inverse scales by 1/nr and 1/na.
 * Replaces perform2DFFT / perform2DIFFT (code/SAR_WK/wk_v5.2.3/task/fft.cc:18,200),
 * which run the same two passes through CNNL FFT plans and a transpose.
 * Power-of-two column lengths 512..4096 are transformed down the columns
 * directly, others through two transposes (scratch in the context). */
sarbp_status sarbp_dft2d(sarbp_ctx *ctx, sarbp_complex64 *data, int32_t na, int32_t nr, int32_t inverse,
                         void *stream);

/* ------------------------------------------------------ CEOS raw ingest -- */

/* Layout of a RADARSAT-1 CEOS raw-data file as the reference's reader sees it
 * (code/data_process/CEOS/read_CEOS_raw.m:13-16,67-80; its values in
 * parentheses). */
typedef struct sarbp_ceos_layout {
    int32_t file_header;     /* bytes before the first block (16252) */
    int32_t header;          /* record header bytes per line (192) */
    int32_t aux;             /* auxiliary bytes per line (50) */
    int32_t cells;           /* range cells per line, 2 bytes (I, Q) each (9288) */
    int32_t replica;         /* replica bytes per block (2880) */
    int32_t replica_line;    /* 1-based line of a block whose record holds the replica, after its aux bytes (7) */
    int32_t lines_per_block; /* (8) */
    int32_t agc_byte;        /* 1-based aux byte whose low 6 bits are the AGC code (50) */
    float gain;              /* gain factor applied with the AGC attenuation (1.5) */
    int32_t reserved;        /* must be 0 */
} sarbp_ceos_layout;

/* Decodes range lines [first_line, first_line + nlines) (0-based in the file)
 * and cells [first_cell, first_cell + ncells) of a CEOS raw-data file into
 * echo [nlines][ncells] complex64: sample byte d -> 2 (d' - 16 [d' > 7]) + 1
 * with d' = d & 15 (read_CEOS_raw.m:135-141), times gain 10^(AGC_dB / 20) per
 * line when apply_agc != 0 (load_DATA_block.m:58-69); agc_db [nlines] (may be
 * NULL) receives code - 24 [code > 31] (extract_AGC.m:45-58).  raw holds the
 * file from byte 0 (host or device, raw_bytes long); from host memory only
 * the blocks holding the requested lines are copied to the device. */
sarbp_status sarbp_ceos_decode(sarbp_ctx *ctx, const uint8_t *raw, uint64_t raw_bytes,
                               const sarbp_ceos_layout *layout, int32_t first_line, int32_t nlines,
                               int32_t first_cell, int32_t ncells, int32_t apply_agc,
                               sarbp_complex64 *echo, int16_t *agc_db, void *stream);

/* ------------------------------------------------------ echo synthesiser -- */

/* Point-target echo with FP64 phase (BPA_SAR.m:80-89; replaces
 * generateEchoKernel, BPA_CUDA_kernels.cu:3-45), plus counter-based complex
 * Gaussian noise at snr_db below the mean noiseless power (no noise when
 * snr_db is NaN).  echo_out [np][ns]. */
sarbp_status sarbp_synthesize_echo(sarbp_ctx *ctx, const sarbp_radar *radar,
                                   const double *apc, int32_t np, int32_t ns,
                                   const sarbp_target *targets, int32_t nt,
                                   double snr_db, uint64_t seed,
                                   sarbp_complex64 *echo_out, void *stream);

/* ------------------------------------------------------------- serving -- */

/* A persistent imaging service on one device.  A worker thread admits
 * submitted jobs while the device-memory budget and the job slots allow,
 * keeps each admitted job's echo, range-compressed data and partial image
 * resident, and advances all admitted jobs together: every step back-projects
 * the next `pulses_per_step` pulses of each job (accumulating into its image),
 * with the step's launches for all jobs captured in one CUDA graph (one branch
 * per job, so their work overlaps on the device).  Jobs that arrive while
 * others run join at the next step.  Each job's result is the same whatever
 * else runs with it (its launches and their order do not depend on the mix).
 * Submit, poll, wait and cancel may be called from any host thread. */
typedef struct sarbp_server sarbp_server;

typedef struct sarbp_server_config {
    int32_t device;
    int32_t max_jobs;           /* jobs resident at once (slots), 1..64 */
    uint64_t hbm_budget_bytes;  /* device memory the server may hold for jobs */
    int32_t pulses_per_step;    /* pulses per job per step (multiple of 16); 0: 512 */
    int32_t use_graphs;         /* 1: capture each step's launches in a CUDA graph; 0: plain streams */
    uint64_t step_updates;      /* 0: every job advances pulses_per_step pulses per step.  Else each
                                   job advances about step_updates / (nx ny) pulses per step (a
                                   multiple of 16, at least 16, at most all of them), so a step
                                   costs every job about the same and small jobs finish in few
                                   steps instead of waiting out a large neighbour's cadence */
} sarbp_server_config;

typedef struct sarbp_job {
    sarbp_radar radar;
    sarbp_grid grid;
    const sarbp_complex64 *echo; /* host [np][ns]; must stay valid until the job ends (pinned: async upload) */
    const double *apc;           /* host [np][3] */
    sarbp_complex64 *image;      /* host [ny][nx] result */
    int32_t np, ns;
    int32_t mode;                /* SARBP_MODE_SPLIT or SARBP_MODE_FP16STORE */
    int32_t reserved;
} sarbp_job;

typedef struct sarbp_job_stats {
    int32_t status;          /* the job's sarbp_status */
    int32_t steps;           /* back-projection steps the job took */
    double queued_ms;        /* entry into sarbp_server_submit -> admitted */
    double latency_ms;       /* entry into sarbp_server_submit (validation and planning included) -> image in host memory */
    double updates;          /* nx * ny * np */
    uint64_t device_bytes;   /* admission footprint */
} sarbp_job_stats;

typedef struct sarbp_server_stats {
    uint64_t submitted, completed, failed, rejected, cancelled;
    uint64_t steps, graph_launches;
    double updates;          /* pixel*pulse updates of completed jobs */
    double busy_s;           /* wall time with at least one job admitted */
    uint64_t bytes_in_use, peak_bytes;
    int32_t active, queued, peak_active, reserved;
    double step_device_s;    /* device time of the back-projection steps (CUDA events around each step) */
    double admit_device_s;   /* device time of admissions: echo and APC upload, range compression */
} sarbp_server_stats;

sarbp_status sarbp_server_create(sarbp_server **out, const sarbp_server_config *cfg);
/* Finishes admitted jobs, cancels queued ones, stops the worker. */
sarbp_status sarbp_server_destroy(sarbp_server *srv);
/* Validates and plans the job, queues it.  SARBP_ERR_BUDGET if the job alone
 * exceeds the budget. */
sarbp_status sarbp_server_submit(sarbp_server *srv, const sarbp_job *job, uint64_t *ticket);
/* SARBP_OK when done, SARBP_ERR_NOT_READY while queued or running, else the job's error. */
sarbp_status sarbp_server_poll(sarbp_server *srv, uint64_t ticket);
/* Waits up to timeout_ms (< 0: forever); SARBP_ERR_TIMEOUT if still running.
 * On completion fills stats (may be NULL), returns the job's status and
 * releases the ticket. */
sarbp_status sarbp_server_wait(sarbp_server *srv, uint64_t ticket, int32_t timeout_ms, sarbp_job_stats *stats);
/* Cancels a queued job (SARBP_ERR_NOT_READY if it was already admitted). */
sarbp_status sarbp_server_cancel(sarbp_server *srv, uint64_t ticket);
sarbp_status sarbp_server_get_stats(sarbp_server *srv, sarbp_server_stats *out);
/* Test switch of a server, not for production use (no reference counterpart):
 * SARBP_SERVER_DEBUG_FAIL_ADMIT_TICKET = t (> 0) refuses the device allocation
 * of ticket t's admission on the host, as a full device would, so that job
 * fails with SARBP_ERR_OUT_OF_MEMORY and the others proceed; 0 clears it. */
enum { SARBP_SERVER_DEBUG_FAIL_ADMIT_TICKET = 1 };
sarbp_status sarbp_server_debug_set(sarbp_server *srv, int32_t key, int64_t value);

/* ------------------------------------------------- reference-layout shim -- */

/* Byte-for-byte layout of the reference's SARParams (BPA_CUDA.h:28-50):
 * 12 floats then 3 ints, 60 bytes. */
typedef struct sarbp_ref_params {
    float c, fc, lambda, Kr, Tr, Br, Fr, vr, H, La, Rg0, Az0;
    int32_t Nfast, Mslow, Ntarget;
} sarbp_ref_params;

/* launchBackProjection (BPA_CUDA_kernels.cu:91-98) with the intended
 * BPA_SAR.m semantics on the reference's data model:
 *   Srnm  [Mslow][Nfast] raw echo, device memory, fast time tr_i = i/Fr
 *         (BPA_CUDA.cpp:44-48), uncentred chirp Kr over Tr;
 *   APC_m = (vr*ta_m, 0, H), ta = linspace(-La/(2vr), La/(2vr), Mslow)
 *         (BPA_CUDA.cpp:35-42);
 *   Image [Na][Nr] device memory, pixel (i, j) on the ground at
 *         (Az0 + (i - Na/2) m, Rg0 + (j - Nr/2) m, 0) (the 1 m pixel of
 *         BPA_CUDA_kernels.cu:56-57, centred on the scene centre);
 *   range compression + 8x upsampling + SPLIT back-projection.
 * Synchronous (the reference synchronises, :97-98).  Uses a process-wide
 * context on the current device. */
sarbp_status sarbp_launch_back_projection(sarbp_complex64 *Srnm, sarbp_complex64 *Image,
                                          const sarbp_ref_params *params, int32_t Na, int32_t Nr);

/* launchGenerateEcho (BPA_CUDA_kernels.cu:79-89): same formula and gates as
 * generateEchoKernel (:18-42), evaluated in FP64.  Ptarget [Ntarget][3] =
 * (Az, Rg, sigma), ta [Mslow], tr [Nfast], Srnm [Mslow][Nfast]: device memory. */
sarbp_status sarbp_launch_generate_echo(sarbp_complex64 *Srnm, const float *Ptarget,
                                        const float *ta, const float *tr,
                                        const sarbp_ref_params *params,
                                        int32_t Mslow, int32_t Nfast);

/* ------------------------------------------------------------ measurement -- */

/* Issue-rate microbenchmarks on the context's device: FP32 FMA lanes/s and
 * MUFU (sin/cos) lanes/s over all its SMs, and the SM count.  The
 * back-projection roofline is built from these (the kernel is FP32/MUFU issue
 * bound, not HBM or tensor bound). */
sarbp_status sarbp_probe_issue_rates(sarbp_ctx *ctx, double *fp32_lanes_per_s,
                                     double *mufu_lanes_per_s, int32_t *sm_count);

/* Time of the last kernel launches issued by the context, measured with CUDA
 * events on the launching stream: range compression and back-projection, ms.
 * Valid after a synchronous call or sarbp_synchronize. */
sarbp_status sarbp_last_timings(sarbp_ctx *ctx, float *rc_ms, float *bp_ms);

/* Number of this library's kernels launched through the context so far. */
int64_t sarbp_kernel_launches(const sarbp_ctx *ctx);

/* ---------------------------------------------------- tests and tuning -- */

/* Switches of one context for tests and tuning sweeps, not for production
 * use; no reference counterpart.  A value of 0 (for the wait fault, -1)
 * restores the default.
 *   SARBP_DEBUG_BP_CHUNK        pulses staged per chunk (16, 8 or 4) where it fits;
 *                               images do not depend on it
 *   SARBP_DEBUG_BP_SEGMENTS     pulse segments per launch (1..64); images agree to
 *                               FP32 rounding
 *   SARBP_DEBUG_BP_CHECKED      1: back-projection kernels that clamp every
 *                               interpolation index and report any clamp
 *                               (SARBP_ERR_DEVICE_CHECK)
 *   SARBP_DEBUG_WAIT_LIMIT_NS   limit of the kernels' bounded staging waits (default 2 s)
 *   SARBP_DEBUG_WAIT_FAULT_CHUNK  >= 0: that pulse chunk's staging barrier in every
 *                               CTA expects 16 bytes more than its copies bring, so
 *                               the wait runs out (SARBP_ERR_TIMEOUT); the kernel
 *                               then lets every copy in flight land before it exits
 *   SARBP_DEBUG_DEVICE_FLAGS    (get only) device check bits of the last call
 *                               that reported any: 1 wait ran out, 2 index clamped,
 *                               8 staging window, 16 a copy did not land in the drain
 *   SARBP_DEBUG_BP_LINEAR_PHASE  SPLIT / FP16STORE phase form of back-projection
 *                               and weighted projection: 1 linear-term form, -1
 *                               series form, 0 the planner's choice (linear-term
 *                               for tiles whose half-diagonal exceeds 12 m) */
enum {
    SARBP_DEBUG_BP_CHUNK = 1,
    SARBP_DEBUG_BP_SEGMENTS = 2,
    SARBP_DEBUG_BP_CHECKED = 3,
    SARBP_DEBUG_WAIT_LIMIT_NS = 4,
    SARBP_DEBUG_WAIT_FAULT_CHUNK = 5,
    SARBP_DEBUG_DEVICE_FLAGS = 6,
    SARBP_DEBUG_BP_LINEAR_PHASE = 7
};
sarbp_status sarbp_debug_set(sarbp_ctx *ctx, int32_t key, int64_t value);
sarbp_status sarbp_debug_get(sarbp_ctx *ctx, int32_t key, int64_t *value);

#ifdef __cplusplus
}
#endif
#endif /* SARBP_H */
