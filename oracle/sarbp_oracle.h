/*
 * sarbp_oracle.h -- FP64 CPU oracle for SAR back-projection imaging.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path and
 * the timed CPU baseline ("port" kind).  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference leg may load it.  The product
 * library (libsarbp) never links or calls it.
 *
 * It restates, in plain C99 + OpenMP and double precision throughout, the
 * processing chain of the reference's MATLAB specification
 *   code/SAR_BP/matlab/BPA_SAR.m
 *     :80-89    echo simulation  (phase pi*Kr*tk^2 - 4*pi*R/lambda, rect gate)
 *     :93-100   matched-filter range compression  ifft(fft(s).*conj(fft(h)))
 *     :106-111  8x range upsampling by mid-spectrum zero insertion
 *     :177-197  back-projection: slant range -> bin -> sample -> *exp(+j4piR/lambda) -> sum
 * and of the reference CUDA echo generator
 *   code/SAR_BP/CUDA/BPA_CUDA_kernels.cu:3-45 (same echo formula and gates).
 *
 * Every primitive is parameterised so that two profiles can be expressed:
 *   - the MATLAB profile (uncentred chirp, strict gates, circular compression of
 *     length Nfast, nearest-bin lookup with MATLAB's 1-based index, 1/(L*N)
 *     amplitude), used to pin this oracle against an independent vectorised
 *     transcription of BPA_SAR.m (tests/golden/);
 *   - the product profile (chirp centred at baseband, linear convolution with
 *     N_fft = nextpow2(Ns+Nc-1), lag shift Nc/2, linear interpolation on the
 *     8x grid, amplitude preserved), which the CUDA path must reproduce.
 *
 * Parity status: the reference ships no golden vectors for back-projection and
 * its BP program cannot serve as an oracle (it does not compile as shipped and
 * its echo is all-zero by construction).  The FFT stage is pinned to the
 * reference's known-answer case (code/fft_simple/fft_kt_sample.cc:5-29); the
 * back-projection stage is parity unpinned by the reference and is anchored on
 * the MATLAB-profile cross-check plus analytic known answers.
 *
 * Complex arrays are interleaved (re, im) doubles, row-major.
 */
#ifndef SARBP_ORACLE_H
#define SARBP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_INTERP_LINEAR = 0,         /* product profile: linear on the upsampled grid */
    ORC_INTERP_NEAREST_MATLAB = 1  /* BPA_SAR.m:184,188: SAR2(m, round(x)) with 1-based index */
};

int orc_version(void);
void orc_set_threads(int n);
int orc_get_threads(void);

/* Unnormalised radix-2 DFT, in place.  sign = -1: X[k] = sum x[n] e^{-j2pi kn/N}
 * (MATLAB fft); sign = +1: the conjugate kernel without 1/N.  n must be a power
 * of two.  Returns 0 on success, -1 on a bad size. */
int orc_fft(double *x, int n, int sign);

/* Matched-filter reference chirp sampled at u_i = i*dt, i in [0, n):
 *   h[i] = exp(j*pi*kr*(u_i - tc)^2) * gate(u_i),
 *   gate = (0 < u < tp) if strict_gate else (0 <= u < tp).
 * MATLAB profile: tc = 0, strict (BPA_SAR.m:93-94).  Product: tc = tp/2. */
void orc_chirp(double *h, int n, double dt, double kr, double tp, double tc, int strict_gate);

/* Range compression + upsampling of np rows of ns samples.
 *   Z[k]  = FFT_nfft(echo row, zero padded)[k] * conj(FFT_nfft(h)[k]) * e^{-j2pi k shift/nfft}
 *   out   = norm * IFFTu_{L*nfft}(Z with (L-1)*nfft zeros inserted after bin
 *           floor((nfft+1)/2)-1), first nout samples          (BPA_SAR.m:106-111)
 *   sar1  = (1/nfft) * IFFTu_nfft(Z)  (optional, NULL to skip) (BPA_SAR.m:100)
 * ns <= nfft, nh <= nfft, nout <= L*nfft.  Returns 0 or -1 on bad sizes. */
int orc_range_compress(const double *echo, int np, int ns, const double *h, int nh,
                       int nfft, int shift, int L, double norm, int nout,
                       double *out, double *sar1);

/* Point-target echo (BPA_SAR.m:80-89, BPA_CUDA_kernels.cu:18-42):
 *   s[p][n] = sum_k sigma_k * gate(u) * exp(j*(pi*kr*(u - tc)^2 - 2*pi*fc*tau_pk)),
 *   u = t_rec0 + n*dt - tau_pk,  tau_pk = 2*|apc_p - tgt_k|/c.
 * tgt is [nt][4] = (x, y, z, sigma).  beam_hw > 0 keeps a target only while
 * |apc_p.x - tgt_k.x| < beam_hw (the azimuth gate |Azk| < La/2 of :88). */
void orc_echo(const double *apc, int np, const double *tgt, int nt,
              double t_rec0, double dt, int ns, double kr, double tp, double tc,
              int strict_gate, double beam_hw, double fc, double c, double *echo);

/* Counter-based complex Gaussian noise, identical stream to the product's echo
 * synthesiser: element i gets sigma/sqrt(2) * (g0 + j g1), Box-Muller on two
 * splitmix64-derived uniforms of (seed, i). */
void orc_add_noise(double *x, int64_t count, double sigma, uint64_t seed);
void orc_noise_sample(uint64_t seed, int64_t i, double *g0, double *g1);
double orc_mean_power(const double *x, int64_t count);

/* Back-projection onto the pixel grid pix(x, y) = origin + x*ux + y*uy for
 * x in [x0, x0+w), y in [y0, y0+h).  img is [h][w].
 *   R = |apc_p - pix|,  b = (2R/c - t0) * binrate,
 *   img += S_p(b) * exp(+j*2*pi*fc*2R/c)            (BPA_SAR.m:182-194)
 * LINEAR: S_p(b) = (1-f) s[i0] + f s[i0+1], i0 = floor(b), samples outside
 * [0, nbins) read as zero.  NEAREST_MATLAB: s[round_half_away(b) - 1]. */
void orc_backproject(const double *rc, int np, int nbins, const double *apc,
                     const double *origin, const double *ux, const double *uy,
                     int x0, int y0, int w, int h,
                     double fc, double c, double t0, double binrate, int interp,
                     double *img);

/* Same as orc_backproject with complex64 range-compressed input (the GPU
 * range compressor's output), so the BP stage can be checked on its own. */
void orc_backproject_c64(const float *rc, int np, int nbins, const double *apc,
                         const double *origin, const double *ux, const double *uy,
                         int x0, int y0, int w, int h,
                         double fc, double c, double t0, double binrate, int interp,
                         double *img);

/* Back-projection with per-pulse corrections (motion compensation / autofocus
 * output; either array may be NULL): R_p = |apc_p - pix| + drange[p] for the bin
 * and the carrier phase, and dphase[p] added to the phase. */
void orc_backproject_corr(const double *rc, int np, int nbins, const double *apc,
                          const double *origin, const double *ux, const double *uy,
                          int x0, int y0, int w, int h,
                          double fc, double c, double t0, double binrate, int interp,
                          const double *drange, const double *dphase, double *img);

/* Adjoint of orc_backproject_corr over the region: out[p] (complex) =
 * sum over pixels of conj(weight) * S_p(b) * exp(j phase_p).  With
 * weight = |I|^2 I this is the per-pulse gradient of the sharpness sum |I|^4:
 * d/d dphase[p] = -4 Im(out[p]). */
void orc_project_weighted(const double *rc, int np, int nbins, const double *apc,
                          const double *origin, const double *ux, const double *uy,
                          int x0, int y0, int w, int h,
                          double fc, double c, double t0, double binrate, int interp,
                          const double *drange, const double *dphase, const double *weight, double *out);

#ifdef __cplusplus
}
#endif
#endif
