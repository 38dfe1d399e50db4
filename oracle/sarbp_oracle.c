/*
 * sarbp_oracle.c -- FP64 CPU oracle (test infrastructure; see sarbp_oracle.h).
 *
 * Restates code/SAR_BP/matlab/BPA_SAR.m (:80-111, :177-197) and the echo
 * formula of code/SAR_BP/CUDA/BPA_CUDA_kernels.cu:3-45 in double precision.
 * Written for clarity and determinism, parallelised over rows with OpenMP.
 */
#define _GNU_SOURCE
#include "sarbp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846
#define ORC_TWO_PI 6.28318530717958647692

static int g_threads = 0;

int orc_version(void) { return 4; }

void orc_set_threads(int n) { g_threads = n; }

int orc_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

/* ------------------------------------------------------------------ FFT -- */

/* tw[k] = exp(-j*2*pi*k/n), k in [0, n/2). */
static double *make_twiddles(int n)
{
    double *tw = (double *)malloc(sizeof(double) * (size_t)(n > 1 ? n : 2));
    for (int k = 0; k < n / 2; ++k) {
        double a = -ORC_TWO_PI * (double)k / (double)n;
        tw[2 * k] = cos(a);
        tw[2 * k + 1] = sin(a);
    }
    return tw;
}

/* Iterative radix-2 decimation-in-time transform with a shared twiddle table. */
static void fft_core(double *x, int n, int sign, const double *tw)
{
    /* bit-reversal permutation */
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double tr = x[2 * i], ti = x[2 * i + 1];
            x[2 * i] = x[2 * j];
            x[2 * i + 1] = x[2 * j + 1];
            x[2 * j] = tr;
            x[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        int step = n / len;
        for (int i = 0; i < n; i += len) {
            for (int k = 0; k < half; ++k) {
                double wr = tw[2 * k * step];
                double wi = sign < 0 ? tw[2 * k * step + 1] : -tw[2 * k * step + 1];
                double *a = x + 2 * (i + k);
                double *b = x + 2 * (i + k + half);
                double br = b[0] * wr - b[1] * wi;
                double bi = b[0] * wi + b[1] * wr;
                b[0] = a[0] - br;
                b[1] = a[1] - bi;
                a[0] += br;
                a[1] += bi;
            }
        }
    }
}

int orc_fft(double *x, int n, int sign)
{
    if (!is_pow2(n)) return -1;
    if (n == 1) return 0;
    double *tw = make_twiddles(n);
    fft_core(x, n, sign, tw);
    free(tw);
    return 0;
}

/* ---------------------------------------------------------------- chirp -- */

void orc_chirp(double *h, int n, double dt, double kr, double tp, double tc, int strict_gate)
{
    for (int i = 0; i < n; ++i) {
        double u = (double)i * dt;
        int on = strict_gate ? (u > 0.0 && u < tp) : (u >= 0.0 && u < tp);
        if (on) {
            double ph = ORC_PI * kr * (u - tc) * (u - tc);
            h[2 * i] = cos(ph);
            h[2 * i + 1] = sin(ph);
        } else {
            h[2 * i] = 0.0;
            h[2 * i + 1] = 0.0;
        }
    }
}

/* ---------------------------------------------------- range compression -- */

int orc_range_compress(const double *echo, int np, int ns, const double *h, int nh,
                       int nfft, int shift, int L, double norm, int nout,
                       double *out, double *sar1)
{
    if (!is_pow2(nfft) || !is_pow2(L) || ns > nfft || nh > nfft || nout > L * nfft || np < 0)
        return -1;
    const int nbig = L * nfft;
    double *tw_small = make_twiddles(nfft);
    double *tw_big = make_twiddles(nbig);

    /* conj(FFT(h)) times the lag-shift ramp e^{-j2pi k shift / nfft} */
    double *filt = (double *)calloc((size_t)2 * nfft, sizeof(double));
    memcpy(filt, h, sizeof(double) * 2 * (size_t)nh);
    fft_core(filt, nfft, -1, tw_small);
    for (int k = 0; k < nfft; ++k) {
        long long m = ((long long)k * (long long)shift) % nfft;
        if (m < 0) m += nfft;
        double a = -ORC_TWO_PI * (double)m / (double)nfft;
        double sr = cos(a), si = sin(a);
        double hr = filt[2 * k], hi = -filt[2 * k + 1]; /* conj */
        filt[2 * k] = hr * sr - hi * si;
        filt[2 * k + 1] = hr * si + hi * sr;
    }
    const int split = (nfft + 1) / 2; /* MATLAB floor((N+1)/2): bins [0, split) stay low */

#pragma omp parallel num_threads(orc_get_threads())
    {
        double *z = (double *)malloc(sizeof(double) * 2 * (size_t)nfft);
        double *big = (double *)malloc(sizeof(double) * 2 * (size_t)nbig);
#pragma omp for schedule(static)
        for (int p = 0; p < np; ++p) {
            memset(z, 0, sizeof(double) * 2 * (size_t)nfft);
            memcpy(z, echo + (size_t)2 * ns * p, sizeof(double) * 2 * (size_t)ns);
            fft_core(z, nfft, -1, tw_small);
            for (int k = 0; k < nfft; ++k) {
                double ar = z[2 * k], ai = z[2 * k + 1];
                double br = filt[2 * k], bi = filt[2 * k + 1];
                z[2 * k] = ar * br - ai * bi;
                z[2 * k + 1] = ar * bi + ai * br;
            }
            memset(big, 0, sizeof(double) * 2 * (size_t)nbig);
            memcpy(big, z, sizeof(double) * 2 * (size_t)split);
            memcpy(big + 2 * (size_t)(nbig - (nfft - split)), z + 2 * (size_t)split,
                   sizeof(double) * 2 * (size_t)(nfft - split));
            if (sar1) {
                fft_core(z, nfft, +1, tw_small);
                double *row = sar1 + (size_t)2 * nfft * p;
                for (int i = 0; i < 2 * nfft; ++i) row[i] = z[i] / (double)nfft;
            }
            fft_core(big, nbig, +1, tw_big);
            double *row = out + (size_t)2 * nout * p;
            for (int i = 0; i < 2 * nout; ++i) row[i] = big[i] * norm;
        }
        free(z);
        free(big);
    }
    free(filt);
    free(tw_small);
    free(tw_big);
    return 0;
}

/* ----------------------------------------------------------------- echo -- */

void orc_echo(const double *apc, int np, const double *tgt, int nt,
              double t_rec0, double dt, int ns, double kr, double tp, double tc,
              int strict_gate, double beam_hw, double fc, double c, double *echo)
{
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int p = 0; p < np; ++p) {
        double *row = echo + (size_t)2 * ns * p;
        memset(row, 0, sizeof(double) * 2 * (size_t)ns);
        const double *a = apc + 3 * (size_t)p;
        for (int k = 0; k < nt; ++k) {
            const double *t = tgt + 4 * (size_t)k;
            if (beam_hw > 0.0 && !(fabs(a[0] - t[0]) < beam_hw)) continue;
            double dx = a[0] - t[0], dy = a[1] - t[1], dz = a[2] - t[2];
            double r = sqrt(dx * dx + dy * dy + dz * dz);
            double tau = 2.0 * r / c;
            double cyc = fc * tau;
            double carrier = -ORC_TWO_PI * (cyc - floor(cyc));
            /* samples whose gate can be open: u = t_rec0 + n dt - tau in [0, tp] */
            long long n_lo = (long long)floor((tau - t_rec0) / dt) - 1;
            long long n_hi = (long long)ceil((tau + tp - t_rec0) / dt) + 1;
            if (n_lo < 0) n_lo = 0;
            if (n_hi > ns - 1) n_hi = ns - 1;
            for (long long n = n_lo; n <= n_hi; ++n) {
                double u = t_rec0 + (double)n * dt - tau;
                int on = strict_gate ? (u > 0.0 && u < tp) : (u >= 0.0 && u < tp);
                if (!on) continue;
                double ph = ORC_PI * kr * (u - tc) * (u - tc) + carrier;
                double s, co;
                sincos(ph, &s, &co);
                row[2 * n] += t[3] * co;
                row[2 * n + 1] += t[3] * s;
            }
        }
    }
}

/* ---------------------------------------------------------------- noise -- */

static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

void orc_noise_sample(uint64_t seed, int64_t i, double *g0, double *g1)
{
    uint64_t h1 = mix64(seed + 0x632BE59BD9B4E019ULL * (uint64_t)(i + 1));
    uint64_t h2 = mix64(h1 ^ 0xD1B54A32D192ED03ULL);
    double u1 = ((double)(h1 >> 11) + 1.0) * (1.0 / 9007199254740992.0); /* (0, 1] */
    double u2 = (double)(h2 >> 11) * (1.0 / 9007199254740992.0);         /* [0, 1) */
    double rad = sqrt(-2.0 * log(u1));
    double s, co;
    sincos(ORC_TWO_PI * u2, &s, &co);
    *g0 = rad * co;
    *g1 = rad * s;
}

void orc_add_noise(double *x, int64_t count, double sigma, uint64_t seed)
{
    const double amp = sigma / sqrt(2.0);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t i = 0; i < count; ++i) {
        double g0, g1;
        orc_noise_sample(seed, i, &g0, &g1);
        x[2 * i] += amp * g0;
        x[2 * i + 1] += amp * g1;
    }
}

double orc_mean_power(const double *x, int64_t count)
{
    double acc = 0.0;
    for (int64_t i = 0; i < count; ++i) acc += x[2 * i] * x[2 * i] + x[2 * i + 1] * x[2 * i + 1];
    return count > 0 ? acc / (double)count : 0.0;
}

/* ------------------------------------------------------- back-projection -- */

static long long round_half_away(double v) { return (long long)(v >= 0.0 ? floor(v + 0.5) : ceil(v - 0.5)); }

/* Sample of pulse p at pixel (px, py, pz) times its phase term, with the
 * optional per-pulse corrections: slant range R + drange[p], phase
 * 2 pi frac(2 fc R / c) + dphase[p].  Linear interpolation (zero outside the
 * row) or the script's nearest bin (BPA_SAR.m:184-188, 1-based round). */
#define ORC_TERM(LOAD_RE, LOAD_IM, p, px, py, pz, out_r, out_i)                              \
    do {                                                                                     \
        const double *a_ = apc + 3 * (size_t)(p);                                            \
        double dx_ = a_[0] - (px), dy_ = a_[1] - (py), dz_ = a_[2] - (pz);                   \
        double r_ = sqrt(dx_ * dx_ + dy_ * dy_ + dz_ * dz_);                                 \
        if (drange) r_ += drange[p];                                                         \
        double b_ = (2.0 * r_ / c - t0) * binrate;                                           \
        double sr_ = 0.0, si_ = 0.0;                                                         \
        size_t rowoff_ = (size_t)nbins * (size_t)(p);                                        \
        if (interp == ORC_INTERP_LINEAR) {                                                   \
            double fl_ = floor(b_);                                                          \
            double f_ = b_ - fl_;                                                            \
            if (fl_ >= -1.0 && fl_ <= (double)nbins - 1.0) {                                 \
                long long i0_ = (long long)fl_;                                              \
                if (i0_ >= 0) {                                                              \
                    sr_ += (1.0 - f_) * LOAD_RE(rowoff_ + (size_t)i0_);                      \
                    si_ += (1.0 - f_) * LOAD_IM(rowoff_ + (size_t)i0_);                      \
                }                                                                            \
                if (i0_ + 1 <= nbins - 1) {                                                  \
                    sr_ += f_ * LOAD_RE(rowoff_ + (size_t)(i0_ + 1));                        \
                    si_ += f_ * LOAD_IM(rowoff_ + (size_t)(i0_ + 1));                        \
                }                                                                            \
            }                                                                                \
        } else {                                                                             \
            long long idx_ = round_half_away(b_) - 1;                                        \
            if (idx_ >= 0 && idx_ < nbins) {                                                 \
                sr_ = LOAD_RE(rowoff_ + (size_t)idx_);                                       \
                si_ = LOAD_IM(rowoff_ + (size_t)idx_);                                       \
            }                                                                                \
        }                                                                                    \
        double cyc_ = 2.0 * fc * r_ / c;                                                     \
        double ph_ = ORC_TWO_PI * (cyc_ - floor(cyc_)) + (dphase ? dphase[p] : 0.0);         \
        double s_, co_;                                                                      \
        sincos(ph_, &s_, &co_);                                                              \
        (out_r) = sr_ * co_ - si_ * s_;                                                      \
        (out_i) = sr_ * s_ + si_ * co_;                                                      \
    } while (0)

#define ORC_BP_BODY(LOAD_RE, LOAD_IM)                                                        \
    _Pragma("omp parallel for collapse(2) schedule(static) num_threads(orc_get_threads())") \
    for (int yy = 0; yy < h; ++yy) {                                                         \
        for (int xx = 0; xx < w; ++xx) {                                                     \
            double px = origin[0] + (double)(x0 + xx) * ux[0] + (double)(y0 + yy) * uy[0];   \
            double py = origin[1] + (double)(x0 + xx) * ux[1] + (double)(y0 + yy) * uy[1];   \
            double pz = origin[2] + (double)(x0 + xx) * ux[2] + (double)(y0 + yy) * uy[2];   \
            double acc_r = 0.0, acc_i = 0.0;                                                 \
            for (int p = 0; p < np; ++p) {                                                   \
                double tr, ti;                                                               \
                ORC_TERM(LOAD_RE, LOAD_IM, p, px, py, pz, tr, ti);                           \
                acc_r += tr;                                                                 \
                acc_i += ti;                                                                 \
            }                                                                                \
            img[2 * ((size_t)yy * w + xx)] = acc_r;                                          \
            img[2 * ((size_t)yy * w + xx) + 1] = acc_i;                                      \
        }                                                                                    \
    }

#define LD_D_RE(i) rc[2 * (i)]
#define LD_D_IM(i) rc[2 * (i) + 1]
#define LD_F_RE(i) ((double)rc[2 * (i)])
#define LD_F_IM(i) ((double)rc[2 * (i) + 1])

void orc_backproject(const double *rc, int np, int nbins, const double *apc,
                     const double *origin, const double *ux, const double *uy,
                     int x0, int y0, int w, int h,
                     double fc, double c, double t0, double binrate, int interp,
                     double *img)
{
    const double *drange = NULL, *dphase = NULL;
    ORC_BP_BODY(LD_D_RE, LD_D_IM)
}

void orc_backproject_c64(const float *rc, int np, int nbins, const double *apc,
                         const double *origin, const double *ux, const double *uy,
                         int x0, int y0, int w, int h,
                         double fc, double c, double t0, double binrate, int interp,
                         double *img)
{
    const double *drange = NULL, *dphase = NULL;
    ORC_BP_BODY(LD_F_RE, LD_F_IM)
}

/* Back-projection with per-pulse corrections (either array may be NULL). */
void orc_backproject_corr(const double *rc, int np, int nbins, const double *apc,
                          const double *origin, const double *ux, const double *uy,
                          int x0, int y0, int w, int h,
                          double fc, double c, double t0, double binrate, int interp,
                          const double *drange, const double *dphase, double *img)
{
    ORC_BP_BODY(LD_D_RE, LD_D_IM)
}

/* Weighted projection, the adjoint of back-projection over the region:
 * out[p] = sum_{pixels} conj(weight[pixel]) * term_p(pixel), term_p the pulse's
 * interpolated sample times its phase term (with corrections).  For the image
 * I = sum_p term_p exp(j phi_p) and weight W = |I|^2 I, d/dphi_p sum |I|^4 =
 * -4 Im(out[p]).  weight: [h][w] complex, out: [np] complex. */
void orc_project_weighted(const double *rc, int np, int nbins, const double *apc,
                          const double *origin, const double *ux, const double *uy,
                          int x0, int y0, int w, int h,
                          double fc, double c, double t0, double binrate, int interp,
                          const double *drange, const double *dphase, const double *weight, double *out)
{
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int p = 0; p < np; ++p) {
        double cr = 0.0, ci = 0.0;
        for (int yy = 0; yy < h; ++yy) {
            for (int xx = 0; xx < w; ++xx) {
                double px = origin[0] + (double)(x0 + xx) * ux[0] + (double)(y0 + yy) * uy[0];
                double py = origin[1] + (double)(x0 + xx) * ux[1] + (double)(y0 + yy) * uy[1];
                double pz = origin[2] + (double)(x0 + xx) * ux[2] + (double)(y0 + yy) * uy[2];
                double tr, ti;
                ORC_TERM(LD_D_RE, LD_D_IM, p, px, py, pz, tr, ti);
                const double wr = weight[2 * ((size_t)yy * w + xx)], wi = weight[2 * ((size_t)yy * w + xx) + 1];
                cr += wr * tr + wi * ti;
                ci += wr * ti - wi * tr;
            }
        }
        out[2 * p] = cr;
        out[2 * p + 1] = ci;
    }
}
