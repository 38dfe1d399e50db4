// sarbp_internal.h -- shared declarations of libsarbp's CUDA translation units.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <atomic>

#include <cmath>
#include <complex>

#include <string>
#include <vector>

#include "sarbp.h"

namespace sarbp {

// Device-side error bits, OR-ed into a context-owned word and read by the host
// after synchronisation.
enum : unsigned {
    kErrWaitTimeout = 1u << 0,   // an mbarrier wait ran out of iterations
    kErrIndexClamp = 1u << 1,    // (checked builds) an interpolation index was clamped
    kErrBadLaunch = 1u << 2,     // a kernel saw inconsistent launch parameters
    kErrWindow = 1u << 3,        // a (tile, pulse) needed more bins than the staging window
    kErrDrainTimeout = 1u << 4,  // after a timed-out wait, a copy in flight did not land within the drain limit
};

// Test and tuning switches of a context (sarbp_debug_set).  Zero / negative
// values leave the planner and the kernels their defaults.
struct Tuning {
    int bp_chunk = 0;              // staged pulse chunk (16, 8, 4) where it fits; 0: planner
    int bp_segments = 0;           // pulse segments (1..64); 0: planner
    int checked = 0;               // 1: clamped, self-reporting back-projection kernels
    long long wait_ns = 0;         // limit of the staging waits; 0: 2 s
    int linear_phase = 0;          // 1 / -1: force the linear-term / series phase form; 0: planner
    int wait_fault_chunk = -1;     // >= 0: that chunk's staging barrier of every CTA is armed with
                                   // kFaultBytes more than its copies deliver (the wait runs out); the
                                   // drain then delivers them, as a late copy would
};
constexpr unsigned kFaultBytes = 16;
constexpr unsigned long long kDefaultWaitNs = 2000000000ull;

// Raises the kernel's dynamic shared-memory limit on the current device to the
// device's opt-in maximum (less the kernel's static shared memory), once per
// (kernel, device).  Launches then need no attribute call of their own (a host
// cost on every launch otherwise), and threads launching the same kernel with
// different sizes cannot lower each other's limit between its setting and
// their launch.  Thread-safe (plan.cpp).
cudaError_t allow_dynamic_smem(const void *kernel);

// SMs of the current device, queried once per device: grid-stride launches
// size their grids as a multiple of it.
inline int current_sms() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return 1;
    }
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return 1;
    }
    cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

// ---------------------------------------------------------------- range compression
struct RcPlan {
    int np;          // pulses in this launch
    int ns;          // echo samples per pulse
    int nfft;        // FFT size (power of two)
    int L;           // upsampling factor
    int nbins;       // L * ns
    int storage;     // sarbp_storage
    float *bound2;   // [2 np] scratch for the split (nfft = 32768) path, else unused
};

// Host-side launchers (rc.cu).  spec: scratch [np][nfft] complex; filt: [nfft]
// matched-filter spectrum; etab: two-level table of E^m = e^{+j2pi m/(L nfft)}:
// etab[i] = E^i for i < 256, etab[256 + i] = E^{256 i} for i < L nfft / 256
// (rc_etab_size entries in all).
cudaError_t launch_rc_forward(const RcPlan &p, const float2 *echo, const float2 *filt,
                              const float2 *etab, float2 *spec, float *scale, cudaStream_t s);
cudaError_t launch_rc_inverse(const RcPlan &p, const float2 *spec, const float2 *etab,
                              const float *scale, void *out, cudaStream_t s);
// The split path (nfft = 32768) writes the FP16 scale in the inverse, so the
// scale pointer passed to launch_rc_inverse must be writable there.
// Loads and configures the kernels a plan's launches use without launching
// them (the module loads here under lazy loading, not at the first launch).
cudaError_t prepare_rc_kernels(const RcPlan &p);
inline int rc_etab_size(int L, int nfft) { return 256 + (L * nfft >= 256 ? L * nfft / 256 : 1); }
bool rc_size_supported(int nfft);

// ---------------------------------------------------------------- back-projection
struct BpGeom {
    double origin[3], ux[3], uy[3];
    double g11, g12, g22;   // ux.ux, ux.uy, uy.uy
    int nx, ny;
};

struct BpPlan {
    const void *rc;          // [np][nbins] c64 or c32h
    const float *scale;      // [np] or null
    int storage;
    int np;                  // pulses
    int nbins;
    int mode;                // sarbp_mode
    const double *apc;       // [np][3] device
    float4 *pref;            // [np][2] per-pulse FP64 references as float pairs (written by launch_bp)
    BpGeom g;
    double fc, c, t0_bins, bin_rate;
    // float pairs of 2 bin_rate / c (bins per metre of range), t0_bins * bin_rate and
    // 2 fc / c (carrier cycles per metre of range) for the float-float tile references
    float kb_h, kb_l, tb_h, tb_l, kc_h, kc_l;
    // float pair of 4 pi fc / c (carrier phase per metre) and the grid metric
    // in FP32: constants of the launch, so the kernel's per-chunk code has no
    // FP64 division or conversion
    float kp_h, kp_l;
    float gf11, gf12, gf22;
    float gf11l, gf12l, gf22l;     // their float-float low parts (linear-term phase increments)
    float2 *image;           // [ny][nx] final image
    float2 *partial;         // [segments][ny][nx] scratch when segments > 1
    int segments;            // pulse segments (1: write image directly)
    int accumulate;
    int win;                 // staged bins per (tile, pulse), multiple of 4
    int nterms;              // polynomial terms for the differential range (3 or 4)
    int lin;                 // 1: linear-term phase (SPLIT / FP16STORE back-projection, large tiles)
    int checked;             // 1: clamp every interpolation index and report clamps
    int pix;                 // pixels per thread (8, 4 or 2): tiles of 32 x (8 pix) pixels
    int chunk;               // pulses per staged chunk (16, 8 or 4)
    unsigned *err;           // device error word
    const double *drange;    // [np] device, per-pulse range corrections (m), or null
    const double *dphase;    // [np] device, per-pulse phase corrections (rad), or null
    const float2 *weight;    // [ny][nx] device, projection weights (launch_project only)
    float2 *proj;            // [tiles][np] device scratch of tile sums (launch_project only)
    unsigned long long wait_ns;  // limit of each bounded staging wait
    int fault_chunk;         // < 0: none; else that chunk's barrier is over-armed (tests, Tuning)
};

cudaError_t launch_bp(const BpPlan &p, cudaStream_t s, int *launches);
// Resident CTAs per SM of the kernel variant launch_bp would run for `p`.
cudaError_t bp_occupancy(const BpPlan &p, int *ctas_per_sm);
// Weighted projection (adjoint of back-projection, SPLIT / FP16STORE arithmetic):
// out[p] = sum over pixels of conj(weight) * pulse p's term, via p.proj
// ([bp_tiles(p)][np] float2 scratch) and a fixed-order reduction in FP64.
cudaError_t launch_project(const BpPlan &p, double2 *out, cudaStream_t s, int *launches);
size_t bp_tiles(const BpPlan &p);
// Geometry extremes the planner sizes tiles and windows from, over a 9 x 9
// lattice of grid points (corners and edges included) and every pulse: the
// nearest and farthest range and the largest |cosine| between the line of sight
// and each grid axis.  The host (plan.cpp) and device (bp.cu) reductions give
// identical bits: FP64 in one fixed operation order without fused multiply-adds,
// correctly rounded square root and division, order-free min / max.
struct BpExtremes {
    double rmin, rmax, cx, sy;
    unsigned nonfinite;  // 1 if an APC coordinate was not finite
};
constexpr int kLattice = 9;  // lattice points per grid axis

__host__ __device__ inline double ext_mul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ inline double ext_add(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ inline double ext_dot(const double *a, const double *b) {
    return ext_add(ext_add(ext_mul(a[0], b[0]), ext_mul(a[1], b[1])), ext_mul(a[2], b[2]));
}
__host__ __device__ inline double ext_sqrt(double x) {
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(x);
#else
    return std::sqrt(x);
#endif
}
__host__ __device__ inline double ext_div(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
// Lattice point (u, v) of the grid: origin + fx ux + fy uy with
// fx = (nx - 1) u / 8, fy = (ny - 1) v / 8 (corners and edges included).
__host__ __device__ inline void ext_lattice(const sarbp_grid &g, int u, int v, double *P) {
    const double fx = (double)((g.nx - 1) * u) / (double)(kLattice - 1);
    const double fy = (double)((g.ny - 1) * v) / (double)(kLattice - 1);
    for (int k = 0; k < 3; ++k) P[k] = ext_add(ext_add(g.origin[k], ext_mul(fx, g.ux[k])), ext_mul(fy, g.uy[k]));
}
// Running maximum of the direction cosine q = |axis.w| / (R |axis|) over points.
// q is evaluated (correctly rounded square root, product and quotient) only
// where the division-free comparison n^2 R_b^2 >= n_b^2 R^2 (1 - 1e-9) against
// the best point so far (n_b, R_b^2) cannot rule the point out: the margin is
// far above the few ulps of rounding in that comparison and in q, so every
// point skipped has a smaller q, and the maximum is the value that evaluating
// q at every point gives.  Along a track that is about one evaluation per
// pulse instead of one per point.
struct ExtCos {
    double best, n, r2;
};
__host__ __device__ inline void ext_cos(ExtCos &c, double n, double r2, double len) {
    const double lhs = ext_mul(ext_mul(n, n), c.r2), rhs = ext_mul(ext_mul(c.n, c.n), r2);
    if (lhs < ext_mul(rhs, 1.0 - 1e-9)) return;
    const double q = ext_div(n, ext_mul(ext_sqrt(r2), len));
    if (q > c.best) {
        c.best = q;
        c.n = n;
        c.r2 = r2;
    }
}
// Reduction state over (pulse, lattice point): squared ranges (the range
// extremes are their square roots: the square root is monotonic and correctly
// rounded, so this equals the extremes of the ranges) and the two cosines
// (zero where R or the axis length is 0).
struct ExtAcc {
    double r2min, r2max;
    ExtCos cx, sy;
};
__host__ __device__ inline void ext_acc_init(ExtAcc &a) {
    a.r2min = 1e300;
    a.r2max = 0.0;
    a.cx = ExtCos{0.0, 0.0, 0.0};
    a.sy = ExtCos{0.0, 0.0, 0.0};
}
// Squared range and |axis . w| of lattice point P against antenna position a.
__host__ __device__ inline void ext_terms(const sarbp_grid &g, const double *P, const double *apc, double &r2,
                                          double &nx, double &ny) {
    double w[3];
    for (int k = 0; k < 3; ++k) w[k] = ext_add(P[k], -apc[k]);
    r2 = ext_dot(w, w);
    nx = fabs(ext_dot(g.ux, w));
    ny = fabs(ext_dot(g.uy, w));
}
__host__ __device__ inline void ext_acc_terms(ExtAcc &a, double r2, double nx, double ny, double lux, double luy) {
    a.r2min = fmin(a.r2min, r2);  // NaN-ignoring on host and device alike
    a.r2max = fmax(a.r2max, r2);
    if (r2 > 0) {
        if (lux > 0) ext_cos(a.cx, nx, r2, lux);
        if (luy > 0) ext_cos(a.sy, ny, r2, luy);
    }
}
__host__ __device__ inline void ext_acc_point(ExtAcc &a, const sarbp_grid &g, double lux, double luy, const double *P,
                                              const double *apc) {
    double r2, nx, ny;
    ext_terms(g, P, apc, r2, nx, ny);
    ext_acc_terms(a, r2, nx, ny, lux, luy);
}
// Range extremes from the squared ones (1e300: no finite point).
inline void ext_ranges(double r2min, double r2max, BpExtremes &e) {
    e.rmin = r2min >= 1e300 ? 1e300 : std::sqrt(r2min);
    e.rmax = std::sqrt(r2max);
}
// Axis lengths |ux|, |uy| as both reductions use them.
void ext_axes(const sarbp_grid &g, double *lux, double *luy);
// Host reduction over apc [np][3] (host memory).
void bp_extremes_host(const double *apc, int np, const sarbp_grid &g, BpExtremes &e);
// Device reduction over apc [np][3] (device memory) into out[0..3] (the four
// extremes as FP64 bit patterns) and out[4] (nonfinite flag): launches the
// initialisation and the reduction on `s`.
cudaError_t launch_bp_extremes(const double *apc, int np, const sarbp_grid &g, unsigned long long *out,
                               cudaStream_t s);

// Host planning (plan.cpp): fills every BpPlan field that does not depend on
// buffers (geometry, constants, tile height, window, series terms, segments
// for launches of `pulses_per_launch` pulses; 0 = all np) from the geometry
// extremes.  On failure returns false with the reason in `why`.
// `tune` (may be null) forces the chunk or the segments and sets the waits'
// limit and fault injection.
bool plan_bp(int sms, const sarbp_radar &r, const sarbp_rc_view &rc, const BpExtremes &ex, int np,
             const sarbp_grid &g, int mode, int pulses_per_launch, BpPlan &p, std::string &why,
             const Tuning *tune = nullptr);
// Two-level table of E^m = e^{+j 2 pi m / (L N)} ([rc_etab_size(L, N)] entries, plan.cpp).
void fft_etab_host(int L, int N, std::vector<float2> &etab);
void fft_etab_fill(int L, int N, float2 *etab);
// Matched-filter spectrum [nfft] and phase table [rc_etab_size] for a layout (plan.cpp).
void rc_tables_host(const sarbp_radar &r, const sarbp_rc_layout &lay, std::vector<float2> &filt,
                    std::vector<float2> &etab);
// The same tables into caller buffers: work [nfft], filt [nfft], etab
// [rc_etab_size] (the allocation-free entry point passes static arrays).
void rc_tables_fill(const sarbp_radar &r, const sarbp_rc_layout &lay, std::complex<double> *work, float2 *filt,
                    float2 *etab);
// In-place unnormalised forward DFT of a power-of-two length N, FP64 (plan.cpp).
void fft_pow2_inplace(std::complex<double> *x, int N);
// Tile geometry the planner needs to size the staging window.
void bp_tile_dims(int pix, int *tile_x, int *tile_y);
// Dynamic shared memory of a BP CTA for a staging window and pulse chunk.
size_t bp_smem_bytes(int storage, int win, int chunk);
int bp_max_chunk();  // largest pulse chunk (16); the planner may choose 8 or 4
// Pulse segments for `tiles` tiles and `npl` pulses per launch on `sms` SMs
// (at least 12 waves of CTAs where the pulses allow; at least 4 chunks per
// segment; partial images within 1 GiB); `force` in 1..64 overrides.
int bp_choose_segments(int tiles, int npl, long long npix, int sms, int force = 0);

// ---------------------------------------------------------------- echo synthesis
cudaError_t launch_echo_synth(const double *apc, int np, int ns, const sarbp_target *tg, int nt,
                              double t_rec0, double fs, double kr, double tp, double tc,
                              double fc, double c, float2 *echo, double *power_acc,
                              cudaStream_t s);
cudaError_t launch_echo_noise(float2 *echo, int64_t count, const double *power_acc,
                              double snr_db, uint64_t seed, cudaStream_t s);
cudaError_t launch_ref_echo(float2 *Srnm, const float *Ptarget, const float *ta, const float *tr,
                            const sarbp_ref_params &p, int Mslow, int Nfast, cudaStream_t s);

// ---------------------------------------------------------------- omega-K (wk.cu)
// Batched 1-D DFT along rows: power-of-two n <= 16384 (m = 0) in shared memory,
// other n <= 8192 by Bluestein through m-point FFTs (m = pow2 >= 2n - 1).
struct DftPlan {
    int n, m;
    const float2 *etab;   // [rc_etab_size(1, m ? m : n)] E table of the shared-memory FFT
    const float2 *chirp;  // [n] w_j = e^{j pi j^2 / n} (Bluestein)
    const float2 *kfwd;   // [m] FFT_m of the circular kernel w, / m (Bluestein forward)
    const float2 *kinv;   // [m] FFT_m of conj(w), / m (Bluestein inverse)
};
// Optional input of a row transform: element i of row b is src[b][i - col0] *
// rowmul[b] inside [col0, col0 + src_cols) and 0 outside (fused zero padding
// and azimuth down-conversion); src = null transforms the rows in place.
struct DftIo {
    const float2 *src = nullptr;
    int src_cols = 0;
    int col0 = 0;
    const float2 *rowmul = nullptr;
};
bool dft_size_supported(int n);
int dft_bluestein_size(int n);
// host FP64 tables for a DftPlan of length n (plan.cpp)
void dft_tables_host(int n, std::vector<float2> &etab, std::vector<float2> &chirp, std::vector<float2> &kfwd,
                     std::vector<float2> &kinv);
// rows x n in place (row stride ld): forward unnormalised, or inverse; times scale
cudaError_t launch_dft_rows(const DftPlan &p, float2 *data, int rows, long long ld, bool inverse, float scale,
                            cudaStream_t s, const DftIo &io = DftIo());
cudaError_t launch_transpose(const float2 *in, float2 *out, int rows, int cols, cudaStream_t s);
// Transforms of length p.n down the ncols columns of a row-major [p.n][ncols]
// array (power-of-two p.n in [512, 4096]), out == in for in place.
bool dft_cols_supported(const DftPlan &p);
// out [NA][NR] = echo [na][nr] placed at (pa, pr) times rowmul[m] per row, zero elsewhere.
cudaError_t launch_wk_pad(const float2 *echo, int na, int nr, const float2 *rowmul, int pa, int pr, int NA, int NR,
                          float2 *out, cudaStream_t s);
cudaError_t launch_dft_cols(const DftPlan &p, const float2 *in, float2 *out, int ncols, bool inverse, float scale,
                            cudaStream_t s);
size_t wk_stolt_smem(int NR);
// FP32 / float-float form of the Stolt stage (eps = q / (f0 + fr)^2 <= 1e-2):
// col_c = (A (f0 + fr) + pi fr^2 / kr) mod 2 pi, col_ip = 1 / (f0 + fr) and row_q as float pairs.
cudaError_t launch_wk_stolt_ff(const float2 *in, float2 *out, int NA, int NR, const float *col_c,
                               const float2 *col_ip, const float2 *row_q, double a4r, double nr_over_fr, int taps,
                               cudaStream_t s);
cudaError_t launch_wk_stolt(const float2 *in, float2 *out, int NA, int NR, const double *col_f2, const double *col_ph,
                            const double *col_fr, const double *row_q, double a4r, double f0, double inv_gap, int taps,
                            cudaStream_t s);

// ---------------------------------------------------------------- CEOS decode (ceos.cu)
struct CeosGeom {
    int header, aux, replica, replica_line, lines_per_block, agc_byte;
    int first_line, nlines, first_cell, ncells, apply_agc;
    long long line_bytes, block_bytes;
    long long raw_offset;  // offset of the device buffer's byte 0 from the start of the first block
};
// echo [nlines][ncells], agc_db [nlines] (may be null); gains[64] = 1.5 10^(dB(code)/20)
cudaError_t launch_ceos_decode(const unsigned char *raw, const CeosGeom &g, const float *gains, float2 *echo,
                               short *agc_db, cudaStream_t s);

// ---------------------------------------------------------------- autofocus (autofocus.cu)
// w = |img|^2 img (w may be null); partial[sharpness_blocks(n)] = per-block sums of |img|^4.
int sharpness_blocks(size_t n);
cudaError_t launch_sharpness_weight(const float2 *img, size_t n, float2 *w, double *partial, cudaStream_t s);

// ---------------------------------------------------------------- probes
cudaError_t run_issue_probe(int sms, double *fp32_lanes_per_s, double *mufu_lanes_per_s,
                            cudaStream_t s);

}  // namespace sarbp
