// plan.cpp -- host-side planning of a back-projection launch (shared by the
// one-shot API and the serving loop).
//
// From the radar, the range-compressed data layout, the APC track and the
// pixel grid it derives everything the BP kernel needs that does not change
// from launch to launch: grid metric terms, float-pair constants, the tile
// height (32 x 64, 32 x 32 or 32 x 16 pixels), the staging window per
// (tile, pulse), the number of series terms and the pulse segmentation.
#include <cmath>
#include <cstdlib>
#include <complex>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "sarbp_internal.h"

namespace sarbp {

cudaError_t allow_dynamic_smem(const void *kernel) {
    static std::mutex m;
    static std::set<std::pair<const void *, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(m);
    if (done.count({kernel, dev})) return cudaSuccess;
    cudaFuncAttributes fa;
    int optin = 0;
    e = cudaFuncGetAttributes(&fa, kernel);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) done.insert({kernel, dev});
    return e;
}

}  // namespace sarbp

namespace sarbp {

void fft_pow2_inplace(std::complex<double> *h, int N) {
    constexpr double kPi = 3.14159265358979323846;
    for (int i = 1, j = 0; i < N; ++i) {
        int bit = N >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(h[i], h[j]);
    }
    for (int len = 2; len <= N; len <<= 1)
        for (int i = 0; i < N; i += len)
            for (int k = 0; k < len / 2; ++k) {
                const double a = -2.0 * kPi * (double)k / (double)len;
                const std::complex<double> w(std::cos(a), std::sin(a));
                const std::complex<double> u = h[i + k], v = h[i + k + len / 2] * w;
                h[i + k] = u + v;
                h[i + k + len / 2] = u - v;
            }
}

namespace {
double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// In-place radix-2 forward DFT (unnormalised) of a power-of-two length, FP64.
void fft_pow2_host(std::vector<std::complex<double>> &h) { fft_pow2_inplace(h.data(), (int)h.size()); }
}  // namespace

// Pulse chunk for a staging window: the largest (16, 8, 4) whose CTA still fits
// twice in an SM's 228 KB of shared memory (1 KB reserved per CTA), else the
// largest that fits once (227 KB per CTA); 0 if none.  `force` = 16, 8 or 4
// takes that chunk where it fits (tuning and tests through sarbp_debug_set:
// results do not depend on it).
int bp_choose_chunk(int storage, int win, int force) {
    constexpr size_t kSmemPerSm = 228u << 10, kSmemPerCta = 227u << 10, kReserve = 1u << 10;
    if ((force == 16 || force == 8 || force == 4) && force <= bp_max_chunk() &&
        bp_smem_bytes(storage, win, force) <= kSmemPerCta)
        return force;
    for (int c = bp_max_chunk(); c >= 4; c /= 2)
        if (2 * (bp_smem_bytes(storage, win, c) + kReserve) <= kSmemPerSm) return c;
    for (int c = bp_max_chunk(); c >= 4; c /= 2)
        if (bp_smem_bytes(storage, win, c) <= kSmemPerCta) return c;
    return 0;
}

void ext_axes(const sarbp_grid &g, double *lux, double *luy) {
    *lux = std::sqrt(ext_dot(g.ux, g.ux));
    *luy = std::sqrt(ext_dot(g.uy, g.uy));
}

// Pulses split over up to 8 host threads (at least 1024 pulses each): min /
// max combine in any order, so the bits do not depend on the split.  About
// 0.6 us per pulse on one core; a submit of 8192 pulses took ~5 ms single-threaded.
void bp_extremes_host(const double *apc, int np, const sarbp_grid &g, BpExtremes &e) {
    double lux, luy;
    ext_axes(g, &lux, &luy);
    double P[kLattice * kLattice][3];
    for (int k = 0; k < kLattice * kLattice; ++k) ext_lattice(g, k / kLattice, k % kLattice, P[k]);
    // each thread accumulates in its own stack copy and stores it once: the
    // threads' slots of `acc` share cache lines, and updating them per point
    // cost 2-4x in false sharing (4096 pulses on 4 threads: 3.2 against 0.9 ms)
    auto run = [&](int p0, int p1, ExtAcc &out, unsigned &bad_out) {
        ExtAcc acc;
        ext_acc_init(acc);
        unsigned bad = 0;
        for (int i = p0; i < p1; ++i) {
            const double *a = apc + 3 * (size_t)i;
            if (!std::isfinite(a[0]) || !std::isfinite(a[1]) || !std::isfinite(a[2])) {
                bad = 1;
                continue;
            }
            for (int k = 0; k < kLattice * kLattice; ++k) ext_acc_point(acc, g, lux, luy, P[k], a);
        }
        out = acc;
        bad_out = bad;
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int nt = (int)std::min<long long>(std::min<unsigned>(hw, 8u), std::max(1, np / 1024));
    std::vector<ExtAcc> acc(nt);
    std::vector<unsigned> bad(nt);
    std::vector<std::thread> pool;
    const int per = (np + nt - 1) / nt;
    int t = 1;
    try {
        for (; t < nt; ++t)
            pool.emplace_back(run, t * per, std::min(np, (t + 1) * per), std::ref(acc[t]), std::ref(bad[t]));
    } catch (...) {  // no thread to be had: the rest on this thread (no exception crosses the C ABI)
        for (int u = t; u < nt; ++u) run(u * per, std::min(np, (u + 1) * per), acc[u], bad[u]);
    }
    run(0, std::min(np, per), acc[0], bad[0]);
    for (auto &th : pool) th.join();
    ExtAcc all = acc[0];
    e.nonfinite = bad[0];
    for (int t = 1; t < nt; ++t) {
        all.r2min = std::fmin(all.r2min, acc[t].r2min);
        all.r2max = std::fmax(all.r2max, acc[t].r2max);
        all.cx.best = std::fmax(all.cx.best, acc[t].cx.best);
        all.sy.best = std::fmax(all.sy.best, acc[t].sy.best);
        e.nonfinite |= bad[t];
    }
    ext_ranges(all.r2min, all.r2max, e);
    e.cx = all.cx.best;
    e.sy = all.sy.best;
}

bool plan_bp(int sms, const sarbp_radar &r, const sarbp_rc_view &rc, const BpExtremes &ex, int np,
             const sarbp_grid &g, int mode, int pulses_per_launch, BpPlan &p, std::string &why,
             const Tuning *tune) {
    std::memset(&p, 0, sizeof p);
    p.wait_ns = tune && tune->wait_ns > 0 ? (unsigned long long)tune->wait_ns : kDefaultWaitNs;
    p.fault_chunk = tune ? tune->wait_fault_chunk : -1;
    p.checked = tune ? tune->checked : 0;
    p.storage = rc.storage;
    p.nbins = rc.nbins;
    p.mode = mode;
    for (int i = 0; i < 3; ++i) {
        p.g.origin[i] = g.origin[i];
        p.g.ux[i] = g.ux[i];
        p.g.uy[i] = g.uy[i];
    }
    p.g.g11 = dot3(g.ux, g.ux);
    p.g.g12 = dot3(g.ux, g.uy);
    p.g.g22 = dot3(g.uy, g.uy);
    p.g.nx = g.nx;
    p.g.ny = g.ny;
    p.fc = r.fc;
    p.c = r.c;
    p.t0_bins = rc.t0_bins;
    p.bin_rate = rc.bin_rate;
    auto split2 = [](double v, float *h, float *l) {
        *h = (float)v;
        *l = (float)(v - (double)*h);
    };
    split2(2.0 / r.c * rc.bin_rate, &p.kb_h, &p.kb_l);
    split2(rc.t0_bins * rc.bin_rate, &p.tb_h, &p.tb_l);
    split2(2.0 * r.fc / r.c, &p.kc_h, &p.kc_l);
    split2(4.0 * 3.141592653589793 * r.fc / r.c, &p.kp_h, &p.kp_l);
    split2(p.g.g11, &p.gf11, &p.gf11l);
    split2(p.g.g12, &p.gf12, &p.gf12l);
    split2(p.g.g22, &p.gf22, &p.gf22l);

    const double lux = std::sqrt(p.g.g11), luy = std::sqrt(p.g.g22);
    double cx = ex.cx, sy = ex.sy;
    const double rmin = ex.rmin;
    cx = std::min(1.0, cx * 1.05 + 0.01);
    sy = std::min(1.0, sy * 1.05 + 0.01);
    const double bpm = 2.0 / r.c * rc.bin_rate;
    // Tile choice: the tallest tile (32 x 64, 32 x 32, 32 x 16 pixels) whose
    // differential-range series truncation stays below kSeriesTol metres and
    // whose staging window fits shared memory.  Series remainder after k terms
    // of sqrt(1+e)-1 times R_T: R_T (5/128) e^4 (k = 3), R_T (7/256) e^5 (k = 4),
    // with e = |n|/R_T^2 <= 2 diag/R_T + diag^2/R_T^2 over the tile.  R_T e^k
    // falls as R_T grows, so the remainder is largest at the nearest tile centre
    // (rmin_tile); x1.1 covers the terms past the first omitted one (|e| < 0.09).
    constexpr double kSeriesTol = 5e-7;  // 1.1e-4 rad of C-band phase at the tile corners
    constexpr double kLinearPhaseHalfDiag = 12.0;  // m: tiles beyond it take the linear-term phase
    why = "no tile size fits";
    bool chosen = false;
#ifdef SARBP_BP_FORCE_PIX
    for (int pix : {SARBP_BP_FORCE_PIX}) {  // tuning builds only
#else
    for (int pix : {8, 4, 2}) {
#endif
        int tx, ty;
        bp_tile_dims(pix, &tx, &ty);
        const double hx = 0.5 * (tx - 1), hy = 0.5 * (ty - 1);
        const double qq_max = hx * hx * p.g.g11 + 2 * hx * hy * std::fabs(p.g.g12) + hy * hy * p.g.g22;
        const double tile_diag = std::sqrt(qq_max);
        const double rmin_tile = rmin - tile_diag;
        if (!(rmin_tile > 20.0 * tile_diag)) {
            why = "an antenna position is within 20 tile diagonals of the grid";
            continue;
        }
        const double half = bpm * (lux * hx * cx + luy * hy * sy + qq_max / (2 * rmin_tile)) * 1.03 + 2.0;
        if (!(half < 4096.0)) {
            why = "tile spans too many range bins";
            continue;
        }
        int win = (int)std::ceil(2 * half) + 8;
        win = (win + 3) & ~3;
        const int chunk = bp_choose_chunk(p.storage, win, tune ? tune->bp_chunk : 0);
        if (!chunk) {
            why = "tile spans too many range bins for shared memory";
            continue;
        }
        const double rt = rmin_tile;
        const double e = (2 * tile_diag * rt + qq_max) / (rt * rt);
        const bool split = mode == SARBP_MODE_SPLIT || mode == SARBP_MODE_FP16STORE;
        if (split && (e >= 0.09 || 1.1 * rt * 0.02734375 * std::pow(e, 5) > kSeriesTol)) {
            why = "tiles too large for the differential-range series";
            continue;
        }
        p.pix = pix;
        p.win = win;
        p.chunk = chunk;
        p.nterms = (1.1 * rt * 0.0390625 * e * e * e * e < kSeriesTol) ? 3 : 4;
        // phase form: the series form's FP32 differential range rounds to 2^-24 of
        // n ~ 2 R_T d, a phase error growing with the tile's extent d (about
        // -82 dB below 12 m of half-diagonal, -67 to -74 dB above); the
        // linear-term form keeps it near -100 dB for ~10% more time
        const int force = tune ? tune->linear_phase : 0;
        p.lin = split && (force > 0 || (force == 0 && tile_diag > kLinearPhaseHalfDiag));
        chosen = true;
        break;
    }
    if (!chosen) return false;
    int tx, ty;
    bp_tile_dims(p.pix, &tx, &ty);
    const int tiles = ((g.nx + tx - 1) / tx) * ((g.ny + ty - 1) / ty);
    const int npl = pulses_per_launch > 0 ? pulses_per_launch : np;
    p.segments = bp_choose_segments(tiles, npl, (long long)g.nx * g.ny, sms, tune ? tune->bp_segments : 0);
    return true;
}

// Pulse segments: every (tile, segment) is one CTA, two resident per SM (the
// SPLIT kernels' register bound).  Finer CTAs fill the last wave and balance
// CTAs that end at different times; measured on GB300 (4096 pulses, config-2
// geometry, ms per call for 1 / 2 / 4 / 8 segments): 1024^2 4.10 / 3.58 / 3.54
// / 3.42, 1536^2 8.00 / 7.94 / 7.68 / 7.58 (5: 7.54), 2048^2 13.82 / 13.30 /
// 13.27 / 13.32; config 1 (512 pulses, 512^2) 0.237 / 0.202 / 0.201 / 0.188.
// Rule: the fewest segments that give at least 12 waves of CTAs, with at least
// 4 chunks of pulses per segment, no empty segment and the partial images (one
// per segment) within 1 GiB.  The count depends on the geometry only (not on
// the staging chunk, which the planner or a forced chunk picks), so a call
// gives the same bits whatever the chunk.  `force` = n (1..64) takes n, for
// sweeps and tests.
int bp_choose_segments(int tiles, int npl, long long npix, int sms, int force) {
    const int kc = bp_max_chunk();
    if (force >= 1 && force <= 64) return force;
    const long long target = 12LL * 2 * std::max(sms, 1);
    const double max_partial = 1024.0 * 1024.0 * 1024.0;
    int best = 1;
    for (int s = 1; s <= 64; ++s) {
        if (s > 1 && (npl / s < 4 * kc || (double)s * (double)npix * 8.0 > max_partial)) break;
        const int n = (npl + s - 1) / s;
        const int pps = (n + kc - 1) / kc * kc;  // as the launch rounds it
        if (s > 1 && (long long)(s - 1) * pps >= npl) continue;  // an empty segment
        best = s;
        if ((long long)tiles * s >= target) break;
    }
    return best;
}

void rc_tables_fill(const sarbp_radar &r, const sarbp_rc_layout &lay, std::complex<double> *h, float2 *filt,
                    float2 *etab) {
    constexpr double kPi = 3.14159265358979323846;
    const int N = lay.nfft, L = r.upsample;
    for (int i = 0; i < N; ++i) h[i] = 0.0;
    for (int i = 0; i < lay.nc && i < N; ++i) {
        const double u = (double)i / r.fs;
        if (u >= 0.0 && u < r.tp) {
            const double ph = kPi * r.kr * (u - r.tc) * (u - r.tc);
            h[i] = std::complex<double>(std::cos(ph), std::sin(ph));
        }
    }
    fft_pow2_inplace(h, N);
    for (int k = 0; k < N; ++k) {
        const long long m = ((long long)k * lay.shift) % N;
        const double a = -2.0 * kPi * (double)m / (double)N;
        const std::complex<double> v = std::conj(h[k]) * std::complex<double>(std::cos(a), std::sin(a)) / (double)N;
        filt[k] = make_float2((float)v.real(), (float)v.imag());
    }
    fft_etab_fill(L, N, etab);
}

void rc_tables_host(const sarbp_radar &r, const sarbp_rc_layout &lay, std::vector<float2> &filt,
                    std::vector<float2> &etab) {
    std::vector<std::complex<double>> h(lay.nfft);
    filt.resize(lay.nfft);
    etab.resize(rc_etab_size(r.upsample, lay.nfft));
    rc_tables_fill(r, lay, h.data(), filt.data(), etab.data());
}

void dft_tables_host(int n, std::vector<float2> &etab, std::vector<float2> &chirp, std::vector<float2> &kfwd,
                     std::vector<float2> &kinv) {
    constexpr double kPi = 3.14159265358979323846;
    const int m = dft_bluestein_size(n);
    fft_etab_host(1, m ? m : n, etab);
    chirp.clear();
    kfwd.clear();
    kinv.clear();
    if (!m) return;
    // w_j = e^{j pi j^2 / n}; j^2 reduced modulo 2n in integers keeps the angle exact
    std::vector<std::complex<double>> w(n), b(m), bc(m);
    chirp.resize(n);
    for (int j = 0; j < n; ++j) {
        const long long r = ((long long)j * j) % (2LL * n);
        const double a = kPi * (double)r / (double)n;
        w[j] = std::complex<double>(std::cos(a), std::sin(a));
        chirp[j] = make_float2((float)w[j].real(), (float)w[j].imag());
    }
    for (int j = 0; j < n; ++j) {
        b[j] = w[j];
        if (j > 0) b[m - j] = w[j];
    }
    for (int j = 0; j < m; ++j) bc[j] = std::conj(b[j]);
    fft_pow2_host(b);
    fft_pow2_host(bc);
    kfwd.resize(m);
    kinv.resize(m);
    for (int j = 0; j < m; ++j) {
        kfwd[j] = make_float2((float)(b[j].real() / m), (float)(b[j].imag() / m));
        kinv[j] = make_float2((float)(bc[j].real() / m), (float)(bc[j].imag() / m));
    }
}

void fft_etab_fill(int L, int N, float2 *etab) {
    constexpr double kPi = 3.14159265358979323846;
    const int n = rc_etab_size(L, N);
    const double LN = (double)L * N;
    for (int i = 0; i < n; ++i) {
        const double a = 2.0 * kPi * (double)(i < 256 ? i : 256 * (i - 256)) / LN;
        etab[i] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
}

void fft_etab_host(int L, int N, std::vector<float2> &etab) {
    etab.resize(rc_etab_size(L, N));
    fft_etab_fill(L, N, etab.data());
}

}  // namespace sarbp
