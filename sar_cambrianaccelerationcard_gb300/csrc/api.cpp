// api.cpp -- C ABI of libsarbp: context, planning, host<->device staging.
//
// Replaces the host orchestration of the reference's BP program
// (code/SAR_BP/CUDA/BPA_CUDA.cpp:11-100, SAR_Processor) with a context that
// owns cached device buffers, validates every argument, returns status codes
// instead of exit() (CHECK_CUDA, BPA_CUDA.h:11-17), and plans the kernels:
// range-compression tables, pulse batching of the spectrum scratch, the
// back-projection staging window and pulse segmentation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "sarbp_internal.h"

using sarbp::BpPlan;
using sarbp::RcPlan;

namespace {

constexpr size_t kSpecScratchBudget = size_t(256) << 20;  // bytes of spectrum scratch per batch

struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need) {
        if (need <= bytes && ptr) return cudaSuccess;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        if (need == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&ptr, need);
        if (e == cudaSuccess) bytes = need;
        else cudaGetLastError();
        return e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T>
    T *as() const { return static_cast<T *>(ptr); }
};

struct DftCache {
    int n = 0, m = 0;
    uint64_t used = 0;
    DevBuf etab, chirp, kf, ki;
    void release() {
        for (DevBuf *b : {&etab, &chirp, &kf, &ki}) b->release();
        n = m = 0;
        used = 0;
    }
};

struct RcTables {
    bool valid = false;
    int nfft = 0, L = 0, nc = 0, shift = 0;
    double kr = 0, fs = 0, tc = 0, tp = 0;
    DevBuf filt, etab;
};

// Omega-K tables on the device (row phasors, axes, Stolt terms) for one
// (parameters, padded size): built on the host and uploaded only when these
// change, then reused by every image; `ready` marks the upload on its stream.
struct WkTables {
    float2 *rowphase = nullptr, *rowq = nullptr, *colip = nullptr;
    float *colc = nullptr;
    const double *tab = nullptr;  // col_f2, col_ph, col_fr [NR] each, row_q [NA]
    double a4r = 0.0;
    bool ff = true;               // float-float Stolt (mapping a small correction)
};
struct WkCache {
    bool valid = false;
    int NA = 0, NR = 0;
    double fr = 0, prf = 0, f0 = 0, r0 = 0, kr = 0, c = 0, vr = 0, f_nc = 0;
    DevBuf row, tab;
    WkTables t;
    cudaEvent_t ready = nullptr;
};

}  // namespace

struct sarbp_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::string err;
    DevBuf echo, spec, rc, scale, apc, image, partial, errword, power, targets, pref;
    DevBuf corr, weight, proj, projout, sharp;  // per-pulse corrections, projection and autofocus scratch
    DevBuf wk0, wk1, wkrow;                       // omega-K ping-pong buffers, CEOS gain table
    WkCache wkc;                                  // omega-K tables
    bool ceos_valid = false;                      // wkrow holds the CEOS gains of ceos_gain
    float ceos_gain = 0.f;
    cudaEvent_t ceos_ready = nullptr;             // their upload
    DftCache dft[4];
    uint64_t dft_clock = 0;
    RcTables tables;
    DevBuf ext;                              // planning extremes [5] (FP64 bits, nonfinite flag)
    unsigned long long *ext_host = nullptr;  // pinned host copy of ext
    cudaEvent_t ev_ext = nullptr;
    cudaStream_t copy_stream = nullptr;      // chunked echo uploads beside range compression
    cudaEvent_t ev_copy = nullptr;
    // Buffers sized by the calls (released by sarbp_trim and sarbp_destroy).
    std::vector<DevBuf *> scratch() {
        std::vector<DevBuf *> v = {&echo,   &spec,  &rc,      &scale,   &apc,     &image,   &partial,
                                   &targets, &pref,  &corr,    &weight,  &proj,    &projout, &sharp,
                                   &wk0,    &wk1,   &wkrow,   &wkc.row, &wkc.tab};
        for (DftCache &d : dft)
            for (DevBuf *b : {&d.etab, &d.chirp, &d.kf, &d.ki}) v.push_back(b);
        return v;
    }
    // Buffers held for the context's lifetime.
    std::vector<DevBuf *> persistent() { return {&errword, &power, &ext, &tables.filt, &tables.etab}; }
    void release_scratch() {
        for (DevBuf *b : scratch()) b->release();
        for (DftCache &d : dft) d.release();  // also forgets the cached sizes
        wkc.valid = false;
        ceos_valid = false;
    }
    int64_t launches = 0;
    sarbp::Tuning tune;           // sarbp_debug_set: forced chunk / segments, checked kernels, wait faults
    unsigned last_device_flags = 0;  // device check word of the last call that reported one
    float rc_ms = 0.f, bp_ms = 0.f;
    bool timed_rc = false, timed_bp = false;
};

namespace {

sarbp_status fail(sarbp_ctx *ctx, sarbp_status st, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return st;
}

sarbp_status cuda_fail(sarbp_ctx *ctx, cudaError_t e, const char *what) {
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, SARBP_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(ctx, SARBP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define SARBP_CUDA(ctx, call, what)                            \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device address of pinned, mapped host memory (cudaHostAlloc / cudaMallocHost,
// torch pin_memory), or nullptr for pageable or device memory.  Kernels can
// write results there directly (NVLink-C2C on GB300), so no download follows.
void *mapped_host_ptr(const void *p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// NVTX range for the duration of a scope (header-only NVTX v3: a no-op
// unless a profiler is attached), naming each stage of a call on the timeline.
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

bool is_pow2(long long n) { return n > 0 && (n & (n - 1)) == 0; }

long long next_pow2(long long n) {
    long long p = 1;
    while (p < n) p <<= 1;
    return p;
}

sarbp_status check_radar(sarbp_ctx *ctx, const sarbp_radar *r) {
    if (!r) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "radar is null");
    if (!(r->c > 0) || !(r->fc > 0) || !(r->fs > 0) || !(r->tp > 0) || !std::isfinite(r->kr) ||
        !std::isfinite(r->tc) || !std::isfinite(r->t_rec0))
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "radar constants must be finite, c/fc/fs/tp > 0");
    if (!is_pow2(r->upsample) || r->upsample > 16)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "upsample must be a power of two in [1, 16]");
    if (r->reserved != 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "radar.reserved must be 0");
    return SARBP_OK;
}

sarbp_status layout(sarbp_ctx *ctx, const sarbp_radar *r, int32_t ns, sarbp_rc_layout *out) {
    sarbp_status st = check_radar(ctx, r);
    if (st != SARBP_OK) return st;
    if (ns <= 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "ns must be > 0");
    const double ncd = std::floor(r->tp * r->fs + 0.5);
    if (!(ncd >= 1 && ncd < (1 << 24))) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "tp*fs out of range");
    const int nc = (int)ncd;
    const long long nfft = next_pow2((long long)ns + nc - 1);
    if ((long long)r->upsample * ns > (1LL << 30) || nfft > (1LL << 30))
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "ns too large");
    out->nc = nc;
    out->nfft = (int32_t)nfft;
    out->shift = nc / 2;
    out->nbins = r->upsample * ns;
    out->t0_bins = r->t_rec0 - (double)out->shift / r->fs;
    out->bin_rate = (double)r->upsample * r->fs;
    return SARBP_OK;
}

sarbp_status ensure_tables(sarbp_ctx *ctx, const sarbp_radar *r, const sarbp_rc_layout &lay) {
    RcTables &t = ctx->tables;
    if (t.valid && t.nfft == lay.nfft && t.L == r->upsample && t.nc == lay.nc && t.shift == lay.shift &&
        t.kr == r->kr && t.fs == r->fs && t.tc == r->tc && t.tp == r->tp)
        return SARBP_OK;
    t.valid = false;
    const int N = lay.nfft, L = r->upsample;
    std::vector<float2> g, et;
    sarbp::rc_tables_host(*r, lay, g, et);
    SARBP_CUDA(ctx, t.filt.ensure(sizeof(float2) * N), "alloc filter");
    SARBP_CUDA(ctx, t.etab.ensure(sizeof(float2) * et.size()), "alloc phase table");
    SARBP_CUDA(ctx, cudaMemcpy(t.filt.ptr, g.data(), sizeof(float2) * N, cudaMemcpyHostToDevice), "upload filter");
    SARBP_CUDA(ctx, cudaMemcpy(t.etab.ptr, et.data(), sizeof(float2) * et.size(), cudaMemcpyHostToDevice),
               "upload phase table");
    t.valid = true;
    t.nfft = N;
    t.L = L;
    t.nc = lay.nc;
    t.shift = lay.shift;
    t.kr = r->kr;
    t.fs = r->fs;
    t.tc = r->tc;
    t.tp = r->tp;
    return SARBP_OK;
}

cudaStream_t pick_stream(sarbp_ctx *ctx, void *stream) {
    return stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
}

sarbp_status check_errword(sarbp_ctx *ctx) {
    unsigned w = 0;
    SARBP_CUDA(ctx, cudaMemcpy(&w, ctx->errword.ptr, sizeof w, cudaMemcpyDeviceToHost), "read device check word");
    if (w == 0) return SARBP_OK;
    ctx->last_device_flags = w;
    SARBP_CUDA(ctx, cudaMemset(ctx->errword.ptr, 0, sizeof(unsigned)), "reset device check word");
    if (w & sarbp::kErrDrainTimeout)
        return fail(ctx, SARBP_ERR_TIMEOUT, "a bounded device wait ran out and a copy in flight did not land (0x%x)", w);
    if (w & sarbp::kErrWaitTimeout)
        return fail(ctx, SARBP_ERR_TIMEOUT, "a bounded device wait ran out; its copies landed (0x%x)", w);
    if (w & sarbp::kErrIndexClamp)
        return fail(ctx, SARBP_ERR_DEVICE_CHECK, "an interpolation index left its staging window (0x%x)", w);
    if (w & sarbp::kErrWindow)
        return fail(ctx, SARBP_ERR_DEVICE_CHECK, "a tile needed more range bins than the staging window (0x%x)", w);
    return fail(ctx, SARBP_ERR_DEVICE_CHECK, "device check word 0x%x", w);
}

// finish a call: synchronise when host memory is involved, read timings and checks
sarbp_status finish(sarbp_ctx *ctx, cudaStream_t s, bool sync) {
    if (!sync) return SARBP_OK;
    SARBP_CUDA(ctx, cudaStreamSynchronize(s), "stream synchronize");
    if (ctx->timed_rc) cudaEventElapsedTime(&ctx->rc_ms, ctx->ev[0], ctx->ev[1]);
    if (ctx->timed_bp) cudaEventElapsedTime(&ctx->bp_ms, ctx->ev[2], ctx->ev[3]);
    return check_errword(ctx);
}

// Range compression of a device-resident echo into a device rc buffer.
sarbp_status rc_device(sarbp_ctx *ctx, const sarbp_radar *r, const sarbp_rc_layout &lay, const float2 *echo,
                       int np, int ns, int storage, void *rc_out, float *scale_out, cudaStream_t s,
                       bool record_events = true) {
    Range range("sarbp: range compression");
    if (!sarbp::rc_size_supported(lay.nfft))
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "range FFT size %d not supported (max 32768: ns + tp*fs - 1 <= 32768)",
                    lay.nfft);
    sarbp_status st = ensure_tables(ctx, r, lay);
    if (st != SARBP_OK) return st;
    const size_t row = sizeof(float2) * (size_t)lay.nfft;
    const int batch = (int)std::max<size_t>(1, std::min<size_t>((size_t)np, kSpecScratchBudget / row));
    // spectra [batch][nfft], then the split path's per-half bounds [2 batch]
    SARBP_CUDA(ctx, ctx->spec.ensure(row * (size_t)batch + sizeof(float) * 2 * (size_t)batch), "alloc spectrum scratch");
    float *bound2 = reinterpret_cast<float *>(static_cast<char *>(ctx->spec.ptr) + row * (size_t)batch);
    float *scale = scale_out;
    if (storage == SARBP_STORE_C32H && !scale) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "fp16 storage needs a scale array");
    const size_t esize = storage == SARBP_STORE_C64 ? 8 : 4;
    if (record_events) cudaEventRecord(ctx->ev[0], s);
    for (int p0 = 0; p0 < np; p0 += batch) {
        RcPlan plan{};
        plan.bound2 = bound2;
        plan.np = std::min(batch, np - p0);
        plan.ns = ns;
        plan.nfft = lay.nfft;
        plan.L = r->upsample;
        plan.nbins = lay.nbins;
        plan.storage = storage;
        SARBP_CUDA(ctx, sarbp::launch_rc_forward(plan, echo + (size_t)p0 * ns, ctx->tables.filt.as<float2>(),
                                                 ctx->tables.etab.as<float2>(), ctx->spec.as<float2>(),
                                                 scale ? scale + p0 : nullptr, s),
                   "range compression (forward)");
        SARBP_CUDA(ctx, sarbp::launch_rc_inverse(plan, ctx->spec.as<float2>(), ctx->tables.etab.as<float2>(),
                                                 scale ? scale + p0 : nullptr,
                                                 static_cast<char *>(rc_out) + (size_t)p0 * lay.nbins * esize, s),
                   "range compression (inverse)");
        ctx->launches += 2;
    }
    if (record_events) {
        cudaEventRecord(ctx->ev[1], s);
        ctx->timed_rc = true;
    }
    return SARBP_OK;
}

// Range compression of a host echo: the upload runs in pulse chunks on the
// context's copy stream and each chunk is range-compressed on `s` as soon as
// its copy lands, so only the first chunk's copy is not hidden.  The copy
// stream first waits for the work already on `s` (earlier users of the
// context's echo buffer).
sarbp_status rc_host_echo_enqueue(sarbp_ctx *ctx, const sarbp_radar *r, const sarbp_rc_layout &lay,
                                  const sarbp_complex64 *echo, int np, int ns, int storage, void *rc_out,
                                  float *scale_out, cudaStream_t s) {
    SARBP_CUDA(ctx, ctx->echo.ensure(sizeof(float2) * (size_t)np * ns), "alloc echo");
    float2 *d_echo = ctx->echo.as<float2>();
    const size_t row = sizeof(float2) * (size_t)ns;
    const int chunk = std::max(256, (np + 7) / 8);
    const size_t esize = storage == SARBP_STORE_C64 ? 8 : 4;
    SARBP_CUDA(ctx, cudaEventRecord(ctx->ev_copy, s), "order echo upload");
    SARBP_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_copy, 0), "order echo upload");
    cudaEventRecord(ctx->ev[0], s);
    for (int p0 = 0; p0 < np; p0 += chunk) {
        const int n = std::min(chunk, np - p0);
        SARBP_CUDA(ctx, cudaMemcpyAsync(d_echo + (size_t)p0 * ns, echo + (size_t)p0 * ns, row * n, cudaMemcpyHostToDevice,
                                        ctx->copy_stream),
                   "upload echo");
        // the wait binds to this record, so one event serves every chunk
        SARBP_CUDA(ctx, cudaEventRecord(ctx->ev_copy, ctx->copy_stream), "upload echo");
        SARBP_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_copy, 0), "upload echo");
        sarbp_status st = rc_device(ctx, r, lay, d_echo + (size_t)p0 * ns, n, ns, storage,
                                    static_cast<char *>(rc_out) + (size_t)p0 * lay.nbins * esize,
                                    scale_out ? scale_out + p0 : nullptr, s, false);
        if (st != SARBP_OK) return st;
    }
    cudaEventRecord(ctx->ev[1], s);
    ctx->timed_rc = true;
    return SARBP_OK;
}

// Waits for the echo uploads still reading the caller's host buffer: an error
// return must not leave copies in flight from memory the caller may free.
void drain_uploads(sarbp_ctx *ctx) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaGetLastError();
}

sarbp_status rc_host_echo(sarbp_ctx *ctx, const sarbp_radar *r, const sarbp_rc_layout &lay, const sarbp_complex64 *echo,
                          int np, int ns, int storage, void *rc_out, float *scale_out, cudaStream_t s) {
    Range range("sarbp: chunked echo upload + range compression");
    const sarbp_status st = rc_host_echo_enqueue(ctx, r, lay, echo, np, ns, storage, rc_out, scale_out, s);
    if (st != SARBP_OK) drain_uploads(ctx);
    return st;
}

sarbp_status check_grid(sarbp_ctx *ctx, const sarbp_grid *g) {
    if (!g) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "grid is null");
    if (g->nx < 0 || g->ny < 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "grid size must be >= 0");
    if ((long long)g->nx * g->ny > (1LL << 31)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "grid too large");
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(g->origin[i]) || !std::isfinite(g->ux[i]) || !std::isfinite(g->uy[i]))
            return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "grid vectors must be finite");
    return SARBP_OK;
}

// Geometry extremes for planning from a device-resident APC: a reduction on the
// stream (after the work already queued there, which may produce the APC), then
// a wait for its 40-byte result only.  Fails on a non-finite APC coordinate.
// Planning extremes in two halves: queue the reduction and its 40-byte
// read-back on s, then (after any work that does not need the plan has been
// queued behind it) wait for the read-back alone.
sarbp_status extremes_enqueue(sarbp_ctx *ctx, const double *apc_dev, int np, const sarbp_grid *g, cudaStream_t s) {
    Range range("sarbp: planning extremes");
    SARBP_CUDA(ctx, sarbp::launch_bp_extremes(apc_dev, np, *g, ctx->ext.as<unsigned long long>(), s),
               "planning extremes");
    ctx->launches += np > 0 ? 2 : 1;
    SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->ext_host, ctx->ext.ptr, 5 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
               "read planning extremes");
    SARBP_CUDA(ctx, cudaEventRecord(ctx->ev_ext, s), "read planning extremes");
    return SARBP_OK;
}

sarbp_status extremes_wait(sarbp_ctx *ctx, sarbp::BpExtremes &e) {
    SARBP_CUDA(ctx, cudaEventSynchronize(ctx->ev_ext), "read planning extremes");
    double v[4];  // squared range extremes, cosines
    std::memcpy(v, ctx->ext_host, sizeof v);
    sarbp::ext_ranges(v[0], v[1], e);
    e.cx = v[2];
    e.sy = v[3];
    e.nonfinite = ctx->ext_host[4] ? 1u : 0u;
    if (e.nonfinite) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "apc must be finite");
    return SARBP_OK;
}

sarbp_status extremes_device(sarbp_ctx *ctx, const double *apc_dev, int np, const sarbp_grid *g, cudaStream_t s,
                             sarbp::BpExtremes &e) {
    sarbp_status st = extremes_enqueue(ctx, apc_dev, np, g, s);
    return st != SARBP_OK ? st : extremes_wait(ctx, e);
}

// Back-projection of device-resident rc + apc into a device image.
sarbp_status bp_device(sarbp_ctx *ctx, const sarbp_radar *r, const sarbp_rc_view &rc, const double *apc_dev,
                       const sarbp::BpExtremes &ex, const sarbp_grid *g, int mode, float2 *image, int accumulate,
                       cudaStream_t s, const double *dr_dev = nullptr, const double *dph_dev = nullptr) {
    Range range("sarbp: back-projection");
    const int np = rc.np;
    if (g->nx == 0 || g->ny == 0) return SARBP_OK;
    if (np == 0) {
        if (!accumulate)
            SARBP_CUDA(ctx, cudaMemsetAsync(image, 0, sizeof(float2) * (size_t)g->nx * g->ny, s), "clear image");
        return SARBP_OK;
    }
    if (rc.nbins % 4 != 0) return fail(ctx, SARBP_ERR_UNSUPPORTED, "nbins must be a multiple of 4");
    if (((uintptr_t)rc.data & 15) != 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc data must be 16-byte aligned");
    BpPlan p;
    std::string why;
    if (!sarbp::plan_bp(ctx->sms, *r, rc, ex, np, *g, mode, 0, p, why, &ctx->tune))
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "%s", why.c_str());
    p.rc = rc.data;
    p.scale = rc.scale;
    p.np = np;
    p.apc = apc_dev;
    p.image = image;
    p.accumulate = accumulate;
    p.err = ctx->errword.as<unsigned>();
    p.drange = dr_dev;
    p.dphase = dph_dev;
    SARBP_CUDA(ctx, ctx->pref.ensure(sizeof(float) * 8 * (size_t)np), "alloc pulse references");
    p.pref = ctx->pref.as<float4>();
    if (p.segments > 1) {
        SARBP_CUDA(ctx, ctx->partial.ensure(sizeof(float2) * (size_t)p.segments * g->nx * g->ny),
                   "alloc partial images");
        p.partial = ctx->partial.as<float2>();
    }
    int launches = 0;
    cudaEventRecord(ctx->ev[2], s);
    SARBP_CUDA(ctx, sarbp::launch_bp(p, s, &launches), "back-projection launch");
    cudaEventRecord(ctx->ev[3], s);
    ctx->timed_bp = true;
    ctx->launches += launches;
    return SARBP_OK;
}

// Weighted projection of device-resident rc + apc against a device weight
// image into out[np] (device, complex128).
sarbp_status project_device(sarbp_ctx *ctx, const sarbp_radar *r, const sarbp_rc_view &rc, const double *apc_dev,
                            const sarbp::BpExtremes &ex, const sarbp_grid *g, int mode, const float2 *weight,
                            double2 *out, cudaStream_t s, const double *dr_dev, const double *dph_dev) {
    Range range("sarbp: weighted projection");
    const int np = rc.np;
    if (np == 0) return SARBP_OK;
    if (rc.nbins % 4 != 0) return fail(ctx, SARBP_ERR_UNSUPPORTED, "nbins must be a multiple of 4");
    if (((uintptr_t)rc.data & 15) != 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc data must be 16-byte aligned");
    BpPlan p;
    std::string why;
    if (!sarbp::plan_bp(ctx->sms, *r, rc, ex, np, *g, mode, 0, p, why, &ctx->tune))
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "%s", why.c_str());
    p.rc = rc.data;
    p.scale = rc.scale;
    p.np = np;
    p.apc = apc_dev;
    p.err = ctx->errword.as<unsigned>();
    p.checked = 0;  // the projection has no checked variant
    p.drange = dr_dev;
    p.dphase = dph_dev;
    p.weight = weight;
    SARBP_CUDA(ctx, ctx->pref.ensure(sizeof(float) * 8 * (size_t)np), "alloc pulse references");
    p.pref = ctx->pref.as<float4>();
    SARBP_CUDA(ctx, ctx->proj.ensure(sizeof(float2) * sarbp::bp_tiles(p) * (size_t)np), "alloc projection scratch");
    p.proj = ctx->proj.as<float2>();
    int launches = 0;
    SARBP_CUDA(ctx, sarbp::launch_project(p, out, s, &launches), "projection launch");
    ctx->launches += launches;
    return SARBP_OK;
}

// Device-side inputs of a back-projection-type call (uploads of host arrays
// into the context's buffers) after validation.
struct BpInputs {
    sarbp_rc_view v{};
    const double *apc_dev = nullptr;
    sarbp::BpExtremes ex{};
    const double *dr_dev = nullptr, *dph_dev = nullptr;
    bool any_host = false;
};

sarbp_status stage_bp_inputs(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_rc_view *rc, const double *apc,
                             const sarbp_grid *grid, int32_t mode, const sarbp_pulse_corr *corr, cudaStream_t s,
                             BpInputs &in) {
    sarbp_status st = check_radar(ctx, radar);
    if (st != SARBP_OK) return st;
    if (!rc) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc view is null");
    st = check_grid(ctx, grid);
    if (st != SARBP_OK) return st;
    if (mode < SARBP_MODE_FP64 || mode > SARBP_MODE_FP16STORE)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown mode %d", mode);
    if (rc->np < 0 || rc->nbins < 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "negative rc size");
    if (rc->storage != SARBP_STORE_C64 && rc->storage != SARBP_STORE_C32H)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown storage %d", rc->storage);
    if (mode == SARBP_MODE_FP16STORE && rc->storage != SARBP_STORE_C32H)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "FP16STORE mode needs SARBP_STORE_C32H data");
    if (!(rc->bin_rate > 0) || !std::isfinite(rc->t0_bins))
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc bin_rate must be > 0 and t0_bins finite");
    if (rc->np > 0 && (!rc->data || !apc)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc data and apc must be non-null");
    if (rc->np > 0 && rc->nbins < 2) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "nbins must be >= 2");
    if (rc->storage == SARBP_STORE_C32H && rc->np > 0 && !rc->scale)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "fp16 storage needs a scale array");
    const size_t esize = rc->storage == SARBP_STORE_C64 ? 8 : 4;
    const int np = rc->np;
    in.v = *rc;
    in.apc_dev = apc;
    if (np == 0) return SARBP_OK;
    // APC on the device for the kernel; the planner's extremes are reduced there
    if (!is_device_ptr(apc)) {
        SARBP_CUDA(ctx, ctx->apc.ensure(sizeof(double) * 3 * np), "alloc apc");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->apc.ptr, apc, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, s),
                   "upload apc");
        in.apc_dev = ctx->apc.as<double>();
        in.any_host = true;
    }
    st = extremes_device(ctx, in.apc_dev, np, grid, s, in.ex);
    if (st != SARBP_OK) return st;
    if (!is_device_ptr(rc->data)) {
        SARBP_CUDA(ctx, ctx->rc.ensure(esize * (size_t)np * rc->nbins), "alloc rc");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->rc.ptr, rc->data, esize * (size_t)np * rc->nbins, cudaMemcpyHostToDevice, s),
                   "upload rc");
        in.v.data = ctx->rc.ptr;
        in.any_host = true;
    }
    if (rc->storage == SARBP_STORE_C32H && !is_device_ptr(rc->scale)) {
        SARBP_CUDA(ctx, ctx->scale.ensure(sizeof(float) * np), "alloc scale");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->scale.ptr, rc->scale, sizeof(float) * np, cudaMemcpyHostToDevice, s),
                   "upload scale");
        in.v.scale = ctx->scale.as<float>();
        in.any_host = true;
    }
    if (corr && (corr->drange || corr->dphase)) {
        SARBP_CUDA(ctx, ctx->corr.ensure(sizeof(double) * 2 * (size_t)np), "alloc corrections");
        const double *src[2] = {corr->drange, corr->dphase};
        const double **dst[2] = {&in.dr_dev, &in.dph_dev};
        for (int k = 0; k < 2; ++k) {
            if (!src[k]) continue;
            if (is_device_ptr(src[k])) {
                *dst[k] = src[k];
            } else {
                for (int i = 0; i < np; ++i)
                    if (!std::isfinite(src[k][i]))
                        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "pulse corrections must be finite");
                double *d = ctx->corr.as<double>() + (size_t)k * np;
                SARBP_CUDA(ctx, cudaMemcpyAsync(d, src[k], sizeof(double) * np, cudaMemcpyHostToDevice, s),
                           "upload corrections");
                *dst[k] = d;
                in.any_host = true;
            }
        }
    }
    return SARBP_OK;
}

// DFT plan for rows of length n (tables cached per length in the context).
sarbp_status get_dft(sarbp_ctx *ctx, int n, sarbp::DftPlan &p) {
    if (!sarbp::dft_size_supported(n))
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "DFT length %d not supported (powers of two <= 16384, others <= 8192)", n);
    DftCache *slot = nullptr;
    for (auto &c : ctx->dft)
        if (c.n == n) slot = &c;
    if (!slot) {
        slot = &ctx->dft[0];
        for (auto &c : ctx->dft)
            if (c.used < slot->used) slot = &c;
        std::vector<float2> etab, chirp, kf, ki;
        sarbp::dft_tables_host(n, etab, chirp, kf, ki);
        slot->n = 0;
        SARBP_CUDA(ctx, slot->etab.ensure(sizeof(float2) * etab.size()), "alloc DFT tables");
        SARBP_CUDA(ctx, cudaMemcpy(slot->etab.ptr, etab.data(), sizeof(float2) * etab.size(), cudaMemcpyHostToDevice),
                   "upload DFT tables");
        slot->m = sarbp::dft_bluestein_size(n);
        if (slot->m) {
            SARBP_CUDA(ctx, slot->chirp.ensure(sizeof(float2) * n), "alloc DFT tables");
            SARBP_CUDA(ctx, slot->kf.ensure(sizeof(float2) * slot->m), "alloc DFT tables");
            SARBP_CUDA(ctx, slot->ki.ensure(sizeof(float2) * slot->m), "alloc DFT tables");
            SARBP_CUDA(ctx, cudaMemcpy(slot->chirp.ptr, chirp.data(), sizeof(float2) * n, cudaMemcpyHostToDevice),
                       "upload DFT tables");
            SARBP_CUDA(ctx, cudaMemcpy(slot->kf.ptr, kf.data(), sizeof(float2) * slot->m, cudaMemcpyHostToDevice),
                       "upload DFT tables");
            SARBP_CUDA(ctx, cudaMemcpy(slot->ki.ptr, ki.data(), sizeof(float2) * slot->m, cudaMemcpyHostToDevice),
                       "upload DFT tables");
        }
        slot->n = n;
    }
    slot->used = ++ctx->dft_clock;
    p.n = n;
    p.m = slot->m;
    p.etab = slot->etab.as<float2>();
    p.chirp = slot->chirp.as<float2>();
    p.kfwd = slot->kf.as<float2>();
    p.kinv = slot->ki.as<float2>();
    return SARBP_OK;
}

void wk_pads(int na, int nr, int *pa, int *pr) {
    // round(Na / 6.0f), round(Nr / 3.0f) as the reference computes them (float, half away from zero)
    *pa = (int)std::lround((float)na / 6.0f);
    *pr = (int)std::lround((float)nr / 3.0f);
}

std::mutex g_shim_mu;
sarbp_ctx *g_shim_ctx = nullptr;
int g_shim_dev = -1;

}  // namespace

extern "C" {

int sarbp_abi_version(void) { return SARBP_ABI_VERSION; }

const char *sarbp_status_string(sarbp_status s) {
    switch (s) {
        case SARBP_OK: return "ok";
        case SARBP_ERR_INVALID_ARGUMENT: return "invalid argument";
        case SARBP_ERR_UNSUPPORTED: return "unsupported";
        case SARBP_ERR_OUT_OF_MEMORY: return "out of memory";
        case SARBP_ERR_CUDA: return "CUDA error";
        case SARBP_ERR_NO_DEVICE: return "no usable device";
        case SARBP_ERR_TIMEOUT: return "device wait timed out";
        case SARBP_ERR_DEVICE_CHECK: return "device-side check failed";
        case SARBP_ERR_NOT_READY: return "not ready";
        case SARBP_ERR_CANCELLED: return "cancelled";
        case SARBP_ERR_BUDGET: return "over memory budget";
        case SARBP_ERR_INTERNAL: return "internal error";
    }
    return "unknown status";
}

sarbp_status sarbp_create(sarbp_ctx **out, int device) {
    if (!out) return SARBP_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return SARBP_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return SARBP_ERR_INVALID_ARGUMENT;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return SARBP_ERR_NO_DEVICE;
    if (prop.major * 10 + prop.minor != 103) return SARBP_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return SARBP_ERR_NO_DEVICE;
    sarbp_ctx *ctx = new sarbp_ctx();
    ctx->device = device;
    ctx->sms = prop.multiProcessorCount;
    bool ok = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) == cudaSuccess;
    for (int i = 0; i < 4 && ok; ++i) ok = cudaEventCreate(&ctx->ev[i]) == cudaSuccess;
    // the planning read-back waits for the stream's earlier work (a whole
    // back-projection when calls come back to back): a blocking wait sleeps
    // and wakes on completion instead of spinning a core for that long, which
    // a busy host may preempt for a scheduler slice
    ok = ok && cudaEventCreateWithFlags(&ctx->ev_ext, cudaEventDisableTiming | cudaEventBlockingSync) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && cudaMallocHost(reinterpret_cast<void **>(&ctx->ext_host), 8 * sizeof(unsigned long long)) == cudaSuccess;
    ok = ok && ctx->ext.ensure(8 * sizeof(unsigned long long)) == cudaSuccess;
    ok = ok && ctx->errword.ensure(sizeof(unsigned)) == cudaSuccess && ctx->power.ensure(sizeof(double)) == cudaSuccess;
    ok = ok && cudaMemset(ctx->errword.ptr, 0, sizeof(unsigned)) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        sarbp_destroy(ctx);
        return SARBP_ERR_CUDA;
    }
    *out = ctx;
    return SARBP_OK;
}

sarbp_status sarbp_destroy(sarbp_ctx *ctx) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->release_scratch();
    for (DevBuf *b : ctx->persistent()) b->release();
    if (ctx->ext_host) cudaFreeHost(ctx->ext_host);
    for (cudaEvent_t &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->ev_ext) cudaEventDestroy(ctx->ev_ext);
    if (ctx->wkc.ready) cudaEventDestroy(ctx->wkc.ready);
    if (ctx->ceos_ready) cudaEventDestroy(ctx->ceos_ready);
    if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SARBP_OK;
}

const char *sarbp_last_error(const sarbp_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

sarbp_status sarbp_synchronize(sarbp_ctx *ctx) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    SARBP_CUDA(ctx, cudaDeviceSynchronize(), "device synchronize");
    if (ctx->timed_rc) cudaEventElapsedTime(&ctx->rc_ms, ctx->ev[0], ctx->ev[1]);
    if (ctx->timed_bp) cudaEventElapsedTime(&ctx->bp_ms, ctx->ev[2], ctx->ev[3]);
    return check_errword(ctx);
}

sarbp_status sarbp_trim(sarbp_ctx *ctx) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->release_scratch();
    return SARBP_OK;
}

size_t sarbp_device_bytes(const sarbp_ctx *ctx) {
    if (!ctx) return 0;
    size_t t = 0;
    sarbp_ctx *c = const_cast<sarbp_ctx *>(ctx);
    for (const DevBuf *b : c->scratch()) t += b->bytes;
    for (const DevBuf *b : c->persistent()) t += b->bytes;
    return t;
}

sarbp_status sarbp_rc_layout_get(const sarbp_radar *radar, int32_t ns, sarbp_rc_layout *out) {
    if (!out) return SARBP_ERR_INVALID_ARGUMENT;
    return layout(nullptr, radar, ns, out);
}

sarbp_status sarbp_range_compress(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_complex64 *echo,
                                  int32_t np, int32_t ns, int32_t storage, void *rc_out, float *rc_scale_out,
                                  void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    sarbp_rc_layout lay;
    sarbp_status st = layout(ctx, radar, ns, &lay);
    if (st != SARBP_OK) return st;
    if (np < 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "np must be >= 0");
    if (storage != SARBP_STORE_C64 && storage != SARBP_STORE_C32H)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown storage %d", storage);
    if (np == 0) return SARBP_OK;
    if (!echo || !rc_out) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "echo and rc_out must be non-null");
    if (storage == SARBP_STORE_C32H && !rc_scale_out)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "fp16 storage needs rc_scale_out");
    cudaStream_t s = pick_stream(ctx, stream);
    const size_t esize = storage == SARBP_STORE_C64 ? 8 : 4;
    const bool dev_in = is_device_ptr(echo), dev_out = is_device_ptr(rc_out);
    const bool dev_sc = storage == SARBP_STORE_C64 || is_device_ptr(rc_scale_out);
    const float2 *d_echo = reinterpret_cast<const float2 *>(echo);
    void *d_rc = rc_out;
    if (!dev_out) {
        SARBP_CUDA(ctx, ctx->rc.ensure(esize * (size_t)np * lay.nbins), "alloc rc");
        d_rc = ctx->rc.ptr;
    }
    float *d_scale = rc_scale_out;
    if (storage == SARBP_STORE_C32H && !dev_sc) {
        SARBP_CUDA(ctx, ctx->scale.ensure(sizeof(float) * np), "alloc scale");
        d_scale = ctx->scale.as<float>();
    }
    ctx->timed_bp = false;
    st = dev_in ? rc_device(ctx, radar, lay, d_echo, np, ns, storage, d_rc, storage == SARBP_STORE_C32H ? d_scale : nullptr, s)
                : rc_host_echo(ctx, radar, lay, echo, np, ns, storage, d_rc, storage == SARBP_STORE_C32H ? d_scale : nullptr, s);
    if (st != SARBP_OK) return st;
    if (!dev_out)
        SARBP_CUDA(ctx, cudaMemcpyAsync(rc_out, d_rc, esize * (size_t)np * lay.nbins, cudaMemcpyDeviceToHost, s),
                   "download rc");
    if (storage == SARBP_STORE_C32H && !dev_sc)
        SARBP_CUDA(ctx, cudaMemcpyAsync(rc_scale_out, d_scale, sizeof(float) * np, cudaMemcpyDeviceToHost, s),
                   "download scale");
    return finish(ctx, s, !dev_in || !dev_out || !dev_sc);
}

sarbp_status sarbp_backproject_ex(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_rc_view *rc,
                                  const double *apc, const sarbp_grid *grid, int32_t mode,
                                  const sarbp_pulse_corr *corr, sarbp_complex64 *image, int32_t accumulate,
                                  void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    cudaStream_t s = pick_stream(ctx, stream);
    if (grid && (size_t)grid->nx * grid->ny > 0 && !image)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "image is null");
    BpInputs in;
    sarbp_status st = stage_bp_inputs(ctx, radar, rc, apc, grid, mode, corr, s, in);
    if (st != SARBP_OK) return st;
    const size_t npix = (size_t)grid->nx * grid->ny;
    if (npix == 0) return SARBP_OK;
    float2 *d_img = reinterpret_cast<float2 *>(image);
    const bool dev_img = is_device_ptr(image);
    bool any_host = in.any_host;
    if (!dev_img) {
        SARBP_CUDA(ctx, ctx->image.ensure(sizeof(float2) * npix), "alloc image");
        d_img = ctx->image.as<float2>();
        if (accumulate)
            SARBP_CUDA(ctx, cudaMemcpyAsync(d_img, image, sizeof(float2) * npix, cudaMemcpyHostToDevice, s), "upload image");
        any_host = true;
    }
    ctx->timed_rc = false;
    st = bp_device(ctx, radar, in.v, in.apc_dev, in.ex, grid, mode, d_img, accumulate, s, in.dr_dev, in.dph_dev);
    if (st != SARBP_OK) return st;
    if (!dev_img)
        SARBP_CUDA(ctx, cudaMemcpyAsync(image, d_img, sizeof(float2) * npix, cudaMemcpyDeviceToHost, s), "download image");
    return finish(ctx, s, any_host);
}

sarbp_status sarbp_bp_plan(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_rc_view *rc, const double *apc,
                           const sarbp_grid *grid, int32_t mode, int32_t host_reduction, sarbp_bp_plan_info *out) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    if (!out) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "out is null");
    std::memset(out, 0, sizeof *out);
    sarbp_status st = check_radar(ctx, radar);
    if (st != SARBP_OK) return st;
    if (!rc) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc view is null");
    st = check_grid(ctx, grid);
    if (st != SARBP_OK) return st;
    if (grid->nx < 1 || grid->ny < 1) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "grid must have pixels");
    if (mode < SARBP_MODE_FP64 || mode > SARBP_MODE_FP16STORE)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown mode %d", mode);
    if (rc->storage != SARBP_STORE_C64 && rc->storage != SARBP_STORE_C32H)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown storage %d", rc->storage);
    if (mode == SARBP_MODE_FP16STORE && rc->storage != SARBP_STORE_C32H)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "FP16STORE mode needs SARBP_STORE_C32H data");
    if (rc->np < 1 || rc->nbins < 2 || rc->nbins % 4 != 0)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc needs np >= 1 and nbins >= 2, a multiple of 4");
    if (!(rc->bin_rate > 0) || !std::isfinite(rc->t0_bins))
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rc bin_rate must be > 0 and t0_bins finite");
    if (!apc) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "apc is null");
    const int np = rc->np;
    sarbp::BpExtremes ex{};
    if (host_reduction) {
        if (is_device_ptr(apc)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "host_reduction needs a host apc");
        sarbp::bp_extremes_host(apc, np, *grid, ex);
        if (ex.nonfinite) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "apc must be finite");
    } else {
        const double *apc_dev = apc;
        if (!is_device_ptr(apc)) {
            SARBP_CUDA(ctx, ctx->apc.ensure(sizeof(double) * 3 * np), "alloc apc");
            SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->apc.ptr, apc, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, ctx->stream),
                       "upload apc");
            apc_dev = ctx->apc.as<double>();
        }
        st = extremes_device(ctx, apc_dev, np, grid, ctx->stream, ex);
        if (st != SARBP_OK) return st;
    }
    sarbp::BpPlan p;
    std::string why;
    if (!sarbp::plan_bp(ctx->sms, *radar, *rc, ex, np, *grid, mode, 0, p, why, &ctx->tune))
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "%s", why.c_str());
    int occ = 0;
    SARBP_CUDA(ctx, sarbp::bp_occupancy(p, &occ), "occupancy");
    sarbp::bp_tile_dims(p.pix, &out->tile_x, &out->tile_y);
    out->window = p.win;
    out->series_terms = p.nterms;
    out->segments = p.segments;
    out->ctas_per_sm = occ;
    out->pulse_chunk = p.chunk;
    out->linear_phase = p.lin;
    out->smem_bytes = sarbp::bp_smem_bytes(p.storage, p.win, p.chunk);
    out->rmin = ex.rmin;
    out->rmax = ex.rmax;
    out->cos_x = ex.cx;
    out->cos_y = ex.sy;
    return SARBP_OK;
}

sarbp_status sarbp_backproject(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_rc_view *rc,
                               const double *apc, const sarbp_grid *grid, int32_t mode, sarbp_complex64 *image,
                               int32_t accumulate, void *stream) {
    return sarbp_backproject_ex(ctx, radar, rc, apc, grid, mode, nullptr, image, accumulate, stream);
}

sarbp_status sarbp_project_weighted(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_rc_view *rc,
                                    const double *apc, const sarbp_grid *grid, int32_t mode,
                                    const sarbp_pulse_corr *corr, const sarbp_complex64 *weight, double *out,
                                    void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    if (mode != SARBP_MODE_SPLIT && mode != SARBP_MODE_FP16STORE)
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "weighted projection runs in SPLIT or FP16STORE mode");
    cudaStream_t s = pick_stream(ctx, stream);
    BpInputs in;
    sarbp_status st = stage_bp_inputs(ctx, radar, rc, apc, grid, mode, corr, s, in);
    if (st != SARBP_OK) return st;
    const int np = rc->np;
    if (np == 0) return SARBP_OK;
    if (!out) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "out is null");
    const size_t npix = (size_t)grid->nx * grid->ny;
    bool any_host = in.any_host;
    double2 *d_out = reinterpret_cast<double2 *>(out);
    const bool dev_out = is_device_ptr(out);
    if (!dev_out) {
        SARBP_CUDA(ctx, ctx->projout.ensure(sizeof(double2) * np), "alloc projection output");
        d_out = ctx->projout.as<double2>();
        any_host = true;
    }
    if (npix == 0) {
        SARBP_CUDA(ctx, cudaMemsetAsync(d_out, 0, sizeof(double2) * np, s), "clear projection");
    } else {
        if (!weight) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "weight is null");
        const float2 *d_w = reinterpret_cast<const float2 *>(weight);
        if (!is_device_ptr(weight)) {
            SARBP_CUDA(ctx, ctx->weight.ensure(sizeof(float2) * npix), "alloc weight");
            SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->weight.ptr, weight, sizeof(float2) * npix, cudaMemcpyHostToDevice, s),
                       "upload weight");
            d_w = ctx->weight.as<float2>();
            any_host = true;
        }
        st = project_device(ctx, radar, in.v, in.apc_dev, in.ex, grid, mode, d_w, d_out, s, in.dr_dev,
                            in.dph_dev);
        if (st != SARBP_OK) return st;
    }
    if (!dev_out)
        SARBP_CUDA(ctx, cudaMemcpyAsync(out, d_out, sizeof(double2) * np, cudaMemcpyDeviceToHost, s), "download projection");
    return finish(ctx, s, any_host);
}

sarbp_status sarbp_autofocus(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_rc_view *rc, const double *apc,
                             const sarbp_grid *grid, int32_t mode, int32_t iterations, const double *drange,
                             double *dphase, sarbp_complex64 *image, double *sharpness, void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_autofocus");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    if (mode != SARBP_MODE_SPLIT && mode != SARBP_MODE_FP16STORE)
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "autofocus runs in SPLIT or FP16STORE mode");
    if (iterations < 0 || iterations > 1000) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "iterations out of range");
    if (!dphase) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "dphase is null");
    if (is_device_ptr(dphase) || (drange && is_device_ptr(drange)) || (sharpness && is_device_ptr(sharpness)))
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "dphase, drange and sharpness are host arrays");
    cudaStream_t s = pick_stream(ctx, stream);
    sarbp_pulse_corr c0{drange, nullptr};
    BpInputs in;
    sarbp_status st = stage_bp_inputs(ctx, radar, rc, apc, grid, mode, &c0, s, in);
    if (st != SARBP_OK) return st;
    const int np = rc->np;
    const size_t npix = (size_t)grid->nx * grid->ny;
    if (np == 0 || npix == 0) return finish(ctx, s, true);
    std::vector<double> ph(dphase, dphase + np);
    for (double v : ph)
        if (!std::isfinite(v)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "dphase must be finite");
    // device state: phases (in the second half of the correction buffer, which
    // stage_bp_inputs sized for 2 np), image, weights, projection, sharpness partials
    SARBP_CUDA(ctx, ctx->corr.ensure(sizeof(double) * 2 * (size_t)np), "alloc corrections");
    double *d_ph = ctx->corr.as<double>() + np;
    const bool dev_img = is_device_ptr(image);
    float2 *d_img = dev_img ? reinterpret_cast<float2 *>(image) : nullptr;
    if (!dev_img) {
        SARBP_CUDA(ctx, ctx->image.ensure(sizeof(float2) * npix), "alloc image");
        d_img = ctx->image.as<float2>();
    }
    SARBP_CUDA(ctx, ctx->weight.ensure(sizeof(float2) * npix), "alloc weight");
    SARBP_CUDA(ctx, ctx->projout.ensure(sizeof(double2) * np), "alloc projection output");
    const int nb = sarbp::sharpness_blocks(npix);
    SARBP_CUDA(ctx, ctx->sharp.ensure(sizeof(double) * nb), "alloc sharpness");
    std::vector<double2> cp(np);
    std::vector<double> part(nb);
    float2 *d_w = ctx->weight.as<float2>();
    for (int it = 0; it <= iterations; ++it) {
        SARBP_CUDA(ctx, cudaMemcpyAsync(d_ph, ph.data(), sizeof(double) * np, cudaMemcpyHostToDevice, s), "upload phases");
        st = bp_device(ctx, radar, in.v, in.apc_dev, in.ex, grid, mode, d_img, 0, s, in.dr_dev, d_ph);
        if (st != SARBP_OK) return st;
        const bool last = it == iterations;
        SARBP_CUDA(ctx, sarbp::launch_sharpness_weight(d_img, npix, last ? nullptr : d_w, ctx->sharp.as<double>(), s),
                   "sharpness");
        ctx->launches += 1;
        if (!last) {
            st = project_device(ctx, radar, in.v, in.apc_dev, in.ex, grid, mode, d_w, ctx->projout.as<double2>(),
                                s, in.dr_dev, d_ph);
            if (st != SARBP_OK) return st;
            SARBP_CUDA(ctx, cudaMemcpyAsync(cp.data(), ctx->projout.ptr, sizeof(double2) * np, cudaMemcpyDeviceToHost, s),
                       "download projection");
        }
        SARBP_CUDA(ctx, cudaMemcpyAsync(part.data(), ctx->sharp.ptr, sizeof(double) * nb, cudaMemcpyDeviceToHost, s),
                   "download sharpness");
        SARBP_CUDA(ctx, cudaStreamSynchronize(s), "autofocus iteration");
        st = check_errword(ctx);
        if (st != SARBP_OK) return st;
        double sum = 0.0;
        for (double v : part) sum += v;
        if (sharpness) sharpness[it] = sum;
        if (last) break;
        double mean = 0.0;
        for (int p = 0; p < np; ++p) {
            ph[p] -= std::atan2(cp[p].y, cp[p].x);
            mean += ph[p];
        }
        mean /= np;
        for (int p = 0; p < np; ++p) ph[p] -= mean;
    }
    std::copy(ph.begin(), ph.end(), dphase);
    if (image && !dev_img)
        SARBP_CUDA(ctx, cudaMemcpyAsync(image, d_img, sizeof(float2) * npix, cudaMemcpyDeviceToHost, s), "download image");
    return finish(ctx, s, true);
}

sarbp_status sarbp_wk_padded_size(int32_t na, int32_t nr, int32_t *na_pad, int32_t *nr_pad) {
    if (na <= 0 || nr <= 0 || !na_pad || !nr_pad) return SARBP_ERR_INVALID_ARGUMENT;
    int pa, pr;
    wk_pads(na, nr, &pa, &pr);
    const long long NA = (long long)na + 2LL * pa, NR = (long long)nr + 2LL * pr;
    if (NA > (1 << 30) || NR > (1 << 30)) return SARBP_ERR_UNSUPPORTED;
    *na_pad = (int32_t)NA;
    *nr_pad = (int32_t)NR;
    return sarbp::dft_size_supported((int)NA) && sarbp::dft_size_supported((int)NR) ? SARBP_OK : SARBP_ERR_UNSUPPORTED;
}

sarbp_status sarbp_dft(sarbp_ctx *ctx, sarbp_complex64 *data, int32_t rows, int32_t n, int32_t inverse, void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_dft");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    if (rows < 0 || n < 1) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "rows must be >= 0 and n >= 1");
    if (rows == 0 || n == 1) return SARBP_OK;
    if (!data) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "data is null");
    sarbp::DftPlan p;
    sarbp_status st = get_dft(ctx, n, p);
    if (st != SARBP_OK) return st;
    cudaStream_t s = pick_stream(ctx, stream);
    const size_t bytes = sizeof(float2) * (size_t)rows * n;
    float2 *d = reinterpret_cast<float2 *>(data);
    const bool dev = is_device_ptr(data);
    if (!dev) {
        SARBP_CUDA(ctx, ctx->wk0.ensure(bytes), "alloc DFT buffer");
        d = ctx->wk0.as<float2>();
        SARBP_CUDA(ctx, cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, s), "upload DFT rows");
    }
    SARBP_CUDA(ctx, sarbp::launch_dft_rows(p, d, rows, n, inverse != 0, inverse ? 1.0f / (float)n : 1.0f, s),
               "DFT launch");
    ctx->launches += 1;
    if (!dev) SARBP_CUDA(ctx, cudaMemcpyAsync(data, d, bytes, cudaMemcpyDeviceToHost, s), "download DFT rows");
    return finish(ctx, s, !dev);
}

sarbp_status sarbp_dft2d(sarbp_ctx *ctx, sarbp_complex64 *data, int32_t na, int32_t nr, int32_t inverse,
                         void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_dft2d");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    if (na < 1 || nr < 1) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "na and nr must be >= 1");
    if ((long long)na * nr > (1LL << 31)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "array too large");
    if (!data) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "data is null");
    if (na == 1 && nr == 1) return SARBP_OK;
    sarbp::DftPlan pr{}, pa{};
    sarbp_status st;
    if (nr > 1 && (st = get_dft(ctx, nr, pr)) != SARBP_OK) return st;
    if (na > 1 && (st = get_dft(ctx, na, pa)) != SARBP_OK) return st;
    if (nr > 1 && na > 1 && na != nr && (st = get_dft(ctx, nr, pr)) != SARBP_OK) return st;  // both still cached
    cudaStream_t s = pick_stream(ctx, stream);
    const size_t bytes = sizeof(float2) * (size_t)na * nr;
    float2 *d = reinterpret_cast<float2 *>(data);
    const bool dev = is_device_ptr(data);
    if (!dev) {
        SARBP_CUDA(ctx, ctx->wk0.ensure(bytes), "alloc DFT buffer");
        d = ctx->wk0.as<float2>();
        SARBP_CUDA(ctx, cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, s), "upload DFT array");
    }
    const bool inv = inverse != 0;
    if (nr > 1) {  // range: along the rows
        SARBP_CUDA(ctx, sarbp::launch_dft_rows(pr, d, na, nr, inv, inv ? 1.0f / (float)nr : 1.0f, s), "row DFT");
        ctx->launches += 1;
    }
    if (na > 1) {  // azimuth: down the columns, through transposes where the column kernel does not apply
        const float sc = inv ? 1.0f / (float)na : 1.0f;
        if (sarbp::dft_cols_supported(pa)) {
            SARBP_CUDA(ctx, sarbp::launch_dft_cols(pa, d, d, nr, inv, sc, s), "column DFT");
            ctx->launches += 1;
        } else {
            SARBP_CUDA(ctx, ctx->wk1.ensure(bytes), "alloc transpose buffer");
            float2 *t = ctx->wk1.as<float2>();
            SARBP_CUDA(ctx, sarbp::launch_transpose(d, t, na, nr, s), "transpose");
            SARBP_CUDA(ctx, sarbp::launch_dft_rows(pa, t, nr, na, inv, sc, s), "column DFT");
            SARBP_CUDA(ctx, sarbp::launch_transpose(t, d, nr, na, s), "transpose");
            ctx->launches += 3;
        }
    }
    if (!dev) SARBP_CUDA(ctx, cudaMemcpyAsync(data, d, bytes, cudaMemcpyDeviceToHost, s), "download DFT array");
    return finish(ctx, s, !dev);
}

// Omega-K parameter checks shared by the pipeline and its stage entry points.
sarbp_status wk_check_params(sarbp_ctx *ctx, const sarbp_wk_params *w) {
    if (!w) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "params is null");
    const double vals[8] = {w->fr, w->prf, w->f0, w->r0, w->kr, w->c, w->vr, w->f_nc};
    for (double v : vals)
        if (!std::isfinite(v)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "omega-K parameters must be finite");
    if (!(w->fr > 0) || !(w->prf > 0) || !(w->f0 > 0) || !(w->c > 0) || !(w->vr > 0) || w->kr == 0.0)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "fr, prf, f0, c, vr must be > 0 and kr != 0");
    if (w->taps < 1 || w->taps > 32) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "taps must be in [1, 32]");
    return SARBP_OK;
}

// Device tables of the omega-K stages for a padded size NA x NR (built on the
// host in FP64, uploaded on s): row phasors of the azimuth down-conversion, the
// Stolt terms per row and column (float-float), and the FP64 tables of the
// FP64 Stolt path.
sarbp_status wk_tables(sarbp_ctx *ctx, const sarbp_wk_params *w, int NA, int NR, cudaStream_t s, WkTables &t) {
    constexpr double kPi = 3.14159265358979323846;
    WkCache &k = ctx->wkc;
    if (k.valid && k.NA == NA && k.NR == NR && k.fr == w->fr && k.prf == w->prf && k.f0 == w->f0 && k.r0 == w->r0 &&
        k.kr == w->kr && k.c == w->c && k.vr == w->vr && k.f_nc == w->f_nc) {
        SARBP_CUDA(ctx, cudaStreamWaitEvent(s, k.ready, 0), "omega-K tables");
        t = k.t;
        return SARBP_OK;
    }
    k.valid = false;
    // host tables (FP64): row phasors exp(-j 2 pi f_nc ta_m), ta_m = (m - NA/2) / prf;
    // frequency axes as the reference builds them (fftshifted index, wk.cc:181-205)
    const double a4r = 4.0 * kPi * w->r0 / w->c;
    std::vector<float2> rowphase(NA), row_qf(NA), col_ip(NR);
    std::vector<float> col_c(NR);
    std::vector<double> tab(3 * (size_t)NR + NA);
    double *col_f2 = tab.data(), *col_ph = col_f2 + NR, *col_fr = col_ph + NR, *row_q = col_fr + NR;
    double qmax = 0.0, pmin = 1e300;
    for (int m = 0; m < NA; ++m) {
        const double ta = (double)(m - NA / 2) / w->prf;
        const double cyc = -w->f_nc * ta;
        const double a = 2.0 * kPi * (cyc - std::nearbyint(cyc));
        rowphase[m] = make_float2((float)std::cos(a), (float)std::sin(a));
        const int idx = m < NA / 2 ? m + NA / 2 : m - NA / 2;
        const double fa = w->f_nc + (double)(idx - NA / 2) * (w->prf / NA);
        row_q[m] = w->c * w->c / (4.0 * w->vr * w->vr) * fa * fa;
        const float qh = (float)row_q[m];
        row_qf[m] = make_float2(qh, (float)(row_q[m] - (double)qh));
        qmax = std::max(qmax, row_q[m]);
    }
    for (int n = 0; n < NR; ++n) {
        const int idx = n < NR / 2 ? n + NR / 2 : n - NR / 2;
        const double fr = (double)(idx - NR / 2) * (w->fr / NR);
        const double P = w->f0 + fr;
        col_f2[n] = P * P;
        col_ph[n] = kPi * fr * fr / w->kr;
        col_fr[n] = fr;
        const double th = a4r * P + col_ph[n];
        col_c[n] = (float)(th - 2.0 * kPi * std::nearbyint(th / (2.0 * kPi)));
        const double ip = 1.0 / P;
        const float iph = (float)ip;
        col_ip[n] = make_float2(iph, (float)(ip - (double)iph));
        pmin = std::min(pmin, P);
    }
    // float-float Stolt stage when the mapping is a small correction (eps <= 1e-2), else FP64
    const bool ff_stolt = pmin > 0.0 && qmax / (pmin * pmin) <= 1e-2;
    const size_t row_bytes = sizeof(float2) * 2 * NA, col_bytes = (sizeof(float) + sizeof(float2)) * NR;
    SARBP_CUDA(ctx, k.row.ensure(row_bytes + col_bytes), "alloc omega-K tables");
    SARBP_CUDA(ctx, k.tab.ensure(sizeof(double) * tab.size()), "alloc omega-K tables");
    float2 *d_rowphase = k.row.as<float2>(), *d_rowq = d_rowphase + NA, *d_colip = d_rowq + NA;
    float *d_colc = reinterpret_cast<float *>(d_colip + NR);
    SARBP_CUDA(ctx, cudaMemcpyAsync(d_rowphase, rowphase.data(), sizeof(float2) * NA, cudaMemcpyHostToDevice, s),
               "upload omega-K tables");
    SARBP_CUDA(ctx, cudaMemcpyAsync(d_rowq, row_qf.data(), sizeof(float2) * NA, cudaMemcpyHostToDevice, s),
               "upload omega-K tables");
    SARBP_CUDA(ctx, cudaMemcpyAsync(d_colip, col_ip.data(), sizeof(float2) * NR, cudaMemcpyHostToDevice, s),
               "upload omega-K tables");
    SARBP_CUDA(ctx, cudaMemcpyAsync(d_colc, col_c.data(), sizeof(float) * NR, cudaMemcpyHostToDevice, s),
               "upload omega-K tables");
    SARBP_CUDA(ctx, cudaMemcpyAsync(k.tab.ptr, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, s),
               "upload omega-K tables");
    if (!k.ready) SARBP_CUDA(ctx, cudaEventCreateWithFlags(&k.ready, cudaEventDisableTiming), "omega-K tables");
    SARBP_CUDA(ctx, cudaEventRecord(k.ready, s), "omega-K tables");
    t.tab = k.tab.as<double>();
    t.rowphase = d_rowphase;
    t.rowq = d_rowq;
    t.colip = d_colip;
    t.colc = d_colc;
    t.a4r = a4r;
    t.ff = ff_stolt;
    k.t = t;
    k.NA = NA;
    k.NR = NR;
    k.fr = w->fr;
    k.prf = w->prf;
    k.f0 = w->f0;
    k.r0 = w->r0;
    k.kr = w->kr;
    k.c = w->c;
    k.vr = w->vr;
    k.f_nc = w->f_nc;
    k.valid = true;
    return SARBP_OK;
}

// Reference-function multiply and Stolt mapping of a 2-D spectrum [NA][NR].
sarbp_status wk_focus_launch(sarbp_ctx *ctx, const sarbp_wk_params *w, const WkTables &t, const float2 *in,
                             float2 *out, int NA, int NR, cudaStream_t s) {
    const double *d_tab = t.tab;
    if (t.ff)
        SARBP_CUDA(ctx, sarbp::launch_wk_stolt_ff(in, out, NA, NR, t.colc, t.colip, t.rowq, t.a4r, NR / w->fr, w->taps, s),
                   "reference-function multiply and Stolt mapping");
    else
        SARBP_CUDA(ctx, sarbp::launch_wk_stolt(in, out, NA, NR, d_tab, d_tab + NR, d_tab + 2 * NR, d_tab + 3 * NR, t.a4r,
                                                w->f0, NR / w->fr, w->taps, s),
                   "reference-function multiply and Stolt mapping");
    ctx->launches += 1;
    return SARBP_OK;
}

sarbp_status sarbp_wk_image(sarbp_ctx *ctx, const sarbp_wk_params *w, const sarbp_complex64 *echo, int32_t na,
                            int32_t nr, sarbp_complex64 *image, void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_wk_image");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    sarbp_status st = wk_check_params(ctx, w);
    if (st != SARBP_OK) return st;
    if (na <= 0 || nr <= 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "echo size must be > 0");
    if (!echo || !image) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "echo and image must be non-null");
    int32_t NA, NR;
    if (sarbp_wk_padded_size(na, nr, &NA, &NR) != SARBP_OK)
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "padded size %d x %d not supported", NA, NR);
    if (sarbp::wk_stolt_smem(NR) > (size_t)(227u << 10))
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "range size %d too large for the Stolt stage", NR);
    int pa, pr;
    wk_pads(na, nr, &pa, &pr);
    sarbp::DftPlan pa_plan, pr_plan;
    st = get_dft(ctx, NR, pr_plan);
    if (st != SARBP_OK) return st;
    st = get_dft(ctx, NA, pa_plan);
    if (st != SARBP_OK) return st;
    cudaStream_t s = pick_stream(ctx, stream);
    WkTables tb;
    st = wk_tables(ctx, w, NA, NR, s, tb);
    if (st != SARBP_OK) return st;
    const size_t npix = (size_t)NA * NR;
    SARBP_CUDA(ctx, ctx->wk0.ensure(sizeof(float2) * npix), "alloc omega-K buffer");
    SARBP_CUDA(ctx, ctx->wk1.ensure(sizeof(float2) * npix), "alloc omega-K buffer");
    float2 *d_rowphase = tb.rowphase;
    const float2 *d_echo = reinterpret_cast<const float2 *>(echo);
    bool any_host = true;  // the host tables above are staged through pageable memory
    if (!is_device_ptr(echo)) {
        SARBP_CUDA(ctx, ctx->echo.ensure(sizeof(float2) * (size_t)na * nr), "alloc echo");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->echo.ptr, echo, sizeof(float2) * (size_t)na * nr, cudaMemcpyHostToDevice, s),
                   "upload echo");
        d_echo = ctx->echo.as<float2>();
    }
    float2 *A = ctx->wk0.as<float2>(), *B = ctx->wk1.as<float2>();
    const bool dev_img = is_device_ptr(image);
    float2 *out = dev_img ? reinterpret_cast<float2 *>(image) : B;
    cudaEventRecord(ctx->ev[0], s);
    // padding rows stay zero through the range FFT; the echo rows are padded,
    // down-converted and transformed in one pass
    SARBP_CUDA(ctx, cudaMemsetAsync(A, 0, sizeof(float2) * (size_t)pa * NR, s), "clear padding");
    SARBP_CUDA(ctx, cudaMemsetAsync(A + (size_t)(pa + na) * NR, 0, sizeof(float2) * (size_t)(NA - pa - na) * NR, s),
               "clear padding");
    sarbp::DftIo io;
    io.src = d_echo;
    io.src_cols = nr;
    io.col0 = pr;
    io.rowmul = d_rowphase + pa;
    SARBP_CUDA(ctx, sarbp::launch_dft_rows(pr_plan, A + (size_t)pa * NR, na, NR, false, 1.0f, s, io), "range FFT");
    // azimuth transforms: down the columns in place (power-of-two lengths up to
    // 4096), else through transposes
    const bool cols = sarbp::dft_cols_supported(pa_plan);
    if (cols) {
        SARBP_CUDA(ctx, sarbp::launch_dft_cols(pa_plan, A, A, NR, false, 1.0f, s), "azimuth FFT");
    } else {
        SARBP_CUDA(ctx, sarbp::launch_transpose(A, B, NA, NR, s), "transpose");
        SARBP_CUDA(ctx, sarbp::launch_dft_rows(pa_plan, B, NR, NA, false, 1.0f, s), "azimuth FFT");
        SARBP_CUDA(ctx, sarbp::launch_transpose(B, A, NR, NA, s), "transpose");
    }
    st = wk_focus_launch(ctx, w, tb, A, B, NA, NR, s);
    if (st != SARBP_OK) return st;
    SARBP_CUDA(ctx, sarbp::launch_dft_rows(pr_plan, B, NA, NR, true, 1.0f / (float)NR, s), "range IFFT");
    if (cols) {
        SARBP_CUDA(ctx, sarbp::launch_dft_cols(pa_plan, B, out, NR, true, 1.0f / (float)NA, s), "azimuth IFFT");
    } else {
        SARBP_CUDA(ctx, sarbp::launch_transpose(B, A, NA, NR, s), "transpose");
        SARBP_CUDA(ctx, sarbp::launch_dft_rows(pa_plan, A, NR, NA, true, 1.0f / (float)NA, s), "azimuth IFFT");
        SARBP_CUDA(ctx, sarbp::launch_transpose(A, out, NR, NA, s), "transpose");
    }
    cudaEventRecord(ctx->ev[1], s);
    ctx->timed_rc = true;  // sarbp_last_timings reports the omega-K time in its rc slot
    ctx->timed_bp = false;
    ctx->launches += cols ? 4 : 8;  // and the Stolt launch counted by wk_focus_launch
    if (!dev_img)
        SARBP_CUDA(ctx, cudaMemcpyAsync(image, out, sizeof(float2) * npix, cudaMemcpyDeviceToHost, s), "download image");
    return finish(ctx, s, any_host);
}

sarbp_status sarbp_wk_preprocess(sarbp_ctx *ctx, const sarbp_wk_params *w, const sarbp_complex64 *echo, int32_t na,
                                 int32_t nr, sarbp_complex64 *out, void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_wk_preprocess");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    sarbp_status st = wk_check_params(ctx, w);
    if (st != SARBP_OK) return st;
    if (na <= 0 || nr <= 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "echo size must be > 0");
    if (!echo || !out) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "echo and out must be non-null");
    int32_t NA, NR;
    if (sarbp_wk_padded_size(na, nr, &NA, &NR) != SARBP_OK)
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "padded size %d x %d not supported", NA, NR);
    int pa, pr;
    wk_pads(na, nr, &pa, &pr);
    cudaStream_t s = pick_stream(ctx, stream);
    WkTables tb;
    st = wk_tables(ctx, w, NA, NR, s, tb);
    if (st != SARBP_OK) return st;
    const float2 *d_echo = reinterpret_cast<const float2 *>(echo);
    if (!is_device_ptr(echo)) {
        SARBP_CUDA(ctx, ctx->echo.ensure(sizeof(float2) * (size_t)na * nr), "alloc echo");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->echo.ptr, echo, sizeof(float2) * (size_t)na * nr, cudaMemcpyHostToDevice, s),
                   "upload echo");
        d_echo = ctx->echo.as<float2>();
    }
    const size_t bytes = sizeof(float2) * (size_t)NA * NR;
    const bool dev_out = is_device_ptr(out);
    float2 *d_out = reinterpret_cast<float2 *>(out);
    if (!dev_out) {
        SARBP_CUDA(ctx, ctx->wk0.ensure(bytes), "alloc omega-K buffer");
        d_out = ctx->wk0.as<float2>();
    }
    SARBP_CUDA(ctx, sarbp::launch_wk_pad(d_echo, na, nr, tb.rowphase, pa, pr, NA, NR, d_out, s), "padding");
    ctx->launches += 1;
    if (!dev_out) SARBP_CUDA(ctx, cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, s), "download");
    return finish(ctx, s, true);  // the host tables are staged through pageable memory
}

sarbp_status sarbp_wk_focus(sarbp_ctx *ctx, const sarbp_wk_params *w, const sarbp_complex64 *spectrum, int32_t na_pad,
                            int32_t nr_pad, sarbp_complex64 *out, void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_wk_focus");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    sarbp_status st = wk_check_params(ctx, w);
    if (st != SARBP_OK) return st;
    if (na_pad <= 0 || nr_pad <= 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "spectrum size must be > 0");
    if (!spectrum || !out) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "spectrum and out must be non-null");
    if (sarbp::wk_stolt_smem(nr_pad) > (size_t)(227u << 10))
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "range size %d too large for the Stolt stage", nr_pad);
    cudaStream_t s = pick_stream(ctx, stream);
    WkTables tb;
    st = wk_tables(ctx, w, na_pad, nr_pad, s, tb);
    if (st != SARBP_OK) return st;
    const size_t bytes = sizeof(float2) * (size_t)na_pad * nr_pad;
    const float2 *d_in = reinterpret_cast<const float2 *>(spectrum);
    if (!is_device_ptr(spectrum)) {
        SARBP_CUDA(ctx, ctx->wk0.ensure(bytes), "alloc omega-K buffer");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->wk0.ptr, spectrum, bytes, cudaMemcpyHostToDevice, s), "upload spectrum");
        d_in = ctx->wk0.as<float2>();
    }
    const bool dev_out = is_device_ptr(out);
    float2 *d_out = reinterpret_cast<float2 *>(out);
    if (!dev_out) {
        SARBP_CUDA(ctx, ctx->wk1.ensure(bytes), "alloc omega-K buffer");
        d_out = ctx->wk1.as<float2>();
    }
    st = wk_focus_launch(ctx, w, tb, d_in, d_out, na_pad, nr_pad, s);
    if (st != SARBP_OK) return st;
    if (!dev_out) SARBP_CUDA(ctx, cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, s), "download");
    return finish(ctx, s, true);
}

sarbp_status sarbp_ceos_decode(sarbp_ctx *ctx, const uint8_t *raw, uint64_t raw_bytes,
                               const sarbp_ceos_layout *l, int32_t first_line, int32_t nlines, int32_t first_cell,
                               int32_t ncells, int32_t apply_agc, sarbp_complex64 *echo, int16_t *agc_db,
                               void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_ceos_decode");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    if (!l) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "layout is null");
    if (l->file_header < 0 || l->header < 0 || l->aux < 1 || l->cells < 1 || l->replica < 0 ||
        l->lines_per_block < 1 || l->replica_line < 1 || l->replica_line > l->lines_per_block ||
        l->agc_byte < 1 || l->agc_byte > l->aux || !std::isfinite(l->gain) || l->reserved != 0)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "inconsistent CEOS layout");
    if ((l->file_header | l->header | l->aux | l->replica) & 1)
        return fail(ctx, SARBP_ERR_UNSUPPORTED, "CEOS layouts with odd header, aux or replica sizes are not supported");
    if (nlines < 0 || ncells < 0 || first_line < 0 || first_cell < 0 || first_cell + (long long)ncells > l->cells)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "line or cell range out of the layout");
    if (nlines == 0 || ncells == 0) return SARBP_OK;
    if (!raw || !echo) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "raw and echo must be non-null");
    sarbp::CeosGeom g{};
    g.header = l->header;
    g.aux = l->aux;
    g.replica = l->replica;
    g.replica_line = l->replica_line;
    g.lines_per_block = l->lines_per_block;
    g.agc_byte = l->agc_byte;
    g.first_line = first_line;
    g.nlines = nlines;
    g.first_cell = first_cell;
    g.ncells = ncells;
    g.apply_agc = apply_agc != 0;
    g.line_bytes = (long long)l->header + l->aux + 2LL * l->cells;
    g.block_bytes = (long long)l->replica + (long long)l->lines_per_block * g.line_bytes;
    const long long b0 = first_line / l->lines_per_block;
    const long long b1 = (first_line + (long long)nlines - 1) / l->lines_per_block + 1;
    const long long lo = l->file_header + b0 * g.block_bytes, hi = l->file_header + b1 * g.block_bytes;
    if ((unsigned long long)hi > raw_bytes)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "raw data end at byte %llu, the lines need %lld",
                    (unsigned long long)raw_bytes, hi);
    cudaStream_t s = pick_stream(ctx, stream);
    bool any_host = false;
    const unsigned char *d_raw;
    if (is_device_ptr(raw)) {
        d_raw = reinterpret_cast<const unsigned char *>(raw);
        g.raw_offset = -(long long)l->file_header;
    } else {
        SARBP_CUDA(ctx, ctx->echo.ensure((size_t)(hi - lo)), "alloc raw buffer");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->echo.ptr, raw + lo, (size_t)(hi - lo), cudaMemcpyHostToDevice, s),
                   "upload raw blocks");
        d_raw = ctx->echo.as<unsigned char>();
        g.raw_offset = b0 * g.block_bytes;
        any_host = true;
    }
    // gain per AGC code: float(gain) * float(10^(dB / 20)), the reader's float
    // arithmetic; uploaded when the layout's gain changes, else reused
    if (ctx->ceos_valid && ctx->ceos_gain == l->gain) {
        SARBP_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ceos_ready, 0), "gain table");
    } else {
        ctx->ceos_valid = false;
        float gains[64];
        for (int code = 0; code < 64; ++code) {
            const int db = code - 24 * (code > 31);
            gains[code] = l->gain * (float)std::pow(10.0, db / 20.0);
        }
        SARBP_CUDA(ctx, ctx->wkrow.ensure(sizeof gains), "alloc gain table");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->wkrow.ptr, gains, sizeof gains, cudaMemcpyHostToDevice, s), "upload gains");
        if (!ctx->ceos_ready)
            SARBP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->ceos_ready, cudaEventDisableTiming), "gain table");
        SARBP_CUDA(ctx, cudaEventRecord(ctx->ceos_ready, s), "gain table");
        ctx->ceos_gain = l->gain;
        ctx->ceos_valid = true;
    }
    float2 *d_echo = reinterpret_cast<float2 *>(echo);
    const size_t out_bytes = sizeof(float2) * (size_t)nlines * ncells;
    const bool dev_echo = is_device_ptr(echo);
    if (!dev_echo) {
        SARBP_CUDA(ctx, ctx->wk0.ensure(out_bytes), "alloc echo");
        d_echo = ctx->wk0.as<float2>();
        any_host = true;
    }
    short *d_agc = nullptr;
    if (agc_db) {
        if (is_device_ptr(agc_db)) {
            d_agc = reinterpret_cast<short *>(agc_db);
        } else {
            SARBP_CUDA(ctx, ctx->sharp.ensure(sizeof(short) * nlines), "alloc agc");
            d_agc = ctx->sharp.as<short>();
            any_host = true;
        }
    }
    SARBP_CUDA(ctx, sarbp::launch_ceos_decode(d_raw, g, ctx->wkrow.as<float>(), d_echo, d_agc, s), "CEOS decode");
    ctx->launches += 1;
    if (!dev_echo) SARBP_CUDA(ctx, cudaMemcpyAsync(echo, d_echo, out_bytes, cudaMemcpyDeviceToHost, s), "download echo");
    if (agc_db && d_agc != reinterpret_cast<short *>(agc_db))
        SARBP_CUDA(ctx, cudaMemcpyAsync(agc_db, d_agc, sizeof(short) * nlines, cudaMemcpyDeviceToHost, s),
                   "download agc");
    return finish(ctx, s, any_host);
}

sarbp_status sarbp_image(sarbp_ctx *ctx, const sarbp_radar *radar, const sarbp_complex64 *echo, int32_t np,
                         int32_t ns, const double *apc, const sarbp_grid *grid, int32_t mode, sarbp_complex64 *image,
                         void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    Range range("sarbp_image");
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    sarbp_rc_layout lay;
    sarbp_status st = layout(ctx, radar, ns, &lay);
    if (st != SARBP_OK) return st;
    st = check_grid(ctx, grid);
    if (st != SARBP_OK) return st;
    if (mode < SARBP_MODE_FP64 || mode > SARBP_MODE_FP16STORE)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown mode %d", mode);
    if (np < 0) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "np must be >= 0");
    const size_t npix = (size_t)grid->nx * grid->ny;
    if (npix == 0) return SARBP_OK;
    if (!image) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "image is null");
    if (np > 0 && (!echo || !apc)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "echo and apc must be non-null");
    cudaStream_t s = pick_stream(ctx, stream);
    const int storage = mode == SARBP_MODE_FP16STORE ? SARBP_STORE_C32H : SARBP_STORE_C64;
    const size_t esize = storage == SARBP_STORE_C64 ? 8 : 4;
    bool any_host = false;
    // APC first: the planner's extremes are reduced on the device ahead of the
    // echo upload and range compression, and waited for only once those are
    // queued behind them (the plan is needed by the back-projection alone)
    const double *apc_dev = apc;
    sarbp::BpExtremes ex{};
    if (np > 0) {
        if (!is_device_ptr(apc)) {
            SARBP_CUDA(ctx, ctx->apc.ensure(sizeof(double) * 3 * np), "alloc apc");
            SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->apc.ptr, apc, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, s),
                       "upload apc");
            apc_dev = ctx->apc.as<double>();
            any_host = true;
        }
        st = extremes_enqueue(ctx, apc_dev, np, grid, s);
        if (st != SARBP_OK) return st;
    }
    const bool host_echo = np > 0 && !is_device_ptr(echo);
    any_host = any_host || host_echo;
    float2 *d_img = reinterpret_cast<float2 *>(image);
    const bool dev_img = is_device_ptr(image);
    // a pinned host image is written by the back-projection itself (no download)
    float2 *mapped_img = dev_img ? nullptr : static_cast<float2 *>(mapped_host_ptr(image));
    if (mapped_img) {
        d_img = mapped_img;
        any_host = true;
    } else if (!dev_img) {
        SARBP_CUDA(ctx, ctx->image.ensure(sizeof(float2) * npix), "alloc image");
        d_img = ctx->image.as<float2>();
        any_host = true;
    }
    ctx->timed_rc = ctx->timed_bp = false;
    sarbp_rc_view v;
    std::memset(&v, 0, sizeof v);
    v.storage = storage;
    v.np = np;
    v.nbins = lay.nbins;
    v.t0_bins = lay.t0_bins;
    v.bin_rate = lay.bin_rate;
    if (np > 0) {
        SARBP_CUDA(ctx, ctx->rc.ensure(esize * (size_t)np * lay.nbins), "alloc rc");
        if (storage == SARBP_STORE_C32H) SARBP_CUDA(ctx, ctx->scale.ensure(sizeof(float) * np), "alloc scale");
        float *d_scale = storage == SARBP_STORE_C32H ? ctx->scale.as<float>() : nullptr;
        st = host_echo ? rc_host_echo(ctx, radar, lay, echo, np, ns, storage, ctx->rc.ptr, d_scale, s)
                       : rc_device(ctx, radar, lay, reinterpret_cast<const float2 *>(echo), np, ns, storage, ctx->rc.ptr,
                                   d_scale, s);
        if (st != SARBP_OK) return st;
        v.data = ctx->rc.ptr;
        v.scale = storage == SARBP_STORE_C32H ? ctx->scale.as<float>() : nullptr;
        st = extremes_wait(ctx, ex);
        if (st != SARBP_OK) {
            if (host_echo) drain_uploads(ctx);
            return st;
        }
    }
    st = bp_device(ctx, radar, v, apc_dev, ex, grid, mode, d_img, 0, s);
    if (st != SARBP_OK) {
        if (host_echo) drain_uploads(ctx);
        return st;
    }
    if (!dev_img && !mapped_img) {
        const cudaError_t e = cudaMemcpyAsync(image, d_img, sizeof(float2) * npix, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) {
            if (host_echo) drain_uploads(ctx);
            return cuda_fail(ctx, e, "download image");
        }
    }
    return finish(ctx, s, any_host);
}

sarbp_status sarbp_synthesize_echo(sarbp_ctx *ctx, const sarbp_radar *radar, const double *apc, int32_t np,
                                   int32_t ns, const sarbp_target *targets, int32_t nt, double snr_db, uint64_t seed,
                                   sarbp_complex64 *echo_out, void *stream) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    ctx->err.clear();
    cudaSetDevice(ctx->device);
    sarbp_status st = check_radar(ctx, radar);
    if (st != SARBP_OK) return st;
    if (np < 0 || ns <= 0 || nt < 0 || nt > 4096)
        return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "need np >= 0, ns > 0, 0 <= nt <= 4096");
    if (np == 0) return SARBP_OK;
    if (!apc || !echo_out || (nt > 0 && !targets)) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "null pointer");
    cudaStream_t s = pick_stream(ctx, stream);
    bool any_host = false;
    const double *d_apc = apc;
    if (!is_device_ptr(apc)) {
        SARBP_CUDA(ctx, ctx->apc.ensure(sizeof(double) * 3 * np), "alloc apc");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->apc.ptr, apc, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, s), "upload apc");
        d_apc = ctx->apc.as<double>();
        any_host = true;
    }
    const sarbp_target *d_tg = targets;
    if (nt > 0 && !is_device_ptr(targets)) {
        SARBP_CUDA(ctx, ctx->targets.ensure(sizeof(sarbp_target) * nt), "alloc targets");
        SARBP_CUDA(ctx, cudaMemcpyAsync(ctx->targets.ptr, targets, sizeof(sarbp_target) * nt, cudaMemcpyHostToDevice, s),
                   "upload targets");
        d_tg = ctx->targets.as<sarbp_target>();
        any_host = true;
    }
    float2 *d_echo = reinterpret_cast<float2 *>(echo_out);
    const bool dev_out = is_device_ptr(echo_out);
    if (!dev_out) {
        SARBP_CUDA(ctx, ctx->echo.ensure(sizeof(float2) * (size_t)np * ns), "alloc echo");
        d_echo = ctx->echo.as<float2>();
        any_host = true;
    }
    const bool noise = !std::isnan(snr_db);
    SARBP_CUDA(ctx, cudaMemsetAsync(ctx->power.ptr, 0, sizeof(double), s), "clear power");
    SARBP_CUDA(ctx, sarbp::launch_echo_synth(d_apc, np, ns, d_tg, nt, radar->t_rec0, radar->fs, radar->kr, radar->tp,
                                             radar->tc, radar->fc, radar->c, d_echo, ctx->power.as<double>(), s),
               "echo synthesis");
    ctx->launches += 1;
    if (noise) {
        SARBP_CUDA(ctx, sarbp::launch_echo_noise(d_echo, (int64_t)np * ns, ctx->power.as<double>(), snr_db, seed, s),
                   "echo noise");
        ctx->launches += 1;
    }
    if (!dev_out)
        SARBP_CUDA(ctx, cudaMemcpyAsync(echo_out, d_echo, sizeof(float2) * (size_t)np * ns, cudaMemcpyDeviceToHost, s),
                   "download echo");
    ctx->timed_rc = ctx->timed_bp = false;
    return finish(ctx, s, any_host);
}

// ------------------------------------------------------- reference shims --

static sarbp_status shim_ctx(sarbp_ctx **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return SARBP_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lk(g_shim_mu);
    if (!g_shim_ctx || g_shim_dev != dev) {
        if (g_shim_ctx) sarbp_destroy(g_shim_ctx);
        g_shim_ctx = nullptr;
        sarbp_status st = sarbp_create(&g_shim_ctx, dev);
        if (st != SARBP_OK) return st;
        g_shim_dev = dev;
    }
    *out = g_shim_ctx;
    return SARBP_OK;
}

sarbp_status sarbp_launch_back_projection(sarbp_complex64 *Srnm, sarbp_complex64 *Image,
                                          const sarbp_ref_params *params, int32_t Na, int32_t Nr) {
    if (!Srnm || !Image || !params || Na < 0 || Nr < 0) return SARBP_ERR_INVALID_ARGUMENT;
    const sarbp_ref_params &q = *params;
    if (q.Mslow <= 0 || q.Nfast <= 0 || !(q.vr != 0.f) || !(q.Fr > 0.f)) return SARBP_ERR_INVALID_ARGUMENT;
    sarbp_ctx *ctx = nullptr;
    sarbp_status st = shim_ctx(&ctx);
    if (st != SARBP_OK) return st;
    sarbp_radar r;
    std::memset(&r, 0, sizeof r);
    r.c = q.c;
    r.fc = q.fc;
    r.fs = q.Fr;
    r.kr = q.Kr;
    r.tp = q.Tr;
    r.tc = 0.0;      // uncentred chirp, as generateEchoKernel emits (BPA_CUDA_kernels.cu:28)
    r.t_rec0 = 0.0;  // tr_i = i / Fr (BPA_CUDA.cpp:44-48)
    r.upsample = 8;
    std::vector<double> apc((size_t)3 * q.Mslow);
    const double ta0 = -(double)q.La / (2.0 * q.vr), ta1 = (double)q.La / (2.0 * q.vr);
    const double step = q.Mslow > 1 ? (ta1 - ta0) / (q.Mslow - 1) : 0.0;
    for (int m = 0; m < q.Mslow; ++m) {
        apc[3 * m] = q.vr * (ta0 + m * step);
        apc[3 * m + 1] = 0.0;
        apc[3 * m + 2] = q.H;
    }
    sarbp_grid g;
    std::memset(&g, 0, sizeof g);
    g.origin[0] = (double)q.Az0 - (double)(Na / 2);
    g.origin[1] = (double)q.Rg0 - (double)(Nr / 2);
    g.uy[0] = 1.0;
    g.ux[1] = 1.0;
    g.nx = Nr;
    g.ny = Na;
    st = sarbp_image(ctx, &r, Srnm, q.Mslow, q.Nfast, apc.data(), &g, SARBP_MODE_SPLIT, Image, nullptr);
    if (st != SARBP_OK) return st;
    return sarbp_synchronize(ctx);
}

sarbp_status sarbp_launch_generate_echo(sarbp_complex64 *Srnm, const float *Ptarget, const float *ta, const float *tr,
                                        const sarbp_ref_params *params, int32_t Mslow, int32_t Nfast) {
    if (!Srnm || !ta || !tr || !params || Mslow < 0 || Nfast < 0) return SARBP_ERR_INVALID_ARGUMENT;
    if (params->Ntarget > 0 && !Ptarget) return SARBP_ERR_INVALID_ARGUMENT;
    sarbp_ctx *ctx = nullptr;
    sarbp_status st = shim_ctx(&ctx);
    if (st != SARBP_OK) return st;
    SARBP_CUDA(ctx, sarbp::launch_ref_echo(reinterpret_cast<float2 *>(Srnm), Ptarget, ta, tr, *params, Mslow, Nfast,
                                           ctx->stream),
               "reference echo");
    ctx->launches += 1;
    SARBP_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "reference echo sync");
    return SARBP_OK;
}

sarbp_status sarbp_debug_set(sarbp_ctx *ctx, int32_t key, int64_t value) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    sarbp::Tuning &t = ctx->tune;
    switch (key) {
        case SARBP_DEBUG_BP_CHUNK:
            if (value != 0 && value != 4 && value != 8 && value != 16)
                return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "pulse chunk must be 0, 4, 8 or 16");
            t.bp_chunk = (int)value;
            return SARBP_OK;
        case SARBP_DEBUG_BP_SEGMENTS:
            if (value < 0 || value > 64) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "segments must be in 0..64");
            t.bp_segments = (int)value;
            return SARBP_OK;
        case SARBP_DEBUG_BP_CHECKED:
            t.checked = value != 0;
            return SARBP_OK;
        case SARBP_DEBUG_WAIT_LIMIT_NS:
            if (value < 0 || value > 60000000000LL)
                return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "wait limit must be in 0..60 s");
            t.wait_ns = value;
            return SARBP_OK;
        case SARBP_DEBUG_WAIT_FAULT_CHUNK:
            t.wait_fault_chunk = value < 0 ? -1 : (int)std::min<int64_t>(value, 1 << 30);
            return SARBP_OK;
        case SARBP_DEBUG_BP_LINEAR_PHASE:
            if (value < -1 || value > 1) return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "linear phase must be -1, 0 or 1");
            t.linear_phase = (int)value;
            return SARBP_OK;
        default:
            return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown debug key %d", (int)key);
    }
}

sarbp_status sarbp_debug_get(sarbp_ctx *ctx, int32_t key, int64_t *value) {
    if (!ctx || !value) return SARBP_ERR_INVALID_ARGUMENT;
    const sarbp::Tuning &t = ctx->tune;
    switch (key) {
        case SARBP_DEBUG_BP_CHUNK: *value = t.bp_chunk; return SARBP_OK;
        case SARBP_DEBUG_BP_SEGMENTS: *value = t.bp_segments; return SARBP_OK;
        case SARBP_DEBUG_BP_CHECKED: *value = t.checked; return SARBP_OK;
        case SARBP_DEBUG_WAIT_LIMIT_NS: *value = t.wait_ns; return SARBP_OK;
        case SARBP_DEBUG_WAIT_FAULT_CHUNK: *value = t.wait_fault_chunk; return SARBP_OK;
        case SARBP_DEBUG_DEVICE_FLAGS: *value = ctx->last_device_flags; return SARBP_OK;
        case SARBP_DEBUG_BP_LINEAR_PHASE: *value = t.linear_phase; return SARBP_OK;
        default: return fail(ctx, SARBP_ERR_INVALID_ARGUMENT, "unknown debug key %d", (int)key);
    }
}

sarbp_status sarbp_probe_issue_rates(sarbp_ctx *ctx, double *fp32_lanes_per_s, double *mufu_lanes_per_s,
                                     int32_t *sm_count) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    SARBP_CUDA(ctx, sarbp::run_issue_probe(ctx->sms, fp32_lanes_per_s, mufu_lanes_per_s, ctx->stream), "issue probe");
    if (sm_count) *sm_count = ctx->sms;
    return SARBP_OK;
}

sarbp_status sarbp_last_timings(sarbp_ctx *ctx, float *rc_ms, float *bp_ms) {
    if (!ctx) return SARBP_ERR_INVALID_ARGUMENT;
    if (rc_ms) *rc_ms = ctx->timed_rc ? ctx->rc_ms : 0.f;
    if (bp_ms) *bp_ms = ctx->timed_bp ? ctx->bp_ms : 0.f;
    return SARBP_OK;
}

int64_t sarbp_kernel_launches(const sarbp_ctx *ctx) { return ctx ? ctx->launches : 0; }

}  // extern "C"
