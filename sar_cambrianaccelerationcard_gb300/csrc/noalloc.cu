// noalloc.cu -- range compression that allocates no device memory.
//
// Some callers cannot call cudaMalloc once they are running: a host program
// whose own allocator has already reserved the GPU's memory at start-up, or a
// latency-bound processing loop that must not stall on an allocation (which
// can synchronise the whole device).  sarbp_range_compress_noalloc serves
// them.  It runs the same range-compression kernels as sarbp_range_compress,
// but every byte of scratch it needs -- the matched-filter spectrum, the
// phase table (FFT twiddles and upsampling ramp) and a batch of per-pulse
// spectra --
// lives in the fixed array below, which every GPU that loads this library
// holds until the process exits.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress (the array's name in
// host code is only a host-side stand-in), uploads the tables of its layout
// and loads the kernels.  Under CUDA's default lazy module loading the array
// and the kernels' code reach the GPU only then, so a caller whose allocator
// later reserves the GPU's memory makes that first call before (a call with
// np = 0 and a valid radar and layout does the set-up and nothing else), or
// runs with CUDA_MODULE_LOADING=EAGER.  Every call whose radar or layout
// differs from the previous one on that device rebuilds the tables and waits
// for their upload, so those calls (the first included) must stay outside
// stream capture.  All calls share the array and it keeps the last call's
// contents; calls whose work overlaps on the GPU (different host threads or
// streams) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <mutex>

#include "sarbp_internal.h"

namespace {

constexpr size_t kScratchBytes = size_t(4) << 20;  // SARBP_NOALLOC_SCRATCH_BYTES
constexpr int kMaxDevices = 64;
constexpr int kMaxN = 32768;  // largest range FFT the kernels support
constexpr int kMaxL = 16;     // largest upsampling factor
constexpr size_t kMaxEtab = 256 + kMaxL * kMaxN / 256;
// The largest tables (filter spectrum and phase table) plus one pulse spectrum
// and its split-path bounds fit, so every supported layout runs here.
static_assert(sizeof(float2) * (kMaxN + kMaxEtab) + 256 + sizeof(float2) * kMaxN + 2 * sizeof(float) <= kScratchBytes,
              "scratch array too small for the largest layout");

static __device__ __align__(256) unsigned char g_rc_scratch[kScratchBytes];

struct TableKey {
    int nfft = 0, L = 0, nc = 0, shift = 0;
    double kr = 0, fs = 0, tc = 0, tp = 0;
    bool operator==(const TableKey &o) const {
        return nfft == o.nfft && L == o.L && nc == o.nc && shift == o.shift && kr == o.kr && fs == o.fs &&
               tc == o.tc && tp == o.tp;
    }
};

std::mutex g_mu;
unsigned char *g_dev_scratch[kMaxDevices] = {};
bool g_have_tables[kMaxDevices] = {};
TableKey g_keys[kMaxDevices];

// host staging for the tables: static storage, no heap
std::complex<double> g_h[kMaxN];
float2 g_filt[kMaxN], g_etab[kMaxEtab];

bool on_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" sarbp_status sarbp_range_compress_noalloc(const sarbp_radar *radar, const sarbp_complex64 *echo,
                                                     int32_t np, int32_t ns, int32_t storage, void *rc_out,
                                                     float *rc_scale_out, void *stream) {
    sarbp_rc_layout lay;
    sarbp_status st = sarbp_rc_layout_get(radar, ns, &lay);
    if (st != SARBP_OK) return st;
    if (np < 0) return SARBP_ERR_INVALID_ARGUMENT;
    if (storage != SARBP_STORE_C64 && storage != SARBP_STORE_C32H) return SARBP_ERR_INVALID_ARGUMENT;
    if (!sarbp::rc_size_supported(lay.nfft) || radar->upsample > kMaxL) return SARBP_ERR_UNSUPPORTED;
    if (np > 0) {
        if (!echo || !rc_out || (storage == SARBP_STORE_C32H && !rc_scale_out)) return SARBP_ERR_INVALID_ARGUMENT;
        if (!on_device(echo) || !on_device(rc_out) || (storage == SARBP_STORE_C32H && !on_device(rc_scale_out)))
            return SARBP_ERR_INVALID_ARGUMENT;  // device memory only: a host buffer would need a staging copy
    }
    const size_t N = (size_t)lay.nfft, L = (size_t)radar->upsample;
    const size_t ne = (size_t)sarbp::rc_etab_size((int)L, (int)N);
    const size_t tables = sizeof(float2) * (N + ne);
    const size_t row = sizeof(float2) * N;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return SARBP_ERR_NO_DEVICE;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_dev_scratch[dev]) {  // once per device, with that device current
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_rc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return SARBP_ERR_CUDA;
        }
        g_dev_scratch[dev] = static_cast<unsigned char *>(p);
    }
    unsigned char *base = g_dev_scratch[dev];
    float2 *d_filt = reinterpret_cast<float2 *>(base);
    float2 *d_etab = d_filt + N;
    float2 *d_spec = reinterpret_cast<float2 *>(base + ((tables + 255) & ~size_t(255)));
    const size_t spec_bytes = kScratchBytes - ((tables + 255) & ~size_t(255));
    // per pulse: one spectrum row and two split-path bounds
    const int batch =
        (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(np, 1), spec_bytes / (row + 2 * sizeof(float))));
    float *d_bound2 = reinterpret_cast<float *>(reinterpret_cast<char *>(d_spec) + row * (size_t)batch);

    TableKey key;
    key.nfft = lay.nfft;
    key.L = radar->upsample;
    key.nc = lay.nc;
    key.shift = lay.shift;
    key.kr = radar->kr;
    key.fs = radar->fs;
    key.tc = radar->tc;
    key.tp = radar->tp;
    if (!g_have_tables[dev] || !(g_keys[dev] == key)) {
        sarbp::rc_tables_fill(*radar, lay, g_h, g_filt, g_etab);  // the allocating path's tables, bit for bit
        // the host staging arrays are reused by the next call: wait for the copies
        if (cudaMemcpyAsync(d_filt, g_filt, sizeof(float2) * N, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(d_etab, g_etab, sizeof(float2) * ne, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            cudaGetLastError();
            g_have_tables[dev] = false;
            return SARBP_ERR_CUDA;
        }
        g_keys[dev] = key;
        g_have_tables[dev] = true;
    }
    sarbp::RcPlan plan{};
    plan.bound2 = d_bound2;
    plan.ns = ns;
    plan.nfft = lay.nfft;
    plan.L = radar->upsample;
    plan.nbins = lay.nbins;
    plan.storage = storage;
    if (np == 0) {  // set-up only: load and configure this layout's kernels
        if (sarbp::prepare_rc_kernels(plan) != cudaSuccess) {
            cudaGetLastError();
            return SARBP_ERR_CUDA;
        }
        return SARBP_OK;
    }
    // No scratch byte needs clearing: every spectrum the inverse kernel reads
    // was written by the forward kernel of the same batch.
    const size_t esize = storage == SARBP_STORE_C64 ? 8 : 4;
    const float2 *e2 = reinterpret_cast<const float2 *>(echo);
    for (int p0 = 0; p0 < np; p0 += batch) {
        plan.np = std::min(batch, np - p0);
        float *sc = storage == SARBP_STORE_C32H ? rc_scale_out + p0 : nullptr;
        if (sarbp::launch_rc_forward(plan, e2 + (size_t)p0 * ns, d_filt, d_etab, d_spec, sc, s) != cudaSuccess ||
            sarbp::launch_rc_inverse(plan, d_spec, d_etab, sc,
                                     static_cast<char *>(rc_out) + (size_t)p0 * lay.nbins * esize, s) != cudaSuccess) {
            cudaGetLastError();
            return SARBP_ERR_CUDA;
        }
    }
    return SARBP_OK;
}
