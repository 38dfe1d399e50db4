// serve.cpp -- continuous-batching imaging service (see sarbp_server_* in sarbp.h).
//
// The reference program images one scene per process run, synchronously
// (main.cpp:3-19, launchBackProjection ends in cudaDeviceSynchronize,
// BPA_CUDA_kernels.cu:98).  Here a worker thread serves a stream of jobs of
// uneven size on one device:
//   * submit (any thread): validate, plan the back-projection (tile, window,
//     segments) and build the range-compression tables on the host, compute
//     the device footprint, queue the job;
//   * admission (worker): in arrival order, every queued job that fits the
//     free budget and a free slot is admitted -- on an admission stream that
//     runs beside the steps, device buffers come from the stream-ordered pool,
//     the APC track is uploaded, the echo goes up in pulse chunks on a copy
//     stream and each chunk is range-compressed into the job's resident buffer
//     as soon as it lands; the job joins the steps once that work has
//     completed;
//   * steps (worker): each step back-projects the next pulses of every
//     admitted job into its resident image (accumulate after the first step):
//     pulses_per_step for every job, or with step_updates set a per-job count
//     of about step_updates / (nx ny), fixed at submit.  The step's launches are captured into one CUDA graph with
//     a branch per job on its own lane stream, so jobs overlap on the device;
//     at most two steps are in flight;
//   * completion: after a job's last step its image is copied back on a
//     download stream and an event recorded; when the event completes the
//     job's memory returns to the budget and waiters are released.
// Every job is computed by the same launches in the same order whatever else
// runs beside it, so its image does not depend on the mix.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "sarbp_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

enum class JobState { Queued, Loading, Active, Finishing, Done, Failed, Cancelled };

// Range-compression tables on the host (matched filter, phase tables), shared
// by every job of the same radar and transform layout.
struct HostTables {
    std::vector<float2> filt, etab;
};
struct TableKey {
    int nfft, L, nc, shift;
    double kr, fs, tc, tp;
    bool operator==(const TableKey &o) const {
        return nfft == o.nfft && L == o.L && nc == o.nc && shift == o.shift && kr == o.kr && fs == o.fs &&
               tc == o.tc && tp == o.tp;
    }
};

struct Job {
    uint64_t id = 0;
    sarbp_job desc{};
    sarbp_rc_layout lay{};
    int storage = SARBP_STORE_C64;
    size_t esize = 8;
    sarbp::BpPlan plan{};          // per-step template (pointers filled at admission)
    std::shared_ptr<const HostTables> tab;  // range-compression tables (host, shared)
    // device: one allocation carved into the buffers below
    size_t bytes = 0;
    unsigned char *dev = nullptr;
    float2 *d_echo = nullptr, *d_img = nullptr, *d_partial = nullptr, *d_filt = nullptr, *d_etab = nullptr;
    void *d_rc = nullptr;
    float *d_scale = nullptr;
    double *d_apc = nullptr;
    float4 *d_pref = nullptr;
    unsigned *d_err = nullptr;
    unsigned *h_err = nullptr;     // pinned copy of the job's device check word
    int lane = -1;
    int pps = 0;                   // pulses this job advances per step
    int next_pulse = 0;
    int steps = 0;
    cudaEvent_t done_ev = nullptr;
    cudaEvent_t ready_ev = nullptr;  // echo uploaded and range-compressed
    cudaEvent_t admit_ev = nullptr;  // start of the admission work (timing)
    std::vector<cudaEvent_t> chunk_done;  // range compression of pulses [b spec_rows, (b + 1) spec_rows) complete
    bool admit_counted = false;      // admission device time added to the stats
    JobState state = JobState::Queued;
    sarbp_status status = SARBP_OK;
    std::string msg;
    Clock::time_point t_submit, t_admit, t_done;
};

}  // namespace

struct sarbp_server {
    sarbp_server_config cfg{};
    int sms = 0;
    std::mutex mu;
    // range-compression tables by (radar, layout): built once per key on the
    // submitting thread (0.5-2.3 ms for 4096-16384-point transforms), 16 kept
    std::mutex tab_mu;
    std::vector<std::pair<TableKey, std::shared_ptr<const HostTables>>> tab_cache;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::thread worker;
    std::deque<Job *> queue;
    std::vector<Job *> active;            // admitted, not yet complete
    std::map<uint64_t, Job *> jobs;       // every unreleased ticket
    uint64_t next_id = 1;
    size_t in_use = 0;
    cudaStream_t s0 = nullptr;            // back-projection steps (graphs)
    cudaStream_t sa = nullptr;            // admission: allocation, upload, range compression
    cudaStream_t sd = nullptr;            // image downloads and frees
    cudaStream_t sc = nullptr;            // admission echo uploads, in pulse chunks
    cudaEvent_t chunk_ev = nullptr;       // a chunk's upload (re-recorded per chunk: each wait takes the latest)
    std::vector<cudaStream_t> lanes;
    std::vector<cudaEvent_t> join;        // one per lane
    cudaEvent_t fork = nullptr;
    cudaEvent_t step_ev[2] = {nullptr, nullptr};   // end of a step (timing)
    cudaEvent_t step_t0[2] = {nullptr, nullptr};   // start of a step (timing)
    int step_parity = 0;
    bool step_pending[2] = {false, false};
    cudaGraphExec_t exec = nullptr;
    float2 *d_spec = nullptr;             // range-compression spectrum scratch
    float *d_bound2 = nullptr;            // split-path bounds for the scratch rows
    size_t spec_rows = 0;
    sarbp_server_stats st{};
    Clock::time_point busy_since;
    bool busy = false;
    uint64_t fail_admit_ticket = 0;       // sarbp_server_debug_set: host-side fault injection (tests)
};

namespace {

constexpr size_t kSpecRows = 256;  // pulses per range-compression batch (scratch rows of up to 32768 points)
constexpr int kMaxN = 32768;

void fail_job(Job *j, sarbp_status st, const std::string &msg) {
    j->status = st;
    j->msg = msg;
    j->state = JobState::Failed;
}

// device footprint of a job, matching the carve in admit()
size_t job_bytes(const Job &j) {
    const size_t np = j.desc.np, ns = j.desc.ns, nb = j.lay.nbins;
    const size_t npix = (size_t)j.desc.grid.nx * j.desc.grid.ny;
    size_t b = 0;
    b += align256(np * ns * 8);                        // echo
    b += align256(np * nb * j.esize);                  // range-compressed data
    b += align256(np * 4);                             // fp16 scales
    b += align256(np * 24);                            // APC
    b += align256(np * 32);                            // pulse references
    b += align256(npix * 8);                           // image
    b += align256((size_t)(j.plan.segments > 1 ? j.plan.segments : 0) * npix * 8);  // partial images
    b += align256(j.tab->filt.size() * 8) + align256(j.tab->etab.size() * 8);
    b += 256;                                          // check word
    return b;
}

// Enqueue admission work for j on the admission stream: carve buffers, upload,
// range-compress, then record the job's ready event.
sarbp_status admit(sarbp_server *S, Job *j) {
    // injected on the host, as a refused allocation would be: no device work
    if (S->fail_admit_ticket != 0 && j->id == S->fail_admit_ticket) return SARBP_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaMallocAsync((void **)&j->dev, j->bytes, S->sa);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SARBP_ERR_OUT_OF_MEMORY;
    }
    cudaEventRecord(j->admit_ev, S->sa);
    const size_t np = j->desc.np, ns = j->desc.ns, nb = j->lay.nbins;
    const size_t npix = (size_t)j->desc.grid.nx * j->desc.grid.ny;
    unsigned char *p = j->dev;
    auto take = [&](size_t n) {
        unsigned char *r = p;
        p += align256(n);
        return r;
    };
    j->d_echo = (float2 *)take(np * ns * 8);
    j->d_rc = take(np * nb * j->esize);
    j->d_scale = (float *)take(np * 4);
    j->d_apc = (double *)take(np * 24);
    j->d_pref = (float4 *)take(np * 32);
    j->d_img = (float2 *)take(npix * 8);
    j->d_partial = (float2 *)take((size_t)(j->plan.segments > 1 ? j->plan.segments : 0) * npix * 8);
    j->d_filt = (float2 *)take(j->tab->filt.size() * 8);
    j->d_etab = (float2 *)take(j->tab->etab.size() * 8);
    j->d_err = (unsigned *)take(sizeof(unsigned));
    // The echo goes up in chunks of spec_rows pulses on the copy stream, and each
    // chunk is range-compressed on the admission stream as soon as it lands, so
    // only the first chunk's upload is exposed.  The copy stream first waits for
    // the admission stream (the allocation above, and earlier admissions).
    e = cudaEventRecord(S->chunk_ev, S->sa);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(S->sc, S->chunk_ev, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(j->d_apc, j->desc.apc, np * 24, cudaMemcpyHostToDevice, S->sa);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(j->d_filt, j->tab->filt.data(), j->tab->filt.size() * 8, cudaMemcpyHostToDevice, S->sa);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(j->d_etab, j->tab->etab.data(), j->tab->etab.size() * 8, cudaMemcpyHostToDevice, S->sa);
    if (e == cudaSuccess) e = cudaMemsetAsync(j->d_err, 0, sizeof(unsigned), S->sa);
    for (size_t p0 = 0; e == cudaSuccess && p0 < np; p0 += S->spec_rows) {
        const size_t rows = std::min(S->spec_rows, np - p0);
        e = cudaMemcpyAsync(j->d_echo + p0 * ns, reinterpret_cast<const float2 *>(j->desc.echo) + p0 * ns,
                            rows * ns * 8, cudaMemcpyHostToDevice, S->sc);
        if (e == cudaSuccess) e = cudaEventRecord(S->chunk_ev, S->sc);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(S->sa, S->chunk_ev, 0);
        if (e != cudaSuccess) break;
        sarbp::RcPlan rp{};
        rp.bound2 = S->d_bound2;
        rp.np = (int)std::min(S->spec_rows, np - p0);
        rp.ns = (int)ns;
        rp.nfft = j->lay.nfft;
        rp.L = j->desc.radar.upsample;
        rp.nbins = (int)nb;
        rp.storage = j->storage;
        float *sc = j->storage == SARBP_STORE_C32H ? j->d_scale + p0 : nullptr;
        e = sarbp::launch_rc_forward(rp, j->d_echo + p0 * ns, j->d_filt, j->d_etab, S->d_spec, sc, S->sa);
        if (e == cudaSuccess)
            e = sarbp::launch_rc_inverse(rp, S->d_spec, j->d_etab, sc,
                                         static_cast<char *>(j->d_rc) + p0 * nb * j->esize, S->sa);
        if (e == cudaSuccess) e = cudaEventRecord(j->chunk_done[p0 / S->spec_rows], S->sa);
    }
    if (e == cudaSuccess) e = cudaEventRecord(j->ready_ev, S->sa);
    if (e != cudaSuccess) {
        cudaGetLastError();
        // chunk copies may still be reading the caller's echo and writing the
        // job's buffer, which the caller frees next: let them finish first
        cudaStreamSynchronize(S->sc);
        cudaGetLastError();
        return SARBP_ERR_CUDA;
    }
    sarbp::BpPlan &bp = j->plan;
    bp.rc = j->d_rc;
    bp.scale = j->storage == SARBP_STORE_C32H ? j->d_scale : nullptr;
    bp.apc = j->d_apc;
    bp.pref = j->d_pref;
    bp.image = j->d_img;
    bp.partial = j->d_partial;
    bp.err = j->d_err;
    return SARBP_OK;
}

// BP launch of pulses [p0, p1) of job j on stream s.
cudaError_t launch_step(Job *j, int p0, int p1, cudaStream_t s) {
    sarbp::BpPlan p = j->plan;
    p.np = p1 - p0;
    p.rc = static_cast<const char *>(j->d_rc) + (size_t)p0 * j->lay.nbins * j->esize;
    p.scale = j->storage == SARBP_STORE_C32H ? j->d_scale + p0 : nullptr;
    p.apc = j->d_apc + 3 * (size_t)p0;
    p.pref = j->d_pref + 2 * (size_t)p0;
    p.accumulate = p0 > 0;
    return sarbp::launch_bp(p, s, nullptr);
}

void release(sarbp_server *S, Job *j) {
    if (j->dev) cudaFreeAsync(j->dev, S->sd);  // after the download, which waited for the last step
    j->dev = nullptr;
    S->in_use -= j->bytes;
    if (j->lane >= 0) j->lane = -1;
}

// Range-compression batch that the job's next step needs (the one holding its
// last pulse): the job joins steps as soon as that batch is complete, while
// later batches are still being compressed.
cudaEvent_t next_step_chunk(const sarbp_server *S, const Job *j) {
    const int p1 = std::min(j->desc.np, j->next_pulse + j->pps);
    return j->chunk_done[(size_t)(p1 - 1) / S->spec_rows];
}

// Device time of step `par` once it has completed (caller holds S->mu).
void fold_step(sarbp_server *S, int par) {
    if (!S->step_pending[par] || cudaEventQuery(S->step_ev[par]) != cudaSuccess) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, S->step_t0[par], S->step_ev[par]) == cudaSuccess) S->st.step_device_s += ms * 1e-3;
    cudaGetLastError();
    S->step_pending[par] = false;
}

void worker_main(sarbp_server *S) {
    cudaSetDevice(S->cfg.device);
    std::vector<bool> lane_busy(S->cfg.max_jobs, false);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        // 1. completions
        for (auto it = S->active.begin(); it != S->active.end();) {
            Job *j = *it;
            if (j->state == JobState::Finishing && cudaEventQuery(j->done_ev) == cudaSuccess) {
                if (*j->h_err) fail_job(j, SARBP_ERR_DEVICE_CHECK, "device check word set");
                else j->state = JobState::Done;
                j->t_done = Clock::now();
                lane_busy[j->lane] = false;
                release(S, j);
                if (j->state == JobState::Done) {
                    S->st.completed++;
                    S->st.updates += (double)j->desc.grid.nx * j->desc.grid.ny * j->desc.np;
                } else {
                    S->st.failed++;
                }
                it = S->active.erase(it);
                S->cv_done.notify_all();
            } else {
                ++it;
            }
        }
        for (Job *j : S->active)
            if (!j->admit_counted && cudaEventQuery(j->ready_ev) == cudaSuccess) {
                if (j->state == JobState::Loading) j->state = JobState::Active;
                float ms = 0.f;
                if (cudaEventElapsedTime(&ms, j->admit_ev, j->ready_ev) == cudaSuccess) S->st.admit_device_s += ms * 1e-3;
                cudaGetLastError();
                j->admit_counted = true;
            }
        fold_step(S, 0);
        fold_step(S, 1);
        if (S->active.empty() && S->busy) {
            S->st.busy_s += std::chrono::duration<double>(Clock::now() - S->busy_since).count();
            S->busy = false;
        }
        // 2. admission, in arrival order, skipping jobs that do not fit yet
        for (auto it = S->queue.begin(); it != S->queue.end();) {
            Job *j = *it;
            if ((int)S->active.size() >= S->cfg.max_jobs) break;
            if (S->in_use + j->bytes > S->cfg.hbm_budget_bytes) {
                ++it;
                continue;
            }
            it = S->queue.erase(it);
            int lane = 0;
            while (lane_busy[lane]) ++lane;
            const sarbp_status st = admit(S, j);
            if (st != SARBP_OK) {
                fail_job(j, st, "admission failed");
                if (j->dev) cudaFreeAsync(j->dev, S->sa);
                j->dev = nullptr;
                S->st.failed++;
                S->cv_done.notify_all();
                continue;
            }
            lane_busy[lane] = true;
            j->lane = lane;
            j->state = JobState::Loading;
            j->t_admit = Clock::now();
            S->in_use += j->bytes;
            S->st.peak_bytes = std::max<uint64_t>(S->st.peak_bytes, S->in_use);
            S->active.push_back(j);
            S->st.peak_active = std::max<int32_t>(S->st.peak_active, (int32_t)S->active.size());
            if (!S->busy) {
                S->busy = true;
                S->busy_since = Clock::now();
            }
        }
        // 3. one step over every admitted job that still has pulses
        std::vector<Job *> step;
        for (Job *j : S->active)
            if (j->state == JobState::Active ||
                (j->state == JobState::Loading && cudaEventQuery(next_step_chunk(S, j)) == cudaSuccess))
                step.push_back(j);
        if (!step.empty()) {
            // at most two steps in flight
            const int par = S->step_parity;
            if (S->step_pending[par]) {
                lk.unlock();
                cudaEventSynchronize(S->step_ev[par]);
                lk.lock();
                fold_step(S, par);
            }
            cudaError_t e = cudaEventRecord(S->step_t0[par], S->s0);
            const bool graph = S->cfg.use_graphs != 0;
            cudaGraph_t g = nullptr;
            if (graph && e == cudaSuccess) e = cudaStreamBeginCapture(S->s0, cudaStreamCaptureModeRelaxed);
            if (e == cudaSuccess) e = cudaEventRecord(S->fork, S->s0);
            for (Job *j : step) {
                if (e != cudaSuccess) break;
                cudaStream_t ls = S->lanes[j->lane];
                const int p0 = j->next_pulse, p1 = std::min(j->desc.np, p0 + j->pps);
                e = cudaStreamWaitEvent(ls, S->fork, 0);
                if (e == cudaSuccess) e = launch_step(j, p0, p1, ls);
                if (e == cudaSuccess) e = cudaEventRecord(S->join[j->lane], ls);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(S->s0, S->join[j->lane], 0);
            }
            if (graph) {
                cudaError_t ee = cudaStreamEndCapture(S->s0, &g);
                if (e == cudaSuccess) e = ee;
                if (e == cudaSuccess) {
                    bool updated = false;
                    if (S->exec) {
                        cudaGraphExecUpdateResultInfo info;
                        updated = cudaGraphExecUpdate(S->exec, g, &info) == cudaSuccess;
                        if (!updated) {
                            cudaGetLastError();
                            cudaGraphExecDestroy(S->exec);
                            S->exec = nullptr;
                        }
                    }
                    if (!updated) e = cudaGraphInstantiate(&S->exec, g, 0);
                    if (e == cudaSuccess) e = cudaGraphLaunch(S->exec, S->s0);
                    if (e == cudaSuccess) S->st.graph_launches++;
                }
                if (g) cudaGraphDestroy(g);
            }
            S->st.steps++;
            if (e != cudaSuccess) cudaGetLastError();
            cudaEventRecord(S->step_ev[par], S->s0);
            bool waited = false;
            for (Job *j : step) {
                if (e != cudaSuccess) {
                    fail_job(j, SARBP_ERR_CUDA, cudaGetErrorString(e));
                    continue;
                }
                j->steps++;
                j->next_pulse = std::min(j->desc.np, j->next_pulse + j->pps);
                if (j->next_pulse >= j->desc.np) {  // last step: copy the image back on the download stream
                    const size_t npix = (size_t)j->desc.grid.nx * j->desc.grid.ny;
                    cudaError_t ce = waited ? cudaSuccess : cudaStreamWaitEvent(S->sd, S->step_ev[par], 0);
                    waited = true;
                    if (ce == cudaSuccess)
                        ce = cudaMemcpyAsync(j->desc.image, j->d_img, npix * 8, cudaMemcpyDeviceToHost, S->sd);
                    if (ce == cudaSuccess)
                        ce = cudaMemcpyAsync(j->h_err, j->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, S->sd);
                    if (ce == cudaSuccess) ce = cudaEventRecord(j->done_ev, S->sd);
                    if (ce != cudaSuccess) fail_job(j, SARBP_ERR_CUDA, cudaGetErrorString(ce));
                    else j->state = JobState::Finishing;
                }
            }
            S->step_pending[par] = true;
            S->step_parity ^= 1;
            // failed jobs leave the active set
            for (auto it = S->active.begin(); it != S->active.end();) {
                Job *j = *it;
                if (j->state == JobState::Failed) {
                    cudaStreamSynchronize(S->s0);
                    cudaStreamWaitEvent(S->sd, S->step_ev[par], 0);
                    lane_busy[j->lane] = false;
                    release(S, j);
                    S->st.failed++;
                    it = S->active.erase(it);
                    S->cv_done.notify_all();
                } else {
                    ++it;
                }
            }
            continue;
        }
        // 4. nothing to launch: wait for a completion, new work or stop
        Job *oldest = nullptr;
        for (Job *j : S->active)
            if (j->state == JobState::Finishing || j->state == JobState::Loading) {
                oldest = j;
                break;
            }
        if (oldest) {
            cudaEvent_t ev = oldest->state == JobState::Loading ? next_step_chunk(S, oldest) : oldest->done_ev;
            lk.unlock();
            cudaEventSynchronize(ev);
            lk.lock();
            continue;
        }
        if (S->stop && S->active.empty()) break;
        S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty(); });
        if (S->stop && S->queue.empty() && S->active.empty()) break;
    }
}

}  // namespace

extern "C" {

sarbp_status sarbp_server_create(sarbp_server **out, const sarbp_server_config *cfg) {
    if (!out || !cfg) return SARBP_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (cfg->max_jobs < 1 || cfg->max_jobs > 64 || cfg->hbm_budget_bytes == 0) return SARBP_ERR_INVALID_ARGUMENT;
    if (cfg->pulses_per_step < 0 || cfg->pulses_per_step % 16 != 0) return SARBP_ERR_INVALID_ARGUMENT;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return SARBP_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= n) return SARBP_ERR_INVALID_ARGUMENT;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, cfg->device) != cudaSuccess || prop.major * 10 + prop.minor != 103)
        return SARBP_ERR_NO_DEVICE;
    cudaSetDevice(cfg->device);
    sarbp_server *S = new sarbp_server();
    S->cfg = *cfg;
    if (S->cfg.pulses_per_step == 0) S->cfg.pulses_per_step = 512;
    S->sms = prop.multiProcessorCount;
    bool ok = cudaStreamCreateWithFlags(&S->s0, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&S->sa, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&S->sd, cudaStreamNonBlocking) == cudaSuccess;
    S->lanes.resize(S->cfg.max_jobs);
    S->join.resize(S->cfg.max_jobs);
    for (int i = 0; ok && i < S->cfg.max_jobs; ++i) {
        ok = cudaStreamCreateWithFlags(&S->lanes[i], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&S->join[i], cudaEventDisableTiming) == cudaSuccess;
    }
    ok = ok && cudaEventCreateWithFlags(&S->fork, cudaEventDisableTiming) == cudaSuccess &&
         cudaEventCreate(&S->step_ev[0]) == cudaSuccess && cudaEventCreate(&S->step_ev[1]) == cudaSuccess &&
         cudaEventCreate(&S->step_t0[0]) == cudaSuccess && cudaEventCreate(&S->step_t0[1]) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&S->sc, cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&S->chunk_ev, cudaEventDisableTiming) == cudaSuccess;
    S->spec_rows = kSpecRows;
    ok = ok && cudaMalloc(&S->d_spec, sizeof(float2) * kSpecRows * kMaxN + sizeof(float) * 2 * kSpecRows) == cudaSuccess;
    if (ok) S->d_bound2 = reinterpret_cast<float *>(S->d_spec + kSpecRows * kMaxN);
    if (ok) {  // keep freed job memory in the pool for the next admissions
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, cfg->device) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    if (!ok) {
        cudaGetLastError();
        sarbp_server_destroy(S);
        return SARBP_ERR_CUDA;
    }
    S->worker = std::thread(worker_main, S);
    *out = S;
    return SARBP_OK;
}

sarbp_status sarbp_server_destroy(sarbp_server *S) {
    if (!S) return SARBP_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        for (Job *j : S->queue) {
            j->state = JobState::Cancelled;
            j->status = SARBP_ERR_CANCELLED;
            S->st.cancelled++;
        }
        S->queue.clear();
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    cudaSetDevice(S->cfg.device);
    for (cudaStream_t st : {S->sc, S->sa, S->s0, S->sd})
        if (st) cudaStreamSynchronize(st);
    for (auto &kv : S->jobs) {
        Job *j = kv.second;
        if (j->done_ev) cudaEventDestroy(j->done_ev);
        if (j->ready_ev) cudaEventDestroy(j->ready_ev);
        if (j->admit_ev) cudaEventDestroy(j->admit_ev);
        for (cudaEvent_t e : j->chunk_done) cudaEventDestroy(e);
        if (j->h_err) cudaFreeHost(j->h_err);
        delete j;
    }
    if (S->exec) cudaGraphExecDestroy(S->exec);
    if (S->d_spec) cudaFree(S->d_spec);
    for (cudaStream_t s : S->lanes)
        if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : S->join)
        if (e) cudaEventDestroy(e);
    if (S->fork) cudaEventDestroy(S->fork);
    for (cudaEvent_t e : S->step_ev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : S->step_t0)
        if (e) cudaEventDestroy(e);
    for (cudaStream_t st : {S->s0, S->sa, S->sd, S->sc})
        if (st) cudaStreamDestroy(st);
    if (S->chunk_ev) cudaEventDestroy(S->chunk_ev);
    delete S;
    return SARBP_OK;
}

static std::shared_ptr<const HostTables> tables_for(sarbp_server *S, const sarbp_radar &r, const sarbp_rc_layout &lay) {
    const TableKey k{lay.nfft, r.upsample, lay.nc, lay.shift, r.kr, r.fs, r.tc, r.tp};
    {
        std::lock_guard<std::mutex> lk(S->tab_mu);
        for (auto &e : S->tab_cache)
            if (e.first == k) return e.second;
    }
    auto t = std::make_shared<HostTables>();
    sarbp::rc_tables_host(r, lay, t->filt, t->etab);  // outside the lock
    std::lock_guard<std::mutex> lk(S->tab_mu);
    if (S->tab_cache.size() >= 16) S->tab_cache.erase(S->tab_cache.begin());
    S->tab_cache.emplace_back(k, t);
    return t;
}

sarbp_status sarbp_server_submit(sarbp_server *S, const sarbp_job *job, uint64_t *ticket) {
    // a job's latency counts from here: validation, planning (geometry extremes
    // on the host) and table set-up are part of it
    const Clock::time_point t_entry = Clock::now();
    if (!S || !job || !ticket) return SARBP_ERR_INVALID_ARGUMENT;
    *ticket = 0;
    const sarbp_job &d = *job;
    if (d.mode != SARBP_MODE_SPLIT && d.mode != SARBP_MODE_FP16STORE) return SARBP_ERR_UNSUPPORTED;
    if (d.np <= 0 || d.ns <= 0 || d.grid.nx <= 0 || d.grid.ny <= 0 || !d.echo || !d.apc || !d.image)
        return SARBP_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < (size_t)3 * d.np; ++i)
        if (!std::isfinite(d.apc[i])) return SARBP_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(d.grid.origin[i]) || !std::isfinite(d.grid.ux[i]) || !std::isfinite(d.grid.uy[i]))
            return SARBP_ERR_INVALID_ARGUMENT;
    if ((long long)d.grid.nx * d.grid.ny > (1LL << 31)) return SARBP_ERR_INVALID_ARGUMENT;
    Job *j = new Job();
    j->desc = d;
    sarbp_status st = sarbp_rc_layout_get(&d.radar, d.ns, &j->lay);
    if (st != SARBP_OK) {
        delete j;
        return st;
    }
    if (!sarbp::rc_size_supported(j->lay.nfft) || j->lay.nbins % 4 != 0) {
        delete j;
        return SARBP_ERR_UNSUPPORTED;
    }
    j->storage = d.mode == SARBP_MODE_FP16STORE ? SARBP_STORE_C32H : SARBP_STORE_C64;
    j->esize = j->storage == SARBP_STORE_C64 ? 8 : 4;
    sarbp_rc_view v{};
    v.storage = j->storage;
    v.np = d.np;
    v.nbins = j->lay.nbins;
    v.t0_bins = j->lay.t0_bins;
    v.bin_rate = j->lay.bin_rate;
    std::string why;
    sarbp::BpExtremes ex;
    sarbp::bp_extremes_host(d.apc, d.np, d.grid, ex);  // same bits as the one-shot calls' device reduction
    j->pps = S->cfg.pulses_per_step;
    if (S->cfg.step_updates > 0) {  // about step_updates pixel*pulse updates per step
        const double px = (double)d.grid.nx * d.grid.ny;
        const double want = std::floor((double)S->cfg.step_updates / px / 16.0) * 16.0;
        const int all = (d.np + 15) / 16 * 16;
        j->pps = (int)std::max(16.0, std::min((double)all, want));
    }
    if (!sarbp::plan_bp(S->sms, d.radar, v, ex, d.np, d.grid, d.mode, j->pps, j->plan, why)) {
        delete j;
        return SARBP_ERR_UNSUPPORTED;
    }
    j->tab = tables_for(S, d.radar, j->lay);
    j->bytes = job_bytes(*j);
    if (j->bytes > S->cfg.hbm_budget_bytes) {
        std::lock_guard<std::mutex> lk(S->mu);
        S->st.rejected++;
        delete j;
        return SARBP_ERR_BUDGET;
    }
    cudaSetDevice(S->cfg.device);
    bool ev_ok = true;
    j->chunk_done.assign((d.np + S->spec_rows - 1) / S->spec_rows, nullptr);
    for (cudaEvent_t &e : j->chunk_done)
        if (ev_ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            ev_ok = false;
            e = nullptr;
        }
    j->chunk_done.erase(std::remove(j->chunk_done.begin(), j->chunk_done.end(), nullptr), j->chunk_done.end());
    if (!ev_ok || cudaEventCreateWithFlags(&j->done_ev, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&j->ready_ev) != cudaSuccess || cudaEventCreate(&j->admit_ev) != cudaSuccess ||
        cudaMallocHost(&j->h_err, sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        if (j->done_ev) cudaEventDestroy(j->done_ev);
        if (j->ready_ev) cudaEventDestroy(j->ready_ev);
        if (j->admit_ev) cudaEventDestroy(j->admit_ev);
        for (cudaEvent_t e : j->chunk_done) cudaEventDestroy(e);
        delete j;
        return SARBP_ERR_CUDA;
    }
    *j->h_err = 0;
    j->t_submit = t_entry;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) {
            cudaEventDestroy(j->done_ev);
            cudaEventDestroy(j->ready_ev);
            cudaEventDestroy(j->admit_ev);
            for (cudaEvent_t e : j->chunk_done) cudaEventDestroy(e);
            cudaFreeHost(j->h_err);
            delete j;
            return SARBP_ERR_CANCELLED;
        }
        j->id = S->next_id++;
        S->jobs[j->id] = j;
        S->queue.push_back(j);
        S->st.submitted++;
        *ticket = j->id;
    }
    S->cv_work.notify_all();
    return SARBP_OK;
}

static sarbp_status job_result(const Job *j) {
    switch (j->state) {
        case JobState::Done: return SARBP_OK;
        case JobState::Failed: return j->status != SARBP_OK ? j->status : SARBP_ERR_INTERNAL;
        case JobState::Cancelled: return SARBP_ERR_CANCELLED;
        default: return SARBP_ERR_NOT_READY;
    }
}

sarbp_status sarbp_server_poll(sarbp_server *S, uint64_t ticket) {
    if (!S) return SARBP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return SARBP_ERR_INVALID_ARGUMENT;
    return job_result(it->second);
}

sarbp_status sarbp_server_wait(sarbp_server *S, uint64_t ticket, int32_t timeout_ms, sarbp_job_stats *stats) {
    if (!S) return SARBP_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return SARBP_ERR_INVALID_ARGUMENT;
    Job *j = it->second;
    auto ready = [&] { return job_result(j) != SARBP_ERR_NOT_READY; };
    if (timeout_ms < 0) S->cv_done.wait(lk, ready);
    else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return SARBP_ERR_TIMEOUT;
    const sarbp_status st = job_result(j);
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        stats->status = st;
        stats->steps = j->steps;
        if (j->state == JobState::Done || j->state == JobState::Failed) {
            stats->queued_ms = j->t_admit.time_since_epoch().count() ? ms_between(j->t_submit, j->t_admit) : 0.0;
            stats->latency_ms = ms_between(j->t_submit, j->t_done);
        }
        stats->updates = (double)j->desc.grid.nx * j->desc.grid.ny * j->desc.np;
        stats->device_bytes = j->bytes;
    }
    S->jobs.erase(it);
    lk.unlock();
    if (j->done_ev) cudaEventDestroy(j->done_ev);
    if (j->ready_ev) cudaEventDestroy(j->ready_ev);
    if (j->admit_ev) cudaEventDestroy(j->admit_ev);
    for (cudaEvent_t e : j->chunk_done) cudaEventDestroy(e);
    if (j->h_err) cudaFreeHost(j->h_err);
    delete j;
    return st;
}

sarbp_status sarbp_server_cancel(sarbp_server *S, uint64_t ticket) {
    if (!S) return SARBP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->jobs.find(ticket);
    if (it == S->jobs.end()) return SARBP_ERR_INVALID_ARGUMENT;
    Job *j = it->second;
    if (j->state != JobState::Queued) return SARBP_ERR_NOT_READY;
    S->queue.erase(std::find(S->queue.begin(), S->queue.end(), j));
    j->state = JobState::Cancelled;
    j->status = SARBP_ERR_CANCELLED;
    S->st.cancelled++;
    S->cv_done.notify_all();
    return SARBP_OK;
}

sarbp_status sarbp_server_debug_set(sarbp_server *S, int32_t key, int64_t value) {
    if (!S) return SARBP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    switch (key) {
        case SARBP_SERVER_DEBUG_FAIL_ADMIT_TICKET:
            if (value < 0) return SARBP_ERR_INVALID_ARGUMENT;
            S->fail_admit_ticket = (uint64_t)value;
            return SARBP_OK;
        default:
            return SARBP_ERR_INVALID_ARGUMENT;
    }
}

sarbp_status sarbp_server_get_stats(sarbp_server *S, sarbp_server_stats *out) {
    if (!S || !out) return SARBP_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    fold_step(S, 0);
    fold_step(S, 1);
    *out = S->st;
    out->bytes_in_use = S->in_use;
    out->active = (int32_t)S->active.size();
    out->queued = (int32_t)S->queue.size();
    if (S->busy) out->busy_s += std::chrono::duration<double>(Clock::now() - S->busy_since).count();
    return SARBP_OK;
}

}  // extern "C"
