// serve.cu — continuous batching of stencil jobs with device-resident state.
//
// No counterpart in the reference (a caller there runs each job as its own mapstencil! loop).
// Clients submit jobs (a host grid, stencil, reduction, boundary, step count); results stay on the device
// until the client fetches them.
//
// Data path (GB300: the copy engines read and write pageable host memory through the host's page tables at
// 90-200 GB/s, while a host memcpy runs at 15-20 GB/s): when the HBM budget allows, submit reserves the job's
// two device parents and copies the caller's grid (dense or pitched) straight into the first one on the
// server's upload stream; the call returns once the copy engine has consumed the host buffer, so the caller
// may reuse it.  Only when the budget is exhausted is the input staged in pinned host memory, and the
// scheduler uploads it once memory frees (jobs are admitted in arrival order).  When a job's run ends its
// result is copied on the download stream into a pinned buffer from a process-wide pool (copy engines
// write pinned memory at ~180 GB/s, a freshly allocated pageable buffer at ~17 GB/s), overlapped with the
// work still running; the job is finished once that copy has landed.  stc_server_fetch_buffer hands the
// pinned buffer itself to the caller (no copy), stc_server_fetch copies it into the caller's memory.
//
// A scheduler thread runs two lanes:
//   * solo lane (large grids, at least 2^21 cells): each job runs alone through stc_map_steps on the solo
//     stream (so it gets the specialised paths: temporal blocking, packed Life, vector kernels), at most
//     three runs queued on the stream at a time;
//   * tick lane (smaller grids): every tick is one batched launch (batch.cu) that advances every active job by
//     up to steps_per_tick steps, whatever its size, stencil or element type; the batch is re-formed every
//     tick (continuous batching), and state never leaves the device between ticks.
// The two lanes run concurrently on the GPU.  Each job's result equals running it alone with stc_map_steps
// (the batch is bit-identical per job).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "batch.h"
#include "profile.h"

namespace stc {

static double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum JobState { JOB_QUEUED = 0, JOB_ACTIVE = 1, JOB_DONE = 2, JOB_CANCELLED = 3, JOB_FAILED = 4 };

struct ServeJob {
    int64_t id = 0;
    stc_grid grid{};            // device-side description (column-major, rows at `pitch` bytes; data unset)
    std::vector<int32_t> offs;
    std::vector<double> wts;
    stc_stencil st{};
    stc_op op{};
    stc_bc bc{};
    int64_t nsteps = 0, remaining = 0;
    size_t bytes = 0;           // one device parent (pitched)
    size_t row = 0, pitch = 0;  // bytes of a row's cells; bytes between device rows (a multiple of 128)
    void* h_in = nullptr;       // pinned staging copy (only when the budget was exhausted at submit)
    void* h_out = nullptr;      // pinned result (from the pool)
    void* d[2] = {nullptr, nullptr};
    cudaEvent_t ev = nullptr;   // upload finished (stream order), then: solo run finished
    int cur = 0;                // parent holding the current state
    bool solo = false;
    bool uploaded = false;      // device parents hold the input (submitted straight, or staged and uploaded)
    bool waited = false;        // the tick stream already waits on the upload
    int state = JOB_QUEUED;
    int status = STC_OK;
    double t_submit = 0, t_done = 0;
};

}  // namespace stc

struct stc_server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<stc::ServeJob*> queue;          // submitted, not yet activated (arrival order)
    std::vector<stc::ServeJob*> active;        // tick lane
    std::vector<stc::ServeJob*> solo_running;  // solo lane, queued on the solo stream
    std::deque<stc::ServeJob*> solo_waiting;   // solo lane, uploaded, not yet queued
    std::vector<stc::ServeJob*> copying;       // runs ended, results being copied to pinned host memory
    std::map<int64_t, stc::ServeJob*> jobs;
    std::deque<int64_t> completed;             // ids that finished (or failed) and were not yet reported
    int64_t next_id = 1;
    size_t budget = 0, used = 0, peak = 0;
    int steps_per_tick = 16;
    int64_t solo_cells = 1ll << 21;
    int64_t admitted = 0, finished = 0, ticks = 0, staged_waiting = 0;
    bool stop = false;
    int device = 0;
    cudaStream_t stream = nullptr;   // ticks
    cudaStream_t solo = nullptr;     // solo runs
    cudaStream_t up = nullptr;       // uploads
    cudaStream_t down = nullptr;     // result downloads
    std::thread worker;
    stc::DeviceCtx* ctx = nullptr;
};

namespace stc {

// ---------------------------------------------------------------------------- pinned host buffers
// Process-wide pool (buffers handed to callers may outlive the server that filled them), by power-of-two
// size class from 64 KiB; at most kPoolKeep bytes stay pooled, the rest is freed on release.
constexpr size_t kPoolKeep = 16ull << 30;
static std::mutex g_pin_mu;
static std::map<size_t, std::vector<void*>> g_pin_free;
static std::map<void*, size_t> g_pin_size;
static size_t g_pin_pooled = 0;

static size_t pin_class(size_t bytes) {
    size_t c = 64 << 10;
    while (c < bytes) c <<= 1;
    return c;
}

static void* pinned_get(size_t bytes) {
    const size_t c = pin_class(bytes);
    {
        std::lock_guard<std::mutex> g(g_pin_mu);
        auto it = g_pin_free.find(c);
        if (it != g_pin_free.end() && !it->second.empty()) {
            void* p = it->second.back();
            it->second.pop_back();
            g_pin_pooled -= c;
            return p;
        }
    }
    void* p = nullptr;
    if (cudaMallocHost(&p, c) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_pin_mu);
    g_pin_size[p] = c;
    return p;
}

static bool pinned_put(void* p) {
    size_t c = 0;
    {
        std::lock_guard<std::mutex> g(g_pin_mu);
        auto it = g_pin_size.find(p);
        if (it == g_pin_size.end()) return false;
        c = it->second;
        if (g_pin_pooled + c <= kPoolKeep) {
            g_pin_free[c].push_back(p);
            g_pin_pooled += c;
            return true;
        }
        g_pin_size.erase(it);
    }
    cudaFreeHost(p);
    return true;
}

static void drop_job(ServeJob* j) {
    if (j->h_in) pinned_put(j->h_in);
    if (j->h_out) pinned_put(j->h_out);
    if (j->ev) cudaEventDestroy(j->ev);
    delete j;
}

constexpr int kSoloInFlight = 3;

static void free_parent(cudaStream_t s, ServeJob* j, int k) {
    if (j->d[k]) {
        cudaFreeAsync(j->d[k], s);
        j->d[k] = nullptr;
    }
}

// Device parents for j, its input uploaded from `host` (rows of grid.size[0] elements at `pitch` bytes) on
// the upload stream, and the event the lanes wait on.  The caller holds the reservation.
static int upload_job(stc_server* s, ServeJob* j, const void* host, size_t pitch) {
    cudaError_t e = cudaMallocAsync(&j->d[0], j->bytes, s->up);
    if (e == cudaSuccess) e = cudaMallocAsync(&j->d[1], j->bytes, s->up);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(j->d[0], j->pitch, host, pitch, j->row, (size_t)j->grid.size[1], cudaMemcpyHostToDevice,
                              s->up);
    if (e == cudaSuccess && !j->ev) e = cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(j->ev, s->up);
    if (e != cudaSuccess) {
        cuda_fail(e);
        free_parent(s->up, j, 0);
        free_parent(s->up, j, 1);
        return STC_ERR_CUDA;
    }
    j->uploaded = true;
    return STC_OK;
}

static void fail_job(stc_server* s, ServeJob* j, int status) {
    j->state = JOB_FAILED;
    j->status = status;
    s->completed.push_back(j->id);
    s->cv_done.notify_all();
}

// Queue a solo job's whole run on the solo stream (after its upload).
static int start_solo(stc_server* s, ServeJob* j) {
    cudaError_t e = cudaStreamWaitEvent(s->solo, j->ev, 0);
    if (e != cudaSuccess) return cuda_fail(e);
    stc_grid a = j->grid, b = j->grid;
    a.data = j->d[0];
    b.data = j->d[1];
    int32_t src_is_b = 0;
    void* prof = prof_begin(s->solo);
    int rc = stc_map_steps(&a, &b, &j->st, &j->op, &j->bc, j->nsteps, &src_is_b, s->solo, STC_ASYNC);
    prof_end(prof, s->solo, "serve_solo", 0.0, (double)j->grid.size[0] * j->grid.size[1] * j->nsteps);
    if (rc) return rc;
    j->cur = src_is_b ? 1 : 0;
    if ((e = cudaEventRecord(j->ev, s->solo)) != cudaSuccess) return cuda_fail(e);
    return STC_OK;
}

// A job's run ended on lane stream `st`: copy its result into a pinned buffer on the download stream (after
// `st`), release both device parents behind the copy, and wait for the copy in the `copying` list.  Holds mu.
static void finish_job(stc_server* s, ServeJob* j, cudaStream_t st) {
    if (j->state == JOB_ACTIVE) {
        const size_t host_bytes = j->row * (size_t)j->grid.size[1];
        j->h_out = pinned_get(host_bytes);
        cudaError_t e = j->h_out ? cudaEventRecord(j->ev, st) : cudaErrorMemoryAllocation;
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s->down, j->ev, 0);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(j->h_out, j->row, j->d[j->cur], j->pitch, j->row, (size_t)j->grid.size[1],
                                  cudaMemcpyDeviceToHost, s->down);
        if (e == cudaSuccess) e = cudaEventRecord(j->ev, s->down);
        if (e == cudaSuccess) {
            s->copying.push_back(j);
        } else {
            cuda_fail(e);
            fail_job(s, j, STC_ERR_CUDA);
        }
    } else {
        s->completed.push_back(j->id);   // cancelled while running
    }
    free_parent(s->down, j, 0);
    free_parent(s->down, j, 1);
    s->used -= 2 * j->bytes;
}

static void serve_loop(stc_server* s) {
    cudaSetDevice(s->device);
    stc_batch tick;
    while (true) {
        std::vector<ServeJob*> to_upload, to_start;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait_for(lk, std::chrono::milliseconds(1), [&] {
                return s->stop || !s->queue.empty() || !s->active.empty() || !s->solo_running.empty() ||
                       !s->solo_waiting.empty() ||
                       !s->copying.empty();
            });
            if (s->stop) break;
            // activation in arrival order; staged inputs wait for the budget
            while (!s->queue.empty()) {
                ServeJob* j = s->queue.front();
                if (j->state == JOB_CANCELLED) {
                    s->queue.pop_front();
                    s->completed.push_back(j->id);
                    if (j->uploaded) {
                        free_parent(s->up, j, 0);
                        free_parent(s->up, j, 1);
                        s->used -= 2 * j->bytes;
                    } else {
                        --s->staged_waiting;
                    }
                    s->cv_done.notify_all();
                    continue;
                }
                if (!j->uploaded) {
                    const size_t need = 2 * j->bytes;
                    if (s->used + need > s->budget) break;
                    s->used += need;
                    s->peak = std::max(s->peak, s->used);
                    --s->staged_waiting;
                    to_upload.push_back(j);
                }
                s->queue.pop_front();
                ++s->admitted;
                to_start.push_back(j);
            }
        }
        for (ServeJob* j : to_upload) {
            const int rc = upload_job(s, j, j->h_in, j->row);
            if (rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                s->used -= 2 * j->bytes;
                fail_job(s, j, rc);
            }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);   // cancel() may run concurrently
            for (ServeJob* j : to_start) {
                if (j->state == JOB_FAILED) continue;
                if (j->state == JOB_QUEUED) j->state = JOB_ACTIVE;   // a cancelled job is retired by its lane
                if (j->solo) s->solo_waiting.push_back(j);
                else s->active.push_back(j);
            }
        }
        // solo lane: at most kSoloInFlight runs queued on the solo stream at a time, so that its launches
        // never fill the stream's launch queue (a full queue blocks the launching thread, and with it the
        // ticks and the retirements)
        while (true) {
            ServeJob* j = nullptr;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                if (s->solo_waiting.empty() || (int)s->solo_running.size() >= kSoloInFlight) break;
                j = s->solo_waiting.front();
                s->solo_waiting.pop_front();
                if (j->state == JOB_CANCELLED) {
                    free_parent(s->solo, j, 0);
                    free_parent(s->solo, j, 1);
                    s->used -= 2 * j->bytes;
                    s->completed.push_back(j->id);
                    s->cv_done.notify_all();
                    continue;
                }
            }
            const int rc = start_solo(s, j);
            std::lock_guard<std::mutex> lk(s->mu);
            if (rc) {
                // the run may be partly queued: release the memory after the stream drains it
                free_parent(s->solo, j, 0);
                free_parent(s->solo, j, 1);
                s->used -= 2 * j->bytes;
                fail_job(s, j, rc);
            } else {
                s->solo_running.push_back(j);
            }
        }
        // solo lane: retire finished runs
        {
            std::vector<ServeJob*> running;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                running = s->solo_running;
            }
            std::vector<ServeJob*> done;
            for (ServeJob* j : running) {
                const cudaError_t q = cudaEventQuery(j->ev);
                if (q == cudaErrorNotReady) continue;
                done.push_back(j);
                if (q != cudaSuccess) j->status = cuda_fail(q);
            }
            if (!done.empty()) {
                // a kernel's bounded wait or inexact conversion is reported on the solo stream's slot
                const int st = take_status(status_slot(s->ctx, s->solo));
                std::lock_guard<std::mutex> lk(s->mu);
                for (ServeJob* j : done) {
                    s->solo_running.erase(std::find(s->solo_running.begin(), s->solo_running.end(), j));
                    if (j->status == STC_OK && st != STC_OK) j->status = st;
                    if (j->status != STC_OK) {
                        free_parent(s->solo, j, 0);
                        free_parent(s->solo, j, 1);
                        s->used -= 2 * j->bytes;
                        fail_job(s, j, j->status);
                    } else {
                        finish_job(s, j, s->solo);
                    }
                }
                s->cv_done.notify_all();
            }
        }
        // results that reached host memory
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (!s->copying.empty()) {
                std::vector<ServeJob*> still;
                bool any = false;
                for (ServeJob* j : s->copying) {
                    const cudaError_t q = cudaEventQuery(j->ev);
                    if (q == cudaErrorNotReady) {
                        still.push_back(j);
                        continue;
                    }
                    any = true;
                    if (q != cudaSuccess) {
                        fail_job(s, j, cuda_fail(q));
                    } else if (j->state == JOB_ACTIVE) {
                        j->state = JOB_DONE;
                        j->t_done = now_s();
                        ++s->finished;
                        s->completed.push_back(j->id);
                    }
                }
                s->copying = still;
                if (any) s->cv_done.notify_all();
            }
        }
        // tick lane
        std::vector<ServeJob*> act;
        bool busy = false;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            act = s->active;
            busy = !s->solo_running.empty() || !s->solo_waiting.empty() || !s->copying.empty();
        }
        if (act.empty()) {
            if (busy) std::this_thread::sleep_for(std::chrono::microseconds(50));   // poll, not spin
            continue;
        }
        tick.specs.clear();
        std::vector<int64_t> chunk(act.size());
        int rc = STC_OK;
        for (size_t i = 0; i < act.size() && !rc; ++i) {
            ServeJob* j = act[i];
            if (!j->waited) {
                cudaError_t e = cudaStreamWaitEvent(s->stream, j->ev, 0);
                if (e != cudaSuccess) rc = cuda_fail(e);
                j->waited = true;
            }
            chunk[i] = std::min<int64_t>(j->remaining, s->steps_per_tick);
            stc_grid a = j->grid, b = j->grid;
            a.data = j->d[j->cur];
            b.data = j->d[1 - j->cur];
            const int r = stc_batch_add(&tick, &a, &b, &j->st, &j->op, &j->bc, chunk[i]);
            if (r < 0) rc = r;
        }
        if (!rc) rc = batch_build(&tick, false, s->stream, s->ctx, false);
        if (!rc) {
            void* prof = prof_begin(s->stream);
            rc = batch_launch(&tick, s->stream);
            prof_end(prof, s->stream, "serve_tick", 0.0, tick.planned_cell_steps);
        }
        if (!rc) {
            cudaError_t e = cudaStreamSynchronize(s->stream);
            if (e != cudaSuccess) rc = cuda_fail(e);
            else rc = take_status(tick.slot);
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            ++s->ticks;
            std::vector<ServeJob*> keep;
            for (size_t i = 0; i < act.size(); ++i) {
                ServeJob* j = act[i];
                if (rc) {
                    free_parent(s->stream, j, 0);
                    free_parent(s->stream, j, 1);
                    s->used -= 2 * j->bytes;
                    fail_job(s, j, rc);
                    continue;
                }
                if (tick.result_in_b[i]) j->cur = 1 - j->cur;
                j->remaining -= chunk[i];
                if (j->remaining <= 0 || j->state == JOB_CANCELLED) finish_job(s, j, s->stream);
                else keep.push_back(j);
            }
            s->active = keep;
            s->cv_done.notify_all();
        }
    }
    batch_free(&tick);
}

static int64_t solo_threshold() {
    const char* e = getenv("STC_SERVE_SOLO_CELLS");
    return e ? atoll(e) : (1ll << 21);
}

}  // namespace stc

using namespace stc;

extern "C" {

int stc_server_create(stc_server** out, double hbm_fraction, int32_t steps_per_tick) {
    if (!out || hbm_fraction <= 0 || hbm_fraction > 1 || steps_per_tick < 1) return STC_ERR_INVALID;
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return cuda_fail(e);
    stc_server* s = new stc_server();
    s->ctx = ctx;
    s->device = ctx->device;
    s->budget = (size_t)(hbm_fraction * (double)free_b);
    s->steps_per_tick = steps_per_tick;
    s->solo_cells = solo_threshold();
    cudaStream_t* st[4] = {&s->stream, &s->solo, &s->up, &s->down};
    for (cudaStream_t* p : st) {
        if ((e = cudaStreamCreateWithFlags(p, cudaStreamNonBlocking)) != cudaSuccess) {
            for (cudaStream_t* q : st)
                if (*q) cudaStreamDestroy(*q);
            delete s;
            return cuda_fail(e);
        }
    }
    s->worker = std::thread(serve_loop, s);
    *out = s;
    return STC_OK;
}

int stc_server_destroy(stc_server* s) {
    if (!s) return STC_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaStream_t st[4] = {s->stream, s->solo, s->up, s->down};
    for (cudaStream_t q : st) cudaStreamSynchronize(q);
    for (auto& kv : s->jobs) {
        ServeJob* j = kv.second;
        free_parent(s->up, j, 0);
        free_parent(s->up, j, 1);
        drop_job(j);
    }
    for (cudaStream_t q : st) {
        cudaStreamSynchronize(q);
        cudaStreamDestroy(q);
    }
    delete s;
    return STC_OK;
}

int stc_server_submit(stc_server* s, const stc_job* job, int64_t* out_id) {
    if (!s || !job || !out_id || job->nsteps < 0) return STC_ERR_INVALID;
    const stc_grid& g = job->grid;
    // the host grid: column-major, rows of size[0] elements at a pitch of stride[1] elements
    if (g.ndims != 2 || !g.data || g.size[0] < 1 || g.size[1] < 1 || g.stride[0] != 1 || g.stride[1] < g.size[0])
        return STC_ERR_INVALID;
    if (job->bc.padding != STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
    const size_t es = (size_t)dtype_size(g.dtype);
    // device rows on 128-byte boundaries, so every grid can be staged by TMA
    const size_t row = (size_t)g.size[0] * es, dpitch = (row + 127) / 128 * 128;
    // validate with the batch rules on placeholder device pointers
    stc_batch probe;
    stc_grid a = g, b = g;
    a.stride[1] = b.stride[1] = (int64_t)(dpitch / es);
    // (disjoint placeholders: the batch rules reject a dest that shares memory with its source)
    const uintptr_t span = (uintptr_t)(dpitch * g.size[1]);
    a.data = (void*)(uintptr_t)0x100;
    b.data = (void*)((uintptr_t)0x200 + span);
    int rc = stc_batch_add(&probe, &a, &b, &job->stencil, &job->op, &job->bc, job->nsteps);
    if (rc < 0) return rc;
    ServeJob* j = new ServeJob();
    j->grid = g;
    j->grid.stride[1] = (int64_t)(dpitch / es);
    j->grid.data = nullptr;
    j->row = row;
    j->pitch = dpitch;
    j->offs.assign(job->stencil.offsets, job->stencil.offsets + job->stencil.len * job->stencil.ndims);
    if (job->stencil.weights) j->wts.assign(job->stencil.weights, job->stencil.weights + job->stencil.len);
    j->st = job->stencil;
    j->st.offsets = j->offs.data();
    j->st.weights = j->wts.empty() ? nullptr : j->wts.data();
    j->op = job->op;
    j->bc = job->bc;
    j->nsteps = j->remaining = job->nsteps;
    j->bytes = dpitch * (size_t)g.size[1];
    // Large grids run alone (specialised paths), except cellular automata whose rows pack into words: their
    // persistent kernel needs every SM to itself, so they stay in the tick lane.
    const bool packs = job->op.code == STC_OP_LIFE && g.size[0] % 32 == 0;
    j->solo = (int64_t)g.size[0] * g.size[1] >= s->solo_cells && !packs;
    j->t_submit = now_s();
    const size_t pitch = (size_t)g.stride[1] * es;
    bool direct = false;
    if (j->nsteps > 0) {
        std::lock_guard<std::mutex> lk(s->mu);
        if (2 * j->bytes > s->budget) {
            // can never be admitted: registered as failed, so poll and fetch report STC_ERR_BUDGET
            j->state = JOB_FAILED;
            j->status = STC_ERR_BUDGET;
            j->id = s->next_id++;
            s->jobs[j->id] = j;
            s->completed.push_back(j->id);
            *out_id = j->id;
            return STC_OK;
        }
        // straight to the device while the budget allows and no staged job waits ahead of this one
        if (s->staged_waiting == 0 && s->used + 2 * j->bytes <= s->budget) {
            s->used += 2 * j->bytes;
            s->peak = std::max(s->peak, s->used);
            direct = true;
        }
    }
    if (direct) {
        if ((rc = upload_job(s, j, g.data, pitch))) {
            std::lock_guard<std::mutex> lk(s->mu);
            s->used -= 2 * j->bytes;
            direct = false;
        }
    }
    if (!direct) {
        // staged: a pinned copy, uploaded when the budget allows (also the nsteps == 0 result)
        j->h_in = pinned_get(row * (size_t)g.size[1]);
        if (!j->h_in) {
            delete j;
            return STC_ERR_CUDA;
        }
        for (int64_t y = 0; y < g.size[1]; ++y)
            std::memcpy((char*)j->h_in + y * row, (const char*)g.data + y * pitch, row);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        j->id = s->next_id++;
        if (j->nsteps == 0) {
            j->state = JOB_DONE;
            j->t_done = j->t_submit;
            ++s->finished;
            s->completed.push_back(j->id);
        } else {
            if (!direct) ++s->staged_waiting;
            s->queue.push_back(j);
        }
        s->jobs[j->id] = j;
        *out_id = j->id;
    }
    s->cv_work.notify_all();
    return STC_OK;
}

int stc_server_poll(stc_server* s, int64_t id) {
    if (!s) return STC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return STC_ERR_INVALID;
    const ServeJob* j = it->second;
    if (j->state == JOB_DONE) return 1;
    if (j->state == JOB_FAILED) return j->status;
    if (j->state == JOB_CANCELLED) return STC_ERR_CANCELLED;
    return 0;
}

// Take a finished job out of the server: its pinned result (the staged input when nsteps == 0).
static int take_result(stc_server* s, int64_t id, size_t out_bytes, bool check_size, ServeJob** out_job) {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return STC_ERR_INVALID;
    ServeJob* j = it->second;
    if (j->state == JOB_FAILED) return j->status;
    if (j->state == JOB_CANCELLED) return STC_ERR_CANCELLED;
    if (j->state != JOB_DONE) return STC_ERR_BUSY;
    if (check_size && out_bytes < j->row * (size_t)j->grid.size[1]) return STC_ERR_SIZE_MISMATCH;
    s->jobs.erase(it);
    if (!j->h_out) {   // nsteps == 0
        j->h_out = j->h_in;
        j->h_in = nullptr;
    }
    *out_job = j;
    return STC_OK;
}

int stc_server_fetch(stc_server* s, int64_t id, void* out, size_t out_bytes, double* out_latency_s) {
    if (!s) return STC_ERR_INVALID;
    ServeJob* j = nullptr;
    int rc = take_result(s, id, out_bytes, out != nullptr, &j);
    if (rc) return rc;
    if (out) std::memcpy(out, j->h_out, j->row * (size_t)j->grid.size[1]);
    if (out_latency_s) *out_latency_s = j->t_done - j->t_submit;
    drop_job(j);
    return STC_OK;
}

int stc_server_fetch_buffer(stc_server* s, int64_t id, void** out_host, size_t* out_bytes, double* out_latency_s) {
    if (!s || !out_host) return STC_ERR_INVALID;
    ServeJob* j = nullptr;
    int rc = take_result(s, id, 0, false, &j);
    if (rc) return rc;
    *out_host = j->h_out;
    if (out_bytes) *out_bytes = j->row * (size_t)j->grid.size[1];
    if (out_latency_s) *out_latency_s = j->t_done - j->t_submit;
    j->h_out = nullptr;   // the caller's until stc_server_release_buffer
    drop_job(j);
    return STC_OK;
}

int stc_server_release_buffer(void* host) {
    if (!host) return STC_ERR_INVALID;
    return pinned_put(host) ? STC_OK : STC_ERR_INVALID;
}

int stc_server_ready(stc_server* s, int64_t* ids, int32_t max_ids, double timeout_s, int32_t* n_out) {
    if (!s || !n_out || max_ids < 0 || (max_ids > 0 && !ids)) return STC_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->completed.empty() && timeout_s > 0)
        s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return !s->completed.empty(); });
    int32_t n = 0;
    while (n < max_ids && !s->completed.empty()) {
        ids[n++] = s->completed.front();
        s->completed.pop_front();
    }
    *n_out = n;
    return STC_OK;
}

int stc_server_cancel(stc_server* s, int64_t id) {
    if (!s) return STC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return STC_ERR_INVALID;
    ServeJob* j = it->second;
    if (j->state == JOB_QUEUED || j->state == JOB_ACTIVE) j->state = JOB_CANCELLED;
    return STC_OK;
}

int stc_server_drain(stc_server* s, double timeout_s) {
    if (!s) return STC_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    auto idle = [&] {
        return s->queue.empty() && s->active.empty() && s->solo_running.empty() && s->solo_waiting.empty() &&
               s->copying.empty();
    };
    while (!idle()) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !idle()) return STC_ERR_TIMEOUT;
    }
    return STC_OK;
}

int stc_server_stats(const stc_server* s, int64_t* admitted, int64_t* finished, int64_t* ticks, int64_t* peak) {
    if (!s) return STC_ERR_INVALID;
    stc_server* m = const_cast<stc_server*>(s);
    std::lock_guard<std::mutex> lk(m->mu);
    if (admitted) *admitted = s->admitted;
    if (finished) *finished = s->finished;
    if (ticks) *ticks = s->ticks;
    if (peak) *peak = (int64_t)s->peak;
    return STC_OK;
}

}  // extern "C"
