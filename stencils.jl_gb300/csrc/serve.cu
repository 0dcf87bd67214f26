// serve.cu — continuous batching of stencil jobs with device-resident state.
//
// No counterpart in the reference (a caller there runs each job as its own mapstencil! loop).
// Clients submit jobs (a host grid, stencil, reduction, boundary, step count).  A scheduler thread:
//   1. admits queued jobs in arrival order while their two device parents fit in the HBM budget
//      (a fraction of the free device memory at creation), copying the input to the device once;
//   2. runs a tick: one batched launch (batch.cu) that advances every admitted job by up to
//      steps_per_tick steps, whatever its grid size, stencil or element type;
//   3. retires jobs that reached their step count: their result is copied to pinned host memory, their
//      device memory returns to the budget, and their latency (submit to result on host) is recorded.
// Jobs that arrive while a tick runs join the next tick as soon as memory allows: the batch is
// re-formed every tick (continuous batching), and state never leaves the device between ticks.
// Each job's result equals running it alone with stc_map_steps (the batch is bit-identical per job).
#include <chrono>
#include <condition_variable>
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
    stc_grid grid{};            // logical grid description (dense column-major)
    std::vector<int32_t> offs;
    std::vector<double> wts;
    stc_stencil st{};
    stc_op op{};
    stc_bc bc{};
    int64_t nsteps = 0, remaining = 0;
    size_t bytes = 0;           // one grid
    void* h_in = nullptr;       // pinned copies
    void* h_out = nullptr;
    void* d[2] = {nullptr, nullptr};
    int cur = 0;                // parent holding the current state
    int state = JOB_QUEUED;
    int status = STC_OK;
    double t_submit = 0, t_done = 0;
};

}  // namespace stc

struct stc_server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<stc::ServeJob*> queue;
    std::vector<stc::ServeJob*> active;
    std::map<int64_t, stc::ServeJob*> jobs;
    int64_t next_id = 1;
    size_t budget = 0, used = 0, peak = 0;
    int steps_per_tick = 16;
    int64_t admitted = 0, finished = 0, ticks = 0;
    bool stop = false;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::thread worker;
    stc::DeviceCtx* ctx = nullptr;
};

namespace stc {

static void free_device(stc_server* s, ServeJob* j) {
    for (int k = 0; k < 2; ++k)
        if (j->d[k]) {
            cudaFreeAsync(j->d[k], s->stream);
            j->d[k] = nullptr;
        }
}

static void serve_loop(stc_server* s) {
    cudaSetDevice(s->device);
    stc_batch tick;
    while (true) {
        std::vector<ServeJob*> to_copy;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait_for(lk, std::chrono::milliseconds(2),
                                [&] { return s->stop || !s->queue.empty() || !s->active.empty(); });
            if (s->stop) break;
            // admission in arrival order while the budget allows
            while (!s->queue.empty()) {
                ServeJob* j = s->queue.front();
                if (j->state == JOB_CANCELLED) { s->queue.pop_front(); continue; }
                const size_t need = 2 * j->bytes;
                if (need > s->budget) {
                    s->queue.pop_front();
                    j->state = JOB_FAILED;
                    j->status = STC_ERR_BUDGET;
                    s->cv_done.notify_all();
                    continue;
                }
                if (s->used + need > s->budget) break;
                s->queue.pop_front();
                s->used += need;
                s->peak = std::max(s->peak, s->used);
                ++s->admitted;
                to_copy.push_back(j);
            }
        }
        // device state for newly admitted jobs (outside the lock)
        for (ServeJob* j : to_copy) {
            cudaError_t e = cudaMallocAsync(&j->d[0], j->bytes, s->stream);
            if (e == cudaSuccess) e = cudaMallocAsync(&j->d[1], j->bytes, s->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(j->d[0], j->h_in, j->bytes, cudaMemcpyHostToDevice, s->stream);
            std::lock_guard<std::mutex> lk(s->mu);
            if (e != cudaSuccess) {
                cuda_fail(e);
                free_device(s, j);
                s->used -= 2 * j->bytes;
                j->state = JOB_FAILED;
                j->status = STC_ERR_CUDA;
                s->cv_done.notify_all();
                continue;
            }
            if (j->state == JOB_CANCELLED) {   // cancelled while its memory was being set up
                free_device(s, j);
                s->used -= 2 * j->bytes;
                s->cv_done.notify_all();
                continue;
            }
            j->state = JOB_ACTIVE;
            j->cur = 0;
            s->active.push_back(j);
        }
        std::vector<ServeJob*> act;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            act = s->active;
        }
        if (act.empty()) continue;
        // one tick: every active job advances by up to steps_per_tick steps
        tick.specs.clear();
        std::vector<int64_t> chunk(act.size());
        int rc = STC_OK;
        for (size_t i = 0; i < act.size(); ++i) {
            ServeJob* j = act[i];
            chunk[i] = std::min<int64_t>(j->remaining, s->steps_per_tick);
            stc_grid a = j->grid, b = j->grid;
            a.data = j->d[j->cur];
            b.data = j->d[1 - j->cur];
            const int r = stc_batch_add(&tick, &a, &b, &j->st, &j->op, &j->bc, chunk[i]);
            if (r < 0) { rc = r; break; }
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
            else
                rc = take_status(tick.slot);
        }
        // retire finished jobs
        std::vector<ServeJob*> done;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            ++s->ticks;
            std::vector<ServeJob*> keep;
            for (size_t i = 0; i < act.size(); ++i) {
                ServeJob* j = act[i];
                if (rc) {
                    j->state = JOB_FAILED;
                    j->status = rc;
                    done.push_back(j);
                    continue;
                }
                if (tick.result_in_b[i]) j->cur = 1 - j->cur;
                j->remaining -= chunk[i];
                if (j->remaining <= 0 || j->state == JOB_CANCELLED) done.push_back(j);
                else keep.push_back(j);
            }
            s->active = keep;
        }
        for (ServeJob* j : done) {
            if (j->state != JOB_FAILED && j->state != JOB_CANCELLED)
                cudaMemcpyAsync(j->h_out, j->d[j->cur], j->bytes, cudaMemcpyDeviceToHost, s->stream);
            free_device(s, j);
        }
        if (!done.empty()) cudaStreamSynchronize(s->stream);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = now_s();
            for (ServeJob* j : done) {
                s->used -= 2 * j->bytes;
                if (j->state == JOB_ACTIVE) {
                    j->state = JOB_DONE;
                    ++s->finished;
                }
                j->t_done = t;
            }
            if (!done.empty()) s->cv_done.notify_all();
        }
    }
    batch_free(&tick);
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
    if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete s;
        return cuda_fail(e);
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
    cudaStreamSynchronize(s->stream);
    for (auto& kv : s->jobs) {
        ServeJob* j = kv.second;
        free_device(s, j);
        if (j->h_in) cudaFreeHost(j->h_in);
        if (j->h_out) cudaFreeHost(j->h_out);
        delete j;
    }
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
    delete s;
    return STC_OK;
}

int stc_server_submit(stc_server* s, const stc_job* job, int64_t* out_id) {
    if (!s || !job || !out_id || job->nsteps < 0) return STC_ERR_INVALID;
    const stc_grid& g = job->grid;
    if (g.ndims != 2 || !g.data || g.size[0] < 1 || g.size[1] < 1 || g.stride[0] != 1 || g.stride[1] != g.size[0])
        return STC_ERR_INVALID;
    if (job->bc.padding != STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
    // validate with the batch rules on placeholder device pointers
    stc_batch probe;
    stc_grid a = g, b = g;
    // (disjoint placeholders: the batch rules reject a dest that shares memory with its source)
    const uintptr_t span = (uintptr_t)(g.size[0] * g.size[1]) * (uintptr_t)dtype_size(g.dtype);
    a.data = (void*)(uintptr_t)0x100;
    b.data = (void*)((uintptr_t)0x200 + span);
    int rc = stc_batch_add(&probe, &a, &b, &job->stencil, &job->op, &job->bc, job->nsteps);
    if (rc < 0) return rc;
    ServeJob* j = new ServeJob();
    j->grid = g;
    j->offs.assign(job->stencil.offsets, job->stencil.offsets + job->stencil.len * job->stencil.ndims);
    if (job->stencil.weights) j->wts.assign(job->stencil.weights, job->stencil.weights + job->stencil.len);
    j->st = job->stencil;
    j->st.offsets = j->offs.data();
    j->st.weights = j->wts.empty() ? nullptr : j->wts.data();
    j->op = job->op;
    j->bc = job->bc;
    j->nsteps = j->remaining = job->nsteps;
    j->bytes = (size_t)g.size[0] * g.size[1] * dtype_size(g.dtype);
    cudaError_t e = cudaMallocHost(&j->h_in, j->bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&j->h_out, j->bytes);
    if (e != cudaSuccess) {
        if (j->h_in) cudaFreeHost(j->h_in);
        delete j;
        return cuda_fail(e);
    }
    std::memcpy(j->h_in, g.data, j->bytes);
    j->grid.data = nullptr;
    j->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        j->id = s->next_id++;
        if (j->nsteps == 0) {
            std::memcpy(j->h_out, j->h_in, j->bytes);
            j->state = JOB_DONE;
            j->t_done = j->t_submit;
            ++s->finished;
        } else {
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

int stc_server_fetch(stc_server* s, int64_t id, void* out, size_t out_bytes, double* out_latency_s) {
    if (!s) return STC_ERR_INVALID;
    ServeJob* j = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(id);
        if (it == s->jobs.end()) return STC_ERR_INVALID;
        j = it->second;
        if (j->state == JOB_FAILED) return j->status;
        if (j->state == JOB_CANCELLED) return STC_ERR_CANCELLED;
        if (j->state != JOB_DONE) return STC_ERR_BUSY;
        if (out && out_bytes < j->bytes) return STC_ERR_SIZE_MISMATCH;
        s->jobs.erase(it);
    }
    if (out) std::memcpy(out, j->h_out, j->bytes);
    if (out_latency_s) *out_latency_s = j->t_done - j->t_submit;
    cudaFreeHost(j->h_in);
    cudaFreeHost(j->h_out);
    delete j;
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
    while (!(s->queue.empty() && s->active.empty())) {
        if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout &&
            !(s->queue.empty() && s->active.empty()))
            return STC_ERR_TIMEOUT;
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
