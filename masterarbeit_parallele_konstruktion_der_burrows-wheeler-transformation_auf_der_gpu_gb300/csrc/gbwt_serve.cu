// gbwt_serve.cu -- serving loop: BWT jobs admitted under a device-memory
// budget, small jobs merged into batched pipeline runs (host code; all GPU
// work goes through the library's own C ABI).
//
// The reference has no serving path: one process builds one BWT
// (main(), K:4793-4815 of Prefix_Free_Parsing_W=5_P=16_kommentiert.cu).
//
// Scheduling.  Jobs wait in arrival order.  A free worker takes the first
// waiting job that fits the budget: a small job (n <= small_max) takes every
// later waiting small job of the same (W, P, alphabet) variant with it, up
// to batch_max bytes, and the worker runs them as one gbwt_pfp_bwt_batch
// call; a large job runs alone.  A job that does not fit stays at the head
// while later jobs that fit pass it; when nothing runs, the head is admitted
// whatever its estimate, so every job eventually runs.  Workers have their
// own storage and stream, so a large job and batches of small ones overlap
// on the device.
#include "gbwt_internal.cuh"
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

namespace gbwt {
namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    const uint8_t *T = nullptr;
    uint8_t *L = nullptr;
    int64_t n = 0;
    int32_t W = 5, P = 16;
    uint32_t flags = 0;
    int64_t status = GBWT_JOB_PENDING;
    int64_t est = 0;
    double submit_us = 0, start_us = 0, end_us = 0;
    int32_t batch = 0, worker = -1;
};

// Device-memory estimates (bytes) of one pipeline call.  Measured scratch
// (gbwt_stats.device_bytes) after 512 MiB of repetitive DNA: 14.8 bytes per
// text byte for one text, 22.5 for a batch of 4096 texts (plus the batch's
// staged input and output, 2 bytes per byte).
int64_t est_single(int64_t n) { return 20 * n + ((int64_t)64 << 20); }
int64_t est_batch(int64_t total, int64_t jobs) { return 28 * total + 64 * jobs + ((int64_t)64 << 20); }

struct Unit {
    std::vector<int64_t> ids;
    std::vector<Job *> jobs;            // stable addresses, taken under the lock
    int64_t total = 0;
    int64_t est = 0;
};

struct Server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job> jobs;               // by ticket; references stay valid on push_back
    std::deque<int64_t> pending;
    int64_t budget = 0, small_max = 0, batch_max = 0;
    int64_t in_use = 0, peak = 0;
    int64_t unfinished = 0;
    int device = 0;
    int nworkers = 1;
    bool simulate = false, stopping = false;
    std::vector<std::thread> threads;
    Clock::time_point t0;

    double now_us() const
    {
        return std::chrono::duration<double, std::micro>(Clock::now() - t0).count();
    }
};

bool same_variant(const Job &a, const Job &b)
{
    return a.W == b.W && a.P == b.P &&
           (a.flags & GBWT_FLAG_SMALL_ALPHABET) == (b.flags & GBWT_FLAG_SMALL_ALPHABET);
}

// Next admissible unit; called with the lock held.
bool pick(Server *s, Unit &u)
{
    const int64_t room = s->budget - s->in_use;
    for (size_t qi = 0; qi < s->pending.size(); qi++) {
        const Job &j = s->jobs[(size_t)s->pending[qi]];
        u.ids.clear();
        u.total = 0;
        if (j.n <= s->small_max) {
            for (size_t r = qi; r < s->pending.size(); r++) {
                const Job &c = s->jobs[(size_t)s->pending[r]];
                if (c.n > s->small_max || !same_variant(c, j)) continue;
                if (!u.ids.empty() && u.total + c.n > s->batch_max) break;
                u.ids.push_back(s->pending[r]);
                u.total += c.n;
            }
            while (u.ids.size() > 1 && est_batch(u.total, (int64_t)u.ids.size()) > room) {
                u.total -= s->jobs[(size_t)u.ids.back()].n;
                u.ids.pop_back();
            }
            u.est = u.ids.size() > 1 ? est_batch(u.total, (int64_t)u.ids.size()) : est_single(u.total);
        } else {
            u.ids.push_back(s->pending[qi]);
            u.total = j.n;
            u.est = est_single(j.n);
        }
        if (u.est <= room || s->in_use == 0) {
            std::deque<int64_t> rest;
            size_t k = 0;
            std::vector<int64_t> taken = u.ids;
            std::sort(taken.begin(), taken.end());
            for (int64_t id : s->pending) {
                if (k < taken.size() && std::binary_search(taken.begin(), taken.end(), id)) {
                    k++;
                    continue;
                }
                rest.push_back(id);
            }
            s->pending.swap(rest);
            u.jobs.clear();
            for (int64_t id : u.ids) u.jobs.push_back(&s->jobs[(size_t)id]);
            return true;
        }
    }
    return false;
}

// Worker-local device state.
struct WorkerState {
    void *st = nullptr;
    uint8_t *din = nullptr, *dout = nullptr;
    size_t dcap = 0;
    std::vector<int64_t> offs;
};

int64_t run_alone(WorkerState &ws, Job &j)
{
    return gbwt_pfp_bwt(ws.st, j.T, j.L, j.n, j.W, j.P, j.flags & GBWT_FLAG_SMALL_ALPHABET);
}

// One batched call; the texts are staged into device memory by the worker.
int64_t run_batch_unit(WorkerState &ws, const Unit &u)
{
    Storage *st = (Storage *)ws.st;
    const size_t need = (size_t)u.total + 16;
    if (ws.dcap < need) {
        if (ws.din) cudaFree(ws.din);
        if (ws.dout) cudaFree(ws.dout);
        ws.din = ws.dout = nullptr;
        ws.dcap = 0;
        if (cudaMalloc(&ws.din, need) != cudaSuccess || cudaMalloc(&ws.dout, need) != cudaSuccess)
            return GBWT_GPU_NOT_ENOUGH_MEMORY;
        ws.dcap = need;
    }
    ws.offs.assign(u.ids.size() + 1, 0);
    for (size_t i = 0; i < u.jobs.size(); i++) {
        const Job &j = *u.jobs[i];
        ws.offs[i + 1] = ws.offs[i] + j.n;
        if (cudaMemcpyAsync(ws.din + ws.offs[i], j.T, (size_t)j.n, cudaMemcpyHostToDevice, st->stream) !=
            cudaSuccess)
            return GBWT_GPU_ERROR;
    }
    const Job &j0 = *u.jobs[0];
    const int64_t rc = gbwt_pfp_bwt_batch(ws.st, ws.din, ws.offs.data(), (int32_t)u.ids.size(), ws.dout, j0.W, j0.P,
                                          (j0.flags & GBWT_FLAG_SMALL_ALPHABET) | GBWT_FLAG_DEVICE_POINTERS);
    if (rc < 0) return rc;
    for (size_t i = 0; i < u.jobs.size(); i++) {
        Job &j = *u.jobs[i];
        if (cudaMemcpyAsync(j.L, ws.dout + ws.offs[i], (size_t)j.n, cudaMemcpyDeviceToHost, st->stream) !=
            cudaSuccess)
            return GBWT_GPU_ERROR;
    }
    return cudaStreamSynchronize(st->stream) == cudaSuccess ? GBWT_NO_ERROR : GBWT_GPU_ERROR;
}

void simulate_unit(const Unit &u)
{
    const double secs = (double)u.total / 1e9 + 20e-6;
    std::this_thread::sleep_for(std::chrono::duration<double>(secs));
    for (Job *j : u.jobs)
        if (j->n) memcpy(j->L, j->T, (size_t)j->n);
}

void worker_main(Server *s, int w)
{
    WorkerState ws;
    int64_t setup_rc = GBWT_NO_ERROR;
    if (!s->simulate) {
        if (cudaSetDevice(s->device) != cudaSuccess) setup_rc = GBWT_GPU_ERROR;
        else setup_rc = gbwt_allocate_device_storage(&ws.st, 0);
    }
    const int64_t keep = s->budget / (int64_t)s->nworkers;
    for (;;) {
        Unit u;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (pick(s, u)) break;
                if (s->stopping && s->pending.empty()) {
                    lk.unlock();
                    if (ws.din) cudaFree(ws.din);
                    if (ws.dout) cudaFree(ws.dout);
                    if (ws.st) gbwt_free_device_storage(ws.st);
                    return;
                }
                s->cv_work.wait(lk);
            }
            s->in_use += u.est;
            s->peak = std::max(s->peak, s->in_use);
            const double t = s->now_us();
            for (Job *jp : u.jobs) {
                Job &j = *jp;
                j.status = GBWT_JOB_RUNNING;
                j.start_us = t;
                j.batch = (int32_t)u.ids.size();
                j.worker = w;
                j.est = u.est;
            }
        }
        std::vector<int64_t> rcs(u.ids.size(), setup_rc);
        if (setup_rc == GBWT_NO_ERROR) {
            if (s->simulate) {
                simulate_unit(u);
            } else if (u.jobs.size() == 1) {
                rcs[0] = run_alone(ws, *u.jobs[0]);
            } else {
                const int64_t rc = run_batch_unit(ws, u);
                if (rc == GBWT_BAD_PARAMETER || rc == GBWT_UNSUPPORTED_INPUT) {
                    // one job's input is invalid: run each alone so only it fails
                    for (size_t i = 0; i < u.jobs.size(); i++) rcs[i] = run_alone(ws, *u.jobs[i]);
                } else {
                    std::fill(rcs.begin(), rcs.end(), rc);
                }
            }
            if (!s->simulate) {
                gbwt_stats stats;
                if (gbwt_get_stats(ws.st, &stats) == GBWT_NO_ERROR &&
                    stats.device_bytes + 2 * (int64_t)ws.dcap > keep) {
                    gbwt_trim_device_storage(ws.st);
                    if (ws.din) cudaFree(ws.din);
                    if (ws.dout) cudaFree(ws.dout);
                    ws.din = ws.dout = nullptr;
                    ws.dcap = 0;
                }
            }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = s->now_us();
            for (size_t i = 0; i < u.jobs.size(); i++) {
                Job &j = *u.jobs[i];
                j.status = rcs[i] < 0 ? rcs[i] : GBWT_NO_ERROR;
                j.end_us = t;
            }
            s->in_use -= u.est;
            s->unfinished -= (int64_t)u.ids.size();
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

void fill_info(const Job &j, gbwt_job_info *info)
{
    if (!info) return;
    info->status = j.status;
    info->n = j.n;
    info->est_bytes = j.est;
    info->submit_us = j.submit_us;
    info->start_us = j.start_us;
    info->end_us = j.end_us;
    info->batch_jobs = j.batch;
    info->worker = j.worker;
}

}  // namespace
}  // namespace gbwt

using namespace gbwt;

extern "C" int64_t gbwt_server_create(void **server, int64_t hbm_budget, int32_t workers, int64_t small_max,
                                      uint32_t flags)
{
    if (!server || workers < 0 || workers > 64) return GBWT_BAD_PARAMETER;
    *server = nullptr;
    Server *s = new (std::nothrow) Server();
    if (!s) return GBWT_NOT_ENOUGH_MEMORY;
    s->simulate = (flags & GBWT_SERVER_SIMULATE) != 0;
    s->small_max = small_max > 0 ? small_max : ((int64_t)16 << 20);
    s->batch_max = std::max<int64_t>(s->small_max, (int64_t)512 << 20);
    if (hbm_budget > 0) {
        s->budget = hbm_budget;
    } else if (s->simulate) {
        s->budget = (int64_t)1 << 34;
    } else {
        size_t free_b = 0, total_b = 0;
        if (cudaGetDevice(&s->device) != cudaSuccess || cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
            delete s;
            return GBWT_GPU_ERROR;
        }
        s->budget = (int64_t)(0.8 * (double)free_b);
    }
    if (!s->simulate && hbm_budget > 0 && cudaGetDevice(&s->device) != cudaSuccess) {
        delete s;
        return GBWT_GPU_ERROR;
    }
    s->t0 = Clock::now();
    const int nw = workers > 0 ? workers : 2;
    s->nworkers = nw;
    try {
        s->threads.reserve((size_t)nw);
        for (int w = 0; w < nw; w++) s->threads.emplace_back(worker_main, s, w);
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stopping = true;
        }
        s->cv_work.notify_all();
        for (auto &t : s->threads) t.join();
        delete s;
        return GBWT_NOT_ENOUGH_MEMORY;
    }
    *server = s;
    return GBWT_NO_ERROR;
}

extern "C" int64_t gbwt_server_drain(void *server, double timeout_s)
{
    Server *s = (Server *)server;
    if (!s) return GBWT_BAD_PARAMETER;
    std::unique_lock<std::mutex> lk(s->mu);
    const auto pred = [&]() { return s->unfinished == 0; };
    if (timeout_s < 0) {
        s->cv_done.wait(lk, pred);
        return GBWT_NO_ERROR;
    }
    return s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred) ? GBWT_NO_ERROR : GBWT_TIMEOUT;
}

extern "C" int64_t gbwt_server_destroy(void *server)
{
    Server *s = (Server *)server;
    if (!s) return GBWT_BAD_PARAMETER;
    gbwt_server_drain(s, -1.0);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->threads) t.join();
    delete s;
    return GBWT_NO_ERROR;
}

extern "C" int64_t gbwt_submit(void *server, const uint8_t *T, uint8_t *L, int64_t n, int32_t W, int32_t P,
                               uint32_t flags, int64_t *ticket)
{
    Server *s = (Server *)server;
    if (!s || !ticket || n < 0 || (n > 0 && (!T || !L)) || W < 1 || W > 64 || P < 1 || P > 65535)
        return GBWT_BAD_PARAMETER;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) return GBWT_BAD_PARAMETER;
        Job j;
        j.T = T;
        j.L = L;
        j.n = n;
        j.W = W;
        j.P = P;
        j.flags = flags;
        j.submit_us = s->now_us();
        *ticket = (int64_t)s->jobs.size();
        s->jobs.push_back(j);
        s->pending.push_back(*ticket);
        s->unfinished++;
    }
    s->cv_work.notify_one();
    return GBWT_NO_ERROR;
}

extern "C" int64_t gbwt_poll(void *server, int64_t ticket, gbwt_job_info *info)
{
    Server *s = (Server *)server;
    if (!s) return GBWT_BAD_PARAMETER;
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket < 0 || ticket >= (int64_t)s->jobs.size()) return GBWT_BAD_PARAMETER;
    const Job &j = s->jobs[(size_t)ticket];
    fill_info(j, info);
    return j.status;
}

extern "C" int64_t gbwt_wait(void *server, int64_t ticket, double timeout_s, gbwt_job_info *info)
{
    Server *s = (Server *)server;
    if (!s) return GBWT_BAD_PARAMETER;
    std::unique_lock<std::mutex> lk(s->mu);
    if (ticket < 0 || ticket >= (int64_t)s->jobs.size()) return GBWT_BAD_PARAMETER;
    const auto done = [&]() {
        const int64_t st = s->jobs[(size_t)ticket].status;
        return st != GBWT_JOB_PENDING && st != GBWT_JOB_RUNNING;
    };
    if (timeout_s < 0) s->cv_done.wait(lk, done);
    else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
    const Job &j = s->jobs[(size_t)ticket];
    fill_info(j, info);
    return j.status;
}

extern "C" int64_t gbwt_server_peak_admitted(void *server)
{
    Server *s = (Server *)server;
    if (!s) return GBWT_BAD_PARAMETER;
    std::lock_guard<std::mutex> lk(s->mu);
    return s->peak;
}
