// Asynchronous batch queue: tbg_batch_submit / tbg_batch_poll / tbg_batch_wait.
//
// A job is a descriptor naming one of the batch entry points (hall
// conductivity, bands, band-resolved or occupied Berry curvature).  Worker
// threads owned by the library pop jobs in submission order and run them
// through the same C-ABI calls a synchronous caller makes; those calls are
// thread-safe and each runs on its own CUDA stream, so jobs of different
// models overlap on the GPU.  The status and message of a finished job are
// kept until the ticket is released by poll (done) or wait.

#include <cuda_runtime.h>

#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "tbgpu_internal.cuh"
#include "../../include/tbgpu.h"

namespace tbg {
namespace {

struct JobRec {
    tbg_job job;
    std::vector<int64_t> kmesh;
    std::vector<double> dirs2, mu;
    int device = 0;
    bool done = false;
    int status = TBG_OK;
    std::string err;
};

struct Queue {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<JobRec>> pending;
    std::unordered_map<int64_t, std::shared_ptr<JobRec>> jobs;
    int64_t next_ticket = 1;
    int want_workers = 4;
    int started = 0;
};

// Never destroyed: workers are detached and may outlive static destructors.
Queue& queue() {
    static Queue* q = new Queue();
    return *q;
}

int run_job(const JobRec& r) {
    const tbg_job& j = r.job;
    switch (j.kind) {
        case TBG_JOB_HALL:
            return tbg_hall_conductivity(j.model, r.kmesh.data(), r.dirs2.data(), j.nmu, r.mu.data(), j.T, j.eta,
                                         j.spin, j.precision, j.out0, nullptr);
        case TBG_JOB_BANDS:
            return tbg_solve_band(j.model, j.nk, j.k, j.out0);
        case TBG_JOB_BERRY:
            return tbg_berry_curvature(j.model, j.nk, j.k, r.dirs2.data(), j.spin, j.eta, j.precision, j.out0,
                                       j.out1);
        case TBG_JOB_OCCUPIED:
            return tbg_occupied_berry_curvature(j.model, j.nk, j.k, r.dirs2.data(), j.spin, j.eta, j.T, r.mu[0],
                                                j.precision, j.out0);
        default:
            return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch: unknown job kind");
    }
}

void worker_loop() {
    Queue& q = queue();
    for (;;) {
        std::shared_ptr<JobRec> r;
        {
            std::unique_lock<std::mutex> lk(q.mu);
            q.cv_work.wait(lk, [&] { return !q.pending.empty(); });
            r = q.pending.front();
            q.pending.pop_front();
        }
        int st = TBG_OK;
        std::string msg;
        if (cudaSetDevice(r->device) != cudaSuccess) {
            st = TBG_E_CUDA;
            msg = "tbg_batch: cudaSetDevice failed";
        } else {
            st = run_job(*r);
            if (st != TBG_OK) {
                char buf[1024];
                tbg_last_error(buf, sizeof(buf));
                msg = buf;
            }
        }
        {
            std::lock_guard<std::mutex> lk(q.mu);
            r->status = st;
            r->err = msg;
            r->done = true;
        }
        q.cv_done.notify_all();
    }
}

// Report a finished job to the caller: status, message in this thread.
int finish(const JobRec& r, int* status) {
    if (status) *status = r.status;
    if (r.status != TBG_OK) set_error(r.status, r.err);
    return TBG_OK;
}

}  // namespace
}  // namespace tbg

using namespace tbg;

extern "C" {

int tbg_batch_set_workers(int n) {
    if (n < 1 || n > 64) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_set_workers: n must be in [1, 64]");
    Queue& q = queue();
    std::lock_guard<std::mutex> lk(q.mu);
    q.want_workers = n;
    return TBG_OK;
}

int tbg_batch_submit(const tbg_job* job, int64_t* ticket) {
    if (!job || !ticket || !job->model) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_submit: null argument");
    int dim = 0, spin = 0;
    int64_t norb = 0, nsta = 0, nR = 0;
    if (int rc = tbg_model_info(job->model, &dim, &spin, &norb, &nsta, &nR)) return rc;
    auto r = std::make_shared<JobRec>();
    r->job = *job;
    switch (job->kind) {
        case TBG_JOB_HALL:
            if (!job->kmesh || !job->dirs2 || !job->mu || job->nmu < 1 || !job->out0)
                return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_submit: hall job needs kmesh, dirs2, mu, out0");
            r->kmesh.assign(job->kmesh, job->kmesh + dim);
            r->dirs2.assign(job->dirs2, job->dirs2 + 2 * dim);
            r->mu.assign(job->mu, job->mu + job->nmu);
            break;
        case TBG_JOB_BANDS:
            if (job->nk < 0 || (job->nk > 0 && (!job->k || !job->out0)))
                return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_submit: bands job needs k and out0");
            break;
        case TBG_JOB_BERRY:
        case TBG_JOB_OCCUPIED:
            if (job->nk < 0 || !job->dirs2 || (job->nk > 0 && (!job->k || !job->out0)) ||
                (job->kind == TBG_JOB_BERRY && job->nk > 0 && !job->out1) ||
                (job->kind == TBG_JOB_OCCUPIED && (!job->mu || job->nmu < 1)))
                return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_submit: berry job arguments");
            r->dirs2.assign(job->dirs2, job->dirs2 + 2 * dim);
            if (job->kind == TBG_JOB_OCCUPIED) r->mu.assign(job->mu, job->mu + 1);
            break;
        default:
            return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_submit: unknown job kind");
    }
    if (cudaGetDevice(&r->device) != cudaSuccess) r->device = 0;
    Queue& q = queue();
    {
        std::lock_guard<std::mutex> lk(q.mu);
        while (q.started < q.want_workers) {
            std::thread(worker_loop).detach();
            ++q.started;
        }
        *ticket = q.next_ticket++;
        q.jobs.emplace(*ticket, r);
        q.pending.push_back(r);
    }
    q.cv_work.notify_one();
    return TBG_OK;
}

int tbg_batch_poll(int64_t ticket, int* done, int* status) {
    if (!done) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_poll: null done");
    Queue& q = queue();
    std::shared_ptr<JobRec> r;
    {
        std::lock_guard<std::mutex> lk(q.mu);
        auto it = q.jobs.find(ticket);
        if (it == q.jobs.end()) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_poll: unknown ticket");
        if (!it->second->done) {
            *done = 0;
            return TBG_OK;
        }
        r = it->second;
        q.jobs.erase(it);
    }
    *done = 1;
    return finish(*r, status);
}

int tbg_batch_wait(int64_t ticket, int* status) {
    Queue& q = queue();
    std::shared_ptr<JobRec> r;
    {
        std::unique_lock<std::mutex> lk(q.mu);
        auto it = q.jobs.find(ticket);
        if (it == q.jobs.end()) return set_error(TBG_E_INVALID_ARGUMENT, "tbg_batch_wait: unknown ticket");
        r = it->second;
        q.cv_done.wait(lk, [&] { return r->done; });
        q.jobs.erase(ticket);
    }
    return finish(*r, status);
}

}  // extern "C"
