// HyperBall job server: continuous batching of independent HyperBall jobs
// under a device-memory budget (no reference counterpart; each job returns
// what HyperBallBuilder::build + run_until_done returns for its graph alone).
//
// Jobs wait in a FIFO queue. The scheduler admits the head job as soon as a
// slot is free (at most max_active jobs past admission) and its estimated
// device footprint fits the budget next to the admitted jobs. Admitted jobs
// go through three stages, each with its own host thread(s):
//   creation  (setup_threads, default 2) hb_create on the job's own stream:
//                            CSR upload, partition, renumbering, transpose;
//                            its steps and results then run on a stream of
//                            the highest priority;
//   stepping  (one thread)   every running job advances one iteration per
//                            step, and the union work of all of them runs as
//                            one kernel launch (hb_multi_step); a job created
//                            meanwhile joins at the next step, a finished one
//                            leaves after the step that stopped it;
//   results   (as many threads) neighbourhood function, sums and registers to
//                            the host, handle destroyed, budget released.
// So requests that arrive while others run are admitted as slots and memory
// free up, and their iterations interleave in the shared kernel. Latency is
// measured from submission to the moment the results are on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "hb_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    hb_handle* h = nullptr;           // from creation to the results stage
    cudaStream_t stream = nullptr;    // creation, at the default priority
    cudaStream_t run_stream = nullptr; // steps and results, at the highest priority
    Csr graph;                // the copied graph (hb_server_submit)
    hb_graph_view borrowed{}; // the caller's graph (hb_server_submit_borrowed), else empty
    bool is_borrowed = false;
    hb_options opts{};
    uint64_t footprint = 0;
    int state = HB_JOB_QUEUED;
    int error = HB_OK;
    std::string message;
    Clock::time_point submitted, started, finished;
    // results
    uint64_t iterations = 0, visited_arcs = 0;
    std::vector<double> nf, sod, harm;
    std::vector<uint8_t> registers;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct hb_server {
    hb_server_options opts{};
    std::mutex mu;
    std::condition_variable cv;        // every stage's wake-ups and job completions
    std::deque<std::shared_ptr<Job>> queue;      // submitted, waiting for admission
    std::deque<std::shared_ptr<Job>> to_create;  // admitted
    std::deque<std::shared_ptr<Job>> ready;      // created, joining the next step
    std::deque<std::shared_ptr<Job>> to_finish;  // stopped (or failed)
    std::map<uint64_t, std::shared_ptr<Job>> jobs;
    std::thread scheduler, stepper;
    std::vector<std::thread> creators, finishers;
    hb_multi* multi = nullptr;
    cudaStream_t step_stream = nullptr;
    uint64_t next_id = 1, used = 0;
    uint64_t steps = 0, job_steps = 0; // stepping statistics (hb_server_stats)
    double step_ms = 0.0;
    uint32_t active = 0;               // admitted and not finished
    bool stopping = false;             // no more admissions
    bool shutdown = false;             // stage threads exit
    std::string err;
};

static thread_local std::string t_server_err;

static int server_err(int code, const std::string& msg) {
    t_server_err = msg;
    return code;
}

// Device bytes a job needs at most: CSR and transpose (u64 offsets, u32
// successors), the CSR's original copy while it is renumbered, both counter
// arrays (one byte per register), the per-node arrays (estimates, two sums,
// in-degrees, renumbering, work lists) and the bitmaps, plus a fixed margin.
uint64_t hb_job_footprint(uint64_t num_nodes, uint64_t num_arcs, int log2m) {
    const uint64_t n = num_nodes, m = num_arcs;
    const uint64_t csr = 8 * (n + 1) + 4 * m;
    return 3 * csr + 2 * n * (1ull << log2m) + 64 * n + (64ull << 20);
}

// The end of a job (results on the host or a failure): bookkeeping under
// the lock, so a shutdown waiting for active == 0 cannot free the server
// under this thread.
static void job_done(hb_server* s, const std::shared_ptr<Job>& job, int r, const std::string& msg) {
    std::lock_guard<std::mutex> lock(s->mu);
    job->finished = Clock::now();
    job->error = r;
    job->message = msg;
    job->state = r ? HB_JOB_FAILED : HB_JOB_DONE;
    job->graph = Csr();  // the graph is no longer needed
    s->used -= job->footprint;
    s->active--;
    s->cv.notify_all();
}

// creation stage: the job's handle on its own stream
static void creator(hb_server* s) {
    for (;;) {
        std::shared_ptr<Job> job;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] { return s->shutdown || !s->to_create.empty(); });
            if (s->to_create.empty()) return;
            job = s->to_create.front();
            s->to_create.pop_front();
        }
        int r = HB_OK;
        std::string msg;
        if (!s->multi) {
            r = HB_ERR_NO_DEVICE;
            msg = "no CUDA device available (this library has no CPU path)";
        } else if (cudaSetDevice(s->opts.device) != cudaSuccess ||
                   cudaStreamCreateWithFlags(&job->stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            r = HB_ERR_CUDA;
            msg = "cudaStreamCreate failed";
        }
        if (!r) {
            hb_options o = job->opts;
            o.stream = job->stream;
            hb_graph_view v = job->is_borrowed ? job->borrowed
                                               : hb_graph_view{job->graph.n, job->graph.m,
                                                               job->graph.offsets.data(),
                                                               job->graph.successors.data()};
            r = hb_create(&v, nullptr, &o, &job->h);
            if (r) msg = hb_global_last_error();
        }
        if (!r) {
            r = hb_multi_start(job->h);
            if (r) msg = hb_last_error(job->h);
        }
        if (!r) {
            // the job's pre- and post-union kernels then go ahead of other
            // jobs' creation work waiting for the SMs
            int least = 0, greatest = 0;
            if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess ||
                cudaStreamCreateWithPriority(&job->run_stream, cudaStreamNonBlocking, greatest) !=
                    cudaSuccess) {
                cudaGetLastError();
                r = HB_ERR_CUDA;
                msg = "cudaStreamCreate failed";
            } else if ((r = hb_multi_set_stream(job->h, job->run_stream))) {
                msg = hb_last_error(job->h);
            }
        }
        if (r) {
            if (job->h) hb_destroy(job->h);
            job->h = nullptr;
            if (job->stream) cudaStreamDestroy(job->stream);
            job->stream = nullptr;
            if (job->run_stream) cudaStreamDestroy(job->run_stream);
            job->run_stream = nullptr;
            job_done(s, job, r, msg);
            continue;
        }
        std::lock_guard<std::mutex> lock(s->mu);
        s->ready.push_back(job);
        s->cv.notify_all();
    }
}

// stepping stage: one iteration of every running job per step, one shared
// union launch
static void stepper(hb_server* s) {
    cudaSetDevice(s->opts.device);
    std::vector<std::shared_ptr<Job>> running;
    std::vector<hb_handle*> hs;
    for (;;) {
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] {
                return !s->ready.empty() || !running.empty() || (s->shutdown && s->to_create.empty());
            });
            if (running.empty() && s->ready.empty() && s->shutdown) return;
            // newly created jobs join at this step
            while (!s->ready.empty() && running.size() < (size_t)hbk::MAX_JOBS) {
                std::shared_ptr<Job> j = s->ready.front();
                s->ready.pop_front();
                if (hb_multi_done(j->h))
                    s->to_finish.push_back(j);  // no nodes: nothing to iterate
                else
                    running.push_back(j);
            }
            s->cv.notify_all();
        }
        if (running.empty()) continue;
        hs.clear();
        for (auto& j : running) hs.push_back(j->h);
        std::string msg;
        const Clock::time_point t0 = Clock::now();
        const int r = hb_multi_step(s->multi, hs.data(), (uint32_t)hs.size(), msg);
        std::lock_guard<std::mutex> lock(s->mu);
        s->steps++;
        s->job_steps += hs.size();
        s->step_ms += ms_between(t0, Clock::now());
        std::vector<std::shared_ptr<Job>> still;
        for (auto& j : running) {
            if (r) {
                j->error = r;
                j->message = msg;
                s->to_finish.push_back(j);
            } else if (hb_multi_done(j->h)) {
                s->to_finish.push_back(j);
            } else {
                still.push_back(j);
            }
        }
        running.swap(still);
        s->cv.notify_all();
    }
}

// results stage
static void finisher(hb_server* s) {
    cudaSetDevice(s->opts.device);
    for (;;) {
        std::shared_ptr<Job> job;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv.wait(lock, [&] { return s->shutdown || !s->to_finish.empty(); });
            if (s->to_finish.empty()) return;
            job = s->to_finish.front();
            s->to_finish.pop_front();
        }
        int r = job->error;
        std::string msg = job->message;
        hb_handle* h = job->h;
        if (!r) {
            job->iterations = hb_num_iterations(h);
            for (uint64_t i = 0; i < job->iterations; i++) {
                hb_iter_stats st{};
                hb_get_iteration_stats(h, i, &st);
                job->visited_arcs += st.visited_arcs;
            }
            const uint64_t n = job->graph.n;
            if (job->iterations) {
                size_t len = 0;
                hb_get_neighborhood_function(h, nullptr, 0, &len);
                job->nf.resize(len);
                r = hb_get_neighborhood_function(h, job->nf.data(), len, &len);
                if (!r && (job->opts.flags & HB_SUM_OF_DISTANCES)) {
                    job->sod.resize(n);
                    r = hb_get_sum_of_distances(h, job->sod.data(), n);
                }
                if (!r && (job->opts.flags & HB_SUM_OF_INVERSE_DISTANCES)) {
                    job->harm.resize(n);
                    r = hb_get_harmonic_centralities(h, job->harm.data(), n);
                }
            }
            if (!r && s->opts.keep_registers) {
                uint64_t cb = 0;
                int rs = 0;
                hb_counter_layout(h, &cb, &rs);
                job->registers.resize(n * cb);
                r = hb_get_registers(h, HB_CURRENT_STATE, job->registers.data(), job->registers.size());
            }
            if (r) msg = hb_last_error(h);
        }
        if (h) hb_destroy(h);
        job->h = nullptr;
        if (job->stream) cudaStreamDestroy(job->stream);
        job->stream = nullptr;
        if (job->run_stream) cudaStreamDestroy(job->run_stream);
        job->run_stream = nullptr;
        job_done(s, job, r, msg);
    }
}

static void schedule(hb_server* s) {
    std::unique_lock<std::mutex> lock(s->mu);
    for (;;) {
        s->cv.wait(lock, [&] {
            if (s->stopping) return true;
            if (s->queue.empty() || s->active >= s->opts.max_active) return false;
            return s->used + s->queue.front()->footprint <= s->opts.hbm_budget_bytes;
        });
        if (s->stopping) return;
        // admit in arrival order while the head fits
        while (!s->queue.empty() && s->active < s->opts.max_active &&
               s->used + s->queue.front()->footprint <= s->opts.hbm_budget_bytes) {
            std::shared_ptr<Job> job = s->queue.front();
            s->queue.pop_front();
            s->used += job->footprint;
            s->active++;
            job->state = HB_JOB_RUNNING;
            job->started = Clock::now();
            s->to_create.push_back(job);
        }
        s->cv.notify_all();
    }
}

void hb_server_options_default(hb_server_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->struct_size = sizeof(hb_server_options);
    o->device = 0;
    o->hbm_budget_bytes = 150ull * 1000 * 1000 * 1000;
    o->max_active = 16;
    o->keep_registers = 0;
    // measured on the 600-job served workload, two runs each: 0, 16 and 38
    // SMs left free gave 1.66/1.49, 1.67/1.84 and 1.41/1.68 e12 updates/s
    o->union_sm_reserve = 16;
}

int hb_server_create(const hb_server_options* opts, hb_server** out) {
    if (!out) return server_err(HB_ERR_INVALID, "out is NULL");
    *out = nullptr;
    hb_server_options o;
    hb_server_options_default(&o);
    if (opts) {
        if (opts->struct_size != sizeof(hb_server_options))
            return server_err(HB_ERR_INVALID, "hb_server_options.struct_size mismatch");
        o = *opts;
    }
    if (o.max_active == 0 || o.max_active > (uint32_t)hbk::MAX_JOBS)
        return server_err(HB_ERR_INVALID, "max_active must be in [1, 48]");
    hb_server* s = new hb_server();
    s->opts = o;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0 && cudaSetDevice(o.device) == cudaSuccess) {
        std::string err;
        // the steps run at the device's highest stream priority, the jobs'
        // creation at the default one
        int least = 0, greatest = 0;
        cudaError_t ce = cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (ce == cudaSuccess)
            ce = cudaStreamCreateWithPriority(&s->step_stream, cudaStreamNonBlocking, greatest);
        int r = ce == cudaSuccess ? hb_multi_create(o.device, s->step_stream, &s->multi, err) : HB_ERR_CUDA;
        if (r) {
            cudaGetLastError();
            if (s->step_stream) cudaStreamDestroy(s->step_stream);
            delete s;
            return server_err(r, "server setup: " + (err.empty() ? std::string("cudaStreamCreate failed") : err));
        }
        if (o.union_sm_reserve) hb_multi_reserve_sms(s->multi, o.union_sm_reserve);
    } else {
        // no device: every job fails at creation with HB_ERR_NO_DEVICE
        cudaGetLastError();
    }
    s->scheduler = std::thread(schedule, s);
    s->stepper = std::thread(stepper, s);
    // creation and results of different jobs overlap (host copies, device
    // set-up kernels on the jobs' own streams) beside the stepping thread.
    // Measured on the 400-job served workload (arrivals at 200/s): 1, 2, 4
    // and 8 workers each gave 0.88, 1.11, 0.98 and 0.87 e12 updates/s; more
    // set-up work in parallel slows the shared steps more than it admits
    // jobs sooner.
    const uint32_t workers = o.setup_threads ? o.setup_threads : std::min<uint32_t>(o.max_active, 2);
    for (uint32_t i = 0; i < workers; i++) {
        s->creators.emplace_back(creator, s);
        s->finishers.emplace_back(finisher, s);
    }
    *out = s;
    return HB_OK;
}

static int submit_impl(hb_server* s, const hb_graph_view* graph, const hb_options* opts, bool borrow,
                       uint64_t* job) {
    if (!s || !graph || !opts || !job) return server_err(HB_ERR_INVALID, "NULL argument");
    if (opts->struct_size != sizeof(hb_options))
        return server_err(HB_ERR_INVALID, "hb_options.struct_size mismatch");
    if (!graph->offsets || (graph->num_arcs && !graph->successors))
        return server_err(HB_ERR_INVALID, "graph arrays must not be NULL");
    if (opts->weights) return server_err(HB_ERR_INVALID, "weights are not supported by the server");
    if (opts->log2m < 4 || opts->log2m > 10) return server_err(HB_ERR_INVALID, "log2m must be in [4, 10]");
    auto j = std::make_shared<Job>();
    j->footprint = hb_job_footprint(graph->num_nodes, graph->num_arcs, opts->log2m);
    if (j->footprint > s->opts.hbm_budget_bytes)
        return server_err(HB_ERR_INVALID, "the job alone needs " + std::to_string(j->footprint) +
                                              " device bytes, more than the budget");
    j->graph.n = graph->num_nodes;
    j->graph.m = graph->num_arcs;
    if (borrow) {
        j->borrowed = *graph;
        j->is_borrowed = true;
    } else {
        j->graph.offsets.assign(graph->offsets, graph->offsets + graph->num_nodes + 1);
        j->graph.successors.assign(graph->successors, graph->successors + graph->num_arcs);
    }
    j->opts = *opts;
    j->opts.device = s->opts.device;
    j->opts.stream = nullptr;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->stopping) return server_err(HB_ERR_INVALID, "server is shutting down");
        j->id = s->next_id++;
        j->submitted = Clock::now();
        s->jobs[j->id] = j;
        s->queue.push_back(j);
        *job = j->id;
    }
    s->cv.notify_all();
    return HB_OK;
}

int hb_server_submit(hb_server* s, const hb_graph_view* graph, const hb_options* opts, uint64_t* job) {
    return submit_impl(s, graph, opts, false, job);
}

int hb_server_submit_borrowed(hb_server* s, const hb_graph_view* graph, const hb_options* opts,
                              uint64_t* job) {
    return submit_impl(s, graph, opts, true, job);
}

static std::shared_ptr<Job> find_job(hb_server* s, uint64_t id) {
    auto it = s->jobs.find(id);
    return it == s->jobs.end() ? nullptr : it->second;
}

int hb_server_wait(hb_server* s, uint64_t job, double timeout_s) {
    if (!s) return server_err(HB_ERR_INVALID, "server is NULL");
    std::unique_lock<std::mutex> lock(s->mu);
    std::shared_ptr<Job> j = find_job(s, job);
    if (!j) return server_err(HB_ERR_INVALID, "unknown job");
    auto done = [&] { return j->state == HB_JOB_DONE || j->state == HB_JOB_FAILED; };
    if (timeout_s < 0) {
        s->cv.wait(lock, done);
    } else if (!s->cv.wait_for(lock, std::chrono::duration<double>(timeout_s), done)) {
        return server_err(HB_ERR_TIMEOUT, "job not finished within the timeout");
    }
    if (j->state == HB_JOB_FAILED) return server_err(j->error, j->message);
    return HB_OK;
}

int hb_server_job_info(hb_server* s, uint64_t job, hb_job_info* info) {
    if (!s || !info) return server_err(HB_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lock(s->mu);
    std::shared_ptr<Job> j = find_job(s, job);
    if (!j) return server_err(HB_ERR_INVALID, "unknown job");
    std::memset(info, 0, sizeof(*info));
    info->state = j->state;
    info->error = j->error;
    info->iterations = j->iterations;
    info->visited_arcs = j->visited_arcs;
    info->register_updates = j->visited_arcs << j->opts.log2m;
    info->footprint_bytes = j->footprint;
    const Clock::time_point now = Clock::now();
    const bool started = j->state != HB_JOB_QUEUED;
    const bool ended = j->state == HB_JOB_DONE || j->state == HB_JOB_FAILED;
    info->queue_ms = ms_between(j->submitted, started ? j->started : now);
    info->run_ms = started ? ms_between(j->started, ended ? j->finished : now) : 0.0;
    info->latency_ms = ms_between(j->submitted, ended ? j->finished : now);
    return HB_OK;
}

static int finished_job(hb_server* s, uint64_t job, std::shared_ptr<Job>& j) {
    if (!s) return server_err(HB_ERR_INVALID, "server is NULL");
    j = find_job(s, job);
    if (!j) return server_err(HB_ERR_INVALID, "unknown job");
    if (j->state != HB_JOB_DONE) return server_err(HB_ERR_NOT_RUN, "job has not finished");
    return HB_OK;
}

int hb_server_get_neighborhood_function(hb_server* s, uint64_t job, double* dst, size_t capacity,
                                        size_t* len) {
    std::lock_guard<std::mutex> lock(s->mu);
    std::shared_ptr<Job> j;
    int r = finished_job(s, job, j);
    if (r) return r;
    if (j->iterations == 0)
        return server_err(HB_ERR_NOT_RUN, "HyperBall was not run (the graph has no nodes)");
    if (len) *len = j->nf.size();
    if (dst) std::copy(j->nf.begin(), j->nf.begin() + std::min(capacity, j->nf.size()), dst);
    return HB_OK;
}

static int server_vec(hb_server* s, uint64_t job, double* dst, size_t len, bool harm) {
    std::lock_guard<std::mutex> lock(s->mu);
    std::shared_ptr<Job> j;
    int r = finished_job(s, job, j);
    if (r) return r;
    if (j->iterations == 0)
        return server_err(HB_ERR_NOT_RUN, "HyperBall was not run (the graph has no nodes)");
    const std::vector<double>& v = harm ? j->harm : j->sod;
    const uint32_t flag = harm ? HB_SUM_OF_INVERSE_DISTANCES : HB_SUM_OF_DISTANCES;
    if (!(j->opts.flags & flag)) return server_err(HB_ERR_NOT_REQUESTED, "output was not requested");
    if (!dst || len != v.size()) return server_err(HB_ERR_INVALID, "len must equal the graph's num_nodes");
    std::copy(v.begin(), v.end(), dst);
    return HB_OK;
}

int hb_server_get_sum_of_distances(hb_server* s, uint64_t job, double* dst, size_t len) {
    return server_vec(s, job, dst, len, false);
}

int hb_server_get_harmonic_centralities(hb_server* s, uint64_t job, double* dst, size_t len) {
    return server_vec(s, job, dst, len, true);
}

int hb_server_get_registers(hb_server* s, uint64_t job, void* dst, size_t bytes) {
    std::lock_guard<std::mutex> lock(s->mu);
    std::shared_ptr<Job> j;
    int r = finished_job(s, job, j);
    if (r) return r;
    if (!s->opts.keep_registers)
        return server_err(HB_ERR_NOT_REQUESTED, "the server does not keep registers (keep_registers = 0)");
    if (!dst || bytes != j->registers.size()) return server_err(HB_ERR_INVALID, "bytes must equal num_nodes * counter bytes");
    std::memcpy(dst, j->registers.data(), bytes);
    return HB_OK;
}

int hb_server_release(hb_server* s, uint64_t job) {
    if (!s) return server_err(HB_ERR_INVALID, "server is NULL");
    std::lock_guard<std::mutex> lock(s->mu);
    std::shared_ptr<Job> j = find_job(s, job);
    if (!j) return server_err(HB_ERR_INVALID, "unknown job");
    if (j->state != HB_JOB_DONE && j->state != HB_JOB_FAILED)
        return server_err(HB_ERR_INVALID, "job has not finished");
    s->jobs.erase(job);
    return HB_OK;
}

void hb_server_destroy(hb_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
        // queued jobs are cancelled
        for (auto& j : s->queue) {
            j->state = HB_JOB_FAILED;
            j->error = HB_ERR_INVALID;
            j->message = "cancelled: the server shut down";
        }
        s->queue.clear();
    }
    s->cv.notify_all();
    if (s->scheduler.joinable()) s->scheduler.join();
    {
        // admitted jobs finish
        std::unique_lock<std::mutex> lock(s->mu);
        s->cv.wait(lock, [&] { return s->active == 0; });
        s->shutdown = true;
    }
    s->cv.notify_all();
    for (auto& t : s->creators) t.join();
    if (s->stepper.joinable()) s->stepper.join();
    for (auto& t : s->finishers) t.join();
    if (s->multi) hb_multi_destroy(s->multi);
    if (s->step_stream) cudaStreamDestroy(s->step_stream);
    delete s;
}

const char* hb_server_last_error(void) { return t_server_err.c_str(); }

int hb_server_stats(hb_server* s, uint64_t* steps, double* step_ms, double* union_ms,
                    uint64_t* job_steps, double* launch_ms) {
    if (!s) return server_err(HB_ERR_INVALID, "server is NULL");
    std::lock_guard<std::mutex> lock(s->mu);
    if (steps) *steps = s->steps;
    if (step_ms) *step_ms = s->step_ms;
    if (job_steps) *job_steps = s->job_steps;
    double ums = 0.0, hms = 0.0;
    if (s->multi) hb_multi_steps(s->multi, nullptr, &ums, &hms, nullptr, nullptr, nullptr);
    if (union_ms) *union_ms = ums;
    if (launch_ms) *launch_ms = hms;
    return HB_OK;
}

int hb_server_step_times(hb_server* s, double* pre_ms, double* union_ms, double* post_ms,
                         double* host_ms, double* wait_ms) {
    if (!s) return server_err(HB_ERR_INVALID, "server is NULL");
    std::lock_guard<std::mutex> lock(s->mu);
    double pre = 0.0, uni = 0.0, post = 0.0, host = 0.0, wait = 0.0;
    if (s->multi) hb_multi_steps(s->multi, nullptr, &uni, &host, &wait, &pre, &post);
    if (pre_ms) *pre_ms = pre;
    if (union_ms) *union_ms = uni;
    if (post_ms) *post_ms = post;
    if (host_ms) *host_ms = host;
    if (wait_ms) *wait_ms = wait;
    return HB_OK;
}
