// server.cu -- nb_server_*: continuous batching of simulation jobs on one GPU.
//
// Three library threads:
//   admit     takes queued jobs first come first served, generates initial
//             conditions when none were given, waits for a slot and for the
//             job's bytes under the budget, allocates the job's buffers from
//             the stream-ordered pool and uploads its state on the upload
//             stream;
//   schedule  runs rounds: the running jobs plus the newly uploaded ones
//             form the batch table of the round, one step is a CUDA graph of
//             the batched kernels (k_batch.cu) replayed for the round's
//             steps, and up to two rounds are in flight so the GPU never
//             waits for the host.  Every job's step budget lives on the
//             device, so a job that ends inside a round stops taking part
//             at once.  Snapshots and final states are copied to fresh
//             device buffers in stream order right after the round;
//   deliver   brings those buffers to the host and hands them to the caller.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/nbgb.h"
#include "nbgb_internal.cuh"
#include "server_policy.hpp"
#include "sysmem.cuh"

using namespace nbgb;
using Clock = std::chrono::steady_clock;

namespace {

struct Job {
    int64_t id = 0;
    nb_config cfg{};
    int steps = 0;
    float dt = 0.0f;
    int n = 0;
    std::vector<float> pos, vel, mass;  // inputs until uploaded
    bool gen_ic = false;
    int64_t bytes = 0;
    char *dmem = nullptr;
    SysMem mem;
    SysDesc desc{};
    cudaEvent_t uploaded = nullptr;
    int done = 0;  // steps enqueued so far
    int state = NB_JOB_QUEUED;
    int status = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    bool have_result = false;
    std::vector<float> res_pos, res_vel;
};
using JobP = std::shared_ptr<Job>;

struct Delivery {
    JobP job;
    int final_state = 0;  // 0 snapshot, 1 final
    int step = 0;
    char *dbuf = nullptr;  // positions float[3n] (+ velocities float[3n]) + Ctrl
    size_t bytes = 0;
    cudaEvent_t ready = nullptr;
};

constexpr size_t kCtrlBytes = (sizeof(Ctrl) + 255) & ~(size_t)255;

}  // namespace

struct nb_server {
    nb_server_config cfg{};
    nb_job_fn fn = nullptr;
    void *user = nullptr;
    int dev = 0, sm = 0, variant = 3;
    cudaStream_t compute = nullptr, upload = nullptr, out = nullptr, cap = nullptr;
    StepFork fork{};  // the captured round step's second branch (direct sums)
    Admission adm{0, 0};
    Clock::time_point t0;

    std::mutex mu;
    std::condition_variable cv_queue, cv_ready, cv_done, cv_deliver;
    std::deque<JobP> queue;
    std::vector<JobP> ready;
    std::deque<Delivery> deliveries;
    std::unordered_map<int64_t, JobP> jobs;
    int64_t next_id = 1;
    bool stop = false, deliver_stop = false;
    std::thread t_admit, t_sched, t_deliver;

    // statistics (under mu)
    std::vector<double> latencies;
    int64_t submitted = 0, completed = 0, failed = 0, running = 0, rounds = 0;
    double body_updates = 0, first_submit = -1, last_done = 0;

    // round resources (scheduler thread only)
    SysDesc *d_sys[2] = {nullptr, nullptr}, *h_sys[2] = {nullptr, nullptr};
    int *d_pref[2] = {nullptr, nullptr}, *h_pref[2] = {nullptr, nullptr};
    int *d_work = nullptr;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int exec_totals[2][kBatchSpaces + 1] = {};
    cudaEvent_t round_ev[2] = {nullptr, nullptr};

    std::string err;
    bool fatal = false;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

static void set_fatal(nb_server *s, const std::string &m) {
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->fatal) s->err = m;
    s->fatal = true;
    s->cv_done.notify_all();
}

// Finishes a job that never ran or that was cancelled (under mu).
static void fail_job_locked(nb_server *s, const JobP &j, int status) {
    j->state = NB_JOB_FAILED;
    j->status = status;
    j->t_done = s->now();
    s->failed += 1;
    s->cv_done.notify_all();
}

// ---------------------------------------------------------------------------
// admit thread
// ---------------------------------------------------------------------------
static int64_t job_bytes(nb_server *s, Job &j) {
    SysMem &m = j.mem;
    m.n = j.n;
    m.tree = j.cfg.algo_config == NB_BARNES_HUT;
    m.quad = m.tree && s->cfg.multipole == NB_MULTIPOLE_QUADRUPOLE;
    m.cap = m.tree ? (j.cfg.cell_capacity > 0 ? j.cfg.cell_capacity : sysmem_default_capacity(j.n)) : 0;
    return (int64_t)(sysmem_layout(m, nullptr) + kCtrlBytes);
}

// Packs the job's state into pinned staging ({x,y,z,m} and {vx,vy,vz,0}
// float4 arrays, then its Ctrl) and uploads it on the upload stream.
static cudaError_t upload_job(nb_server *s, Job &j, char *&stage, size_t &stage_cap) {
    cudaError_t e = cudaMallocAsync((void **)&j.dmem, (size_t)j.bytes, s->upload);
    if (e != cudaSuccess) return e;
    sysmem_layout(j.mem, j.dmem);
    j.mem.ctrl = reinterpret_cast<Ctrl *>(j.dmem + (size_t)j.bytes - kCtrlBytes);
    const size_t n = (size_t)j.n;
    const size_t need = 32 * n + sizeof(Ctrl);
    if (need > stage_cap) {
        if (stage) cudaFreeHost(stage);
        stage_cap = need + need / 4;
        if ((e = cudaMallocHost((void **)&stage, stage_cap)) != cudaSuccess) {
            stage = nullptr;
            stage_cap = 0;
            return e;
        }
    }
    float4 *body = reinterpret_cast<float4 *>(stage), *vel = body + n;
    for (size_t i = 0; i < n; ++i) {
        body[i] = make_float4(j.pos[3 * i], j.pos[3 * i + 1], j.pos[3 * i + 2], j.mass[i]);
        vel[i] = j.vel.empty() ? make_float4(0.f, 0.f, 0.f, 0.f)
                               : make_float4(j.vel[3 * i], j.vel[3 * i + 1], j.vel[3 * i + 2], 0.0f);
    }
    Ctrl *init = reinterpret_cast<Ctrl *>(vel + n);
    memset(init, 0, sizeof(Ctrl));
    init->budget = j.steps;
    if ((e = cudaMemcpyAsync(j.mem.body[0], body, 16 * n, cudaMemcpyHostToDevice, s->upload)) != cudaSuccess ||
        (e = cudaMemcpyAsync(j.mem.vel, vel, 16 * n, cudaMemcpyHostToDevice, s->upload)) != cudaSuccess ||
        (e = cudaMemsetAsync(j.mem.acc, 0, 16 * n, s->upload)) != cudaSuccess ||
        (e = cudaMemcpyAsync(j.mem.ctrl, init, sizeof(Ctrl), cudaMemcpyHostToDevice, s->upload)) != cudaSuccess)
        return e;
    int *top_counts = nullptr;
    size_t top_bytes = 0;
    sysmem_top_counts(j.mem, &top_counts, &top_bytes);
    if (top_bytes && (e = cudaMemsetAsync(top_counts, 0, top_bytes, s->upload)) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&j.uploaded, cudaEventDisableTiming)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(j.uploaded, s->upload)) != cudaSuccess) return e;
    j.desc = sysmem_desc(j.mem, j.cfg, j.dt);
    // the staging is reused by the next job
    return cudaStreamSynchronize(s->upload);
}

static void admit_loop(nb_server *s) {
    cudaSetDevice(s->dev);
    char *stage = nullptr;  // pinned upload staging, grown to the largest job
    size_t stage_cap = 0;
    struct FreeStage {
        char *&p;
        ~FreeStage() {
            if (p) cudaFreeHost(p);
        }
    } free_stage{stage};
    while (true) {
        JobP j;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_queue.wait(lk, [&] { return s->stop || !s->queue.empty(); });
            if (s->stop) return;
            j = s->queue.front();
        }
        if (j->gen_ic) {
            j->pos.resize(3 * (size_t)j->n);
            j->vel.resize(3 * (size_t)j->n);
            j->mass.resize((size_t)j->n);
            nb_status st = nb_generate_ic(&j->cfg, j->pos.data(), j->vel.data(), j->mass.data());
            if (st != NB_OK) {
                std::lock_guard<std::mutex> g(s->mu);
                s->queue.pop_front();
                fail_job_locked(s, j, st);
                continue;
            }
        }
        j->bytes = job_bytes(s, *j);
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (!s->adm.can_ever_fit(j->bytes)) {
                s->queue.pop_front();
                fail_job_locked(s, j, NB_ERR_OUT_OF_MEMORY);
                continue;
            }
            s->cv_queue.wait(lk, [&] { return s->stop || s->adm.fits(j->bytes); });
            if (s->stop) return;
            s->adm.reserve(j->bytes);
            s->queue.pop_front();
        }
        cudaError_t e = upload_job(s, *j, stage, stage_cap);
        j->pos = std::vector<float>();
        j->vel = std::vector<float>();
        j->mass = std::vector<float>();
        std::lock_guard<std::mutex> g(s->mu);
        if (e != cudaSuccess) {
            if (j->dmem) cudaFreeAsync(j->dmem, s->upload);
            j->dmem = nullptr;
            s->adm.release(j->bytes);
            fail_job_locked(s, j, e == cudaErrorMemoryAllocation ? NB_ERR_OUT_OF_MEMORY : NB_ERR_CUDA);
            s->cv_queue.notify_all();
            continue;
        }
        j->state = NB_JOB_RUNNING;
        j->t_admit = s->now();
        s->running += 1;
        s->ready.push_back(j);
        s->cv_ready.notify_all();
    }
}

// ---------------------------------------------------------------------------
// schedule thread
// ---------------------------------------------------------------------------
// Copies the current body buffer (+ velocities when final) and the status
// word of job j to a new device buffer, in stream order after the round.
// Unpacks the current positions (+ velocities when final) of job j into a
// new device buffer in the reference's float[3N] layout, and copies its
// status word after them, in stream order after the round.
static size_t copy_out_ctrl_offset(int n, bool final_state) {
    const size_t b = (final_state ? 24 : 12) * (size_t)n;
    return (b + 15) & ~(size_t)15;
}

static cudaError_t enqueue_copy_out(nb_server *s, const JobP &j, bool final_state, std::deque<Delivery> &out) {
    Delivery d;
    d.job = j;
    d.final_state = final_state ? 1 : 0;
    d.step = j->done;
    const size_t n = (size_t)j->n;
    const size_t off = copy_out_ctrl_offset(j->n, final_state);
    d.bytes = off + sizeof(Ctrl);
    cudaError_t e = cudaMallocAsync((void **)&d.dbuf, d.bytes, s->compute);
    if (e != cudaSuccess) return e;
    const float4 *cur = j->mem.body[j->done & 1];  // every step flips the current buffer
    float *pos3 = reinterpret_cast<float *>(d.dbuf);
    float *vel3 = final_state ? pos3 + 3 * n : nullptr;
    if ((e = launch_unpack(cur, final_state ? j->mem.vel : nullptr, nullptr, pos3, vel3, nullptr, j->n,
                           s->compute)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(d.dbuf + off, j->mem.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToDevice, s->compute)) !=
        cudaSuccess)
        return e;
    out.push_back(d);
    return cudaSuccess;
}

static cudaError_t launch_round(nb_server *s, std::vector<JobP> &run, int steps, int buf,
                                std::deque<Delivery> &outs, std::vector<JobP> &finished) {
    const int ns = (int)run.size();
    for (int k = 0; k < ns; ++k) s->h_sys[buf][k] = run[k]->desc;
    int totals[kBatchSpaces];
    batch_prefixes(s->h_sys[buf], ns, batch_direct_block_bodies(s->variant), s->h_pref[buf], totals);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(s->d_sys[buf], s->h_sys[buf], sizeof(SysDesc) * ns, cudaMemcpyHostToDevice,
                             s->compute)) != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(s->d_pref[buf], s->h_pref[buf], sizeof(int) * batch_prefix_ints(ns),
                             cudaMemcpyHostToDevice, s->compute)) != cudaSuccess)
        return e;
    const int key[kBatchSpaces + 1] = {ns, totals[0], totals[1], totals[2], totals[3], totals[4]};
    if (!s->exec[buf] || memcmp(key, s->exec_totals[buf], sizeof(key)) != 0) {
        // the kernels read everything else from the device tables; only the
        // totals (grid sizes) and the system count live in the graph
        const BatchTables t = batch_tables(s->d_sys[buf], ns, s->d_pref[buf], totals, s->d_work);
        const int method = s->cfg.numerical_method;
        const int comp = s->cfg.precision == NB_PRECISION_COMPENSATED;
        const int quad = s->cfg.multipole == NB_MULTIPOLE_QUADRUPOLE;
        if ((e = cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
        int nl = 0;
        cudaError_t le = launch_batch_step(t, method, comp, quad, s->variant, TreeShape{}, s->sm, s->cap, &s->fork,
                                           &nl);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(s->cap, &g);
        if (le != cudaSuccess) e = le;
        if (e == cudaSuccess) {
            bool updated = false;
            if (s->exec[buf]) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(s->exec[buf], g, &info) == cudaSuccess;
                cudaGetLastError();
            }
            if (!updated) {
                if (s->exec[buf]) cudaGraphExecDestroy(s->exec[buf]);
                s->exec[buf] = nullptr;
                e = cudaGraphInstantiate(&s->exec[buf], g, 0);
            }
        }
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return e;
        memcpy(s->exec_totals[buf], key, sizeof(key));
    }
    for (int i = 0; i < steps; ++i)
        if ((e = cudaGraphLaunch(s->exec[buf], s->compute)) != cudaSuccess) return e;
    // what the round leaves: snapshots, final states, freed job buffers
    std::vector<JobP> keep;
    for (auto &j : run) {
        j->done = steps_after(j->done, j->steps, steps);
        if (j->done == j->steps) {
            if ((e = enqueue_copy_out(s, j, true, outs)) != cudaSuccess) return e;
            finished.push_back(j);
        } else {
            if (snapshot_due(j->done, j->steps, s->cfg.snapshot_every))
                if ((e = enqueue_copy_out(s, j, false, outs)) != cudaSuccess) return e;
            keep.push_back(j);
        }
    }
    for (auto &j : finished) {
        if ((e = cudaFreeAsync(j->dmem, s->compute)) != cudaSuccess) return e;
        j->dmem = nullptr;
    }
    run.swap(keep);
    return cudaSuccess;
}

static void schedule_loop(nb_server *s) {
    cudaSetDevice(s->dev);
    std::vector<JobP> run;
    std::deque<int> inflight;
    int r = 0;
    while (true) {
        if (inflight.size() == 2) {
            cudaEventSynchronize(s->round_ev[inflight.front()]);
            inflight.pop_front();
        }
        std::vector<JobP> fresh;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (run.empty() && s->ready.empty()) {
                if (!inflight.empty()) {
                    lk.unlock();
                    cudaEventSynchronize(s->round_ev[inflight.front()]);
                    inflight.pop_front();
                    continue;
                }
                s->cv_ready.wait(lk, [&] { return s->stop || !s->ready.empty(); });
            }
            if (s->stop) break;
            fresh.swap(s->ready);
        }
        cudaError_t e = cudaSuccess;
        for (auto &j : fresh) {
            if (e == cudaSuccess) e = cudaStreamWaitEvent(s->compute, j->uploaded, 0);
            // the wait is enqueued; the event is released once it has completed
            cudaEventDestroy(j->uploaded);
            j->uploaded = nullptr;
            run.push_back(j);
        }
        std::vector<int> remaining;
        for (auto &j : run) remaining.push_back(j->steps - j->done);
        const int steps = round_steps(remaining, s->cfg.snapshot_every);
        const int buf = r & 1;
        std::deque<Delivery> outs;
        std::vector<JobP> finished;
        if (e == cudaSuccess) e = launch_round(s, run, steps, buf, outs, finished);
        for (auto &d : outs) {
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d.ready, cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaEventRecord(d.ready, s->compute);
        }
        if (e == cudaSuccess) e = cudaEventRecord(s->round_ev[buf], s->compute);
        if (e != cudaSuccess) {
            set_fatal(s, std::string("round launch: ") + cudaGetErrorString(e));
            break;
        }
        inflight.push_back(buf);
        ++r;
        std::lock_guard<std::mutex> g(s->mu);
        s->rounds += 1;
        for (auto &j : finished) s->adm.release(j->bytes);
        if (!finished.empty()) s->cv_queue.notify_all();
        for (auto &d : outs) s->deliveries.push_back(d);
        if (!outs.empty()) s->cv_deliver.notify_all();
    }
    // stopping: let the rounds in flight finish, then cancel what is left
    for (int b : inflight) cudaEventSynchronize(s->round_ev[b]);
    cudaStreamSynchronize(s->compute);
    std::lock_guard<std::mutex> g(s->mu);
    for (auto &j : run) {
        if (j->dmem) cudaFreeAsync(j->dmem, s->compute);
        j->dmem = nullptr;
        s->running -= 1;
        fail_job_locked(s, j, NB_ERR_STATE);
    }
    for (auto &j : s->ready) {
        if (j->dmem) cudaFreeAsync(j->dmem, s->compute);
        j->dmem = nullptr;
        s->running -= 1;
        fail_job_locked(s, j, NB_ERR_STATE);
    }
    s->ready.clear();
    cudaStreamSynchronize(s->compute);
}

// ---------------------------------------------------------------------------
// deliver thread
// ---------------------------------------------------------------------------
static void deliver_loop(nb_server *s) {
    cudaSetDevice(s->dev);
    char *pinned = nullptr;  // host staging, grown to the largest delivery
    size_t pinned_cap = 0;
    while (true) {
        Delivery d;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_deliver.wait(lk, [&] { return s->deliver_stop || !s->deliveries.empty(); });
            if (s->deliveries.empty()) break;
            d = s->deliveries.front();
            s->deliveries.pop_front();
        }
        const int n = d.job->n;
        cudaError_t e = cudaSuccess;
        if (d.bytes > pinned_cap) {
            if (pinned) cudaFreeHost(pinned);
            pinned_cap = d.bytes + d.bytes / 4;
            e = cudaMallocHost((void **)&pinned, pinned_cap);
            if (e != cudaSuccess) {
                pinned = nullptr;
                pinned_cap = 0;
            }
        }
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s->out, d.ready, 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(pinned, d.dbuf, d.bytes, cudaMemcpyDeviceToHost, s->out);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->out);
        cudaFreeAsync(d.dbuf, s->out);
        cudaEventDestroy(d.ready);
        Ctrl c{};
        if (e == cudaSuccess) memcpy(&c, pinned + copy_out_ctrl_offset(n, d.final_state != 0), sizeof(Ctrl));
        const int status = e != cudaSuccess ? NB_ERR_CUDA : c.status;
        const float *pos = reinterpret_cast<const float *>(pinned);
        const float *vel = pos + 3 * (size_t)n;
        const JobP &j = d.job;
        if (!d.final_state) {
            if (s->fn && status == 0) s->fn(s->user, j->id, NB_JOB_EVENT_SNAPSHOT, d.step, pos, nullptr, n);
            continue;
        }
        {
            std::lock_guard<std::mutex> g(s->mu);
            j->t_done = s->now();
            j->status = status;
            j->state = status ? NB_JOB_FAILED : NB_JOB_DONE;
            s->running -= 1;
            if (status) {
                s->failed += 1;
            } else {
                s->completed += 1;
                s->body_updates += (double)n * (double)j->steps;
                s->latencies.push_back(j->t_done - j->t_submit);
                s->last_done = std::max(s->last_done, j->t_done);
                if (!s->fn) {
                    j->res_pos.assign(pos, pos + 3 * (size_t)n);
                    j->res_vel.assign(vel, vel + 3 * (size_t)n);
                    j->have_result = true;
                }
            }
        }
        if (s->fn) {
            if (status) s->fn(s->user, j->id, NB_JOB_EVENT_FAILED, status, nullptr, nullptr, n);
            else s->fn(s->user, j->id, NB_JOB_EVENT_DONE, j->steps, pos, vel, n);
        }
        std::lock_guard<std::mutex> g(s->mu);
        s->cv_done.notify_all();
    }
    if (pinned) cudaFreeHost(pinned);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void nb_server_config_default(nb_server_config *c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->device = 0;
    c->max_jobs = 1024;
    c->hbm_budget_bytes = 120LL * 1000 * 1000 * 1000;
    c->snapshot_every = 10;
    c->numerical_method = NB_EULER;
    c->precision = NB_PRECISION_FP32;
    c->multipole = NB_MULTIPOLE_MONOPOLE;
    c->direct_variant = -1;
}

nb_status nb_server_create(const nb_server_config *c, nb_job_fn fn, void *user, nb_server **out) {
    if (!c || !out || c->max_jobs < 1 || c->hbm_budget_bytes <= 0 || c->snapshot_every < 0)
        return NB_ERR_INVALID_ARGUMENT;
    if (c->direct_variant >= batch_direct_variants()) return NB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NB_ERR_NO_DEVICE;
    if (c->device < 0 || c->device >= ndev) return NB_ERR_INVALID_ARGUMENT;
    nb_server *s = new nb_server();
    s->cfg = *c;
    s->fn = fn;
    s->user = user;
    s->dev = c->device;
    s->variant = c->direct_variant >= 0 ? c->direct_variant : 3;
    s->adm = Admission(c->hbm_budget_bytes, c->max_jobs);
    s->t0 = Clock::now();
    auto bad = [&](nb_status st) {
        nb_server_destroy(s);
        return st;
    };
    if (cudaSetDevice(s->dev) != cudaSuccess) return bad(NB_ERR_CUDA);
    cudaDeviceGetAttribute(&s->sm, cudaDevAttrMultiProcessorCount, s->dev);
    // freed job buffers stay in the pool for the next jobs
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, s->dev) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    const size_t ns = (size_t)c->max_jobs;
    bool ok = cudaStreamCreateWithFlags(&s->compute, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->upload, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->out, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->fork.aux, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->fork.fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&s->fork.join, cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc(&s->d_work, sizeof(int)) == cudaSuccess;
    for (int b = 0; b < 2 && ok; ++b) {
        ok = cudaMalloc(&s->d_sys[b], sizeof(SysDesc) * ns) == cudaSuccess &&
             cudaMalloc(&s->d_pref[b], sizeof(int) * batch_prefix_device_ints((int)ns)) == cudaSuccess &&
             cudaMallocHost(&s->h_sys[b], sizeof(SysDesc) * ns) == cudaSuccess &&
             cudaMallocHost(&s->h_pref[b], sizeof(int) * batch_prefix_ints((int)ns)) == cudaSuccess &&
             cudaEventCreateWithFlags(&s->round_ev[b], cudaEventDisableTiming) == cudaSuccess;
    }
    if (!ok) return bad(NB_ERR_OUT_OF_MEMORY);
    s->t_admit = std::thread(admit_loop, s);
    s->t_sched = std::thread(schedule_loop, s);
    s->t_deliver = std::thread(deliver_loop, s);
    *out = s;
    return NB_OK;
}

nb_status nb_server_submit(nb_server *s, const nb_config *cfg, int32_t steps, float dt, const float *pos3,
                           const float *vel3, const float *mass, int64_t *job) {
    if (!s || !cfg || steps < 1 || !std::isfinite(dt)) return NB_ERR_INVALID_ARGUMENT;
    const nb_config &c = *cfg;
    if (c.num_of_bodies < 1 || c.algo_config < NB_BARNES_HUT || c.algo_config > NB_BRUTE_FORCE_LOCAL)
        return NB_ERR_INVALID_ARGUMENT;
    if (pos3 && !mass) return NB_ERR_INVALID_ARGUMENT;
    if (c.numerical_method != s->cfg.numerical_method || c.precision != s->cfg.precision ||
        c.multipole != s->cfg.multipole || c.device != s->cfg.device)
        return NB_ERR_UNSUPPORTED;
    if (c.algo_config != NB_BARNES_HUT && c.force_law != NB_FORCE_PLUMMER) return NB_ERR_UNSUPPORTED;
    const float eps =
        c.algo_config == NB_BARNES_HUT ? c.epsilon : (c.direct_epsilon >= 0.0f ? c.direct_epsilon : c.epsilon);
    if (!(eps > 0.0f)) return NB_ERR_UNSUPPORTED;
    if (c.algo_config == NB_BARNES_HUT) {
        const long long cap = c.cell_capacity > 0 ? c.cell_capacity : sysmem_default_capacity(c.num_of_bodies);
        if ((long long)c.num_of_bodies + cap + 1 >= (1LL << 26) - 1) return NB_ERR_UNSUPPORTED;
    }
    auto j = std::make_shared<Job>();
    j->cfg = c;
    j->steps = steps;
    j->dt = dt;
    j->n = c.num_of_bodies;
    const size_t n = (size_t)j->n;
    if (pos3) {
        j->pos.assign(pos3, pos3 + 3 * n);
        j->mass.assign(mass, mass + n);
        if (vel3) j->vel.assign(vel3, vel3 + 3 * n);
    } else {
        j->gen_ic = true;
    }
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop || s->fatal) return NB_ERR_STATE;
    j->id = s->next_id++;
    j->t_submit = s->now();
    if (s->first_submit < 0) s->first_submit = j->t_submit;
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    s->submitted += 1;
    s->cv_queue.notify_all();
    if (job) *job = j->id;
    return NB_OK;
}

nb_status nb_server_job_info(nb_server *s, int64_t job, nb_job_info *out) {
    if (!s || !out) return NB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->jobs.find(job);
    if (it == s->jobs.end()) return NB_ERR_INVALID_ARGUMENT;
    const Job &j = *it->second;
    out->state = j.state;
    out->status = j.status;
    out->steps = j.steps;
    out->n = j.n;
    out->t_submit = j.t_submit;
    out->t_admit = j.t_admit;
    out->t_done = j.t_done;
    out->bytes = j.bytes;
    return NB_OK;
}

nb_status nb_server_wait(nb_server *s, int64_t job, double timeout_s) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    JobP j;
    if (job >= 0) {
        auto it = s->jobs.find(job);
        if (it == s->jobs.end()) return NB_ERR_INVALID_ARGUMENT;
        j = it->second;
    }
    auto finished = [&] {
        if (s->fatal) return true;
        if (j) return j->state == NB_JOB_DONE || j->state == NB_JOB_FAILED;
        return s->completed + s->failed == s->submitted;
    };
    if (timeout_s < 0) {
        s->cv_done.wait(lk, finished);
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished)) {
        return NB_ERR_SPIN_TIMEOUT;
    }
    if (s->fatal) return NB_ERR_CUDA;
    if (j && j->state == NB_JOB_FAILED) return (nb_status)j->status;
    return NB_OK;
}

nb_status nb_server_result(nb_server *s, int64_t job, float *pos3, float *vel3) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->jobs.find(job);
    if (it == s->jobs.end()) return NB_ERR_INVALID_ARGUMENT;
    Job &j = *it->second;
    if (j.state == NB_JOB_FAILED) return (nb_status)j.status;
    if (j.state != NB_JOB_DONE || !j.have_result) return NB_ERR_STATE;
    if (pos3) memcpy(pos3, j.res_pos.data(), sizeof(float) * j.res_pos.size());
    if (vel3) memcpy(vel3, j.res_vel.data(), sizeof(float) * j.res_vel.size());
    j.res_pos = std::vector<float>();
    j.res_vel = std::vector<float>();
    j.have_result = false;
    return NB_OK;
}

nb_status nb_server_get_stats(nb_server *s, nb_server_stats *out) {
    if (!s || !out) return NB_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(s->mu);
    memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->queued = (int64_t)s->queue.size();
    out->running = s->running;
    out->rounds = s->rounds;
    out->bytes_in_use = s->adm.in_use();
    out->peak_bytes = s->adm.peak();
    out->peak_jobs = s->adm.peak_jobs();
    out->body_updates = s->body_updates;
    out->first_submit_s = s->first_submit;
    out->last_done_s = s->last_done;
    out->latency_p50_s = percentile(s->latencies, 50.0);
    out->latency_p99_s = percentile(s->latencies, 99.0);
    out->latency_max_s = percentile(s->latencies, 100.0);
    double sum = 0;
    for (double v : s->latencies) sum += v;
    out->latency_mean_s = s->latencies.empty() ? 0.0 : sum / (double)s->latencies.size();
    return NB_OK;
}

nb_status nb_server_destroy(nb_server *s) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        s->cv_queue.notify_all();
        s->cv_ready.notify_all();
    }
    if (s->t_admit.joinable()) s->t_admit.join();
    if (s->t_sched.joinable()) s->t_sched.join();
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->deliver_stop = true;
        s->cv_deliver.notify_all();
    }
    if (s->t_deliver.joinable()) s->t_deliver.join();
    cudaSetDevice(s->dev);
    {
        std::lock_guard<std::mutex> g(s->mu);
        for (auto &j : s->queue) fail_job_locked(s, j, NB_ERR_STATE);
        s->queue.clear();
        for (auto &kv : s->jobs) {
            if (kv.second->uploaded) cudaEventDestroy(kv.second->uploaded);
            kv.second->uploaded = nullptr;
        }
    }
    if (s->upload) cudaStreamSynchronize(s->upload);
    for (int b = 0; b < 2; ++b) {
        if (s->exec[b]) cudaGraphExecDestroy(s->exec[b]);
        cudaFree(s->d_sys[b]);
        cudaFree(s->d_pref[b]);
        if (s->h_sys[b]) cudaFreeHost(s->h_sys[b]);
        if (s->h_pref[b]) cudaFreeHost(s->h_pref[b]);
        if (s->round_ev[b]) cudaEventDestroy(s->round_ev[b]);
    }
    cudaFree(s->d_work);
    if (s->fork.fork) cudaEventDestroy(s->fork.fork);
    if (s->fork.join) cudaEventDestroy(s->fork.join);
    for (cudaStream_t st : {s->compute, s->upload, s->out, s->cap, s->fork.aux})
        if (st) cudaStreamDestroy(st);
    delete s;
    return NB_OK;
}

const char *nb_server_last_error_message(const nb_server *s) { return s ? s->err.c_str() : "null handle"; }

}  // extern "C"
