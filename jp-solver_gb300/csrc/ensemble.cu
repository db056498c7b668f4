// Ensembles and the solve server: many independent Taylor-Green solves on one GPU.
//
// No counterpart in the reference, which runs one solve per process.  An ensemble batches the steps
// of many solves: uniform cubes in one stream-collide launch per storage format per lattice step
// (k_stream_collide takes up to kMaxBatch cubes of any sizes), AMR solves in one launch per stage of
// the coarse step over the blocks of all of them (amr_batch_step).  The server adds continuous
// batching on top: requests wait until their HBM estimate fits the pool and a slot is free, join
// between ticks while other solves run, advance together, and leave with a result.  Each solve does
// exactly what the `uniform` / `amr` programs do for it (same steps, diagnostic cadence, regrid
// cadence, VALID gate), so its numbers do not depend on what else is running.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "amr_kernels.h"
#include "jp.h"
#include "kernels.h"
#include "solver.h"

namespace jp {

#define ECK(call, what)                                     \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
    } while (0)

// One batched lattice step of `members` (uniform, same device) on `st`: one launch per
// (storage, vec, threads) class and per kMaxBatch cubes.  Swaps each member's buffers.
static jp_status batched_step(const std::vector<jp_solver*>& members, cudaStream_t st) {
    // in-place cubes group by the parity of their step count too (local or stream step)
    std::map<long long, std::vector<jp_solver*>> groups;
    for (jp_solver* m : members)
        groups[((long long)m->inplace << 42) | ((long long)(m->inplace ? m->step_count & 1 : 0) << 40) |
               ((long long)m->storage << 32) | ((long long)m->vec << 16) | (long long)m->tpb].push_back(m);
    for (auto& g : groups) {
        const std::vector<jp_solver*>& v = g.second;
        for (size_t i = 0; i < v.size(); i += kMaxBatch) {
            const size_t cnt = std::min(v.size() - i, (size_t)kMaxBatch);
            UniSolve us[kMaxBatch];
            for (size_t k = 0; k < cnt; ++k) {
                jp_solver* m = v[i + k];
                std::memset(&us[k], 0, sizeof us[k]);
                us[k].src = m->fa;
                us[k].dst = m->inplace ? m->fa : m->fb;
                us[k].n = m->n;
                us[k].omega = float(m->info.omega);
                us[k].omega_d = m->info.omega;
            }
            if (v[i]->inplace) {
                ECK(launch_stream_collide_inplace(v[i]->storage, us, (int)cnt, int(v[i]->step_count & 1), v[i]->vec,
                                                  v[i]->tpb, st), "batched in-place step");
            } else {
                ECK(launch_stream_collide(v[i]->storage, us, (int)cnt, v[i]->vec, v[i]->tpb, st), "batched stream_collide");
            }
            for (size_t k = 0; k < cnt; ++k) {
                if (!v[i + k]->inplace) std::swap(v[i + k]->fa, v[i + k]->fb);
                ++v[i + k]->step_count;
            }
        }
    }
    return JP_OK;
}

}  // namespace jp

using namespace jp;

// ------------------------------------------------------------------------------------------------
// ensemble

struct jp_ensemble {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    AmrFork fk;  // the level-0 branch of the AMR members' coarse steps
    std::vector<jp_solver*> members;
    // persistent AMR coarse steps (jp_ensemble_set_persistent): barrier state of each launch of a
    // jp_ensemble_step (one per kAmrBatchMax members), its error fields kept until jp_ensemble_sync
    int persist = 0, persist_grid = 0;
    long long limit_ns = kPersistLimitNs;
    amr::PersistSync* sync = nullptr;
    amr::PersistSync* sync_host = nullptr;  // pinned copy read by jp_ensemble_sync
    static constexpr int kSyncSlots = 64;
    static constexpr long long kPersistLimitNs = 2000000000LL;
};

extern "C" {

jp_status jp_ensemble_create(int32_t device, jp_ensemble** out) {
    if (!out) return fail(JP_ERR_INVALID, "null argument");
    *out = nullptr;
    ECK(cudaSetDevice(device), "cudaSetDevice");
    jp_ensemble* e = new (std::nothrow) jp_ensemble();
    if (!e) return fail(JP_ERR_NOMEM, "host allocation");
    e->device = device;
    cudaError_t err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming);
    if (err == cudaSuccess) err = e->fk.create(e->stream);
    if (err != cudaSuccess) {
        jp_ensemble_destroy(e);
        return cuda_fail(err, "ensemble stream");
    }
    *out = e;
    return JP_OK;
}

void jp_ensemble_destroy(jp_ensemble* e) {
    if (!e) return;
    if (e->stream) {
        cudaStreamSynchronize(e->stream);
        cudaStreamDestroy(e->stream);
    }
    e->fk.destroy();
    if (e->done) cudaEventDestroy(e->done);
    if (e->sync) cudaFree(e->sync);
    if (e->sync_host) cudaFreeHost(e->sync_host);
    delete e;
}

jp_status jp_ensemble_set_persistent(jp_ensemble* e, int32_t mode, int64_t wait_limit_ns, int32_t grid) {
    if (!e) return fail(JP_ERR_INVALID, "null ensemble");
    if (mode != 0 && mode != 1) return fail(JP_ERR_INVALID, "persistent mode %d (0 or 1)", mode);
    if (wait_limit_ns < 0 || grid < 0) return fail(JP_ERR_INVALID, "negative wait limit or grid");
    ECK(cudaSetDevice(e->device), "cudaSetDevice");
    if (mode && !e->sync) {
        const size_t bytes = sizeof(amr::PersistSync) * jp_ensemble::kSyncSlots;
        ECK(cudaMalloc(&e->sync, bytes), "cudaMalloc barrier state");
        ECK(cudaMallocHost(&e->sync_host, bytes), "cudaMallocHost barrier state");
        ECK(cudaMemsetAsync(e->sync, 0, bytes, e->stream), "barrier state");
    }
    e->persist = mode;
    e->limit_ns = wait_limit_ns ? wait_limit_ns : jp_ensemble::kPersistLimitNs;
    e->persist_grid = grid;
    return JP_OK;
}

jp_status jp_ensemble_sync(jp_ensemble* e) {
    if (!e) return fail(JP_ERR_INVALID, "null ensemble");
    ECK(cudaSetDevice(e->device), "cudaSetDevice");
    if (!e->sync) {
        ECK(cudaStreamSynchronize(e->stream), "ensemble sync");
        return JP_OK;
    }
    const size_t bytes = sizeof(amr::PersistSync) * jp_ensemble::kSyncSlots;
    ECK(cudaMemcpyAsync(e->sync_host, e->sync, bytes, cudaMemcpyDeviceToHost, e->stream), "barrier state D2H");
    ECK(cudaMemsetAsync(e->sync, 0, bytes, e->stream), "barrier state");
    ECK(cudaStreamSynchronize(e->stream), "ensemble sync");
    for (int c = 0; c < jp_ensemble::kSyncSlots; ++c)
        if (e->sync_host[c].err)
            return fail(JP_ERR_TIMEOUT, "persistent coarse steps: a grid barrier wait ran past %lld ns (launch %d, "
                        "phase %d of coarse step %d)", e->limit_ns, c, e->sync_host[c].phase + 1, e->sync_host[c].step);
    return JP_OK;
}

jp_status jp_ensemble_add(jp_ensemble* e, jp_solver* s) {
    if (!e || !s) return fail(JP_ERR_INVALID, "null argument");
    if (s->device != e->device) return fail(JP_ERR_INVALID, "solver on device %d, ensemble on %d", s->device, e->device);
    if (std::find(e->members.begin(), e->members.end(), s) != e->members.end()) return JP_OK;
    e->members.push_back(s);
    return JP_OK;
}

jp_status jp_ensemble_remove(jp_ensemble* e, jp_solver* s) {
    if (!e || !s) return fail(JP_ERR_INVALID, "null argument");
    auto it = std::find(e->members.begin(), e->members.end(), s);
    if (it == e->members.end()) return fail(JP_ERR_INVALID, "solver is not a member");
    e->members.erase(it);
    return JP_OK;
}

jp_status jp_ensemble_step(jp_ensemble* e, int64_t nsteps) {
    if (!e) return fail(JP_ERR_INVALID, "null ensemble");
    if (nsteps < 0) return fail(JP_ERR_INVALID, "negative step count");
    ECK(cudaSetDevice(e->device), "cudaSetDevice");
    for (jp_solver* m : e->members) {  // after each member's pending work
        if (m->kind == JP_UNIFORM && nsteps > 0) {  // populations staged for the next step
            const jp_status taken = uniform_take_staged(m);
            if (taken != JP_OK) return taken;
        }
        ECK(cudaEventRecord(m->ev1, m->stream), "event");
        ECK(cudaStreamWaitEvent(e->stream, m->ev1, 0), "wait");
    }
    // uniform members in batched stream-collide launches; AMR members in batched coarse steps, one
    // group per compatible launch shape (block edge, storage, step threads, skip flags)
    std::vector<jp_solver*> uni;
    std::vector<std::vector<jp_solver*>> amr;
    for (jp_solver* m : e->members) {
        if (m->kind == JP_UNIFORM) {
            uni.push_back(m);
            continue;
        }
        bool placed = false;
        for (auto& g : amr)
            if (amr_batch_compatible(g[0], m)) {
                g.push_back(m);
                placed = true;
                break;
            }
        if (!placed) amr.push_back({m});
    }
    // persistent launches: all nsteps coarse steps of a group at once
    std::vector<bool> in_persist(amr.size(), false);
    if (e->persist && nsteps > 0)
        for (size_t k = 0; k < amr.size(); ++k) {
            bool ok = true;
            for (jp_solver* m : amr[k]) ok = ok && amr_persist_ok(m);
            if (!ok) continue;
            jp_status st = amr_persist_steps(amr[k], std::vector<long long>(amr[k].size(), nsteps), e->stream, e->sync,
                                             jp_ensemble::kSyncSlots, e->limit_ns, e->persist_grid);
            if (st != JP_OK) return st;
            in_persist[k] = true;
        }
    for (int64_t i = 0; i < nsteps; ++i) {
        jp_status st = batched_step(uni, e->stream);
        if (st != JP_OK) return st;
        for (size_t k = 0; k < amr.size(); ++k) {
            if (in_persist[k]) continue;
            st = amr_batch_step(amr[k], e->stream, &e->fk);
            if (st != JP_OK) return st;
        }
    }
    ECK(cudaEventRecord(e->done, e->stream), "event");
    for (jp_solver* m : e->members) ECK(cudaStreamWaitEvent(m->stream, e->done, 0), "wait");  // before later work
    return JP_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// server

namespace {

struct Job {
    jp_request req{};
    jp_solver* s = nullptr;
    jp_info info{};
    long long step = 0, steps = 0, diagK = 1, adapt = 0;
    bool dynamic = false, need_diag = true;
    int inflight = 0;       // diagnostics launched and not yet read back
    bool admitted = false;  // holds `bytes` of the pool budget
    bool requeue = false;   // an AMR worker could not get the memory: back to the queue head
    // AMR: `step` is the program loop's s_; events (regrid, diagnostic) of step s_ are handled once
    // (events_done) before the solve takes its next coarse steps in the batch (round_steps).  A worker
    // creates the solve (task 1) or regrids it (task 2, plus the diagnostic of that step when dg).
    long long sstep = 1;
    bool events_done = false, dg = false;
    int task = 0;
    int lane = 0;           // AMR: the batch lane (stream) the solve advances in
    jp_status error = JP_OK;
    int samples = 0;
    double E0 = -1, prevE = 1e30, Elast = 0, peak = -1, peak_ts = -1, mass0 = -1, drift = 0;
    bool mono = true;
    double t_submit = 0, t_start = 0;
    long long bytes = 0;
};

long long estimate_bytes(const jp_config& c) {
    const long long n = c.n;
    const int Qn = 19;
    if (c.kind == JP_UNIFORM) {
        const long long elem = c.storage == JP_FP64 ? 8 : (c.storage == JP_FP32 ? 4 : 2);
        const long long field = diag_pop_ok(c.storage, (int)n) ? 0 : (c.storage == JP_FP64 ? 32 : 16) * n * n * n;
        const long long arrays = (c.flags & JP_FLAG_INPLACE) ? 1 : 2;  // in place: one population array
        return arrays * Qn * elem * n * n * n + field + (1 << 20);
    }
    // AMR: the pools of amr_create with the level-2 pool at its upper bound
    const long long mb = c.mb, mb3 = mb * mb * mb, sh = 6 * mb * mb + 12 * mb;
    const long long cgx = n / mb, cnb0 = cgx * cgx * cgx;
    const long long cap_nref0 = c.l1_mode == JP_REFINE_ALL
                                    ? cnb0
                                    : std::min(cnb0, std::max(1LL, (long long)std::ceil(c.frac1 * cnb0 * 1.4)));
    const long long cap1 = 8 * cap_nref0;
    const long long cap_nref1 = c.l2_mode == JP_REFINE_ALL
                                    ? cap1
                                    : std::min(cap1, std::max(1LL, (long long)std::ceil(2.5 * c.frac2 * cap1) + 8));
    const long long cap2 = 8 * cap_nref1;
    const long long elem = c.storage == JP_FP32 ? 4 : 2;
    const long long blk = Qn * mb3 * elem, gh = Qn * sh * elem;
    const long long n2 = 4 * n;
    return 3 * cnb0 * blk + cap1 * (3 * blk + gh) + cap2 * (2 * blk + gh) + 16 * n2 * n2 * n2 + (8 << 20);
}

}  // namespace

struct jp_server {
    jp_server_config cfg{};
    cudaStream_t stream = nullptr;     // batched uniform launches and their diagnostics
    cudaMemPool_t pool = nullptr;      // device memory of every served solve (stream-ordered)
    std::deque<Job*> queue;            // submitted, not admitted
    std::vector<Job*> active;          // admitted uniform solves
    std::vector<jp_result> done;
    double budget = 0;
    long long used = 0;
    std::chrono::steady_clock::time_point t0;
    // Uniform diagnostics are read back one tick late: tick t launches its diagnostics and steps,
    // then collects tick t-1's results, so the GPU always has the next tick queued while the host
    // waits.  Two sets of slots alternate.
    struct DiagBatch {
        double* dev = nullptr;    // 3 doubles per entry
        double* host = nullptr;   // pinned copy
        int cap = 0;
        cudaEvent_t done = nullptr;
        std::vector<std::pair<Job*, long long>> entries;  // job, step the values belong to
    } diag[2];
    int diag_cur = 0;
    // device time of batched launches: timing events around a round's launches on a stream, read
    // once they have completed (four rounds later)
    struct Span {
        cudaEvent_t a = nullptr, b = nullptr;
        bool live = false;
    };
    Span uspan[4];
    int uspan_tick = 0;
    // AMR solves advance in lanes, each a thread with its own stream and a share of the solves.  A
    // lane's rounds launch the diagnostics due, batched coarse steps with one launch per stage over
    // the lane's solves (amr_batch_step), and read the previous round's diagnostics back.  Creation and
    // regrids, which need read-backs, run on worker threads on each solve's own stream while its
    // lane goes on without it; a solve that leaves for a regrid waits only for its own lane's queue.
    struct AmrDiag {
        cudaEvent_t done = nullptr;
        std::vector<std::pair<Job*, long long>> entries;  // job, step; values in the solver's host slot
    };
    struct Lane {
        std::thread th;
        std::mutex mu;
        std::condition_variable cv;
        std::deque<Job*> inbox;          // created or regridded solves (re)joining the lane
        std::vector<Job*> active;        // the lane thread's own
        cudaStream_t stream = nullptr;
        AmrFork fk;  // the level-0 branch of the lane's batched coarse steps
        AmrDiag adiag[2];
        int diag_cur = 0;
        Span span[4];
        int span_tick = 0;
    };
    static constexpr int kLanes = 8;
    Lane lane[kLanes];
    int lane_load[kLanes] = {};        // admitted AMR solves per lane (tick thread)
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_todo, cv_fin;
    std::deque<Job*> amr_todo;         // worker tasks
    std::vector<Job*> amr_fin;         // AMR solves to retire (or to requeue) by the tick thread
    int amr_live = 0;                  // admitted AMR solves not yet retired (tick thread only)
    std::atomic<bool> stop{false};
    std::mutex stats_mu;
    jp_server_stats stats{};
    void add(double jp_server_stats::*field, double seconds, int64_t jp_server_stats::*count = nullptr,
             int64_t n = 1) {
        std::lock_guard<std::mutex> lk(stats_mu);
        stats.*field += seconds;
        if (count) stats.*count += n;
    }
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

double seconds_since(std::chrono::steady_clock::time_point t) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}
using clk = std::chrono::steady_clock;

void finish(jp_server* sv, Job* j, jp_status status) {
    jp_result r;
    std::memset(&r, 0, sizeof r);
    r.id = j->req.id;
    r.status = status;
    r.steps = j->steps;
    r.samples = j->samples;
    r.peak_tstar = j->peak_ts;
    r.peak_enstrophy = j->peak;
    r.energy_ratio = j->E0 > 0 ? j->Elast / j->E0 : 0.0;
    r.mass_drift = j->drift;
    r.valid = status == JP_OK && std::isfinite(j->peak) && j->peak_ts > 4.0 && j->peak_ts < 10.0 && j->mono &&
              j->drift < 5e-4;
    r.t_submit = j->t_submit;
    r.t_start = j->t_start;
    r.t_end = sv->now();
    r.bytes = j->bytes;
    sv->done.push_back(r);
    if (j->s) {
        const auto t = clk::now();
        jp_destroy(j->s);
        sv->add(&jp_server_stats::destroy_s, seconds_since(t));
    }
    if (j->admitted) sv->used -= j->bytes;
    {
        std::lock_guard<std::mutex> lk(sv->stats_mu);
        ++sv->stats.solves;
    }
    delete j;
}

// diagnostics bookkeeping of the programs' loops (src/tgv3d_uniform.cu:173-188)
void record(Job* j, const double d[3], long long step) {
    const double E = d[0], ens = d[1], mass = d[2];
    const double ts = double(step) * j->req.cfg.u0 * j->info.kf;
    if (j->mass0 < 0) j->mass0 = mass;
    j->drift = std::max(j->drift, std::fabs(mass - j->mass0) / j->mass0);
    if (j->E0 < 0) j->E0 = E;
    if (E > j->prevE * 1.0000001) j->mono = false;
    j->prevE = E;
    j->Elast = E;
    if (ens > j->peak) {
        j->peak = ens;
        j->peak_ts = ts;
    }
    ++j->samples;
}

// the device time of a round's launches on a stream: open before, close after; a slot is folded
// into the statistics when it comes round again
cudaError_t span_open(jp_server* sv, jp_server::Span (&ring)[4], int tick, double jp_server_stats::*field,
                      cudaStream_t st) {
    auto& sp = ring[tick & 3];
    cudaError_t e = cudaSuccess;
    if (!sp.a) e = cudaEventCreate(&sp.a);
    if (e == cudaSuccess && !sp.b) e = cudaEventCreate(&sp.b);
    if (e == cudaSuccess && sp.live) {
        float ms = 0.f;
        if (wait_event(sp.b) == cudaSuccess && cudaEventElapsedTime(&ms, sp.a, sp.b) == cudaSuccess)
            sv->add(field, ms * 1e-3);
        sp.live = false;
    }
    if (e == cudaSuccess) e = cudaEventRecord(sp.a, st);
    return e;
}
cudaError_t span_close(jp_server::Span (&ring)[4], int tick, cudaStream_t st) {
    auto& sp = ring[tick & 3];
    sp.live = true;
    return cudaEventRecord(sp.b, st);
}

// A worker's part of an AMR solve, on the solve's own stream: creation with the initial build and
// the diagnostic of step 0 (task 1), or a regrid and, when due at the same step, the diagnostic
// (task 2).  Everything else happens in the tick's batched launches.
void amr_task(jp_server* sv, Job* j) {
    if (cudaSetDevice(sv->cfg.device) != cudaSuccess) {
        j->error = JP_ERR_CUDA;
        return;
    }
    jp_status st = JP_OK;
    if (j->task == 1) {
        auto t = clk::now();
        st = create_solver(&j->req.cfg, sv->pool, &j->s);
        if (st == JP_OK) st = amr_prepare_diag(j->s);
        sv->add(&jp_server_stats::create_s, seconds_since(t));
        if (st != JP_OK) {
            if (j->s) jp_destroy(j->s);
            j->s = nullptr;
            if (st == JP_ERR_NOMEM) j->requeue = true;  // the estimate was optimistic: wait for memory
            else j->error = st;
            return;
        }
        jp_get_info(j->s, &j->info);
        j->steps = j->info.steps;
        j->diagK = j->req.diag_every > 0 ? j->req.diag_every : std::max(1LL, j->steps / 160);
        j->dynamic = j->req.cfg.l1_mode == JP_REFINE_SENSOR || j->req.cfg.l2_mode == JP_REFINE_SENSOR;
        j->adapt = j->req.cfg.adapt_every > 0 ? j->req.cfg.adapt_every : 100;
        j->sstep = (j->req.cfg.flags & JP_FLAG_GRAPH) ? 2 : 1;  // the program steps two at a time then
        j->step = 0;
        j->dg = true;  // step 0 has a diagnostic and no regrid
    } else {
        auto t = clk::now();
        st = jp_regrid(j->s);
        sv->add(&jp_server_stats::regrid_s, seconds_since(t), &jp_server_stats::regrids);
    }
    if (st == JP_OK && j->dg) {  // into slot 2 of the solver's pinned read-back area (slots 0, 1: tick)
        auto t = clk::now();
        double* d = j->s->diag_host + 6;
        st = amr_diag_async(j->s, j->s->stream, d);
        if (st == JP_OK && wait_stream(j->s) != cudaSuccess) st = fail(JP_ERR_CUDA, "diagnostics");
        sv->add(&jp_server_stats::diag_s, seconds_since(t), &jp_server_stats::diags);
        if (st == JP_OK) record(j, d, j->step);
    }
    j->error = st;
    j->events_done = true;
}

void worker_main(jp_server* sv) {
    for (;;) {
        Job* j = nullptr;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv_todo.wait(lk, [sv] { return sv->stop.load() || !sv->amr_todo.empty(); });
            if (sv->stop.load()) return;
            j = sv->amr_todo.front();
            sv->amr_todo.pop_front();
        }
        amr_task(sv, j);
        if (j->requeue || j->error != JP_OK) {  // the tick thread requeues or retires it
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->amr_fin.push_back(j);
            }
            sv->cv_fin.notify_all();
        } else {  // back to its lane
            auto& L = sv->lane[j->lane];
            {
                std::lock_guard<std::mutex> lk(L.mu);
                L.inbox.push_back(j);
            }
            L.cv.notify_one();
        }
    }
}

void to_worker(jp_server* sv, Job* j, int task);

// Coarse steps of an AMR solve in one lane round: up to the next step the program would visit
// (steps sstep apart) at which the solve has an event (a regrid, a diagnostic, the end), at most
// kRoundSteps.  Fewer, longer rounds leave less of a solve's time to the lane's per-round host work
// and read-back; the events still fall on the program's steps.
constexpr long long kRoundSteps = 8;
long long round_steps(const Job* j) {
    const long long cap = std::max(j->sstep, (kRoundSteps / j->sstep) * j->sstep);
    long long e = j->step;
    do {
        e += j->sstep;
    } while (e - j->step < cap && e < j->steps && !(j->dynamic && e % j->adapt == 0) && e % j->diagK != 0);
    return e - j->step;
}

// One round of a lane: the events of each solve's current step (a regrid sends the solve to a
// worker, its stream ordered after the lane's work so far, and a diagnostic of the same step goes
// with it; a diagnostic alone is launched on the lane's stream into this round's read-back slot; a
// solve with a diagnostic in flight waits a round before a regrid, so its samples are recorded in
// order), the batched coarse steps of the solves that move (each up to its next event, round_steps:
// the program's steps, two at a time with graph replay), the previous round's read-backs, and the
// retirement of solves that are over.
// Returns whether anything was launched or read back.
bool lane_round(jp_server* sv, jp_server::Lane& L) {
    bool busy = false;
    auto fail_all = [&](jp_status st) {
        for (Job* j : L.active)
            if (j->error == JP_OK) j->error = st;
    };
    auto& cur = L.adiag[L.diag_cur];
    cur.entries.clear();
    for (size_t i = 0; i < L.active.size();) {
        Job* j = L.active[i];
        if (j->events_done || j->step > j->steps || j->error != JP_OK) {
            ++i;
            continue;
        }
        const bool rg = j->dynamic && j->step > 0 && j->step % j->adapt == 0, dg = j->step % j->diagK == 0;
        if (rg) {
            if (j->inflight) {
                ++i;
                continue;
            }
            if (cudaEventRecord(j->s->ev0, L.stream) != cudaSuccess ||
                cudaStreamWaitEvent(j->s->stream, j->s->ev0, 0) != cudaSuccess) {
                j->error = fail(JP_ERR_CUDA, "lane event");
                ++i;
                continue;
            }
            j->dg = dg;
            L.active.erase(L.active.begin() + i);
            to_worker(sv, j, 2);
            busy = true;
            continue;
        }
        if (dg) {
            const auto ta = clk::now();
            jp_status st = amr_diag_async(j->s, L.stream, j->s->diag_host + 3 * L.diag_cur);
            sv->add(&jp_server_stats::diag_s, seconds_since(ta), &jp_server_stats::diags);
            if (st != JP_OK) {
                j->error = st;
                ++i;
                continue;
            }
            cur.entries.push_back({j, j->step});
            ++j->inflight;
            busy = true;
        }
        j->events_done = true;
        ++i;
    }
    if (!cur.entries.empty() && cudaEventRecord(cur.done, L.stream) != cudaSuccess) fail_all(JP_ERR_CUDA);
    // batched coarse steps, one group per launch shape
    std::vector<std::vector<Job*>> groups;
    for (Job* j : L.active) {
        if (!j->events_done || j->step >= j->steps || j->error != JP_OK) continue;
        bool placed = false;
        for (auto& g : groups)
            if (amr_batch_compatible(g[0]->s, j->s)) {
                g.push_back(j);
                placed = true;
                break;
            }
        if (!placed) groups.push_back({j});
    }
    if (!groups.empty()) {
        const auto tab = clk::now();
        long long moved = 0;
        if (span_open(sv, L.span, L.span_tick, &jp_server_stats::amr_gpu_s, L.stream) != cudaSuccess)
            fail_all(JP_ERR_CUDA);
        for (auto& g : groups) {
            jp_status st = JP_OK;
            std::vector<long long> ks(g.size());
            long long kmax = 0;
            for (size_t i = 0; i < g.size(); ++i) kmax = std::max(kmax, ks[i] = round_steps(g[i]));
            for (long long t = 0; t < kmax && st == JP_OK; ++t) {
                std::vector<jp_solver*> ms;
                for (size_t i = 0; i < g.size(); ++i)
                    if (ks[i] > t) ms.push_back(g[i]->s);
                // a group of one with graph replay replays its captured step instead (one launch)
                const bool alone = ms.size() == 1 && (ms[0]->cfg.flags & JP_FLAG_GRAPH);
                st = alone ? amr_graph_step_on(ms[0], L.stream) : amr_batch_step(ms, L.stream, &L.fk);
                moved += (long long)ms.size();
            }
            for (size_t i = 0; i < g.size(); ++i) {
                if (st != JP_OK) g[i]->error = st;
                g[i]->step += ks[i];
                g[i]->events_done = false;
            }
        }
        span_close(L.span, L.span_tick, L.stream);
        ++L.span_tick;
        sv->add(&jp_server_stats::step_s, seconds_since(tab), &jp_server_stats::coarse_steps, moved);
        busy = true;
    }
    // the previous round's diagnostics
    auto& prev = L.adiag[L.diag_cur ^ 1];
    if (!prev.entries.empty()) {
        const auto tw = clk::now();
        const cudaError_t e = wait_event(prev.done);
        for (auto& en : prev.entries) {
            if (e == cudaSuccess) record(en.first, en.first->s->diag_host + 3 * (L.diag_cur ^ 1), en.second);
            else if (en.first->error == JP_OK) en.first->error = fail(JP_ERR_CUDA, "diagnostics");
            --en.first->inflight;
        }
        prev.entries.clear();
        sv->add(&jp_server_stats::diag_s, seconds_since(tw));
        busy = true;
    }
    L.diag_cur ^= 1;
    // retire solves that take no more steps and have nothing in flight; their frees are ordered
    // after the lane's last work on them
    std::vector<Job*> over;
    for (size_t i = 0; i < L.active.size();) {
        Job* j = L.active[i];
        const bool done = j->step > j->steps || (j->step == j->steps && j->events_done) || j->error != JP_OK;
        if (done && j->inflight == 0) {
            if (cudaEventRecord(j->s->ev0, L.stream) != cudaSuccess ||
                cudaStreamWaitEvent(j->s->stream, j->s->ev0, 0) != cudaSuccess)
                cudaStreamSynchronize(L.stream);
            L.active.erase(L.active.begin() + i);
            over.push_back(j);
        } else {
            ++i;
        }
    }
    if (!over.empty()) {
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            for (Job* j : over) sv->amr_fin.push_back(j);
        }
        sv->cv_fin.notify_all();
        busy = true;
    }
    return busy;
}

void lane_main(jp_server* sv, int l) {
    jp_server::Lane& L = sv->lane[l];
    cudaSetDevice(sv->cfg.device);
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(L.mu);
            if (L.active.empty())
                L.cv.wait_for(lk, std::chrono::milliseconds(2), [&] { return sv->stop.load() || !L.inbox.empty(); });
            if (sv->stop.load()) return;
            while (!L.inbox.empty()) {  // (re)join after the worker's work on the solve's own stream
                Job* j = L.inbox.front();
                L.inbox.pop_front();
                if (cudaEventRecord(j->s->ev1, j->s->stream) != cudaSuccess ||
                    cudaStreamWaitEvent(L.stream, j->s->ev1, 0) != cudaSuccess)
                    j->error = fail(JP_ERR_CUDA, "lane event");
                L.active.push_back(j);
            }
        }
        if (L.active.empty()) continue;
        if (!lane_round(sv, L)) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

void to_worker(jp_server* sv, Job* j, int task) {
    j->task = task;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->amr_todo.push_back(j);
    }
    sv->cv_todo.notify_one();
}

}  // namespace

extern "C" {

jp_status jp_server_create(const jp_server_config* cfg, jp_server** out) {
    if (!cfg || !out) return fail(JP_ERR_INVALID, "null argument");
    *out = nullptr;
    ECK(cudaSetDevice(cfg->device), "cudaSetDevice");
    jp_server* sv = new (std::nothrow) jp_server();
    if (!sv) return fail(JP_ERR_NOMEM, "host allocation");
    sv->cfg = *cfg;
    if (sv->cfg.tick_steps <= 0) sv->cfg.tick_steps = 64;
    if (sv->cfg.workers <= 0) sv->cfg.workers = (int)std::min(32u, std::max(4u, std::thread::hardware_concurrency()));
    sv->t0 = std::chrono::steady_clock::now();
    // stream priorities: the solves' own streams (creation, regrids, read-backs) run at the highest;
    // with uniform_first the uniform batches share it and the AMR lanes take the lowest
    int lo = 0, hi = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithPriority(&sv->stream, cudaStreamNonBlocking, sv->cfg.uniform_first ? hi : lo);
    for (int l = 0; l < jp_server::kLanes && e == cudaSuccess; ++l) {
        e = cudaStreamCreateWithPriority(&sv->lane[l].stream, cudaStreamNonBlocking, lo);
        if (e == cudaSuccess) e = sv->lane[l].fk.create(sv->lane[l].stream);
        for (auto& d : sv->lane[l].adiag)
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d.done, cudaEventDisableTiming);
    }
    size_t fr = 0, tot = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&fr, &tot);
    if (e == cudaSuccess) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = cfg->device;
        e = cudaMemPoolCreate(&sv->pool, &props);
    }
    if (e == cudaSuccess) {  // keep freed memory in the pool for the next solves
        uint64_t keep = UINT64_MAX;
        e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e != cudaSuccess) {
        jp_server_destroy(sv);
        return cuda_fail(e, "server setup");
    }
    sv->budget = cfg->pool_gb > 0 ? cfg->pool_gb * double(1ull << 30) : 0.75 * double(fr);
    for (int w = 0; w < sv->cfg.workers; ++w) sv->workers.emplace_back(worker_main, sv);
    for (int l = 0; l < jp_server::kLanes; ++l) sv->lane[l].th = std::thread(lane_main, sv, l);
    *out = sv;
    return JP_OK;
}

void jp_server_destroy(jp_server* sv) {
    if (!sv) return;
    cudaSetDevice(sv->cfg.device);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop.store(true);
    }
    sv->cv_todo.notify_all();
    for (auto& L : sv->lane) {
        { std::lock_guard<std::mutex> lk(L.mu); }
        L.cv.notify_all();
    }
    for (std::thread& t : sv->workers) t.join();  // a running task ends first
    for (auto& L : sv->lane)
        if (L.th.joinable()) L.th.join();
    if (sv->stream) cudaStreamSynchronize(sv->stream);
    for (auto& L : sv->lane)
        if (L.stream) cudaStreamSynchronize(L.stream);
    for (Job* j : sv->active) {
        if (j->s) jp_destroy(j->s);
        delete j;
    }
    for (auto& L : sv->lane) {
        for (Job* j : L.active) {
            if (j->s) jp_destroy(j->s);
            delete j;
        }
        for (Job* j : L.inbox) {
            if (j->s) jp_destroy(j->s);
            delete j;
        }
    }
    for (Job* j : sv->amr_todo) {
        if (j->s) jp_destroy(j->s);
        delete j;
    }
    for (Job* j : sv->amr_fin) {
        if (j->s) jp_destroy(j->s);
        delete j;
    }
    auto drop_spans = [](jp_server::Span (&ring)[4]) {
        for (auto& sp : ring) {
            if (sp.a) cudaEventDestroy(sp.a);
            if (sp.b) cudaEventDestroy(sp.b);
        }
    };
    for (auto& L : sv->lane) {
        for (auto& d : L.adiag)
            if (d.done) cudaEventDestroy(d.done);
        drop_spans(L.span);
    }
    drop_spans(sv->uspan);
    for (auto& L : sv->lane) {
        L.fk.destroy();
        if (L.stream) cudaStreamDestroy(L.stream);
    }
    for (Job* j : sv->queue) delete j;
    for (auto& b : sv->diag) {
        if (b.dev) cudaFree(b.dev);
        if (b.host) cudaFreeHost(b.host);
        if (b.done) cudaEventDestroy(b.done);
    }
    if (sv->stream) cudaStreamDestroy(sv->stream);
    if (sv->pool) {
        cudaDeviceSynchronize();
        cudaMemPoolDestroy(sv->pool);
    }
    delete sv;
}

jp_status jp_server_submit(jp_server* sv, const jp_request* req) {
    if (!sv || !req) return fail(JP_ERR_INVALID, "null argument");
    Job* j = new (std::nothrow) Job();
    if (!j) return fail(JP_ERR_NOMEM, "host allocation");
    j->req = *req;
    j->req.cfg.device = sv->cfg.device;
    j->t_submit = sv->now();
    j->bytes = estimate_bytes(j->req.cfg);
    if ((double)j->bytes > sv->budget) {
        jp_result r;
        std::memset(&r, 0, sizeof r);
        r.id = req->id;
        r.status = JP_ERR_NOMEM;
        r.t_submit = r.t_start = r.t_end = j->t_submit;
        r.bytes = j->bytes;
        sv->done.push_back(r);
        delete j;
        return fail(JP_ERR_NOMEM, "request %lld needs %lld bytes, pool budget is %.0f", (long long)req->id, j->bytes,
                    sv->budget);
    }
    sv->queue.push_back(j);
    return JP_OK;
}

static jp_status server_tick(jp_server* sv, int32_t* n_active, int32_t* n_queued);

jp_status jp_server_tick(jp_server* sv, int32_t* n_active, int32_t* n_queued) {
    if (!sv) return fail(JP_ERR_INVALID, "null server");
    const auto t = clk::now();
    const jp_status st = server_tick(sv, n_active, n_queued);
    sv->add(&jp_server_stats::tick_s, seconds_since(t));
    return st;
}

jp_status jp_server_get_stats(const jp_server* sv, jp_server_stats* out) {
    if (!sv || !out) return fail(JP_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(const_cast<jp_server*>(sv)->stats_mu);
    *out = sv->stats;
    return JP_OK;
}

}  // extern "C"

static jp_status server_tick(jp_server* sv, int32_t* n_active, int32_t* n_queued) {
    ECK(cudaSetDevice(sv->cfg.device), "cudaSetDevice");
    // 1. retire the AMR solves the workers finished (their memory is back in the pool)
    std::vector<Job*> fin, requeued;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        fin.swap(sv->amr_fin);
    }
    for (Job* j : fin) {  // from the lanes (over) and the workers (failed, or no memory yet)
        --sv->amr_live;
        --sv->lane_load[j->lane];
        if (j->requeue) {
            j->requeue = false;
            j->admitted = false;
            sv->used -= j->bytes;
            sv->queue.push_front(j);
            requeued.push_back(j);
        } else {
            finish(sv, j, j->error);
        }
    }
    // 2. admission in submission order while the budget and the slots allow.  An AMR solve also
    //    needs a free worker; while none is free it keeps its place and later uniform solves may
    //    pass it (they need no worker).  Memory is strictly first come, first served.
    for (auto it = sv->queue.begin(); it != sv->queue.end();) {
        if (sv->cfg.max_active > 0 && (int)sv->active.size() + sv->amr_live >= sv->cfg.max_active) break;
        Job* j = *it;
        if (std::find(requeued.begin(), requeued.end(), j) != requeued.end()) break;  // no memory: next tick
        if (j->req.cfg.kind == JP_AMR && sv->amr_live >= 4 * amr::kAmrBatchMax) {  // enough to fill the batch
            ++it;
            continue;
        }
        if ((double)(sv->used + j->bytes) > sv->budget) break;
        it = sv->queue.erase(it);
        j->t_start = sv->now();
        if (j->req.cfg.kind == JP_AMR) {
            j->admitted = true;
            sv->used += j->bytes;
            ++sv->amr_live;
            j->lane = int(std::min_element(sv->lane_load, sv->lane_load + jp_server::kLanes) - sv->lane_load);
            ++sv->lane_load[j->lane];
            to_worker(sv, j, 1);
            continue;
        }
        const auto tc = clk::now();
        jp_status st = create_solver(&j->req.cfg, sv->pool, &j->s);
        sv->add(&jp_server_stats::create_s, seconds_since(tc));
        if (st == JP_ERR_NOMEM) {  // the estimate was optimistic: wait for memory to free up
            j->s = nullptr;
            sv->queue.insert(it, j);
            break;
        }
        if (st != JP_OK) {
            j->s = nullptr;
            finish(sv, j, st);
            continue;
        }
        j->admitted = true;
        sv->used += j->bytes;
        jp_solver* s = j->s;
        jp_get_info(s, &j->info);
        j->steps = j->info.steps;
        j->diagK = j->req.diag_every > 0 ? j->req.diag_every : std::max(1LL, j->steps / 240);
        // an FP64 solve's diagnostics read a macro field, ready before the server's stream uses it
        // (the float storages' diagnostics read the populations)
        cudaError_t e = cudaSuccess;
        if (!diag_pop_ok(s->storage, s->n)) {
            e = dev_alloc(s, &s->field, (s->storage == JP_FP64 ? 8 : 4) * 4 * (size_t)s->cells);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        }
        if (e != cudaSuccess) {
            finish(sv, j, cuda_fail(e, "macro field"));
            continue;
        }
        sv->active.push_back(j);
    }
    // 3. the tick's uniform work on the server's stream: up to tick_steps batched steps, and each
    // diagnostic at the step it belongs to (macro field and reduction of that solve, into its own
    // slot of this tick's batch), so a solve sampled every step still advances tick_steps steps per
    // tick.  One read-back of all slots at the end.
    auto& cur = sv->diag[sv->diag_cur];
    cur.entries.clear();
    const long long T = sv->cfg.tick_steps;
    int slots = 0;  // diagnostics this tick can reach: the one due now and those at multiples of diagK
    for (Job* j : sv->active)
        if (j->error == JP_OK) {
            const long long last = std::min(j->steps, j->step + T);
            slots += (j->need_diag ? 1 : 0) + int(last / j->diagK - j->step / j->diagK);
        }
    if (slots > cur.cap) {  // these slots were read back last tick: free to replace
        if (cur.dev) cudaFree(cur.dev);
        if (cur.host) cudaFreeHost(cur.host);
        cur.dev = nullptr;
        cur.host = nullptr;
        cur.cap = std::max(2 * slots, 64);
        ECK(cudaMalloc(&cur.dev, sizeof(double) * 3 * cur.cap), "cudaMalloc diag slots");
        ECK(cudaMallocHost(&cur.host, sizeof(double) * 3 * cur.cap), "cudaMallocHost diag slots");
    }
    if (!cur.done) ECK(cudaEventCreateWithFlags(&cur.done, cudaEventDisableTiming), "diag event");
    double diag_host_s = 0.0;
    auto launch_diags = [&]() -> jp_status {  // the diagnostics due at the solves' current steps
        const auto td = clk::now();
        for (Job* j : sv->active) {
            if (j->error != JP_OK || !j->need_diag) continue;
            if ((int)cur.entries.size() >= cur.cap) return fail(JP_ERR_CAPACITY, "diagnostic slots exhausted");
            jp_solver* s = j->s;
            double* slot = cur.dev + 3 * cur.entries.size();
            if (diag_pop_ok(s->storage, s->n)) {
                ECK(launch_diag_pop(s->storage, s->aa_layout(), s->fa, s->n, s->partials, slot, nullptr, sv->stream),
                    "diag");  // a wait that gave up leaves NaN diagnostics, which fail the solve's check
            } else {
                const bool dbl = s->storage == JP_FP64;
                ECK(launch_macro(s->storage, s->fa, s->field, s->n, sv->stream, s->aa_layout()), "macro");
                ECK(launch_diag_field(dbl, !dbl, s->field, s->n, s->partials, slot, sv->stream), "diag");
            }
            cur.entries.push_back({j, j->step});
            j->need_diag = false;
            ++j->inflight;
        }
        diag_host_s += seconds_since(td);
        return JP_OK;
    };
    std::vector<Job*> moving;
    std::vector<jp_solver*> members;
    const auto tsb = clk::now();
    bool spanned = false;
    for (long long t = 0;; ++t) {
        const jp_status dst = launch_diags();
        if (dst != JP_OK) return dst;
        if (t == T) break;
        moving.clear();
        members.clear();
        for (Job* j : sv->active)
            if (j->error == JP_OK && j->step < j->steps) {
                moving.push_back(j);
                members.push_back(j->s);
            }
        if (members.empty()) break;
        if (!spanned) {
            ECK(span_open(sv, sv->uspan, sv->uspan_tick, &jp_server_stats::uniform_gpu_s, sv->stream), "span");
            spanned = true;
        }
        jp_status st = batched_step(members, sv->stream);
        if (st != JP_OK) return st;
        for (Job* j : moving)
            if (++j->step % j->diagK == 0) j->need_diag = true;  // launched before the next step
    }
    if (spanned) {
        ECK(span_close(sv->uspan, sv->uspan_tick, sv->stream), "span");
        ++sv->uspan_tick;
        sv->add(&jp_server_stats::step_s, seconds_since(tsb) - diag_host_s);
    }
    if (!cur.entries.empty()) {
        ECK(cudaMemcpyAsync(cur.host, cur.dev, sizeof(double) * 3 * cur.entries.size(), cudaMemcpyDeviceToHost,
                            sv->stream), "diag D2H");
        ECK(cudaEventRecord(cur.done, sv->stream), "diag event");
        sv->add(&jp_server_stats::diag_s, diag_host_s, &jp_server_stats::diags, (int64_t)cur.entries.size());
    }
    // 5. the previous tick's diagnostics (the GPU meanwhile works on this tick's launches)
    auto& prev = sv->diag[sv->diag_cur ^ 1];
    if (!prev.entries.empty()) {
        const auto tw = clk::now();
        ECK(wait_event(prev.done), "diag");
        for (size_t k = 0; k < prev.entries.size(); ++k) {
            record(prev.entries[k].first, prev.host + 3 * k, prev.entries[k].second);
            --prev.entries[k].first->inflight;
        }
        prev.entries.clear();
        sv->add(&jp_server_stats::diag_s, seconds_since(tw));
    }
    sv->diag_cur ^= 1;
    // retire finished uniform solves: all steps issued, every diagnostic read back.  A solve whose
    // step count is not a multiple of its diagnostic interval ends with steps that no diagnostic
    // follows, and they may still run on the server's stream: its memory goes back to the pool on
    // its own stream, ordered after everything the server's stream holds so far.  A solve that
    // failed is retired the same way once no read-back of it is pending.
    for (size_t i = 0; i < sv->active.size();) {
        Job* j = sv->active[i];
        const bool done = j->step >= j->steps && !j->need_diag && j->inflight == 0;
        if (done || (j->error != JP_OK && j->inflight == 0)) {
            sv->active.erase(sv->active.begin() + i);
            if (cudaEventRecord(j->s->ev0, sv->stream) != cudaSuccess ||
                cudaStreamWaitEvent(j->s->stream, j->s->ev0, 0) != cudaSuccess)
                cudaStreamSynchronize(sv->stream);
            finish(sv, j, j->error);
        } else {
            ++i;
        }
    }
    // 6. nothing launched here while AMR solves run in their lanes: wait briefly for one to end
    if (!spanned && sv->amr_live > 0) {
        std::unique_lock<std::mutex> lk(sv->mu);
        sv->cv_fin.wait_for(lk, std::chrono::milliseconds(1), [sv] { return !sv->amr_fin.empty(); });
    }
    if (n_active) *n_active = (int32_t)sv->active.size() + sv->amr_live;
    if (n_queued) *n_queued = (int32_t)sv->queue.size();
    return JP_OK;
}

extern "C" {

int32_t jp_server_poll(jp_server* sv, jp_result* out, int32_t max) {
    if (!sv || !out || max <= 0) return 0;
    const int32_t n = (int32_t)std::min<size_t>((size_t)max, sv->done.size());
    for (int32_t i = 0; i < n; ++i) out[i] = sv->done[i];
    sv->done.erase(sv->done.begin(), sv->done.begin() + n);
    return n;
}

double jp_server_clock(const jp_server* sv) { return sv ? sv->now() : 0.0; }

}  // extern "C"
