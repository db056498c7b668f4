// Ensembles and the solve server: many independent Taylor-Green solves on one GPU.
//
// No counterpart in the reference, which runs one solve per process.  An ensemble batches the
// stream-collide of many uniform cubes into one launch per storage format per lattice step
// (k_stream_collide takes up to kMaxBatch cubes of any sizes).  The server adds continuous
// batching on top: requests wait until their HBM estimate fits the pool and a slot is free, join
// between ticks while other solves run, advance together, and leave with a result.  Each solve does
// exactly what the `uniform` / `amr` programs do for it (same steps, diagnostic cadence, regrid
// cadence, VALID gate), so its numbers do not depend on what else is running.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <vector>

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
    std::map<long long, std::vector<jp_solver*>> groups;
    for (jp_solver* m : members)
        groups[((long long)m->storage << 32) | ((long long)m->vec << 16) | (long long)m->tpb].push_back(m);
    for (auto& g : groups) {
        const std::vector<jp_solver*>& v = g.second;
        for (size_t i = 0; i < v.size(); i += kMaxBatch) {
            const size_t cnt = std::min(v.size() - i, (size_t)kMaxBatch);
            UniSolve us[kMaxBatch];
            for (size_t k = 0; k < cnt; ++k) {
                jp_solver* m = v[i + k];
                std::memset(&us[k], 0, sizeof us[k]);
                us[k].src = m->fa;
                us[k].dst = m->fb;
                us[k].n = m->n;
                us[k].omega = float(m->info.omega);
                us[k].omega_d = m->info.omega;
            }
            ECK(launch_stream_collide(v[i]->storage, us, (int)cnt, v[i]->vec, v[i]->tpb, st), "batched stream_collide");
            for (size_t k = 0; k < cnt; ++k) {
                std::swap(v[i + k]->fa, v[i + k]->fb);
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
    std::vector<jp_solver*> members;
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
    if (e->done) cudaEventDestroy(e->done);
    delete e;
}

jp_status jp_ensemble_add(jp_ensemble* e, jp_solver* s) {
    if (!e || !s) return fail(JP_ERR_INVALID, "null argument");
    if (s->kind != JP_UNIFORM) return fail(JP_ERR_INVALID, "ensembles hold uniform solvers");
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
        ECK(cudaEventRecord(m->ev1, m->stream), "event");
        ECK(cudaStreamWaitEvent(e->stream, m->ev1, 0), "wait");
    }
    for (int64_t i = 0; i < nsteps; ++i) {
        jp_status st = batched_step(e->members, e->stream);
        if (st != JP_OK) return st;
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
    bool dynamic = false, need_diag = true, regridded = false;
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
        const long long field = (c.storage == JP_FP64 ? 32 : 16) * n * n * n;
        return 2 * Qn * elem * n * n * n + field + (1 << 20);
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
    const long long blk = Qn * mb3 * 4, gh = Qn * sh * 4;
    const long long n2 = 4 * n;
    return 3 * cnb0 * blk + cap1 * (3 * blk + gh) + cap2 * (2 * blk + gh) + 16 * n2 * n2 * n2 + (8 << 20);
}

}  // namespace

struct jp_server {
    jp_server_config cfg{};
    cudaStream_t stream = nullptr;
    std::deque<Job*> queue;
    std::vector<Job*> active;
    std::vector<jp_result> done;
    double budget = 0;
    long long used = 0;
    std::chrono::steady_clock::time_point t0;
    double* dev_diag = nullptr;   // 3 doubles per uniform job with a pending diagnostic
    double* host_diag = nullptr;
    int diag_cap = 0;
    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

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
        jp_destroy(j->s);
        sv->used -= j->bytes;
    }
    delete j;
}

// diagnostics bookkeeping of the programs' loops (src/tgv3d_uniform.cu:173-188)
void record(Job* j, const double d[3]) {
    const double E = d[0], ens = d[1], mass = d[2];
    const double ts = double(j->step) * j->req.cfg.u0 * j->info.kf;
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
    j->need_diag = false;
}

long long next_event(const Job* j) {
    long long e = std::min(j->steps, (j->step / j->diagK + 1) * j->diagK);
    if (j->dynamic && j->adapt > 0) e = std::min(e, (j->step / j->adapt + 1) * j->adapt);
    return e;
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
    sv->t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking);
    size_t fr = 0, tot = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&fr, &tot);
    if (e != cudaSuccess) {
        jp_server_destroy(sv);
        return cuda_fail(e, "server setup");
    }
    sv->budget = cfg->pool_gb > 0 ? cfg->pool_gb * double(1ull << 30) : 0.75 * double(fr);
    *out = sv;
    return JP_OK;
}

void jp_server_destroy(jp_server* sv) {
    if (!sv) return;
    cudaSetDevice(sv->cfg.device);
    if (sv->stream) cudaStreamSynchronize(sv->stream);
    for (Job* j : sv->active) {
        if (j->s) jp_destroy(j->s);
        delete j;
    }
    for (Job* j : sv->queue) delete j;
    if (sv->dev_diag) cudaFree(sv->dev_diag);
    if (sv->host_diag) cudaFreeHost(sv->host_diag);
    if (sv->stream) cudaStreamDestroy(sv->stream);
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

jp_status jp_server_tick(jp_server* sv, int32_t* n_active, int32_t* n_queued) {
    if (!sv) return fail(JP_ERR_INVALID, "null server");
    ECK(cudaSetDevice(sv->cfg.device), "cudaSetDevice");
    // 1. admission: FIFO while the head fits the budget and a slot is free
    while (!sv->queue.empty() && (sv->cfg.max_active <= 0 || (int)sv->active.size() < sv->cfg.max_active)) {
        Job* j = sv->queue.front();
        if ((double)(sv->used + j->bytes) > sv->budget) break;
        sv->queue.pop_front();
        j->t_start = sv->now();
        jp_status st = jp_create(&j->req.cfg, &j->s);
        if (st == JP_ERR_NOMEM) {  // the estimate was optimistic: wait for memory to free up
            sv->queue.push_front(j);
            break;
        }
        if (st != JP_OK) {
            j->s = nullptr;
            finish(sv, j, st);
            continue;
        }
        sv->used += j->bytes;
        jp_get_info(j->s, &j->info);
        j->steps = j->info.steps;
        const bool amr = j->req.cfg.kind == JP_AMR;
        j->diagK = j->req.diag_every > 0 ? j->req.diag_every : std::max(1LL, j->steps / (amr ? 160 : 240));
        j->dynamic = amr && (j->req.cfg.l1_mode == JP_REFINE_SENSOR || j->req.cfg.l2_mode == JP_REFINE_SENSOR);
        j->adapt = j->req.cfg.adapt_every > 0 ? j->req.cfg.adapt_every : 100;
        sv->active.push_back(j);
    }
    // 2. regrid (AMR, before the diagnostic of the same step) and diagnostics due now
    std::vector<Job*> uni_diag;
    // a failing call ends only its own solve: the job leaves with that status at the next retirement
    for (Job* j : sv->active) {
        if (j->error != JP_OK) continue;
        if (j->req.cfg.kind == JP_AMR && j->dynamic && j->step > 0 && j->step % j->adapt == 0 && !j->regridded) {
            jp_status st = jp_regrid(j->s);
            j->regridded = true;
            if (st != JP_OK) {
                j->error = st;
                continue;
            }
        }
        if (!j->need_diag) continue;
        if (j->req.cfg.kind == JP_AMR) {
            double d[3];
            jp_status st = jp_diag(j->s, d);
            if (st != JP_OK) {
                j->error = st;
                continue;
            }
            record(j, d);
        } else {
            uni_diag.push_back(j);
        }
    }
    if (!uni_diag.empty()) {
        if ((int)uni_diag.size() > sv->diag_cap) {
            if (sv->dev_diag) cudaFree(sv->dev_diag);
            if (sv->host_diag) cudaFreeHost(sv->host_diag);
            sv->diag_cap = std::max<int>(2 * (int)uni_diag.size(), 64);
            ECK(cudaMalloc(&sv->dev_diag, sizeof(double) * 3 * sv->diag_cap), "cudaMalloc diag slots");
            ECK(cudaMallocHost(&sv->host_diag, sizeof(double) * 3 * sv->diag_cap), "cudaMallocHost diag slots");
        }
        for (size_t k = 0; k < uni_diag.size(); ++k) {
            jp_solver* s = uni_diag[k]->s;
            if (!s->field) {
                const size_t fb = (s->storage == JP_FP64 ? 8 : 4) * 4 * (size_t)s->cells;
                ECK(cudaMalloc(&s->field, fb), "cudaMalloc macro field");
            }
            const bool dbl = s->storage == JP_FP64;
            ECK(launch_macro(s->storage, s->fa, s->field, s->n, sv->stream), "macro");
            ECK(launch_diag_field(dbl, !dbl, s->field, s->n, s->partials, sv->dev_diag + 3 * k, sv->stream), "diag");
        }
        ECK(cudaMemcpyAsync(sv->host_diag, sv->dev_diag, sizeof(double) * 3 * uni_diag.size(), cudaMemcpyDeviceToHost,
                            sv->stream), "diag D2H");
        ECK(cudaStreamSynchronize(sv->stream), "diag");
        for (size_t k = 0; k < uni_diag.size(); ++k) record(uni_diag[k], sv->host_diag + 3 * k);
    }
    // 3. retire finished solves (after the batched launches that touched them)
    bool any_done = false;
    for (Job* j : sv->active) any_done |= (j->step >= j->steps && !j->need_diag) || j->error != JP_OK;
    if (any_done) ECK(cudaStreamSynchronize(sv->stream), "retire");
    for (size_t i = 0; i < sv->active.size();) {
        Job* j = sv->active[i];
        if ((j->step >= j->steps && !j->need_diag) || j->error != JP_OK) {
            sv->active.erase(sv->active.begin() + i);
            finish(sv, j, j->error);
        } else {
            ++i;
        }
    }
    // 4. advance: uniform solves in batched launches, AMR solves on their own streams
    std::vector<std::pair<Job*, long long>> uni;
    long long kmax = 0;
    for (Job* j : sv->active) {
        if (j->error != JP_OK) continue;
        const long long target = next_event(j);
        if (j->req.cfg.kind == JP_AMR) {
            const long long k = std::min(target - j->step, std::max(1LL, (long long)sv->cfg.tick_steps / 4));
            if (k <= 0) continue;
            jp_status st = jp_step(j->s, k);
            if (st != JP_OK) {
                j->error = st;
                continue;
            }
            j->step += k;
            j->regridded = false;
        } else {
            const long long k = std::min(target - j->step, (long long)sv->cfg.tick_steps);
            uni.push_back({j, k});
            kmax = std::max(kmax, k);
        }
    }
    std::vector<jp_solver*> members;
    for (long long t = 0; t < kmax; ++t) {
        members.clear();
        for (auto& p : uni)
            if (p.second > t) members.push_back(p.first->s);
        jp_status st = batched_step(members, sv->stream);
        if (st != JP_OK) return st;
    }
    for (auto& p : uni) p.first->step += p.second;
    for (Job* j : sv->active) {
        if (j->step % j->diagK == 0) j->need_diag = true;  // diagnostics at the new step (next tick)
    }
    if (n_active) *n_active = (int32_t)sv->active.size();
    if (n_queued) *n_queued = (int32_t)sv->queue.size();
    return JP_OK;
}

int32_t jp_server_poll(jp_server* sv, jp_result* out, int32_t max) {
    if (!sv || !out || max <= 0) return 0;
    const int32_t n = (int32_t)std::min<size_t>((size_t)max, sv->done.size());
    for (int32_t i = 0; i < n; ++i) out[i] = sv->done[i];
    sv->done.erase(sv->done.begin(), sv->done.begin() + n);
    return n;
}

double jp_server_clock(const jp_server* sv) { return sv ? sv->now() : 0.0; }

}  // extern "C"
