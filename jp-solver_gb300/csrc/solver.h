// Solver object behind the opaque jp_solver handle, and the per-kind implementations the C ABI
// dispatches to.  Internal to libjpsolver.so.
#pragma once
#include "jp.h"
#include "kernels.h"

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <vector>

namespace jp {
struct AmrState;
namespace amr {
struct PersistSync;
}

jp_status fail(jp_status st, const char* fmt, ...);
jp_status cuda_fail(cudaError_t e, const char* what);
size_t storage_bytes(int storage);

// Device memory of a solver: from its stream-ordered pool on its own stream when it has one (solves
// run by a server: no device-wide synchronisation when they come and go), else cudaMalloc/cudaFree.
cudaError_t dev_alloc(jp_solver* s, void** p, size_t bytes);
void dev_free(jp_solver* s, void* p);
// Small pinned host buffers (<= 256 bytes: diagnostic and count read-backs) from process-wide slabs
// that are never returned to the driver, so creating and destroying solvers never calls
// cudaFreeHost (which synchronises the device).
void* pinned_slot_alloc();
void pinned_slot_free(void* p);
// jp_create with a stream-ordered memory pool (nullptr: plain allocations).  A solver with a pool
// belongs to a server and waits for its stream politely (wait_stream).
jp_status create_solver(const jp_config* cfg, cudaMemPool_t pool, jp_solver** out);
// Wait until the solver's stream has drained.  A served solver polls an event, yielding the core and
// then sleeping in short slices, so that many solves waiting at once leave the host cores to the
// threads that issue work; otherwise cudaStreamSynchronize.
cudaError_t wait_stream(jp_solver* s);
// wait for an event without spinning on a core (yield, then sleep between polls)
cudaError_t wait_event(cudaEvent_t ev);
double stored_to_double(int storage, const void* base, size_t idx, int q);
void double_to_stored(int storage, void* base, size_t idx, int q, double v);
}  // namespace jp

struct jp_solver {
    jp_config cfg{};
    jp_info info{};
    int kind = 0;
    int device = 0;
    int storage = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;  // device allocations come from here when set (see dev_alloc)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_wait = nullptr;  // wait_stream of a served solver
    int64_t step_count = 0;
    bool initialized = false;  // false between jp_create with JP_FLAG_DEFER_INIT and jp_init_tgv

    // uniform cube (flat [q][z][y][x])
    int n = 0;
    long long cells = 0;
    size_t elem = 0;           // bytes per stored population
    void* fa = nullptr;        // state at the current time
    void* fb = nullptr;        // next state (null when in place)
    bool inplace = false;      // JP_FLAG_INPLACE: one array, AA steps (uniform_aa.cu)
    void* field = nullptr;     // macro field (float4 or double4 per cell), allocated on first use
    double* partials = nullptr;  // diagnostic block partials + error word (kDiagPartials)
    double* diag_dev = nullptr;  // 3 doubles (+ the error word's copy, uniform)
    double* diag_host = nullptr; // 4 doubles, pinned
    int vec = 0, tpb = 0;
    float* outbuf = nullptr;   // device Q / speed / velocity for output frames, allocated on first use
    // populations staged for the next step (jp_stage_populations): uploaded into `staging` on
    // copy_stream while the solver's stream works, swapped in as fa by the next step
    void* staging = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_staged = nullptr;        // the upload has landed
    cudaEvent_t ev_staging_free = nullptr;  // the work that used the buffer before it was swapped out is done
    bool staged = false;

    jp::AmrState* amr = nullptr;

    // layout of fa for launch_macro: 0 flat, 1 / 2 in place after an even / odd step count
    int aa_layout() const { return inplace ? 1 + int(step_count & 1) : 0; }
};

namespace jp {
// uniform (solver_uniform.cu)
jp_status uniform_create(jp_solver* s);
void uniform_free(jp_solver* s);
jp_status uniform_init(jp_solver* s);
jp_status uniform_step(jp_solver* s, int64_t nsteps);
// upload populations for the next step on the copy stream (jp_stage_populations)
jp_status uniform_stage_populations(jp_solver* s, int layout, int dtype, const void* host, int64_t count);
// take staged populations as the state (the next step's first action); no-op when none are staged
jp_status uniform_take_staged(jp_solver* s);
jp_status uniform_diag(jp_solver* s, double out[3]);
jp_status uniform_get_populations(jp_solver* s, int level, int layout, int dtype, void* host, int64_t count);
jp_status uniform_set_populations(jp_solver* s, int level, int layout, int dtype, const void* host, int64_t count);
jp_status uniform_get_macro(jp_solver* s, float* host, int64_t count);
jp_status uniform_get_output_fields(jp_solver* s, float* q, float* speed, float* vel, int64_t count);
jp_status output_fields_from(jp_solver* s, const void* field, bool field_is_double, bool float_diff, int n, float* q,
                             float* speed, float* vel);
jp_status common_setup(jp_solver* s);
// drop populations staged for the next step, after their copy has finished reading the host buffer
jp_status uniform_discard_staged(jp_solver* s);
// element of fa that holds population q of cell (x, y, z) at the current step count
size_t uniform_slot(const jp_solver* s, int q, int x, int y, int z);
// fa as stored <-> the flat [q][z][y][x] order of the two-array step (host copies; identity unless in place)
void uniform_raw_to_flat(const jp_solver* s, const unsigned char* raw, unsigned char* flat);
void uniform_flat_to_raw(const jp_solver* s, const unsigned char* flat, unsigned char* raw);

// AMR (solver_amr.cu)
jp_status amr_create(jp_solver* s);
void amr_destroy(jp_solver* s);
jp_status amr_init(jp_solver* s);
jp_status amr_step(jp_solver* s, int64_t nsteps);
jp_status amr_diag(jp_solver* s, double out[3]);
jp_status amr_population_count(const jp_solver* s, int level, int64_t* count);
jp_status amr_get_populations(jp_solver* s, int level, int layout, int dtype, void* host, int64_t count);
jp_status amr_set_populations(jp_solver* s, int level, int layout, int dtype, const void* host, int64_t count);
jp_status amr_regrid(jp_solver* s);
// the fine steps' mapping: vec 4 (rows) or 1 (a cell per thread, tpb threads per CTA); autotuner
jp_status amr_set_step_map(jp_solver* s, int vec, int tpb);
// a side stream (at the priority of the stream it branches from) and the two events of the level-0
// branch of a coarse step
struct AmrFork {
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t fork2 = nullptr, join2 = nullptr;  // the second branch: level-1 blocks outside the skin
    cudaError_t create(cudaStream_t like);
    void destroy();
};
// one coarse step of many AMR solvers, one launch per stage over all of them, on `st` (the level-0
// stages on fork->side when a fork is given)
jp_status amr_batch_step(const std::vector<jp_solver*>& members, cudaStream_t st, const AmrFork* fork = nullptr);
bool amr_batch_compatible(const jp_solver* a, const jp_solver* b);
// whether a solver's coarse step can run in the persistent launch (amr_persist_supported)
bool amr_persist_ok(const jp_solver* s);
// steps[i] coarse steps of members[i] (batch-compatible, amr_persist_ok) in persistent launches on
// `st`, up to kAmrBatchMax members per launch; launch c waits at its grid barriers on sync[c] (of
// nsync, zeroed by the caller once: the error fields stay set until the caller clears them), at most
// limit_ns per wait; grid = CTAs per launch (0: all that can be resident).  *launches (optional)
// counts the launches.
jp_status amr_persist_steps(const std::vector<jp_solver*>& members, const std::vector<long long>& steps,
                            cudaStream_t st, amr::PersistSync* sync, int nsync, long long limit_ns, int grid,
                            int* launches = nullptr);
jp_status amr_prepare_diag(jp_solver* s);
jp_status amr_graph_step_on(jp_solver* s, cudaStream_t st);
jp_status amr_save_state(jp_solver* s, std::FILE* f);
jp_status amr_load_state(jp_solver* s, std::FILE* f);
jp_status amr_diag_async(jp_solver* s, cudaStream_t st, double* host_out);
jp_status amr_get_counts(jp_solver* s, jp_amr_counts* out);
jp_status amr_get_table(jp_solver* s, int table, int32_t* host, int64_t capacity, int64_t* count);
jp_status amr_get_sensor(jp_solver* s, int level, float* host, int64_t capacity, int64_t* count);
jp_status amr_set_sensor_override(jp_solver* s, const float* sen0, const float* sen1_by_pos);
jp_status amr_get_output_fields(jp_solver* s, float* q, float* speed, float* vel, int64_t count);
}  // namespace jp
