// C ABI of the engine (include/jp.h): solver lifecycle, stepping, diagnostics and population I/O.
// The reference's equivalents live inline in the two main() functions (src/tgv3d_uniform.cu:142-203,
// src/tgv3d_amr.cu:643-907); each entry point names the lines it replaces in include/jp.h.
#include "jp.h"
#include "kernels.h"
#include "lattice.cuh"
#include "solver.h"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace jp {

static thread_local std::string g_err;

jp_status fail(jp_status st, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return st;
}

jp_status cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(JP_ERR_NOMEM, "%s: %s", what, cudaGetErrorString(e));
    }
    return fail(JP_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

size_t storage_bytes(int storage) {
    switch (storage) {
        case JP_FP32: return 4;
        case JP_FP16: return 2;
        case JP_BF16: return 2;
        case JP_FP64: return 8;
    }
    return 0;
}

// host-side conversion of one stored element to double (unshifted)
double stored_to_double(int storage, const void* base, size_t idx, int q) {
    switch (storage) {
        case JP_FP32: return double(static_cast<const float*>(base)[idx]);
        case JP_FP64: return static_cast<const double*>(base)[idx];
        case JP_FP16: {
            __half_raw r;
            r.x = static_cast<const uint16_t*>(base)[idx];
            return double(wf(q)) + double(__half2float(__half(r)));
        }
        case JP_BF16: {
            __nv_bfloat16_raw r;
            r.x = static_cast<const uint16_t*>(base)[idx];
            return double(wf(q)) + double(__bfloat162float(__nv_bfloat16(r)));
        }
    }
    return 0.0;
}

void double_to_stored(int storage, void* base, size_t idx, int q, double v) {
    switch (storage) {
        case JP_FP32: static_cast<float*>(base)[idx] = float(v); break;
        case JP_FP64: static_cast<double*>(base)[idx] = v; break;
        case JP_FP16: {
            __half h = __float2half_rn(float(v - double(wf(q))));
            static_cast<uint16_t*>(base)[idx] = __half_raw(h).x;
            break;
        }
        case JP_BF16: {
            __nv_bfloat16 h = __float2bfloat16_rn(float(v - double(wf(q))));
            static_cast<uint16_t*>(base)[idx] = __nv_bfloat16_raw(h).x;
            break;
        }
    }
}

}  // namespace jp

using namespace jp;

// ------------------------------------------------------------------------------------------------

jp_status jp::create_solver(const jp_config* cfg, cudaMemPool_t pool, jp_solver** out) {
    if (!cfg || !out) return fail(JP_ERR_INVALID, "jp_create: null argument");
    *out = nullptr;
    if (cfg->kind != JP_UNIFORM && cfg->kind != JP_AMR) return fail(JP_ERR_INVALID, "unknown solver kind %d", cfg->kind);
    if (cfg->storage < 0 || cfg->storage > 3) return fail(JP_ERR_INVALID, "unknown storage %d", cfg->storage);
    if (cfg->mb != 4 && cfg->mb != 8 && cfg->mb != 16) return fail(JP_ERR_INVALID, "mb must be 4, 8 or 16 (got %d)", cfg->mb);
    if (cfg->n <= 0 || cfg->n % cfg->mb != 0) return fail(JP_ERR_INVALID, "N%%MB: n=%d is not a positive multiple of mb=%d", cfg->n, cfg->mb);
    if (!(cfg->re > 0.0) || !(cfg->u0 > 0.0) || !(cfg->tstar >= 0.0)) return fail(JP_ERR_INVALID, "re, u0 must be > 0 and tstar >= 0");
    jp_solver* s = new (std::nothrow) jp_solver();
    if (!s) return fail(JP_ERR_NOMEM, "host allocation");
    s->cfg = *cfg;
    s->pool = pool;
    jp_status st = (cfg->kind == JP_UNIFORM) ? uniform_create(s) : amr_create(s);
    if (st != JP_OK) {
        std::string keep = g_err;
        jp_destroy(s);
        g_err = keep;
        return st;
    }
    *out = s;
    return JP_OK;
}

extern "C" {

const char* jp_last_error(void) { return g_err.c_str(); }
int32_t jp_abi_version(void) { return JP_ABI_VERSION; }
const char* jp_build_info(void) {
    return "jp-solver GB300 engine: D3Q19 BGK, sm_103a, storages fp32/fp16s/bf16s/fp64";
}
int64_t jp_launch_count(void) { return launch_count(); }
size_t jp_sizeof(int32_t which) {
    switch (which) {
        case 0: return sizeof(jp_config);
        case 1: return sizeof(jp_info);
        case 2: return sizeof(jp_amr_counts);
        case 3: return sizeof(jp_server_config);
        case 4: return sizeof(jp_request);
        case 5: return sizeof(jp_result);
        case 6: return sizeof(jp_server_stats);
    }
    return 0;
}

void jp_config_default(jp_config* c, int32_t kind) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->kind = kind;
    c->u0 = 0.05;
    c->tstar = 12.0;
    c->storage = JP_FP32;
    c->mb = 8;
    c->device = 0;
    c->develop_steps = 300;
    c->adapt_every = 100;
    c->max_gb = 0.0;
    if (kind == JP_AMR) {
        c->n = 32;
        c->re = 800.0;
        c->frac1 = 0.35;
        c->frac2 = 0.35;
        c->l1_mode = JP_REFINE_ALL;
        c->l2_mode = JP_REFINE_ALL;
    } else {
        c->n = 128;
        c->re = 1600.0;
        c->frac1 = 0.35;
        c->frac2 = 0.35;
    }
}

jp_status jp_create(const jp_config* cfg, jp_solver** out) { return create_solver(cfg, nullptr, out); }


void jp_destroy(jp_solver* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    // pooled memory is freed in stream order behind the solver's last work; plain cudaFree waits
    if (s->stream && !s->pool) cudaStreamSynchronize(s->stream);
    if (s->kind == JP_AMR) amr_destroy(s);
    uniform_free(s);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->ev_wait) cudaEventDestroy(s->ev_wait);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

jp_status jp_get_info(const jp_solver* s, jp_info* out) {
    if (!s || !out) return fail(JP_ERR_INVALID, "jp_get_info: null argument");
    *out = s->info;
    out->step_count = s->step_count;
    return JP_OK;
}

jp_status jp_init_tgv(jp_solver* s) {
    if (!s) return fail(JP_ERR_INVALID, "null solver");
    cudaSetDevice(s->device);
    return s->kind == JP_UNIFORM ? uniform_init(s) : amr_init(s);
}

jp_status jp_step(jp_solver* s, int64_t nsteps) {
    if (!s) return fail(JP_ERR_INVALID, "null solver");
    if (nsteps < 0) return fail(JP_ERR_INVALID, "negative step count");
    if (!s->initialized) return fail(JP_ERR_STATE, "solver created with JP_FLAG_DEFER_INIT: call jp_init_tgv first");
    cudaSetDevice(s->device);
    return s->kind == JP_UNIFORM ? uniform_step(s, nsteps) : amr_step(s, nsteps);
}

jp_status jp_sync(jp_solver* s) {
    if (!s) return fail(JP_ERR_INVALID, "null solver");
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "jp_sync");
    return JP_OK;
}

jp_status jp_diag(jp_solver* s, double out[3]) {
    if (!s || !out) return fail(JP_ERR_INVALID, "jp_diag: null argument");
    if (!s->initialized) return fail(JP_ERR_STATE, "solver created with JP_FLAG_DEFER_INIT: call jp_init_tgv first");
    cudaSetDevice(s->device);
    return s->kind == JP_UNIFORM ? uniform_diag(s, out) : amr_diag(s, out);
}

jp_status jp_population_count(const jp_solver* s, int32_t level, int64_t* count) {
    if (!s || !count) return fail(JP_ERR_INVALID, "null argument");
    if (s->kind == JP_UNIFORM) {
        if (level != 0) return fail(JP_ERR_INVALID, "uniform solver has only level 0");
        *count = (int64_t)Q * s->cells;
        return JP_OK;
    }
    return amr_population_count(s, level, count);
}

jp_status jp_get_populations(jp_solver* s, int32_t level, int32_t layout, int32_t dtype, void* host, int64_t count) {
    if (!s || !host) return fail(JP_ERR_INVALID, "null argument");
    if (dtype != JP_F32 && dtype != JP_F64) return fail(JP_ERR_INVALID, "bad dtype %d", dtype);
    cudaSetDevice(s->device);
    if (s->kind == JP_UNIFORM) return uniform_get_populations(s, level, layout, dtype, host, count);
    return amr_get_populations(s, level, layout, dtype, host, count);
}

jp_status jp_set_populations(jp_solver* s, int32_t level, int32_t layout, int32_t dtype, const void* host, int64_t count) {
    if (!s || !host) return fail(JP_ERR_INVALID, "null argument");
    if (dtype != JP_F32 && dtype != JP_F64) return fail(JP_ERR_INVALID, "bad dtype %d", dtype);
    cudaSetDevice(s->device);
    if (s->kind == JP_UNIFORM) return uniform_set_populations(s, level, layout, dtype, host, count);
    return amr_set_populations(s, level, layout, dtype, host, count);
}

jp_status jp_stage_populations(jp_solver* s, int32_t layout, int32_t dtype, const void* host, int64_t count) {
    if (!s || !host) return fail(JP_ERR_INVALID, "null argument");
    if (s->kind != JP_UNIFORM) return fail(JP_ERR_UNSUPPORTED, "jp_stage_populations: uniform solvers only");
    cudaSetDevice(s->device);
    return uniform_stage_populations(s, layout, dtype, host, count);
}

jp_status jp_get_macro(jp_solver* s, float* host, int64_t count) {
    if (!s || !host) return fail(JP_ERR_INVALID, "null argument");
    if (s->kind != JP_UNIFORM) return fail(JP_ERR_UNSUPPORTED, "jp_get_macro: uniform solvers only");
    cudaSetDevice(s->device);
    return uniform_get_macro(s, host, count);
}

jp_status jp_get_output_fields(jp_solver* s, float* q, float* speed, float* velocity, int64_t count) {
    if (!s) return fail(JP_ERR_INVALID, "null solver");
    cudaSetDevice(s->device);
    return s->kind == JP_UNIFORM ? uniform_get_output_fields(s, q, speed, velocity, count)
                                 : amr_get_output_fields(s, q, speed, velocity, count);
}

jp_status jp_memory_info(jp_solver* s, int64_t* free_bytes, int64_t* total_bytes) {
    if (!s || !free_bytes || !total_bytes) return fail(JP_ERR_INVALID, "null argument");
    cudaSetDevice(s->device);
    size_t f = 0, t = 0;
    cudaError_t e = cudaMemGetInfo(&f, &t);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
    *free_bytes = (int64_t)f;
    *total_bytes = (int64_t)t;
    return JP_OK;
}

static jp_status need_amr(const jp_solver* s) {
    if (!s) return fail(JP_ERR_INVALID, "null solver");
    if (s->kind != JP_AMR) return fail(JP_ERR_INVALID, "not an AMR solver");
    return JP_OK;
}

jp_status jp_regrid(jp_solver* s) {
    jp_status st = need_amr(s);
    if (st != JP_OK) return st;
    if (!s->initialized) return fail(JP_ERR_STATE, "solver created with JP_FLAG_DEFER_INIT: call jp_init_tgv first");
    cudaSetDevice(s->device);
    return amr_regrid(s);
}

jp_status jp_amr_get_counts(jp_solver* s, jp_amr_counts* out) {
    jp_status st = need_amr(s);
    if (st != JP_OK) return st;
    if (!out) return fail(JP_ERR_INVALID, "null argument");
    return amr_get_counts(s, out);
}

jp_status jp_get_table(jp_solver* s, int32_t table, int32_t* host, int64_t capacity, int64_t* count) {
    jp_status st = need_amr(s);
    if (st != JP_OK) return st;
    if (!host && capacity > 0) return fail(JP_ERR_INVALID, "null buffer");
    cudaSetDevice(s->device);
    return amr_get_table(s, table, host, capacity, count);
}

jp_status jp_get_sensor(jp_solver* s, int32_t level, float* host, int64_t capacity, int64_t* count) {
    jp_status st = need_amr(s);
    if (st != JP_OK) return st;
    if (!host && capacity > 0) return fail(JP_ERR_INVALID, "null buffer");
    cudaSetDevice(s->device);
    return amr_get_sensor(s, level, host, capacity, count);
}

jp_status jp_set_sensor_override(jp_solver* s, const float* sen0, const float* sen1_by_pos) {
    jp_status st = need_amr(s);
    if (st != JP_OK) return st;
    cudaSetDevice(s->device);
    return amr_set_sensor_override(s, sen0, sen1_by_pos);
}

jp_status jp_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return fail(JP_ERR_INVALID, "null argument");
    cudaError_t e = cudaMallocHost(ptr, bytes);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return cuda_fail(e, "cudaMallocHost");
    }
    return JP_OK;
}
void jp_host_free(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
}

jp_status jp_step_timed(jp_solver* s, int64_t nsteps, float* ms) {
    if (!s || !ms) return fail(JP_ERR_INVALID, "null argument");
    cudaSetDevice(s->device);
    cudaError_t e = cudaEventRecord(s->ev0, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    jp_status st = jp_step(s, nsteps);
    if (st != JP_OK) return st;
    e = cudaEventRecord(s->ev1, s->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(s->ev1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, s->ev0, s->ev1);
    if (e != cudaSuccess) return cuda_fail(e, "jp_step_timed");
    return JP_OK;
}

}  // extern "C"
