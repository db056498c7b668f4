// Uniform periodic solver: one cube in the flat layout, double-buffered, stepped by the batched
// stream-collide kernel (batch of one), with the device diagnostic reduction.
// Reference: main() of src/tgv3d_uniform.cu:142-203.
#include "jp.h"
#include "kernels.h"
#include "lattice.cuh"
#include "solver.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace jp {

#define JP_CK(call, what)                                   \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
    } while (0)

// nu, tau and the step count exactly as the reference derives them (src/tgv3d_uniform.cu:151-153,
// src/tgv3d_amr.cu:659-664).
jp_status common_setup(jp_solver* s) {
    const jp_config& c = s->cfg;
    s->kind = c.kind;
    s->device = c.device;
    s->storage = c.storage;
    int ndev = 0;
    JP_CK(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount");
    if (c.device < 0 || c.device >= ndev) return fail(JP_ERR_INVALID, "device %d out of range (%d devices)", c.device, ndev);
    JP_CK(cudaSetDevice(c.device), "cudaSetDevice");
    if (s->pool) {
        // a served solve: its own stream carries the short latency-bound work (creation, regrids,
        // read-backs) that the batched launches of the other solves must not hold up
        int lo = 0, hi = 0;
        JP_CK(cudaDeviceGetStreamPriorityRange(&lo, &hi), "cudaDeviceGetStreamPriorityRange");
        JP_CK(cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, hi), "cudaStreamCreate");
    } else {
        JP_CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    }
    JP_CK(cudaEventCreate(&s->ev0), "cudaEventCreate");
    JP_CK(cudaEventCreate(&s->ev1), "cudaEventCreate");
    jp_info& in = s->info;
    std::memset(&in, 0, sizeof in);
    in.kind = c.kind;
    in.n = c.n;
    in.mb = c.mb;
    in.storage = c.storage;
    in.cells = (int64_t)c.n * c.n * c.n;
    const double N = double(c.n);
    in.nu = c.u0 * N / (2.0 * M_PI * c.re);
    in.tau = 3.0 * in.nu + 0.5;
    in.omega = double(float(1.0 / in.tau));
    if (c.storage == JP_FP64) in.omega = 1.0 / in.tau;
    in.tau1 = 2.0 * in.tau - 0.5;
    in.tau2 = 2.0 * in.tau1 - 0.5;
    in.kf = 2.0 * M_PI / N;
    in.steps = (int64_t)(long)(c.tstar / (c.u0 * in.kf) + 0.5);
    return JP_OK;
}

static int pick_vec(int storage, int n, int want) {
    const int cand[4] = {8, 4, 2, 1};
    for (int v : cand) {
        if (want && v != want) continue;
        if (!vec_supported(storage, v)) continue;
        if (want == 0 && v > default_vec(storage)) continue;
        if (n % v) continue;
        if (((long long)n * n * n / v) % 32) continue;
        return v;
    }
    return 0;
}

jp_status uniform_create(jp_solver* s) {
    jp_status st = common_setup(s);
    if (st != JP_OK) return st;
    const jp_config& c = s->cfg;
    s->n = c.n;
    s->cells = (long long)c.n * c.n * c.n;
    s->elem = storage_bytes(c.storage);
    s->inplace = (c.flags & JP_FLAG_INPLACE) != 0;
    s->tpb = c.threads_per_block ? c.threads_per_block : 128;
    if (s->tpb != 64 && s->tpb != 128 && s->tpb != 256 && s->tpb != 512)
        return fail(JP_ERR_INVALID, "threads_per_block must be 64, 128, 256 or 512");
    if (s->inplace) {
        // the in-place steps run the storage's default vector width, whole x-rows per CUDA block
        s->vec = default_vec(c.storage);
        if ((c.vec && c.vec != s->vec) || c.n % s->vec)
            return fail(JP_ERR_INVALID, "in-place streaming needs vec=%d dividing n=%d", s->vec, c.n);
        if (!inplace_tpb(c.storage, s->vec, s->tpb, c.n))
            return fail(JP_ERR_INVALID, "in-place streaming: an x-row of n=%d does not fit one CUDA block", c.n);
    } else {
        s->vec = pick_vec(c.storage, c.n, c.vec);
        if (!s->vec) return fail(JP_ERR_INVALID, "no vector width fits n=%d (requested vec=%d)", c.n, c.vec);
    }
    const size_t bytes = (size_t)Q * s->cells * s->elem;
    s->info.bytes_state = (int64_t)((s->inplace ? 1 : 2) * bytes);
    JP_CK(dev_alloc(s, &s->fa, bytes), "cudaMalloc populations");
    if (!s->inplace) JP_CK(dev_alloc(s, &s->fb, bytes), "cudaMalloc populations");
    JP_CK(dev_alloc(s, (void**)&s->partials, sizeof(double) * kDiagPartials), "cudaMalloc partials");
    JP_CK(cudaMemsetAsync(diag_err_word(s->partials), 0, sizeof(int), s->stream), "clear diag error word");
    JP_CK(dev_alloc(s, (void**)&s->diag_dev, sizeof(double) * 4), "cudaMalloc diag");
    s->diag_host = (double*)pinned_slot_alloc();
    if (!s->diag_host) return fail(JP_ERR_NOMEM, "pinned host slot");
    if (s->cfg.flags & JP_FLAG_DEFER_INIT) return JP_OK;
    return uniform_init(s);
}

void uniform_free(jp_solver* s) {
    if (s->copy_stream) cudaStreamSynchronize(s->copy_stream);  // an upload in flight ends first
    dev_free(s, s->staging);
    if (s->ev_staged) cudaEventDestroy(s->ev_staged);
    if (s->ev_staging_free) cudaEventDestroy(s->ev_staging_free);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    s->staging = nullptr;
    s->ev_staged = s->ev_staging_free = nullptr;
    s->copy_stream = nullptr;
    s->staged = false;
    dev_free(s, s->fa);
    dev_free(s, s->fb);
    dev_free(s, s->field);
    dev_free(s, s->partials);
    dev_free(s, s->diag_dev);
    pinned_slot_free(s->diag_host);
    dev_free(s, s->outbuf);
    s->outbuf = nullptr;
    s->fa = s->fb = s->field = nullptr;
    s->partials = s->diag_dev = s->diag_host = nullptr;
}

// An explicit new state discards populations staged before it.  The staged copy may still be
// reading the caller's pinned buffer: wait for it, so the buffer is free once the call returns.
jp_status uniform_discard_staged(jp_solver* s) {
    if (!s->staged) return JP_OK;
    s->staged = false;
    JP_CK(cudaEventSynchronize(s->ev_staged), "staged copy");
    return JP_OK;
}

jp_status uniform_init(jp_solver* s) {
    {
        const jp_status ds = uniform_discard_staged(s);
        if (ds != JP_OK) return ds;
    }
    // the per-axis trigonometry table of the initial state lives in the diagnostic partials buffer
    // (3n <= 3 * kDiagBlocks doubles for n <= kDiagBlocks), which is free between diagnostics
    double* tab = s->partials;
    double* own = nullptr;
    if (s->n > kDiagBlocks) {
        JP_CK(dev_alloc(s, (void**)&own, sizeof(double) * 3 * s->n), "cudaMalloc init table");
        tab = own;
    }
    cudaError_t e = launch_init_tgv(s->storage, s->fa, s->n, s->cfg.u0, s->info.kf, tab, s->stream, s->inplace);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    dev_free(s, own);
    JP_CK(e, "init_tgv");
    JP_CK(cudaStreamSynchronize(s->stream), "init_tgv");
    s->step_count = 0;
    s->initialized = true;
    return JP_OK;
}

// The state for the next step, uploaded while the solver's stream still works on the current one.
// The copy runs on copy_stream into a second state buffer; the next step waits for it on the device
// and swaps the buffers, and the buffer swapped out takes the upload after that, once the work queued
// before the swap (which may still read or write it) is done.  An uploading call overlaps the
// previous call's steps: at N=512 FP32 the 10.2 GB upload (~49 ms at the box's ~210 GB/s) hides
// behind 81 steps (~240 ms).
jp_status uniform_stage_populations(jp_solver* s, int layout, int dtype, const void* host, int64_t count) {
    if (s->inplace) return fail(JP_ERR_UNSUPPORTED, "jp_stage_populations: not for in-place solvers");
    if (count != (int64_t)Q * s->cells) return fail(JP_ERR_INVALID, "count %lld != 19*n^3", (long long)count);
    const bool native = layout == JP_LAYOUT_FLAT &&
                        ((dtype == JP_F32 && s->storage == JP_FP32) || (dtype == JP_F64 && s->storage == JP_FP64));
    if (!native)
        return fail(JP_ERR_UNSUPPORTED, "jp_stage_populations: flat layout in the storage's own type (FP32 or FP64)");
    if (s->staged) return fail(JP_ERR_STATE, "jp_stage_populations: populations are already staged for the next step");
    const size_t bytes = (size_t)count * s->elem;
    if (!s->staging) {
        JP_CK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking), "copy stream");
        JP_CK(cudaEventCreateWithFlags(&s->ev_staged, cudaEventDisableTiming), "cudaEventCreate");
        JP_CK(cudaEventCreateWithFlags(&s->ev_staging_free, cudaEventDisableTiming), "cudaEventCreate");
        JP_CK(dev_alloc(s, &s->staging, bytes), "cudaMalloc staging populations");
        JP_CK(cudaEventRecord(s->ev_staging_free, s->stream), "cudaEventRecord");  // after a pooled allocation
        s->info.bytes_state += (int64_t)bytes;
    }
    JP_CK(cudaStreamWaitEvent(s->copy_stream, s->ev_staging_free, 0), "cudaStreamWaitEvent");
    JP_CK(cudaMemcpyAsync(s->staging, host, bytes, cudaMemcpyHostToDevice, s->copy_stream), "staged populations H2D");
    JP_CK(cudaEventRecord(s->ev_staged, s->copy_stream), "cudaEventRecord");
    s->staged = true;
    return JP_OK;
}

jp_status uniform_take_staged(jp_solver* s) {
    if (!s->staged) return JP_OK;
    JP_CK(cudaStreamWaitEvent(s->stream, s->ev_staged, 0), "cudaStreamWaitEvent");
    std::swap(s->fa, s->staging);
    JP_CK(cudaEventRecord(s->ev_staging_free, s->stream), "cudaEventRecord");
    s->staged = false;
    return JP_OK;
}

jp_status uniform_step(jp_solver* s, int64_t nsteps) {
    const jp_status taken = uniform_take_staged(s);
    if (taken != JP_OK) return taken;
    UniSolve u;
    std::memset(&u, 0, sizeof u);
    u.n = s->n;
    u.omega = float(s->info.omega);
    u.omega_d = s->info.omega;
    if (s->inplace) {
        u.src = u.dst = s->fa;
        for (int64_t i = 0; i < nsteps; ++i) {
            cudaError_t e = launch_stream_collide_inplace(s->storage, &u, 1, int(s->step_count & 1), s->vec, s->tpb,
                                                          s->stream);
            if (e != cudaSuccess) return cuda_fail(e, "in-place step launch");
            ++s->step_count;
        }
        return JP_OK;
    }
    for (int64_t i = 0; i < nsteps; ++i) {
        u.src = s->fa;
        u.dst = s->fb;
        cudaError_t e = launch_stream_collide(s->storage, &u, 1, s->vec, s->tpb, s->stream);
        if (e != cudaSuccess) return cuda_fail(e, "stream_collide launch");
        std::swap(s->fa, s->fb);
        ++s->step_count;
    }
    return JP_OK;
}

static jp_status ensure_field(jp_solver* s) {
    if (s->field) return JP_OK;
    const size_t fb = (s->storage == JP_FP64 ? sizeof(double) : sizeof(float)) * 4 * (size_t)s->cells;
    JP_CK(dev_alloc(s, &s->field, fb), "cudaMalloc macro field");
    return JP_OK;
}

jp_status uniform_diag(jp_solver* s, double out[3]) {
    const bool pop = diag_pop_ok(s->storage, s->n);
    if (pop) {  // float storages: straight from the populations; diag_dev[3] takes the error word
        JP_CK(launch_diag_pop(s->storage, s->aa_layout(), s->fa, s->n, s->partials, s->diag_dev, s->diag_dev + 3,
                              s->stream),
              "diag");
    } else {  // FP64 terms from an FP64 macro field (or a cube beyond 32-bit cell indices)
        const jp_status st = ensure_field(s);
        if (st != JP_OK) return st;
        const bool dbl = s->storage == JP_FP64;
        JP_CK(launch_macro(s->storage, s->fa, s->field, s->n, s->stream, s->aa_layout()), "macro");
        JP_CK(launch_diag_field(dbl, !dbl, s->field, s->n, s->partials, s->diag_dev, s->stream), "diag");
    }
    JP_CK(cudaMemcpyAsync(s->diag_host, s->diag_dev, (pop ? 4 : 3) * sizeof(double), cudaMemcpyDeviceToHost,
                          s->stream),
          "diag D2H");
    JP_CK(cudaStreamSynchronize(s->stream), "diag");
    if (pop && s->diag_host[3] != 0.0)
        return fail(JP_ERR_TIMEOUT, "diagnostic: a wait between the kernel's warps gave up (its sums are NaN)");
    out[0] = s->diag_host[0];
    out[1] = s->diag_host[1];
    out[2] = s->diag_host[2];
    return JP_OK;
}

// index of population q of cell (x,y,z) in the blocked layout [block][q][cell] of edge mb
static inline size_t blocked_index(int n, int mb, int q, int x, int y, int z) {
    const int gx = n / mb;
    const size_t b = ((size_t)(z / mb) * gx + (y / mb)) * gx + (x / mb);
    const size_t cell = ((size_t)(z % mb) * mb + (y % mb)) * mb + (x % mb);
    return (b * Q + q) * (size_t)mb * mb * mb + cell;
}

size_t uniform_slot(const jp_solver* s, int q, int x, int y, int z) {
    const int n = s->n;
    if (s->inplace) {
        if (s->step_count & 1) {
            q = opp(q);
        } else {
            x = (x + cx(q) + n) % n;
            y = (y + cy(q) + n) % n;
            z = (z + cz(q) + n) % n;
        }
    }
    return (size_t)q * s->cells + ((size_t)z * n + y) * n + x;
}

void uniform_raw_to_flat(const jp_solver* s, const unsigned char* raw, unsigned char* flat) {
    const size_t e = s->elem;
    const int n = s->n;
    if (!s->inplace) {
        std::memcpy(flat, raw, (size_t)Q * s->cells * e);
        return;
    }
    for (int q = 0; q < Q; ++q)
        for (int z = 0; z < n; ++z)
            for (int y = 0; y < n; ++y)
                for (int x = 0; x < n; ++x)
                    std::memcpy(flat + e * ((size_t)q * s->cells + ((size_t)z * n + y) * n + x),
                                raw + e * uniform_slot(s, q, x, y, z), e);
}

void uniform_flat_to_raw(const jp_solver* s, const unsigned char* flat, unsigned char* raw) {
    const size_t e = s->elem;
    const int n = s->n;
    if (!s->inplace) {
        std::memcpy(raw, flat, (size_t)Q * s->cells * e);
        return;
    }
    for (int q = 0; q < Q; ++q)
        for (int z = 0; z < n; ++z)
            for (int y = 0; y < n; ++y)
                for (int x = 0; x < n; ++x)
                    std::memcpy(raw + e * uniform_slot(s, q, x, y, z),
                                flat + e * ((size_t)q * s->cells + ((size_t)z * n + y) * n + x), e);
}

jp_status uniform_get_populations(jp_solver* s, int level, int layout, int dtype, void* host, int64_t count) {
    if (level != 0) return fail(JP_ERR_INVALID, "uniform solver has only level 0");
    if (count != (int64_t)Q * s->cells) return fail(JP_ERR_INVALID, "count %lld != 19*n^3", (long long)count);
    if (layout != JP_LAYOUT_FLAT && layout != JP_LAYOUT_BLOCKED) return fail(JP_ERR_INVALID, "bad layout %d", layout);
    const size_t bytes = (size_t)count * s->elem;
    const bool native = layout == JP_LAYOUT_FLAT && !s->inplace &&
                        ((dtype == JP_F32 && s->storage == JP_FP32) || (dtype == JP_F64 && s->storage == JP_FP64));
    if (native) {
        JP_CK(cudaMemcpyAsync(host, s->fa, bytes, cudaMemcpyDeviceToHost, s->stream), "populations D2H");
        JP_CK(cudaStreamSynchronize(s->stream), "populations D2H");
        return JP_OK;
    }
    std::vector<unsigned char> raw(bytes);
    JP_CK(cudaMemcpyAsync(raw.data(), s->fa, bytes, cudaMemcpyDeviceToHost, s->stream), "populations D2H");
    JP_CK(cudaStreamSynchronize(s->stream), "populations D2H");
    const int n = s->n, mb = s->cfg.mb;
    for (int q = 0; q < Q; ++q)
        for (int z = 0; z < n; ++z)
            for (int y = 0; y < n; ++y)
                for (int x = 0; x < n; ++x) {
                    const size_t src = uniform_slot(s, q, x, y, z);
                    const size_t dst = layout == JP_LAYOUT_FLAT ? (size_t)q * s->cells + ((size_t)z * n + y) * n + x
                                                                : blocked_index(n, mb, q, x, y, z);
                    const double v = stored_to_double(s->storage, raw.data(), src, q);
                    if (dtype == JP_F32) static_cast<float*>(host)[dst] = float(v);
                    else static_cast<double*>(host)[dst] = v;
                }
    return JP_OK;
}

jp_status uniform_set_populations(jp_solver* s, int level, int layout, int dtype, const void* host, int64_t count) {
    if (level != 0) return fail(JP_ERR_INVALID, "uniform solver has only level 0");
    if (count != (int64_t)Q * s->cells) return fail(JP_ERR_INVALID, "count %lld != 19*n^3", (long long)count);
    if (layout != JP_LAYOUT_FLAT && layout != JP_LAYOUT_BLOCKED) return fail(JP_ERR_INVALID, "bad layout %d", layout);
    const size_t bytes = (size_t)count * s->elem;
    {
        const jp_status ds = uniform_discard_staged(s);
        if (ds != JP_OK) return ds;
    }
    const bool native = layout == JP_LAYOUT_FLAT && !s->inplace &&
                        ((dtype == JP_F32 && s->storage == JP_FP32) || (dtype == JP_F64 && s->storage == JP_FP64));
    if (native) {
        // asynchronous from pinned memory; stream order puts it before the next step
        JP_CK(cudaMemcpyAsync(s->fa, host, bytes, cudaMemcpyHostToDevice, s->stream), "populations H2D");
        return JP_OK;
    }
    std::vector<unsigned char> raw(bytes);
    const int n = s->n, mb = s->cfg.mb;
    for (int q = 0; q < Q; ++q)
        for (int z = 0; z < n; ++z)
            for (int y = 0; y < n; ++y)
                for (int x = 0; x < n; ++x) {
                    const size_t dst = uniform_slot(s, q, x, y, z);
                    const size_t src = layout == JP_LAYOUT_FLAT ? (size_t)q * s->cells + ((size_t)z * n + y) * n + x
                                                                : blocked_index(n, mb, q, x, y, z);
                    const double v = dtype == JP_F32 ? double(static_cast<const float*>(host)[src])
                                                     : static_cast<const double*>(host)[src];
                    double_to_stored(s->storage, raw.data(), dst, q, v);
                }
    JP_CK(cudaMemcpyAsync(s->fa, raw.data(), bytes, cudaMemcpyHostToDevice, s->stream), "populations H2D");
    JP_CK(cudaStreamSynchronize(s->stream), "populations H2D");
    return JP_OK;
}

// Q / speed / velocity of a device macro field of edge n, copied to host arrays of n^3 (vel: 3 n^3).
jp_status output_fields_from(jp_solver* s, const void* field, bool field_is_double, bool float_diff, int n, float* q,
                             float* speed, float* vel) {
    const size_t cells = (size_t)n * n * n;
    if (!s->outbuf) JP_CK(dev_alloc(s, (void**)&s->outbuf, sizeof(float) * 5 * cells), "cudaMalloc output fields");
    float* dq = s->outbuf;
    float* ds = dq + cells;
    float* dv = ds + cells;
    JP_CK(launch_qspeed(field_is_double, float_diff, field, n, dq, ds, vel ? dv : nullptr, s->stream), "qspeed");
    if (q) JP_CK(cudaMemcpyAsync(q, dq, sizeof(float) * cells, cudaMemcpyDeviceToHost, s->stream), "Q D2H");
    if (speed) JP_CK(cudaMemcpyAsync(speed, ds, sizeof(float) * cells, cudaMemcpyDeviceToHost, s->stream), "speed D2H");
    if (vel) JP_CK(cudaMemcpyAsync(vel, dv, sizeof(float) * 3 * cells, cudaMemcpyDeviceToHost, s->stream), "vel D2H");
    JP_CK(cudaStreamSynchronize(s->stream), "output fields");
    return JP_OK;
}

jp_status uniform_get_output_fields(jp_solver* s, float* q, float* speed, float* vel, int64_t count) {
    if (count != (int64_t)s->cells) return fail(JP_ERR_INVALID, "count %lld != n^3", (long long)count);
    jp_status st = ensure_field(s);
    if (st != JP_OK) return st;
    JP_CK(launch_macro(s->storage, s->fa, s->field, s->n, s->stream, s->aa_layout()), "macro");
    const bool dbl = s->storage == JP_FP64;
    return output_fields_from(s, s->field, dbl, !dbl, s->n, q, speed, vel);
}

jp_status uniform_get_macro(jp_solver* s, float* host, int64_t count) {
    if (count != 4 * (int64_t)s->cells) return fail(JP_ERR_INVALID, "count %lld != 4*n^3", (long long)count);
    jp_status st = ensure_field(s);
    if (st != JP_OK) return st;
    JP_CK(launch_macro(s->storage, s->fa, s->field, s->n, s->stream, s->aa_layout()), "macro");
    if (s->storage == JP_FP64) {
        std::vector<double> tmp((size_t)count);
        JP_CK(cudaMemcpyAsync(tmp.data(), s->field, (size_t)count * 8, cudaMemcpyDeviceToHost, s->stream), "macro D2H");
        JP_CK(cudaStreamSynchronize(s->stream), "macro D2H");
        for (int64_t i = 0; i < count; ++i) host[i] = float(tmp[(size_t)i]);
        return JP_OK;
    }
    JP_CK(cudaMemcpyAsync(host, s->field, (size_t)count * 4, cudaMemcpyDeviceToHost, s->stream), "macro D2H");
    JP_CK(cudaStreamSynchronize(s->stream), "macro D2H");
    return JP_OK;
}

}  // namespace jp
