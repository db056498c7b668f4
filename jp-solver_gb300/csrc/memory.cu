// Device and pinned-host memory of the solvers, and how a served solver waits for its stream.
//
// A solver created by the server allocates from the server's stream-ordered pool on its own stream
// (cudaMallocFromPoolAsync / cudaFreeAsync): solves come and go while others run, and cudaFree would
// synchronise the whole device at every retirement.  Everything else uses cudaMalloc / cudaFree.
// The few bytes each solver reads back per diagnostic or adaptation live in pinned slots carved
// from slabs that stay for the life of the process (cudaFreeHost also synchronises the device).
#include <chrono>
#include <mutex>
#include <thread>
#include <vector>

#include "solver.h"

namespace jp {

cudaError_t dev_alloc(jp_solver* s, void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 1;
    if (s->pool) return cudaMallocFromPoolAsync(p, bytes, s->pool, s->stream);
    return cudaMalloc(p, bytes);
}

void dev_free(jp_solver* s, void* p) {
    if (!p) return;
    if (s->pool) {
        cudaFreeAsync(p, s->stream);
    } else {
        cudaFree(p);
    }
}

cudaError_t wait_stream(jp_solver* s) {
    if (!s->pool) return cudaStreamSynchronize(s->stream);
    if (!s->ev_wait) {
        cudaError_t e = cudaEventCreateWithFlags(&s->ev_wait, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaEventRecord(s->ev_wait, s->stream);
    if (e != cudaSuccess) return e;
    return wait_event(s->ev_wait);
}

// The server's threads (tick, lanes, workers) outnumber the host cores; a spinning
// cudaEventSynchronize in each would keep them all runnable.  This wait polls, yielding the core for
// the first 200 us and sleeping between polls after that.
cudaError_t wait_event(cudaEvent_t ev) {
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaEventQuery(ev);
        if (e != cudaErrorNotReady) return e;
        if (std::chrono::steady_clock::now() - t0 < std::chrono::microseconds(200)) {
            std::this_thread::yield();
        } else {
            std::this_thread::sleep_for(std::chrono::microseconds(40));
        }
    }
}

namespace {
constexpr size_t kSlot = 256;          // bytes per slot (the largest read-back is 40 bytes)
constexpr size_t kSlab = 256 * kSlot;  // 64 KiB per cudaHostAlloc
std::mutex g_slot_mutex;
std::vector<void*> g_free_slots;
}  // namespace

void* pinned_slot_alloc() {
    std::lock_guard<std::mutex> lock(g_slot_mutex);
    if (g_free_slots.empty()) {
        void* slab = nullptr;
        if (cudaHostAlloc(&slab, kSlab, cudaHostAllocPortable) != cudaSuccess) return nullptr;
        for (size_t k = kSlab / kSlot; k-- > 0;) g_free_slots.push_back((char*)slab + k * kSlot);
    }
    void* p = g_free_slots.back();
    g_free_slots.pop_back();
    return p;
}

void pinned_slot_free(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> lock(g_slot_mutex);
    g_free_slots.push_back(p);
}

}  // namespace jp
