// State files: a solve written to disk and continued later, in the same process or another one.
//
// No counterpart in the reference (its runs start from the initial state every time).  A file holds
// a header (magic, ABI version, the configuration that fixes the state's shape and physics, the step
// count) and the kind's payload: for a uniform cube the stored populations in the flat [q][z][y][x]
// order of the two-array step (an in-place solver reorders on the host, so files move between the two); for an AMR solve its counts, block tables and the populations of the blocks in use
// (amr_save_state).  Loading into a solver created with the same kind, n, mb, storage, Re, u0 and
// refinement modes continues bit for bit where the saved solve was.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "jp.h"
#include "lattice.cuh"
#include "solver.h"

using namespace jp;

#define JP_CK(call, what)                                   \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
    } while (0)

namespace {

struct StateHeader {
    char magic[8];           // "JPSTATE\0"
    int32_t abi;             // JP_ABI_VERSION
    int32_t kind, n, mb, storage, l1_mode, l2_mode;
    int32_t pad;
    double re, u0;
    int64_t step_count;
    int64_t reserved[4];
};
const char kMagic[8] = {'J', 'P', 'S', 'T', 'A', 'T', 'E', 0};

struct File {
    std::FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

}  // namespace

extern "C" {

jp_status jp_save_state(jp_solver* s, const char* path) {
    if (!s || !path) return fail(JP_ERR_INVALID, "jp_save_state: null argument");
    JP_CK(cudaSetDevice(s->device), "cudaSetDevice");
    File file;
    file.f = std::fopen(path, "wb");
    if (!file.f) return fail(JP_ERR_INVALID, "cannot open %s for writing", path);
    StateHeader h;
    std::memset(&h, 0, sizeof h);
    std::memcpy(h.magic, kMagic, sizeof kMagic);
    h.abi = JP_ABI_VERSION;
    h.kind = s->cfg.kind;
    h.n = s->cfg.n;
    h.mb = s->cfg.mb;
    h.storage = s->cfg.storage;
    h.l1_mode = s->cfg.l1_mode;
    h.l2_mode = s->cfg.l2_mode;
    h.re = s->cfg.re;
    h.u0 = s->cfg.u0;
    h.step_count = s->step_count;
    if (std::fwrite(&h, sizeof h, 1, file.f) != 1) return fail(JP_ERR_INVALID, "write failed: %s", path);
    if (s->kind == JP_AMR) return amr_save_state(s, file.f);
    JP_CK(cudaStreamSynchronize(s->stream), "save");
    const size_t bytes = (size_t)Q * s->cells * s->elem;
    std::vector<unsigned char> raw(bytes);
    JP_CK(cudaMemcpy(raw.data(), s->fa, bytes, cudaMemcpyDeviceToHost), "populations D2H");
    if (s->inplace) {
        std::vector<unsigned char> flat(bytes);
        uniform_raw_to_flat(s, raw.data(), flat.data());
        raw.swap(flat);
    }
    if (std::fwrite(raw.data(), 1, bytes, file.f) != bytes) return fail(JP_ERR_INVALID, "write failed: %s", path);
    return JP_OK;
}

jp_status jp_load_state(jp_solver* s, const char* path) {
    if (!s || !path) return fail(JP_ERR_INVALID, "jp_load_state: null argument");
    JP_CK(cudaSetDevice(s->device), "cudaSetDevice");
    File file;
    file.f = std::fopen(path, "rb");
    if (!file.f) return fail(JP_ERR_INVALID, "cannot open %s", path);
    StateHeader h;
    if (std::fread(&h, sizeof h, 1, file.f) != 1 || std::memcmp(h.magic, kMagic, sizeof kMagic) != 0)
        return fail(JP_ERR_INVALID, "%s is not a state file", path);
    if (h.abi != JP_ABI_VERSION) return fail(JP_ERR_INVALID, "state file ABI %d, library %d", h.abi, JP_ABI_VERSION);
    const jp_config& c = s->cfg;
    if (h.kind != c.kind || h.n != c.n || h.mb != c.mb || h.storage != c.storage || h.re != c.re || h.u0 != c.u0 ||
        (c.kind == JP_AMR && (h.l1_mode != c.l1_mode || h.l2_mode != c.l2_mode)))
        return fail(JP_ERR_INVALID, "state file %s was written by a different configuration", path);
    if (s->kind == JP_AMR) {
        jp_status st = amr_load_state(s, file.f);
        if (st != JP_OK) return st;
    } else {
        const size_t bytes = (size_t)Q * s->cells * s->elem;
        std::vector<unsigned char> raw(bytes);
        if (std::fread(raw.data(), 1, bytes, file.f) != bytes) return fail(JP_ERR_INVALID, "state file truncated");
        if (s->inplace) {
            std::vector<unsigned char> st(bytes);
            s->step_count = h.step_count;  // the in-place layout follows the step count's parity
            uniform_flat_to_raw(s, raw.data(), st.data());
            raw.swap(st);
        }
        JP_CK(cudaStreamSynchronize(s->stream), "load");
        JP_CK(cudaMemcpy(s->fa, raw.data(), bytes, cudaMemcpyHostToDevice), "populations H2D");
        const jp_status ds = uniform_discard_staged(s);  // the loaded state replaces them
        if (ds != JP_OK) return ds;
    }
    s->step_count = h.step_count;
    s->initialized = true;
    return JP_OK;
}

}  // extern "C"
