// Autotuner: picks the uniform step's thread mapping or the AMR block edge by timing candidates on
// the device (an extension: the reference fixes MB and the mapping at compile time).
#include <cstring>
#include <vector>

#include "jp.h"
#include "kernels.h"
#include "solver.h"

using namespace jp;

extern "C" jp_status jp_autotune(jp_config* cfg, int32_t steps, double* best) {
    if (!cfg || !best) return fail(JP_ERR_INVALID, "jp_autotune: null argument");
    if (steps <= 0) return fail(JP_ERR_INVALID, "jp_autotune: steps must be positive");
    *best = 0.0;
    if (cfg->kind == JP_UNIFORM) {
        // one solver, the mapping switched between timings (same buffers, same state shape)
        jp_config c = *cfg;
        c.vec = 0;
        c.threads_per_block = 0;
        jp_solver* s = nullptr;
        jp_status st = jp_create(&c, &s);
        if (st != JP_OK) return st;
        const int vecs[4] = {1, 2, 4, 8};
        const int tpbs[4] = {64, 128, 256, 512};
        int bv = s->vec, bt = s->tpb;
        const double cells = double(s->cells);
        for (int v : vecs) {
            if (!vec_supported(s->storage, v) || s->n % v || ((long long)s->cells / v) % 32) continue;
            if (s->inplace && v != s->vec) continue;  // the in-place steps run the storage's default width
            for (int t : tpbs) {
                s->vec = v;
                s->tpb = t;
                float ms = 0.f;
                st = jp_step(s, 2);
                if (st == JP_OK) st = jp_step_timed(s, steps, &ms);
                if (st != JP_OK) {
                    jp_destroy(s);
                    return st;
                }
                const double lups = cells * steps / (double(ms) * 1e-3);
                if (lups > *best) {
                    *best = lups;
                    bv = v;
                    bt = t;
                }
            }
        }
        jp_destroy(s);
        cfg->vec = bv;
        cfg->threads_per_block = bt;
        return JP_OK;
    }
    // AMR: block edges that divide n x threads per CTA of the level steps; work-normalised
    // throughput of the 1:2:4 step on the grid each edge builds
    const int mbs[3] = {4, 8, 16};
    int bmb = cfg->mb, btpb = cfg->threads_per_block, bvec = cfg->vec;
    for (int mb : mbs) {
        if (cfg->n % mb) continue;
        jp_config c = *cfg;
        c.mb = mb;
        c.threads_per_block = 0;
        c.vec = 0;
        jp_solver* s = nullptr;
        jp_status st = jp_create(&c, &s);
        if (st == JP_ERR_NOMEM || st == JP_ERR_CAPACITY) continue;
        if (st != JP_OK) return st;
        jp_amr_counts k;
        st = jp_amr_get_counts(s, &k);
        const double work = (double(k.cnb0) + 2.0 * k.nf1 + 4.0 * k.nf2) * double(mb) * mb * mb * steps;
        // candidates: rows of four cells (vec 4, MB >= 8), then a cell per thread at each CTA size
        std::vector<std::pair<int, int>> maps;
        if (mb >= 8) maps.push_back({4, 0});
        for (int t : (mb == 4 ? std::vector<int>{64} : std::vector<int>{128, 256, 512})) maps.push_back({1, t});
        for (const auto& m : maps) {
            float ms = 0.f;
            if (st == JP_OK) st = amr_set_step_map(s, m.first, m.second);
            if (st == JP_OK) st = jp_step(s, 1);
            if (st == JP_OK) st = jp_step_timed(s, steps, &ms);
            if (st != JP_OK) break;
            const double lups = work / (double(ms) * 1e-3);
            if (lups > *best) {
                *best = lups;
                bmb = mb;
                btpb = m.second;
                bvec = m.first;
            }
        }
        jp_destroy(s);
        if (st != JP_OK) return st;
    }
    cfg->mb = bmb;
    cfg->threads_per_block = btpb;
    cfg->vec = bvec;
    return JP_OK;
}
