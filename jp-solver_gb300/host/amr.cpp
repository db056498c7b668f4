// `amr`: drop-in for the reference's three-level AMR Taylor-Green program (src/tgv3d_amr.cu:643-907),
// driving the GB300 engine through the C ABI.  Same flags and defaults (including --adapt, --maxgb,
// --graph, --skipprep, --skiprestr, --bench and --buffer, which the reference parses and this
// program implements: sensor marks dilated by that many block layers; 0 by default), same stdout lines,
// exit codes and .vti/.vtp frames.  Additions: --prec fp32|fp16|bf16 (population storage), --mb,
// --vec (fine steps: 4 = rows of four cells per thread, 1 = a cell per thread), --tpb (threads per
// CTA of the per-cell steps), --develop, --device, --autotune 1 (MB x step mapping), --diag-every.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cli_common.h"
#include "jp.h"

using namespace cli;

static std::vector<int> table(jp_solver* s, int id) {
    int64_t n = 0;
    jp_get_table(s, id, nullptr, 0, &n);
    std::vector<int> t((size_t)std::max<int64_t>(n, 1));
    ck(jp_get_table(s, id, t.data(), (int64_t)t.size(), &n), "table");
    t.resize((size_t)n);
    return t;
}

// level-1 and level-2 block boxes in 4*N0 coordinates (src/tgv3d_amr.cu:617-625)
static std::vector<Box> boxes(jp_solver* s, int cgx, int l1gx, int MB) {
    std::vector<Box> bs;
    const std::vector<int> pcb = table(s, JP_TABLE_L1PCB), oct = table(s, JP_TABLE_L1OCT);
    for (size_t b = 0; b < pcb.size(); ++b) {
        const int cb = pcb[b], o = oct[b], qx = o & 1, qy = (o >> 1) & 1, qz = o >> 2;
        const int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
        bs.push_back({double((cbx * 2 * MB + qx * MB) * 2), double((cby * 2 * MB + qy * MB) * 2),
                      double((cbz * 2 * MB + qz * MB) * 2), 2.0 * MB, 1});
    }
    const std::vector<int> pl1 = table(s, JP_TABLE_L2PL1), o2 = table(s, JP_TABLE_L2OCT), f1pos = table(s, JP_TABLE_F1POS);
    for (size_t b = 0; b < pl1.size(); ++b) {
        const int p = f1pos[pl1[b]], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
        const int o = o2[b], qx = o & 1, qy = (o >> 1) & 1, qz = o >> 2;
        bs.push_back({double(px * 2 * MB + qx * MB), double(py * 2 * MB + qy * MB), double(pz * 2 * MB + qz * MB),
                      double(MB), 2});
    }
    return bs;
}

int main(int argc, char** argv) {
    const int N = argi(argc, argv, "--n", 32);
    const double Re = argd(argc, argv, "--re", 800.0), u0 = argd(argc, argv, "--u0", 0.05);
    const double tstar = argd(argc, argv, "--tstar", 12.0);
    const double frac1 = argd(argc, argv, "--frac1", 0.35), frac2 = argd(argc, argv, "--frac2", 0.35);
    const int buffer = argi(argc, argv, "--buffer", 0);  // mark dilation in block layers (src/tgv3d_amr.cu:648)
    const char* l1mode = args(argc, argv, "--l1", "all");
    const char* l2mode = args(argc, argv, "--l2", "all");
    const char* vtk = args(argc, argv, "--vtk", nullptr);
    const int frames = argi(argc, argv, "--frames", 240);
    const bool bench = argd(argc, argv, "--bench", 0.0) > 0.5;
    const bool skipprep = argd(argc, argv, "--skipprep", 0.0) > 0.5;
    const bool skiprestr = argd(argc, argv, "--skiprestr", 0.0) > 0.5;
    const bool usegraph = argd(argc, argv, "--graph", 0.0) > 0.5;
    const int MBarg = argi(argc, argv, "--mb", 8);
    if (MBarg <= 0 || N % MBarg) {
        std::fprintf(stderr, "N%%MB\n");
        return 2;
    }
    const bool dynamic = !std::strcmp(l1mode, "sensor") || !std::strcmp(l2mode, "sensor");
    const int adaptEvery = argi(argc, argv, "--adapt", 100);
    jp_config cfg;
    jp_config_default(&cfg, JP_AMR);
    cfg.n = N;
    cfg.re = Re;
    cfg.u0 = u0;
    cfg.tstar = tstar;
    cfg.frac1 = frac1;
    cfg.frac2 = frac2;
    cfg.l1_mode = refine_of(l1mode);
    cfg.l2_mode = refine_of(l2mode);
    cfg.adapt_every = adaptEvery;
    cfg.max_gb = argd(argc, argv, "--maxgb", 0.0);
    cfg.mb = MBarg;
    cfg.develop_steps = argi(argc, argv, "--develop", 300);
    cfg.buffer = buffer;
    cfg.device = argi(argc, argv, "--device", 0);
    cfg.threads_per_block = argi(argc, argv, "--tpb", 0);
    cfg.vec = argi(argc, argv, "--vec", 0);
    cfg.storage = storage_of(args(argc, argv, "--prec", "fp32"));
    cfg.flags = (skipprep ? JP_FLAG_SKIP_PREP : 0) | (skiprestr ? JP_FLAG_SKIP_RESTRICT : 0) | (usegraph ? JP_FLAG_GRAPH : 0);
    if (argd(argc, argv, "--autotune", 0.0) > 0.5) {
        double best = 0.0;
        ck(jp_autotune(&cfg, 4, &best), "autotune");
        std::printf("[autotune] MB=%d vec=%d threads/block=%d  %.1f MLUPS(work)\n", cfg.mb, cfg.vec, cfg.threads_per_block,
                    best / 1e6);
    }
    const int MB = cfg.mb;  // the block edge in use (--mb, or the autotuner's pick)
    jp_solver* s = nullptr;
    ck(jp_create(&cfg, &s), "create");
    jp_info info;
    ck(jp_get_info(s, &info), "info");
    jp_amr_counts c;
    ck(jp_amr_get_counts(s, &c), "counts");
    const long steps = (long)info.steps;
    const int cgx = N / MB, l1gx = 2 * cgx, N1 = 2 * N, N2 = 4 * N;
    std::printf("[jp-solver amr] 3-level 3D. N0=%d N1=%d N2=%d Re=%g L1=%s(%d blk) L2=%s(%d blk) tau0=%.4f steps=%ld%s\n", N,
                N1, N2, Re, l1mode, c.nf1, l2mode, c.nf2, info.tau, steps, vtk ? " (vti+vtp)" : "");

    if (bench) {  // time the pure step loop, report MLUPS(work) and memory (src/tgv3d_amr.cu:839-864)
        for (int w = 0; w < 20; ++w) {
            if (dynamic && w % adaptEvery == 0) ck(jp_regrid(s), "regrid");
            ck(jp_step(s, 1), "step");
        }
        ck(jp_sync(s), "sync");
        int64_t freeA = 0, totA = 0;
        ck(jp_memory_info(s, &freeA, &totA), "memory");
        const long bsteps = std::min(steps, 600L);
        ck(jp_amr_get_counts(s, &c), "counts");
        const double MB3 = double(MB) * MB * MB;
        // work per coarse step from the counts before the timed loop, as the reference counts it (:843)
        double work = double(c.cnb0 + 2.0 * c.nf1 + 4.0 * c.nf2) * MB3;
        float ms = 0.f;
        if (usegraph) {
            ck(jp_step_timed(s, 2 * (bsteps / 2), &ms), "bench");
            work *= double(2 * (bsteps / 2));
        } else if (!dynamic) {
            ck(jp_step_timed(s, bsteps, &ms), "bench");
            work *= double(bsteps);
        } else {  // regrids inside the timed loop, timed on the wall clock like the reference's events
            const auto t0 = std::chrono::steady_clock::now();
            for (long s_ = 0; s_ < bsteps;) {
                if (s_ % adaptEvery == 0) ck(jp_regrid(s), "regrid");
                const long next = std::min(bsteps, (s_ / adaptEvery + 1) * adaptEvery);
                ck(jp_step(s, next - s_), "step");
                s_ = next;
            }
            ck(jp_sync(s), "sync");
            ms = float(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
            work *= double(bsteps);
        }
        const double poolGB = double(info.bytes_state) / 1073741824.0;
        std::printf("[bench%s] AMR N0=%d(fine %d): %.3f s  work=%.3e updates  %.1f MLUPS(work)  pools %.3f GB  ctx+pools %.3f GB  (L1=%d L2=%d)\n",
                    usegraph ? "+graph" : "", N, N2, ms / 1e3, work, work / (double(ms) * 1e3), poolGB,
                    double(totA - freeA) / 1073741824.0, c.nf1, c.nf2);
        jp_destroy(s);
        return 0;
    }

    std::vector<float> Qh, spdh, novel;
    int fi = 0;
    const long diagK = std::max(1L, (long)argi(argc, argv, "--diag-every", (int)std::max(1L, steps / 160)));
    const long frameK = vtk ? std::max(1L, steps / std::max(1, frames)) : 0;
    double E0 = -1, peak_ens = -1, peak_ts = -1, prevE = 1e30, mass0 = -1, mass_drift = 0;
    bool mono = true;
    const long sstep = usegraph ? 2 : 1;  // the reference's graph replays two steps at a time
    const size_t NN2 = size_t(N2) * N2 * N2;
    for (long s_ = 0; s_ <= steps; s_ += sstep) {
        if (dynamic && s_ > 0 && s_ % adaptEvery == 0) ck(jp_regrid(s), "regrid");
        if (s_ % diagK == 0) {
            double d[3];
            ck(jp_diag(s, d), "diag");
            const double E = d[0], ens = d[1], mass = d[2], ts = double(s_) * u0 * info.kf;
            if (mass0 < 0) mass0 = mass;
            mass_drift = std::max(mass_drift, std::fabs(mass - mass0) / mass0);
            if (E0 < 0) E0 = E;
            if (E > prevE * 1.0000001) mono = false;
            prevE = E;
            if (ens > peak_ens) {
                peak_ens = ens;
                peak_ts = ts;
            }
            std::printf("  t*=%.3f E/E0=%.5f enstrophy=%.6e mass_drift=%.2e\n", ts, E / E0, ens, mass_drift);
        }
        if (frameK && s_ % frameK == 0 && fi < frames) {
            Qh.resize(NN2);
            spdh.resize(NN2);
            ck(jp_get_output_fields(s, Qh.data(), spdh.data(), nullptr, (int64_t)NN2), "output fields");
            char nm[512];
            std::snprintf(nm, sizeof nm, "%s_%04d.vti", vtk, fi);
            write_vti(nm, Qh, spdh, novel, N2);
            std::snprintf(nm, sizeof nm, "%s_%04d.vtp", vtk, fi);
            write_boxes(nm, boxes(s, cgx, l1gx, MB));
            fi++;
        }
        if (s_ < steps) ck(jp_step(s, sstep), "step");
    }
    ck(jp_sync(s), "sync");
    ck(jp_amr_get_counts(s, &c), "counts");
    std::printf("  enstrophy peak at t*=%.3f (value %.6e)\n", peak_ts, peak_ens);
    std::printf("  energy monotonic: %s  mass drift %.2e\n", mono ? "yes" : "NO", mass_drift);
    std::printf("  pool high-water: L1 %ld/%d blocks (%.0f%%), L2 %ld/%d (%.0f%%)  [full-refine would be %d/%d]\n",
                (long)c.hw_nf1, c.cap1, 100.0 * c.hw_nf1 / c.cap1, (long)c.hw_nf2, c.cap2,
                c.cap2 ? 100.0 * c.hw_nf2 / c.cap2 : 0.0, c.ng1, c.ng1 * 8);
    const bool ok = std::isfinite(peak_ens) && peak_ts > 4.0 && peak_ts < 10.0 && mono && mass_drift < 5e-4;
    std::printf("  %s\n", ok ? "VALID (breakdown present, energy monotonic, mass held)" : "CHECK");
    if (vtk) std::printf("  wrote %d frames %s_0000.vti/.vtp ..\n", fi, vtk);
    jp_destroy(s);
    return ok ? 0 : 1;
}
