// `uniform`: drop-in for the reference's uniform Taylor-Green program (src/tgv3d_uniform.cu:142-203),
// driving the GB300 engine through the C ABI.  Same flags and defaults, same stdout lines, same exit
// codes (0 VALID, 1 CHECK, 2 error or N%MB), same .vti frames.  Additions on top: --prec
// fp32|fp16|bf16|fp64 storage, --mb, --tpb/--vec thread mapping, --diag-every, --bench 1 (time the
// step loop without diagnostics), --device, --inplace 1 (AA streaming in one population array).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "cli_common.h"
#include "jp.h"

using namespace cli;

int main(int argc, char** argv) {
    const int N = argi(argc, argv, "--n", 128);
    const double Re = argd(argc, argv, "--re", 1600.0), u0 = argd(argc, argv, "--u0", 0.05);
    const double tstar = argd(argc, argv, "--tstar", 12.0);
    const char* vtk = args(argc, argv, "--vtk", nullptr);
    const int frames = argi(argc, argv, "--frames", 160);
    const int MB = argi(argc, argv, "--mb", 8);
    const bool bench = argd(argc, argv, "--bench", 0.0) > 0.5;
    if (MB <= 0 || N % MB) {
        std::fprintf(stderr, "N%%MB\n");
        return 2;
    }
    jp_config cfg;
    jp_config_default(&cfg, JP_UNIFORM);
    cfg.n = N;
    cfg.re = Re;
    cfg.u0 = u0;
    cfg.tstar = tstar;
    cfg.mb = MB;
    cfg.storage = storage_of(args(argc, argv, "--prec", "fp32"));
    cfg.threads_per_block = argi(argc, argv, "--tpb", 0);
    cfg.vec = argi(argc, argv, "--vec", 0);
    cfg.device = argi(argc, argv, "--device", 0);
    if (argd(argc, argv, "--inplace", 0.0) > 0.5) cfg.flags |= JP_FLAG_INPLACE;
    if (argd(argc, argv, "--autotune", 0.0) > 0.5) {
        double best = 0.0;
        ck(jp_autotune(&cfg, 10, &best), "autotune");
        std::printf("[autotune] vec=%d threads/block=%d  %.1f MLUPS\n", cfg.vec, cfg.threads_per_block, best / 1e6);
    }
    jp_solver* s = nullptr;
    ck(jp_create(&cfg, &s), "create");
    jp_info info;
    ck(jp_get_info(s, &info), "info");
    const int gx = N / MB, nb = gx * gx * gx;
    const long steps = (long)info.steps;
    std::printf("[jp-solver uniform] TGV3D N=%d MB=%d blocks=%d Re=%g nu=%g tau=%.4f steps=%ld t*max=%.1f%s\n", N, MB,
                nb, Re, info.nu, info.tau, steps, tstar, vtk ? "  (writing vti)" : "");

    if (bench) {
        // step loop only, no diagnostics or output; GLUPS = N^3 * steps / device time
        const long bsteps = std::min(steps, 600L);
        ck(jp_step(s, 20), "warm-up");
        float ms = 0.f;
        ck(jp_step_timed(s, bsteps, &ms), "bench");
        const double cells = double(N) * N * N;
        const double bpu = cfg.storage == JP_FP64 ? 304.0 : (cfg.storage == JP_FP32 ? 152.0 : 76.0);
        std::printf("[bench] uniform N=%d: %.3f s  %ld steps  %.1f MLUPS  %.1f GB/s (%.0f B/update)  state %.2f GB%s\n",
                    N, ms / 1e3, bsteps, cells * bsteps / (ms * 1e3), cells * bsteps * bpu / (ms * 1e6), bpu,
                    double(info.bytes_state) / 1e9, (cfg.flags & JP_FLAG_INPLACE) ? " (in place)" : "");
        jp_destroy(s);
        return 0;
    }

    const long diagK = std::max(1L, (long)argi(argc, argv, "--diag-every", (int)std::max(1L, steps / 240)));
    const long frameK = vtk ? std::max(1L, steps / std::max(1, frames)) : 0;
    double E0 = -1, peak_ens = -1, peak_ts = -1, prevE = 1e30, mass0 = -1, mass_drift = 0;
    bool energy_mono = true;
    int fi = 0;
    std::vector<float> Qf, spd, vel;
    const size_t cells = size_t(N) * N * N;
    for (long s_ = 0; s_ <= steps;) {
        if (s_ % diagK == 0) {
            double d[3];
            ck(jp_diag(s, d), "diag");
            const double E = d[0], ens = d[1], mass = d[2];
            const double ts = double(s_) * u0 * info.kf;
            if (mass0 < 0) mass0 = mass;
            mass_drift = std::max(mass_drift, std::fabs(mass - mass0) / mass0);
            if (E0 < 0) E0 = E;
            if (E > prevE * 1.0000001) energy_mono = false;
            prevE = E;
            if (ens > peak_ens) {
                peak_ens = ens;
                peak_ts = ts;
            }
            std::printf("  t*=%.3f  E/E0=%.5f  enstrophy=%.6e  mass_drift=%.2e\n", ts, E / E0, ens, mass_drift);
        }
        if (frameK && s_ % frameK == 0 && fi < frames) {
            Qf.resize(cells);
            spd.resize(cells);
            vel.resize(3 * cells);
            ck(jp_get_output_fields(s, Qf.data(), spd.data(), vel.data(), (int64_t)cells), "output fields");
            char nm[512];
            std::snprintf(nm, sizeof nm, "%s_%04d.vti", vtk, fi++);
            write_vti(nm, Qf, spd, vel, N);
        }
        if (s_ >= steps) break;
        // advance to the next diagnostic or frame in one call
        long next = std::min(steps, (s_ / diagK + 1) * diagK);
        if (frameK) next = std::min(next, (s_ / frameK + 1) * frameK);
        ck(jp_step(s, next - s_), "step");
        s_ = next;
    }
    ck(jp_sync(s), "sync");
    std::printf("  enstrophy peak at t*=%.3f (value %.6e)\n", peak_ts, peak_ens);
    std::printf("  energy monotonic: %s   mass drift %.2e\n", energy_mono ? "yes" : "NO", mass_drift);
    const bool ok = std::isfinite(peak_ens) && peak_ts > 4.0 && peak_ts < 10.0 && energy_mono && mass_drift < 5e-4;
    std::printf("  %s\n", ok ? "VALID (enstrophy peaks then falls, energy monotonic, mass held in FP32)" : "CHECK (see values)");
    if (vtk) std::printf("  wrote %d vti frames %s_0000.vti ..\n", fi, vtk);
    jp_destroy(s);
    return ok ? 0 : 1;
}
