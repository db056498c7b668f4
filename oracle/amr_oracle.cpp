// ORACLE - test infrastructure only.  A CPU restatement of the reference's three-level block AMR
// (src/tgv3d_amr.cu of josepedro/jp-solver): the level kernels, the coarse-fine interface, the
// adaptation pipeline and the composite diagnostics, with the host orchestration of its main()
// (gpurce_init, gpurce_regrid, base_step).  Used by the tests as the checker; the engine never calls it.
//
// Layouts are the reference's: populations float[blk][19][MB^3], ghosts float[blk][19][(MB+2)^3],
// int32 tables with -1 = absent.  Thrust's sort / exclusive_scan / copy_if become std::sort and
// plain loops (the order statistic, the prefix sum and the ordered compaction are uniquely defined).
// Compiled with -ffp-contract=off: identical bits on x86 and Arm.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

const int cvx[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int cvy[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int cvz[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
const float cw[19] = {1.f / 3,
                      1.f / 18, 1.f / 18, 1.f / 18, 1.f / 18, 1.f / 18, 1.f / 18,
                      1.f / 36, 1.f / 36, 1.f / 36, 1.f / 36, 1.f / 36, 1.f / 36,
                      1.f / 36, 1.f / 36, 1.f / 36, 1.f / 36, 1.f / 36, 1.f / 36};
const int Q = 19;

// src/tgv3d_amr.cu:52-55
inline float feq_q(int q, float rho, float ux, float uy, float uz) {
    float cu = 3.f * (cvx[q] * ux + cvy[q] * uy + cvz[q] * uz);
    return cw[q] * rho * (1.f + cu + 0.5f * cu * cu - 1.5f * (ux * ux + uy * uy + uz * uz));
}
// src/tgv3d_amr.cu:56-67: project the non-equilibrium part onto its second-order moments.
inline void regularize(float* n) {
    float Pxx = 0, Pyy = 0, Pzz = 0, Pxy = 0, Pxz = 0, Pyz = 0;
    for (int q = 0; q < Q; ++q) {
        float v = n[q];
        Pxx += cvx[q] * cvx[q] * v;
        Pyy += cvy[q] * cvy[q] * v;
        Pzz += cvz[q] * cvz[q] * v;
        Pxy += cvx[q] * cvy[q] * v;
        Pxz += cvx[q] * cvz[q] * v;
        Pyz += cvy[q] * cvz[q] * v;
    }
    for (int q = 0; q < Q; ++q) {
        float Qxx = cvx[q] * cvx[q] - 1.f / 3.f, Qyy = cvy[q] * cvy[q] - 1.f / 3.f, Qzz = cvz[q] * cvz[q] - 1.f / 3.f;
        float Qxy = cvx[q] * cvy[q], Qxz = cvx[q] * cvz[q], Qyz = cvy[q] * cvz[q];
        n[q] = 4.5f * cw[q] * (Qxx * Pxx + Qyy * Pyy + Qzz * Pzz + 2.f * (Qxy * Pxy + Qxz * Pxz + Qyz * Pyz));
    }
}
inline void moments(const float* f, float& rho, float& ux, float& uy, float& uz) {
    rho = 0;
    ux = 0;
    uy = 0;
    uz = 0;
    for (int q = 0; q < Q; ++q) {
        rho += f[q];
        ux += cvx[q] * f[q];
        uy += cvy[q] * f[q];
        uz += cvz[q] * f[q];
    }
    ux /= rho;
    uy /= rho;
    uz /= rho;
}
inline int pmod(int a, int n) { return ((a % n) + n) % n; }

struct Amr {
    // geometry (src/tgv3d_amr.cu:37,658)
    int N, MB, MB3, EB, EB3, HALF, cgx, cnb0, l1gx, N1, N2, NG1;
    double re, u0, frac1, frac2;
    int l1mode, l2mode, develop;  // 0 all, 1 slab, 2 sensor
    bool dynamic;
    double tau0, tau1, tau2, nqs01, nqi10, nqs12, nqi21, kf;
    float om0, om1, om2;
    long steps;
    // pools (src/tgv3d_amr.cu:675-709)
    int cap_nref0, cap1, cap_nref1, cap2;
    long hw_nf1 = 0, hw_nf2 = 0;
    double budget;
    size_t PB;
    std::vector<float> c0a, c0b, f1a, f1b, gh1, prep0, prep1, f2a, f2b, gh2;
    std::vector<int> ref0, fof0, rl0, l1pcb, l1oct, f1pos, l1grid, ref1, fof1, rl1, l2pl1, l2oct, skin0, skin1;
    std::vector<int> o_ref0, o_fof0, o_l1grid, o_ref1, o_fof1, deep;
    std::vector<float> sen0, sen1;
    int nref0 = 0, nf1 = 0, nref1 = 0, nf2 = 0, n_skin0 = 0, n_skin1 = 0, ndeep = 0;
    bool ov = false;
    std::vector<float> ov_sen0, ov_sen1pos;
    int error = 0;  // 3 = pool capacity exceeded
    // off: the reference's behaviour (an overflow is an error here, an out-of-bounds write there);
    // on: the engine's pool growth (capacity at least doubled, budget permitting, payloads kept)
    bool grow = false;

    bool grow_l1(int needed) {
        int cap = ((std::max(needed, 2 * cap1) + 7) / 8) * 8;
        if (!pool_fits(cap, cap2)) return false;
        size_t blkn = (size_t)Q * MB3;
        f1a.resize(cap * blkn, 0.f);
        f1b.resize(cap * blkn, 0.f);
        prep1.resize(cap * blkn, 0.f);
        gh1.resize((size_t)cap * Q * EB3, 0.f);
        for (std::vector<int>* t : {&rl0, &l1pcb, &l1oct, &f1pos, &ref1, &rl1, &deep, &skin1}) t->resize(cap, 0);
        fof1.resize(cap, -1);
        sen1.resize(cap, 0.f);
        cap1 = cap;
        return true;
    }
    bool grow_l2(int needed) {
        int cap = ((std::max(needed, 2 * cap2) + 7) / 8) * 8;
        if (!pool_fits(cap1, cap)) return false;
        size_t blkn = (size_t)Q * MB3;
        f2a.resize(cap * blkn, 0.f);
        f2b.resize(cap * blkn, 0.f);
        gh2.resize((size_t)cap * Q * EB3, 0.f);
        l2pl1.resize(cap, 0);
        l2oct.resize(cap, 0);
        cap2 = cap;
        return true;
    }

    size_t blk(int b, int q) const { return ((size_t)b * Q + q) * MB3; }
    size_t gblk(int b, int q) const { return ((size_t)b * Q + q) * EB3; }

    // ---- level kernels --------------------------------------------------------------------------

    // k_init_tgv3d (src/tgv3d_amr.cu:431-440)
    void init_tgv(std::vector<float>& f) {
        for (int b = 0; b < cnb0; ++b) {
            int bx = b % cgx, by = (b / cgx) % cgx, bz = b / (cgx * cgx);
            for (int cell = 0; cell < MB3; ++cell) {
                int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
                double x = (bx * MB + i + 0.5) * kf, y = (by * MB + j + 0.5) * kf, z = (bz * MB + k + 0.5) * kf;
                double ux = u0 * sin(x) * cos(y) * cos(z), uy = -u0 * cos(x) * sin(y) * cos(z);
                double p = (u0 * u0 / 16.0) * (cos(2 * x) + cos(2 * y)) * (cos(2 * z) + 2.0), rho = 1.0 + 3.0 * p;
                for (int q = 0; q < Q; ++q) f[blk(b, q) + cell] = feq_q(q, float(rho), float(ux), float(uy), 0.f);
            }
        }
    }
    // k_step_L0 (src/tgv3d_amr.cu:203-220)
    void step_L0(const std::vector<float>& fa, std::vector<float>& fb) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < cnb0; ++b) {
            int bx = b % cgx, by = (b / cgx) % cgx, bz = b / (cgx * cgx);
            for (int cell = 0; cell < MB3; ++cell) {
                int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
                int gi = bx * MB + i, gj = by * MB + j, gk = bz * MB + k;
                float fin[Q];
                for (int q = 0; q < Q; ++q) {
                    int sgi = (gi - cvx[q] + N) % N, sgj = (gj - cvy[q] + N) % N, sgk = (gk - cvz[q] + N) % N;
                    int sbx = sgi / MB, sby = sgj / MB, sbz = sgk / MB, nbk = (sbz * cgx + sby) * cgx + sbx;
                    int sc = ((sgk - sbz * MB) * MB + (sgj - sby * MB)) * MB + (sgi - sbx * MB);
                    fin[q] = fa[blk(nbk, q) + sc];
                }
                collide(fin, om0, &fb[blk(b, 0)], cell);
            }
        }
    }
    void collide(float* fin, float om, float* out0, int cell) {
        float rho, ux, uy, uz;
        moments(fin, rho, ux, uy, uz);
        for (int q = 0; q < Q; ++q) out0[(size_t)q * MB3 + cell] = fin[q] - om * (fin[q] - feq_q(q, rho, ux, uy, uz));
    }
    // pr = feq + nqs*regularize(f - feq) of one cell
    void prep_cell(const float* f, float nqs, float* out) {
        float rho, ux, uy, uz;
        moments(f, rho, ux, uy, uz);
        float nq[Q];
        for (int q = 0; q < Q; ++q) nq[q] = f[q] - feq_q(q, rho, ux, uy, uz);
        regularize(nq);
        for (int q = 0; q < Q; ++q) out[q] = feq_q(q, rho, ux, uy, uz) + nqs * nq[q];
    }
    // k_prep_list (src/tgv3d_amr.cu:160-171)
    void prep_list(const std::vector<float>& fin, std::vector<float>& pr, const std::vector<int>& list, int nlist,
                   float nqs) {
#pragma omp parallel for schedule(static)
        for (int li = 0; li < nlist; ++li) {
            int b = list[li];
            for (int cell = 0; cell < MB3; ++cell) {
                float f[Q], o[Q];
                for (int q = 0; q < Q; ++q) f[q] = fin[blk(b, q) + cell];
                prep_cell(f, nqs, o);
                for (int q = 0; q < Q; ++q) pr[blk(b, q) + cell] = o[q];
            }
        }
    }
    // prolong_prep_L0 (src/tgv3d_amr.cu:122-132)
    void prolong_prep_L0(const std::vector<float>& pr, int cfi, int cfj, int cfk, float* out) {
        double xc = (double(cfi) + 0.5) / 2.0 - 0.5, yc = (double(cfj) + 0.5) / 2.0 - 0.5, zc = (double(cfk) + 0.5) / 2.0 - 0.5;
        int ib = int(floor(xc)), jb = int(floor(yc)), kb = int(floor(zc));
        float tx = float(xc - ib), ty = float(yc - jb), tz = float(zc - kb);
        for (int q = 0; q < Q; ++q) out[q] = 0;
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    float wgt = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
                    int ci = pmod(ib + di, N), cj = pmod(jb + dj, N), ck = pmod(kb + dk, N);
                    int cbx = ci / MB, cby = cj / MB, cbz = ck / MB, cb = (cbz * cgx + cby) * cgx + cbx;
                    int cc = ((ck - cbz * MB) * MB + (cj - cby * MB)) * MB + (ci - cbx * MB);
                    for (int q = 0; q < Q; ++q) out[q] += wgt * pr[blk(cb, q) + cc];
                }
    }
    // prolong_prep_L1 (src/tgv3d_amr.cu:133-144): corners outside L1 are dropped and the rest renormalised
    void prolong_prep_L1(const std::vector<float>& pr, int gfi, int gfj, int gfk, float* out) {
        double xc = (double(gfi) + 0.5) / 2.0 - 0.5, yc = (double(gfj) + 0.5) / 2.0 - 0.5, zc = (double(gfk) + 0.5) / 2.0 - 0.5;
        int ib = int(floor(xc)), jb = int(floor(yc)), kb = int(floor(zc));
        float tx = float(xc - ib), ty = float(yc - jb), tz = float(zc - kb), wsum = 0;
        for (int q = 0; q < Q; ++q) out[q] = 0;
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    float wgt = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
                    int ci = pmod(ib + di, N1), cj = pmod(jb + dj, N1), ck = pmod(kb + dk, N1);
                    int lbx = ci / MB, lby = cj / MB, lbz = ck / MB, lb = l1grid[(lbz * l1gx + lby) * l1gx + lbx];
                    if (lb < 0) continue;
                    int cc = ((ck - lbz * MB) * MB + (cj - lby * MB)) * MB + (ci - lbx * MB);
                    wsum += wgt;
                    for (int q = 0; q < Q; ++q) out[q] += wgt * pr[blk(lb, q) + cc];
                }
        if (wsum > 0.f && wsum < 0.999f) {
            float inv = 1.f / wsum;
            for (int q = 0; q < Q; ++q) out[q] *= inv;
        }
    }
    // prolong_L0 / prolong_L1 (src/tgv3d_amr.cu:70-118): the same trilinear, computing each corner's
    // regularised source on the fly (used by seed and migrate)
    void prolong_L0(const std::vector<float>& cf, int cfi, int cfj, int cfk, float nqs, float* out) {
        double xc = (double(cfi) + 0.5) / 2.0 - 0.5, yc = (double(cfj) + 0.5) / 2.0 - 0.5, zc = (double(cfk) + 0.5) / 2.0 - 0.5;
        int ib = int(floor(xc)), jb = int(floor(yc)), kb = int(floor(zc));
        float tx = float(xc - ib), ty = float(yc - jb), tz = float(zc - kb);
        for (int q = 0; q < Q; ++q) out[q] = 0;
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    float wgt = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
                    int ci = pmod(ib + di, N), cj = pmod(jb + dj, N), ck = pmod(kb + dk, N);
                    int cbx = ci / MB, cby = cj / MB, cbz = ck / MB, cb = (cbz * cgx + cby) * cgx + cbx;
                    int cc = ((ck - cbz * MB) * MB + (cj - cby * MB)) * MB + (ci - cbx * MB);
                    float fq[Q], p[Q];
                    for (int q = 0; q < Q; ++q) fq[q] = cf[blk(cb, q) + cc];
                    prep_cell(fq, nqs, p);
                    for (int q = 0; q < Q; ++q) out[q] += wgt * p[q];
                }
    }
    void prolong_L1(const std::vector<float>& f1, const std::vector<int>& grid, int gfi, int gfj, int gfk, float nqs,
                    float* out) {
        double xc = (double(gfi) + 0.5) / 2.0 - 0.5, yc = (double(gfj) + 0.5) / 2.0 - 0.5, zc = (double(gfk) + 0.5) / 2.0 - 0.5;
        int ib = int(floor(xc)), jb = int(floor(yc)), kb = int(floor(zc));
        float tx = float(xc - ib), ty = float(yc - jb), tz = float(zc - kb), wsum = 0;
        for (int q = 0; q < Q; ++q) out[q] = 0;
        for (int dk = 0; dk < 2; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    float wgt = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
                    int ci = pmod(ib + di, N1), cj = pmod(jb + dj, N1), ck = pmod(kb + dk, N1);
                    int lbx = ci / MB, lby = cj / MB, lbz = ck / MB, lb = grid[(lbz * l1gx + lby) * l1gx + lbx];
                    if (lb < 0) continue;
                    int cc = ((ck - lbz * MB) * MB + (cj - lby * MB)) * MB + (ci - lbx * MB);
                    float fq[Q], p[Q];
                    for (int q = 0; q < Q; ++q) fq[q] = f1[blk(lb, q) + cc];
                    prep_cell(fq, nqs, p);
                    wsum += wgt;
                    for (int q = 0; q < Q; ++q) out[q] += wgt * p[q];
                }
        if (wsum > 0.f && wsum < 0.999f) {
            float inv = 1.f / wsum;
            for (int q = 0; q < Q; ++q) out[q] *= inv;
        }
    }
    // k_fillcf_L1p (src/tgv3d_amr.cu:173-186)
    void fill_L1p() {
#pragma omp parallel for schedule(static)
        for (int fb = 0; fb < nf1; ++fb) {
            int cb = l1pcb[fb], oct = l1oct[fb], qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2;
            int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
            int ox = cbx * 2 * MB + qx * MB, oy = cby * 2 * MB + qy * MB, oz = cbz * 2 * MB + qz * MB;
            for (int s = 0; s < EB3; ++s) {
                int ei = s % EB, ej = (s / EB) % EB, ek = s / (EB * EB), i = ei - 1, j = ej - 1, k = ek - 1;
                if (i >= 0 && i < MB && j >= 0 && j < MB && k >= 0 && k < MB) continue;
                int gfi = pmod(ox + i, N1), gfj = pmod(oy + j, N1), gfk = pmod(oz + k, N1);
                int scb = ((gfk / (2 * MB)) * cgx + (gfj / (2 * MB))) * cgx + (gfi / (2 * MB));
                if (ref0[scb]) continue;
                float out[Q];
                prolong_prep_L0(prep0, gfi, gfj, gfk, out);
                for (int q = 0; q < Q; ++q) gh1[gblk(fb, q) + s] = out[q];
            }
        }
    }
    // k_fillcf_L2p (src/tgv3d_amr.cu:187-202)
    void fill_L2p() {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nf2; ++b) {
            int pl1 = l2pl1[b], oct = l2oct[b], qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2;
            int p = f1pos[pl1], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
            int ox = px * 2 * MB + qx * MB, oy = py * 2 * MB + qy * MB, oz = pz * 2 * MB + qz * MB;
            for (int s = 0; s < EB3; ++s) {
                int ei = s % EB, ej = (s / EB) % EB, ek = s / (EB * EB), i = ei - 1, j = ej - 1, k = ek - 1;
                if (i >= 0 && i < MB && j >= 0 && j < MB && k >= 0 && k < MB) continue;
                int g2i = pmod(ox + i, N2), g2j = pmod(oy + j, N2), g2k = pmod(oz + k, N2);
                int lbx = g2i / (2 * MB), lby = g2j / (2 * MB), lbz = g2k / (2 * MB), lb = l1grid[(lbz * l1gx + lby) * l1gx + lbx];
                if (lb >= 0 && ref1[lb]) continue;
                float out[Q];
                prolong_prep_L1(prep1, g2i, g2j, g2k, out);
                for (int q = 0; q < Q; ++q) gh2[gblk(b, q) + s] = out[q];
            }
        }
    }
    // k_step_L1 (src/tgv3d_amr.cu:241-274)
    void step_L1(const std::vector<float>& fa, std::vector<float>& fbuf) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nf1; ++b) {
            int cb = l1pcb[b], oct = l1oct[b], qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2;
            int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
            int sref[27], sfof[27];
            for (int c = 0; c < 27; ++c) {
                int dx = c % 3 - 1, dy = (c / 3) % 3 - 1, dz = c / 9 - 1;
                int nx = (cbx + dx + cgx) % cgx, ny = (cby + dy + cgx) % cgx, nz = (cbz + dz + cgx) % cgx,
                    ncb = (nz * cgx + ny) * cgx + nx;
                sref[c] = ref0[ncb];
                sfof[c] = fof0[ncb];
            }
            int ox = cbx * 2 * MB + qx * MB, oy = cby * 2 * MB + qy * MB, oz = cbz * 2 * MB + qz * MB;
            for (int cell = 0; cell < MB3; ++cell) {
                int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB), gfi = ox + i, gfj = oy + j, gfk = oz + k;
                float fin[Q];
                for (int q = 0; q < Q; ++q) {
                    int sfi = (gfi - cvx[q] + N1) % N1, sfj = (gfj - cvy[q] + N1) % N1, sfk = (gfk - cvz[q] + N1) % N1;
                    int scbx = sfi / (2 * MB), scby = sfj / (2 * MB), scbz = sfk / (2 * MB);
                    int ddx = scbx - cbx, ddy = scby - cby, ddz = scbz - cbz;
                    if (ddx > 1) ddx -= cgx; else if (ddx < -1) ddx += cgx;
                    if (ddy > 1) ddy -= cgx; else if (ddy < -1) ddy += cgx;
                    if (ddz > 1) ddz -= cgx; else if (ddz < -1) ddz += cgx;
                    int sidx = (ddz + 1) * 9 + (ddy + 1) * 3 + (ddx + 1);
                    if (sref[sidx]) {
                        int sqx = (sfi % (2 * MB)) / MB, sqy = (sfj % (2 * MB)) / MB, sqz = (sfk % (2 * MB)) / MB;
                        int sfb = sfof[sidx] + (sqz * 4 + sqy * 2 + sqx), sc = ((sfk % MB) * MB + (sfj % MB)) * MB + (sfi % MB);
                        fin[q] = fa[blk(sfb, q) + sc];
                    } else {
                        int ei = i - cvx[q] + 1, ej = j - cvy[q] + 1, ek = k - cvz[q] + 1;
                        fin[q] = gh1[gblk(b, q) + (ek * EB + ej) * EB + ei];
                    }
                }
                collide(fin, om1, &fbuf[blk(b, 0)], cell);
            }
        }
    }
    // k_step_L2 (src/tgv3d_amr.cu:331-356)
    void step_L2(const std::vector<float>& fa, std::vector<float>& fbuf) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nf2; ++b) {
            int pl1 = l2pl1[b], oct = l2oct[b], qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2;
            int p = f1pos[pl1], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
            int ox = px * 2 * MB + qx * MB, oy = py * 2 * MB + qy * MB, oz = pz * 2 * MB + qz * MB;
            for (int cell = 0; cell < MB3; ++cell) {
                int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB), g2i = ox + i, g2j = oy + j, g2k = oz + k;
                float fin[Q];
                for (int q = 0; q < Q; ++q) {
                    int sfi = (g2i - cvx[q] + N2) % N2, sfj = (g2j - cvy[q] + N2) % N2, sfk = (g2k - cvz[q] + N2) % N2;
                    int lbx = sfi / (2 * MB), lby = sfj / (2 * MB), lbz = sfk / (2 * MB), lb = l1grid[(lbz * l1gx + lby) * l1gx + lbx];
                    if (lb >= 0 && ref1[lb]) {
                        int sqx = (sfi % (2 * MB)) / MB, sqy = (sfj % (2 * MB)) / MB, sqz = (sfk % (2 * MB)) / MB;
                        int sfb = fof1[lb] + (sqz * 4 + sqy * 2 + sqx), sc = ((sfk % MB) * MB + (sfj % MB)) * MB + (sfi % MB);
                        fin[q] = fa[blk(sfb, q) + sc];
                    } else {
                        int ei = i - cvx[q] + 1, ej = j - cvy[q] + 1, ek = k - cvz[q] + 1;
                        fin[q] = gh2[gblk(b, q) + (ek * EB + ej) * EB + ei];
                    }
                }
                collide(fin, om2, &fbuf[blk(b, 0)], cell);
            }
        }
    }
    // k_restrict_L1 / k_restrict_L2 (src/tgv3d_amr.cu:275-298, 357-381): each covered coarse cell becomes
    // the regularised average of its 8 children, with the non-equilibrium part rescaled by nqi.
    void restrict_(std::vector<float>& cf, const std::vector<float>& ff, const std::vector<int>& rl,
                   const std::vector<int>& fof, int n_ref, float nqi) {
#pragma omp parallel for schedule(static)
        for (int r = 0; r < n_ref; ++r) {
            int cb = rl[r];
            for (int cell = 0; cell < MB3; ++cell) {
                int lci = cell % MB, lcj = (cell / MB) % MB, lck = cell / (MB * MB);
                int qx = lci / HALF, qy = lcj / HALF, qz = lck / HALF, oct = qz * 4 + qy * 2 + qx, fb = fof[cb] + oct;
                int fi0 = 2 * (lci % HALF), fj0 = 2 * (lcj % HALF), fk0 = 2 * (lck % HALF);
                float avg[Q];
                for (int q = 0; q < Q; ++q) avg[q] = 0;
                for (int dk = 0; dk < 2; ++dk)
                    for (int dj = 0; dj < 2; ++dj)
                        for (int di = 0; di < 2; ++di) {
                            int sc = ((fk0 + dk) * MB + (fj0 + dj)) * MB + (fi0 + di);
                            for (int q = 0; q < Q; ++q) avg[q] += 0.125f * ff[blk(fb, q) + sc];
                        }
                float rho, ux, uy, uz;
                moments(avg, rho, ux, uy, uz);
                float nq[Q];
                for (int q = 0; q < Q; ++q) nq[q] = avg[q] - feq_q(q, rho, ux, uy, uz);
                regularize(nq);
                int cc = (lck * MB + lcj) * MB + lci;
                for (int q = 0; q < Q; ++q) cf[blk(cb, q) + cc] = feq_q(q, rho, ux, uy, uz) + nqi * nq[q];
            }
        }
    }
    // k_seed_L1 (src/tgv3d_amr.cu:299-308)
    void seed_L1() {
#pragma omp parallel for schedule(static)
        for (int fb = 0; fb < nf1; ++fb) {
            int cb = l1pcb[fb], oct = l1oct[fb], qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2;
            int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
            for (int cell = 0; cell < MB3; ++cell) {
                int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
                float out[Q];
                prolong_L0(c0a, cbx * 2 * MB + qx * MB + i, cby * 2 * MB + qy * MB + j, cbz * 2 * MB + qz * MB + k,
                           float(nqs01), out);
                for (int q = 0; q < Q; ++q) f1a[blk(fb, q) + cell] = out[q];
            }
        }
    }
    // k_seed_L2 (src/tgv3d_amr.cu:382-393)
    void seed_L2() {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nf2; ++b) {
            int pl1 = l2pl1[b], oct = l2oct[b], qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2;
            int p = f1pos[pl1], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
            for (int cell = 0; cell < MB3; ++cell) {
                int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
                float out[Q];
                prolong_L1(f1a, l1grid, px * 2 * MB + qx * MB + i, py * 2 * MB + qy * MB + j, pz * 2 * MB + qz * MB + k,
                           float(nqs12), out);
                for (int q = 0; q < Q; ++q) f2a[blk(b, q) + cell] = out[q];
            }
        }
    }
    // k_migrate_L1 (src/tgv3d_amr.cu:397-411): old f1a -> new f1b, then swap
    void migrate_L1() {
#pragma omp parallel for schedule(static)
        for (int nfb = 0; nfb < nf1; ++nfb) {
            int cb = l1pcb[nfb], oct = l1oct[nfb];
            for (int cell = 0; cell < MB3; ++cell) {
                if (o_ref0[cb]) {
                    int ofb = o_fof0[cb] + oct;
                    for (int q = 0; q < Q; ++q) f1b[blk(nfb, q) + cell] = f1a[blk(ofb, q) + cell];
                } else {
                    int qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2, cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
                    int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
                    float out[Q];
                    prolong_L0(c0a, cbx * 2 * MB + qx * MB + i, cby * 2 * MB + qy * MB + j, cbz * 2 * MB + qz * MB + k,
                               float(nqs01), out);
                    for (int q = 0; q < Q; ++q) f1b[blk(nfb, q) + cell] = out[q];
                }
            }
        }
        std::swap(f1a, f1b);
    }
    // k_migrate_L2 (src/tgv3d_amr.cu:414-430): keyed by the L1 grid position
    void migrate_L2() {
#pragma omp parallel for schedule(static)
        for (int nfb = 0; nfb < nf2; ++nfb) {
            int pl1 = l2pl1[nfb], oct = l2oct[nfb], p = f1pos[pl1];
            int old_l1b = o_l1grid[p];
            for (int cell = 0; cell < MB3; ++cell) {
                if (old_l1b >= 0 && o_ref1[old_l1b]) {
                    int of2 = o_fof1[old_l1b] + oct;
                    for (int q = 0; q < Q; ++q) f2b[blk(nfb, q) + cell] = f2a[blk(of2, q) + cell];
                } else {
                    int px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx), qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2;
                    int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
                    float out[Q];
                    prolong_L1(f1a, l1grid, px * 2 * MB + qx * MB + i, py * 2 * MB + qy * MB + j, pz * 2 * MB + qz * MB + k,
                               float(nqs12), out);
                    for (int q = 0; q < Q; ++q) f2b[blk(nfb, q) + cell] = out[q];
                }
            }
        }
        std::swap(f2a, f2b);
    }
    // k_sensor (src/tgv3d_amr.cu:442-453): per block max over cells of |f - feq|_2 / rho
    void sensor(const std::vector<float>& ff, int nblk, std::vector<float>& d) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nblk; ++b) {
            float m = -INFINITY;
            for (int cell = 0; cell < MB3; ++cell) {
                float f[Q];
                for (int q = 0; q < Q; ++q) f[q] = ff[blk(b, q) + cell];
                float rho, ux, uy, uz;
                moments(f, rho, ux, uy, uz);
                float s = 0;
                for (int q = 0; q < Q; ++q) {
                    float d2 = f[q] - feq_q(q, rho, ux, uy, uz);
                    s += d2 * d2;
                }
                s = sqrtf(s) / rho;
                m = cell == 0 ? s : fmaxf(m, s);
            }
            d[b] = m;
        }
    }

    // ---- adaptation (src/tgv3d_amr.cu:455-513 and the Thrust calls of :722-815) ----------------

    bool is_deep(int b) {
        int p = f1pos[b], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
        const int nb6[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
        for (int d = 0; d < 6; ++d) {
            int nx = (px + nb6[d][0] + l1gx) % l1gx, ny = (py + nb6[d][1] + l1gx) % l1gx, nz = (pz + nb6[d][2] + l1gx) % l1gx;
            if (l1grid[(nz * l1gx + ny) * l1gx + nx] < 0) return false;
        }
        return true;
    }
    static float order_stat(std::vector<float> v, int n, int tgt) {
        std::sort(v.begin(), v.begin() + n);
        return v[n - tgt];
    }
    void compute_sen0() {
        if (ov) {
            for (int b = 0; b < cnb0; ++b) sen0[b] = ov_sen0[b];
        } else {
            sensor(c0a, cnb0, sen0);
        }
    }
    void compute_sen1() {
        if (ov) {
            for (int b = 0; b < nf1; ++b) sen1[b] = ov_sen1pos[f1pos[b]];
        } else {
            sensor(f1a, nf1, sen1);
        }
    }
    void mark_l0_sensor() {
        compute_sen0();
        int tgt0 = std::min(cap_nref0, std::max(1, (int)(frac1 * cnb0)));
        float thr = order_stat(sen0, cnb0, tgt0);
        for (int i = 0; i < cnb0; ++i) ref0[i] = (sen0[i] >= thr) ? 1 : 0;
    }
    // exclusive scan of ref0, then the L1 tables (k_scatter_L1)
    bool build_l1() {
        std::vector<int> rank(cnb0);
        int acc = 0;
        for (int i = 0; i < cnb0; ++i) {
            rank[i] = acc;
            acc += ref0[i];
        }
        nref0 = acc;
        nf1 = 8 * nref0;
        hw_nf1 = std::max(hw_nf1, (long)nf1);
        if (nf1 > cap1 && !(grow && grow_l1(nf1))) { error = 3; return false; }
        std::fill(l1grid.begin(), l1grid.end(), -1);
        std::fill(fof0.begin(), fof0.end(), -1);
        for (int cb = 0; cb < cnb0; ++cb) {
            if (!ref0[cb]) { fof0[cb] = -1; continue; }
            int r = rank[cb];
            fof0[cb] = 8 * r;
            rl0[r] = cb;
            int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
            for (int oct = 0; oct < 8; ++oct) {
                int qx = oct & 1, qy = (oct >> 1) & 1, qz = oct >> 2, fb = 8 * r + oct;
                int px = cbx * 2 + qx, py = cby * 2 + qy, pz = cbz * 2 + qz, pos = (pz * l1gx + py) * l1gx + px;
                l1pcb[fb] = cb;
                l1oct[fb] = oct;
                f1pos[fb] = pos;
                l1grid[pos] = fb;
            }
        }
        return true;
    }
    // deep mask, threshold over the deep sensors, mark (k_deepmask, copy_if, sort, k_mark_ref1)
    void mark_l1(bool all_mode, bool init) {
        compute_sen1();
        for (int b = 0; b < nf1; ++b) deep[b] = is_deep(b) ? 1 : 0;
        std::fill(ref1.begin(), ref1.end(), 0);
        if (all_mode) {
            for (int b = 0; b < nf1; ++b) ref1[b] = deep[b];
            ndeep = 0;
            for (int b = 0; b < nf1; ++b) ndeep += deep[b];
            return;
        }
        std::vector<float> ds;
        for (int b = 0; b < nf1; ++b)
            if (deep[b]) ds.push_back(sen1[b]);
        ndeep = (int)ds.size();
        if (ndeep > 0) {
            int tgt1 = init ? std::max(1, (int)(frac2 * ndeep)) : std::min(cap_nref1, std::max(1, (int)(frac2 * ndeep)));
            float thr = order_stat(ds, ndeep, tgt1);
            for (int b = 0; b < nf1; ++b) ref1[b] = (deep[b] && sen1[b] >= thr) ? 1 : 0;
        }
    }
    // exclusive scan of ref1 (counts only); k_scatter_L2 is scatter_l2()
    std::vector<int> rank1;
    void scan_l2() {
        rank1.assign(nf1, 0);
        int acc = 0;
        for (int i = 0; i < nf1; ++i) {
            rank1[i] = acc;
            acc += ref1[i];
        }
        nref1 = acc;
        nf2 = 8 * nref1;
        hw_nf2 = std::max(hw_nf2, (long)nf2);
    }
    void scatter_l2() {
        std::fill(fof1.begin(), fof1.end(), -1);
        for (int b = 0; b < nf1; ++b) {
            if (!ref1[b]) continue;
            int r = rank1[b];
            fof1[b] = 8 * r;
            rl1[r] = b;
            for (int oct = 0; oct < 8; ++oct) {
                l2pl1[8 * r + oct] = b;
                l2oct[8 * r + oct] = oct;
            }
        }
    }
    // k_dilate_L0 / k_dilate_L1 + copy_if over a counting iterator
    void skins() {
        n_skin0 = 0;
        for (int cb = 0; cb < cnb0; ++cb) {
            int bx = cb % cgx, by = (cb / cgx) % cgx, bz = cb / (cgx * cgx), f = 0;
            for (int dz = -1; dz <= 1 && !f; ++dz)
                for (int dy = -1; dy <= 1 && !f; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        int nx = (bx + dx + cgx) % cgx, ny = (by + dy + cgx) % cgx, nz = (bz + dz + cgx) % cgx;
                        if (ref0[(nz * cgx + ny) * cgx + nx]) { f = 1; break; }
                    }
            if (f) skin0[n_skin0++] = cb;
        }
        n_skin1 = 0;
        for (int b = 0; b < nf1; ++b) {
            int p = f1pos[b], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx), f = 0;
            for (int dz = -1; dz <= 1 && !f; ++dz)
                for (int dy = -1; dy <= 1 && !f; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        int nx = (px + dx + l1gx) % l1gx, ny = (py + dy + l1gx) % l1gx, nz = (pz + dz + l1gx) % l1gx,
                            nb = l1grid[(nz * l1gx + ny) * l1gx + nx];
                        if (nb >= 0 && ref1[nb]) { f = 1; break; }
                    }
            if (f) skin1[n_skin1++] = b;
        }
    }

    bool pool_fits(long c1, long c2) const { return (double)((size_t)(c1 + c2) * PB * 6 / 5) < budget; }

    // gpurce_init (src/tgv3d_amr.cu:776-815)
    void initial_build() {
        if (l1mode == 0) std::fill(ref0.begin(), ref0.end(), 1);
        else if (l1mode == 1) {
            for (int cb = 0; cb < cnb0; ++cb) ref0[cb] = (cb / (cgx * cgx) < cgx / 2) ? 1 : 0;
        } else {
            for (int s = 0; s < develop; ++s) {
                step_L0(c0a, c0b);
                std::swap(c0a, c0b);
            }
            mark_l0_sensor();
        }
        if (!build_l1()) return;
        if (nf1) {
            std::fill(gh1.begin(), gh1.begin() + (size_t)nf1 * Q * EB3, 0.f);
            seed_L1();
        }
        nref1 = 0;
        nf2 = 0;
        if (nf1) {
            mark_l1(l2mode == 0, true);
            scan_l2();
            cap_nref1 = std::max(1, (int)std::ceil(nref1 * 2.5));
            if (l2mode == 0) cap_nref1 = std::max(cap_nref1, nf1);
            cap_nref1 = std::min(cap_nref1, cap1);
            while (cap_nref1 > 1 && !pool_fits(cap1, 8L * cap_nref1)) cap_nref1--;
            cap2 = 8 * cap_nref1;
        } else {
            cap_nref1 = 1;
            cap2 = 8;
        }
        if (nf2 > cap2) { error = 3; return; }
        f2a.assign((size_t)cap2 * Q * MB3, 0.f);
        f2b.assign((size_t)cap2 * Q * MB3, 0.f);
        gh2.assign((size_t)cap2 * Q * EB3, 0.f);
        l2pl1.assign(cap2, 0);
        l2oct.assign(cap2, 0);
        scatter_l2();
        if (nf2) seed_L2();
        skins();
    }
    // gpurce_regrid (src/tgv3d_amr.cu:722-764)
    void regrid() {
        o_ref0 = ref0;
        o_fof0 = fof0;
        o_l1grid = l1grid;
        o_ref1 = ref1;
        o_fof1 = fof1;
        mark_l0_sensor();
        if (!build_l1()) return;
        if (nf1) migrate_L1();
        nref1 = 0;
        nf2 = 0;
        if (nf1) {
            mark_l1(false, false);
            scan_l2();
            if (nf2 > cap2 && !(grow && grow_l2(nf2))) { error = 3; return; }
            scatter_l2();
            if (nf2) migrate_L2();
        }
        skins();
    }
    // base_step (src/tgv3d_amr.cu:821-837)
    void base_step() {
        step_L0(c0a, c0b);
        std::swap(c0a, c0b);
        if (nf1) {
            prep_list(c0a, prep0, skin0, n_skin0, float(nqs01));
            fill_L1p();
            for (int s1 = 0; s1 < 2; ++s1) {
                if (nf2) {
                    prep_list(f1a, prep1, skin1, n_skin1, float(nqs12));
                    fill_L2p();
                    for (int s2 = 0; s2 < 2; ++s2) {
                        step_L2(f2a, f2b);
                        std::swap(f2a, f2b);
                    }
                    restrict_(f1a, f2a, rl1, fof1, nref1, float(nqi21));
                }
                step_L1(f1a, f1b);
                std::swap(f1a, f1b);
            }
            restrict_(c0a, f1a, rl0, fof0, nref0, float(nqi10));
        }
    }
    // cmacro + k_composite + k_diag_reduce (src/tgv3d_amr.cu:515-549), summed in cell order in double
    void diag(double out[3]) {
        long NN = (long)N2 * N2 * N2;
        std::vector<float> F((size_t)NN * 4);
#pragma omp parallel for schedule(static)
        for (long idx = 0; idx < NN; ++idx) {
            int gi = idx % N2, gj = (idx / N2) % N2, gk = idx / ((long)N2 * N2);
            int lbx = gi / (2 * MB), lby = gj / (2 * MB), lbz = gk / (2 * MB), lb = l1grid[(lbz * l1gx + lby) * l1gx + lbx];
            const float* src;
            size_t b;
            int sc;
            if (lb >= 0 && ref1[lb]) {
                int qx = (gi % (2 * MB)) / MB, qy = (gj % (2 * MB)) / MB, qz = (gk % (2 * MB)) / MB;
                b = fof1[lb] + (qz * 4 + qy * 2 + qx);
                sc = ((gk % MB) * MB + (gj % MB)) * MB + (gi % MB);
                src = f2a.data();
            } else if (lb >= 0) {
                int g1i = gi / 2, g1j = gj / 2, g1k = gk / 2;
                b = lb;
                sc = ((g1k % MB) * MB + (g1j % MB)) * MB + (g1i % MB);
                src = f1a.data();
            } else {
                int c0i = gi / 4, c0j = gj / 4, c0k = gk / 4, cbx = c0i / MB, cby = c0j / MB, cbz = c0k / MB;
                b = (cbz * cgx + cby) * cgx + cbx;
                sc = ((c0k % MB) * MB + (c0j % MB)) * MB + (c0i % MB);
                src = c0a.data();
            }
            float r = 0, x = 0, y = 0, z = 0;
            for (int q = 0; q < Q; ++q) {
                float v = src[(b * Q + q) * MB3 + sc];
                r += v;
                x += cvx[q] * v;
                y += cvy[q] * v;
                z += cvz[q] * v;
            }
            F[idx * 4 + 0] = r;
            F[idx * 4 + 1] = x / r;
            F[idx * 4 + 2] = y / r;
            F[idx * 4 + 3] = z / r;
        }
        int Nn = N2;
        double acc[3] = {0, 0, 0};
        for (long idx = 0; idx < NN; ++idx) {
            int i = idx % Nn, j = (idx / Nn) % Nn, k = idx / ((long)Nn * Nn);
            int ip = (i + 1) % Nn, im = (i - 1 + Nn) % Nn, jp = (j + 1) % Nn, jm = (j - 1 + Nn) % Nn, kp = (k + 1) % Nn,
                km = (k - 1 + Nn) % Nn;
            auto V = [&](int a, int b, int c, int comp) -> double { return F[(((long)c * Nn + b) * Nn + a) * 4 + 1 + comp]; };
            double u = F[idx * 4 + 1], v = F[idx * 4 + 2], w = F[idx * 4 + 3], rho = F[idx * 4 + 0];
            double dudy = (V(i, jp, k, 0) - V(i, jm, k, 0)) * 0.5, dudz = (V(i, j, kp, 0) - V(i, j, km, 0)) * 0.5;
            double dvdx = (V(ip, j, k, 1) - V(im, j, k, 1)) * 0.5, dvdz = (V(i, j, kp, 1) - V(i, j, km, 1)) * 0.5;
            double dwdx = (V(ip, j, k, 2) - V(im, j, k, 2)) * 0.5, dwdy = (V(i, jp, k, 2) - V(i, jm, k, 2)) * 0.5;
            double ox = dwdy - dvdz, oy = dudz - dwdx, oz = dvdx - dudy;
            acc[0] += 0.5 * (u * u + v * v + w * w);
            acc[1] += 0.5 * (ox * ox + oy * oy + oz * oz);
            acc[2] += rho;
        }
        double inv = 1.0 / double(NN);
        out[0] = acc[0] * inv;
        out[1] = acc[1] * inv;
        out[2] = acc[2] * inv;
    }
};

Amr* make(int N, int MB, double re, double u0, double tstar, int l1mode, int l2mode, double frac1, double frac2,
          int develop, double budget_bytes) {
    Amr* a = new Amr();
    a->N = N;
    a->MB = MB;
    a->MB3 = MB * MB * MB;
    a->EB = MB + 2;
    a->EB3 = a->EB * a->EB * a->EB;
    a->HALF = MB / 2;
    a->cgx = N / MB;
    a->cnb0 = a->cgx * a->cgx * a->cgx;
    a->l1gx = 2 * a->cgx;
    a->N1 = 2 * N;
    a->N2 = 4 * N;
    a->NG1 = a->l1gx * a->l1gx * a->l1gx;
    a->re = re;
    a->u0 = u0;
    a->frac1 = frac1;
    a->frac2 = frac2;
    a->l1mode = l1mode;
    a->l2mode = l2mode;
    a->develop = develop;
    a->dynamic = (l1mode == 2 || l2mode == 2);
    // src/tgv3d_amr.cu:659-664
    double nu = u0 * double(N) / (2.0 * M_PI * re);
    a->tau0 = 3.0 * nu + 0.5;
    a->tau1 = 2.0 * a->tau0 - 0.5;
    a->tau2 = 2.0 * a->tau1 - 0.5;
    a->om0 = float(1.0 / a->tau0);
    a->om1 = float(1.0 / a->tau1);
    a->om2 = float(1.0 / a->tau2);
    a->nqs01 = (a->tau1 - 1.0) / (2.0 * (a->tau0 - 1.0));
    a->nqi10 = (2.0 * (a->tau0 - 1.0)) / (a->tau1 - 1.0);
    a->nqs12 = (a->tau2 - 1.0) / (2.0 * (a->tau1 - 1.0));
    a->nqi21 = (2.0 * (a->tau1 - 1.0)) / (a->tau2 - 1.0);
    a->kf = 2.0 * M_PI / double(N);
    a->steps = long(tstar / (u0 * a->kf) + 0.5);
    // pool caps (src/tgv3d_amr.cu:675-691)
    a->budget = budget_bytes;
    a->PB = size_t(Q) * 4 * (2 * a->MB3 + a->EB3);
    a->cap_nref0 = (l1mode == 0) ? a->cnb0 : std::min(a->cnb0, std::max(1, (int)std::ceil(frac1 * a->cnb0 * 1.4)));
    while (a->cap_nref0 > 1 && !a->pool_fits(8L * a->cap_nref0, 0)) a->cap_nref0--;
    a->cap1 = 8 * a->cap_nref0;
    a->cap_nref1 = INT_MAX;
    a->cap2 = 0;
    size_t c0 = (size_t)a->cnb0 * Q * a->MB3, c1 = (size_t)a->cap1 * Q * a->MB3;
    a->c0a.assign(c0, 0.f);
    a->c0b.assign(c0, 0.f);
    a->prep0.assign(c0, 0.f);
    a->f1a.assign(c1, 0.f);
    a->f1b.assign(c1, 0.f);
    a->prep1.assign(c1, 0.f);
    a->gh1.assign((size_t)a->cap1 * Q * a->EB3, 0.f);
    a->ref0.assign(a->cnb0, 0);
    a->fof0.assign(a->cnb0, -1);
    a->rl0.assign(a->cap1, 0);
    a->l1pcb.assign(a->cap1, 0);
    a->l1oct.assign(a->cap1, 0);
    a->f1pos.assign(a->cap1, 0);
    a->l1grid.assign(a->NG1, -1);
    a->ref1.assign(a->cap1, 0);
    a->fof1.assign(a->cap1, -1);
    a->rl1.assign(a->cap1, 0);
    a->deep.assign(a->cap1, 0);
    a->skin0.assign(a->cnb0, 0);
    a->skin1.assign(a->cap1, 0);
    a->sen0.assign(a->cnb0, 0.f);
    a->sen1.assign(a->cap1, 0.f);
    a->init_tgv(a->c0a);
    return a;
}

}  // namespace

extern "C" {

void* orc_amr_create(int N, int MB, double re, double u0, double tstar, int l1mode, int l2mode, double frac1,
                     double frac2, int develop, double budget_bytes) {
    if (MB <= 0 || N % MB) return nullptr;
    return make(N, MB, re, u0, tstar, l1mode, l2mode, frac1, frac2, develop, budget_bytes);
}
void orc_amr_destroy(void* h) { delete static_cast<Amr*>(h); }

// sensor override: sen0 per coarse block (cnb0), sen1 per L1 grid position (l1gx^3); NULL clears
void orc_amr_set_sensor_override(void* h, const float* sen0, const float* sen1pos) {
    Amr* a = static_cast<Amr*>(h);
    if (!sen0 || !sen1pos) { a->ov = false; return; }
    a->ov = true;
    a->ov_sen0.assign(sen0, sen0 + a->cnb0);
    a->ov_sen1pos.assign(sen1pos, sen1pos + a->NG1);
}
void orc_amr_set_growth(void* h, int on) { static_cast<Amr*>(h)->grow = on != 0; }
int orc_amr_initial_build(void* h) {
    Amr* a = static_cast<Amr*>(h);
    a->initial_build();
    return a->error;
}
int orc_amr_regrid(void* h) {
    Amr* a = static_cast<Amr*>(h);
    a->regrid();
    return a->error;
}
int orc_amr_step(void* h, long n) {
    Amr* a = static_cast<Amr*>(h);
    for (long i = 0; i < n; ++i) a->base_step();
    return a->error;
}
void orc_amr_diag(void* h, double* out) { static_cast<Amr*>(h)->diag(out); }

// counts: nref0 nf1 nref1 nf2 n_skin0 n_skin1 cap1 cap2 cnb0 NG1 hw_nf1 hw_nf2 ndeep cap_nref0 cap_nref1 steps
void orc_amr_counts(void* h, long* out) {
    Amr* a = static_cast<Amr*>(h);
    long v[16] = {a->nref0, a->nf1, a->nref1, a->nf2, a->n_skin0, a->n_skin1, a->cap1, a->cap2, a->cnb0, a->NG1,
                  a->hw_nf1, a->hw_nf2, a->ndeep, a->cap_nref0, a->cap_nref1, a->steps};
    std::memcpy(out, v, sizeof v);
}

// table ids follow the engine's JP_TABLE_* numbering
int orc_amr_get_table(void* h, int id, int* out, long cap) {
    Amr* a = static_cast<Amr*>(h);
    const std::vector<int>* t = nullptr;
    long n = 0;
    switch (id) {
        case 0: t = &a->ref0; n = a->cnb0; break;
        case 1: t = &a->fof0; n = a->cnb0; break;
        case 2: t = &a->rl0; n = a->nref0; break;
        case 3: t = &a->l1pcb; n = a->nf1; break;
        case 4: t = &a->l1oct; n = a->nf1; break;
        case 5: t = &a->f1pos; n = a->nf1; break;
        case 6: t = &a->l1grid; n = a->NG1; break;
        case 7: t = &a->ref1; n = a->nf1; break;
        case 8: t = &a->fof1; n = a->nf1; break;
        case 9: t = &a->rl1; n = a->nref1; break;
        case 10: t = &a->l2pl1; n = a->nf2; break;
        case 11: t = &a->l2oct; n = a->nf2; break;
        case 12: t = &a->skin0; n = a->n_skin0; break;
        case 13: t = &a->skin1; n = a->n_skin1; break;
        case 14: t = &a->deep; n = a->nf1; break;
        default: return -1;
    }
    if (n > cap) return -2;
    std::memcpy(out, t->data(), sizeof(int) * n);
    return (int)n;
}
int orc_amr_get_sensor(void* h, int level, float* out, long cap) {
    Amr* a = static_cast<Amr*>(h);
    long n = level == 0 ? a->cnb0 : a->nf1;
    if (n > cap) return -2;
    std::memcpy(out, level == 0 ? a->sen0.data() : a->sen1.data(), sizeof(float) * n);
    return (int)n;
}
// populations of a level (active blocks only), reference blocked layout
long orc_amr_get_pops(void* h, int level, float* out, long cap) {
    Amr* a = static_cast<Amr*>(h);
    const std::vector<float>& f = level == 0 ? a->c0a : (level == 1 ? a->f1a : a->f2a);
    long nb = level == 0 ? a->cnb0 : (level == 1 ? a->nf1 : a->nf2);
    long n = nb * Q * a->MB3;
    if (n > cap) return -2;
    std::memcpy(out, f.data(), sizeof(float) * n);
    return n;
}
long orc_amr_set_pops(void* h, int level, const float* in, long count) {
    Amr* a = static_cast<Amr*>(h);
    std::vector<float>& f = level == 0 ? a->c0a : (level == 1 ? a->f1a : a->f2a);
    long nb = level == 0 ? a->cnb0 : (level == 1 ? a->nf1 : a->nf2);
    long n = nb * Q * a->MB3;
    if (count != n) return -2;
    std::memcpy(f.data(), in, sizeof(float) * n);
    return n;
}
void orc_amr_params(void* h, double* out) {
    Amr* a = static_cast<Amr*>(h);
    double v[12] = {a->tau0, a->tau1, a->tau2, a->om0, a->om1, a->om2, a->nqs01, a->nqi10, a->nqs12, a->nqi21, a->kf,
                    (double)a->steps};
    std::memcpy(out, v, sizeof v);
}

}  // extern "C"
