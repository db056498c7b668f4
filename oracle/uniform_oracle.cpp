// ORACLE - test infrastructure only.  A CPU restatement of the reference's uniform D3Q19 path, used
// by the tests (as the checker), by __graft_entry__.smoke() and by bench.py's CPU baseline.  The
// engine never calls it.
//
// Restates src/tgv3d_uniform.cu of josepedro/jp-solver in plain C++ (OpenMP over blocks), in the
// reference's own layout: populations float[nblk][19][MB^3], block b = (bz*gx+by)*gx+bx, cell
// (k*MB+j)*MB+i.  Arithmetic follows the reference expression by expression and is compiled with
// -ffp-contract=off, so x86 and Arm hosts give identical bits.
//
// Pinned against the reference's own kernels run on a GB300 (tests/golden/make_golden.py, fixtures in
// tests/golden/uniform_*.npz, checked by tests/test_oracle_golden.py).
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
const double cwd[19] = {1.0 / 3,
                        1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                        1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                        1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};

// src/tgv3d_uniform.cu:35-38
template <class R> inline R feq_q(int q, R rho, R ux, R uy, R uz);
template <> inline float feq_q<float>(int q, float rho, float ux, float uy, float uz) {
    float cu = 3.f * (cvx[q] * ux + cvy[q] * uy + cvz[q] * uz);
    return cw[q] * rho * (1.f + cu + 0.5f * cu * cu - 1.5f * (ux * ux + uy * uy + uz * uz));
}
template <> inline double feq_q<double>(int q, double rho, double ux, double uy, double uz) {
    double cu = 3.0 * (cvx[q] * ux + cvy[q] * uy + cvz[q] * uz);
    return cwd[q] * rho * (1.0 + cu + 0.5 * cu * cu - 1.5 * (ux * ux + uy * uy + uz * uz));
}

// src/tgv3d_uniform.cu:40-61 (k_step): pull with a periodic modulo per population, BGK relax.
template <class R>
void step(const R* fa, R* fb, int N, int MB, R omega) {
    const int gx = N / MB, nb = gx * gx * gx, MB3 = MB * MB * MB;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        const int bx = b % gx, by = (b / gx) % gx, bz = b / (gx * gx);
        for (int cell = 0; cell < MB3; ++cell) {
            const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
            const int gi = bx * MB + i, gj = by * MB + j, gk = bz * MB + k;
            R fin[19];
            for (int q = 0; q < 19; ++q) {
                int sgi = (gi - cvx[q] + N) % N, sgj = (gj - cvy[q] + N) % N, sgk = (gk - cvz[q] + N) % N;
                int sbx = sgi / MB, sby = sgj / MB, sbz = sgk / MB;
                int nbk = (sbz * gx + sby) * gx + sbx;
                int sc = ((sgk - sbz * MB) * MB + (sgj - sby * MB)) * MB + (sgi - sbx * MB);
                fin[q] = fa[((size_t)nbk * 19 + q) * MB3 + sc];
            }
            R rho = 0, ux = 0, uy = 0, uz = 0;
            for (int q = 0; q < 19; ++q) {
                rho += fin[q];
                ux += cvx[q] * fin[q];
                uy += cvy[q] * fin[q];
                uz += cvz[q] * fin[q];
            }
            ux /= rho;
            uy /= rho;
            uz /= rho;
            for (int q = 0; q < 19; ++q)
                fb[((size_t)b * 19 + q) * MB3 + cell] = fin[q] - omega * (fin[q] - feq_q<R>(q, rho, ux, uy, uz));
        }
    }
}

// src/tgv3d_uniform.cu:63-77 (k_init_tgv3d).  The float variant rounds rho and u to float before the
// float equilibrium, as the reference does; the double variant stays in double.
template <class R>
void init_tgv(R* f, int N, int MB, double u0) {
    const int gx = N / MB, nb = gx * gx * gx, MB3 = MB * MB * MB;
    const double kf = 2.0 * M_PI / double(N);
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        const int bx = b % gx, by = (b / gx) % gx, bz = b / (gx * gx);
        for (int cell = 0; cell < MB3; ++cell) {
            const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
            double x = (bx * MB + i + 0.5) * kf, y = (by * MB + j + 0.5) * kf, z = (bz * MB + k + 0.5) * kf;
            double ux = u0 * sin(x) * cos(y) * cos(z);
            double uy = -u0 * cos(x) * sin(y) * cos(z);
            double uz = 0.0;
            double p = (u0 * u0 / 16.0) * (cos(2 * x) + cos(2 * y)) * (cos(2 * z) + 2.0);
            double rho = 1.0 + 3.0 * p;
            for (int q = 0; q < 19; ++q)
                f[((size_t)b * 19 + q) * MB3 + cell] = feq_q<R>(q, R(rho), R(ux), R(uy), R(uz));
        }
    }
}

// src/tgv3d_uniform.cu:79-90 (k_macro): (rho, ux, uy, uz) to a linear (gk*N+gj)*N+gi field.
template <class R>
void macro(const R* f, int N, int MB, R* out) {
    const int gx = N / MB, nb = gx * gx * gx, MB3 = MB * MB * MB;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nb; ++b) {
        const int bx = b % gx, by = (b / gx) % gx, bz = b / (gx * gx);
        for (int cell = 0; cell < MB3; ++cell) {
            const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
            const int gi = bx * MB + i, gj = by * MB + j, gk = bz * MB + k;
            R rho = 0, ux = 0, uy = 0, uz = 0;
            for (int q = 0; q < 19; ++q) {
                R v = f[((size_t)b * 19 + q) * MB3 + cell];
                rho += v;
                ux += cvx[q] * v;
                uy += cvy[q] * v;
                uz += cvz[q] * v;
            }
            size_t idx = (((size_t)gk * N) + gj) * N + gi;
            out[idx * 4 + 0] = rho;
            out[idx * 4 + 1] = ux / rho;
            out[idx * 4 + 2] = uy / rho;
            out[idx * 4 + 3] = uz / rho;
        }
    }
}

inline size_t idx3(int i, int j, int k, int N) { return ((size_t)k * N + j) * N + i; }

// src/tgv3d_uniform.cu:98-108 (grad_at): the difference of two field values is taken in the field's
// type, then widened and halved.
template <class R>
void grad_at(const R* F, int N, int i, int j, int k, double g[3][3]) {
    const int ip = (i + 1) % N, im = (i - 1 + N) % N, jp = (j + 1) % N, jm = (j - 1 + N) % N, kp = (k + 1) % N,
              km = (k - 1 + N) % N;
    for (int c = 0; c < 3; ++c) {
        double dxc = (F[idx3(ip, j, k, N) * 4 + 1 + c] - F[idx3(im, j, k, N) * 4 + 1 + c]) * 0.5;
        double dyc = (F[idx3(i, jp, k, N) * 4 + 1 + c] - F[idx3(i, jm, k, N) * 4 + 1 + c]) * 0.5;
        double dzc = (F[idx3(i, j, kp, N) * 4 + 1 + c] - F[idx3(i, j, km, N) * 4 + 1 + c]) * 0.5;
        g[c][0] = dxc;
        g[c][1] = dyc;
        g[c][2] = dzc;
    }
}

// src/tgv3d_uniform.cu:173-183: mean 1/2|u|^2, mean 1/2|omega|^2, mean rho, summed in the
// reference's loop order (k, j, i) in double.
template <class R>
void diag(const R* F, int N, double out[3]) {
    double E = 0, ens = 0, mass = 0;
    for (int k = 0; k < N; ++k)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                size_t p = idx3(i, j, k, N);
                mass += F[p * 4 + 0];
                double u = F[p * 4 + 1], v = F[p * 4 + 2], w = F[p * 4 + 3];
                E += 0.5 * (u * u + v * v + w * w);
                double g[3][3];
                grad_at<R>(F, N, i, j, k, g);
                double ox = g[2][1] - g[1][2], oy = g[0][2] - g[2][0], oz = g[1][0] - g[0][1];
                ens += 0.5 * (ox * ox + oy * oy + oz * oz);
            }
    double invn = 1.0 / (double(N) * N * N);
    out[0] = E * invn;
    out[1] = ens * invn;
    out[2] = mass * invn;
}

// src/tgv3d_uniform.cu:112-121 (write_vti): speed |u| and velocity from the field's float values
// widened to double; Q = -1/2 sum_ab g_ab g_ba of grad_at's gradient, in double, rounded to float.
void qspeed(const float* F, int N, float* Qo, float* spd, float* vel) {
#pragma omp parallel for schedule(static)
    for (int k = 0; k < N; ++k)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                size_t p = idx3(i, j, k, N);
                double u = F[p * 4 + 1], v = F[p * 4 + 2], w = F[p * 4 + 3];
                spd[p] = float(std::sqrt(u * u + v * v + w * w));
                if (vel) {
                    vel[p * 3 + 0] = float(u);
                    vel[p * 3 + 1] = float(v);
                    vel[p * 3 + 2] = float(w);
                }
                double g[3][3];
                grad_at<float>(F, N, i, j, k, g);
                double Qc = 0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) Qc -= 0.5 * g[a][b] * g[b][a];
                Qo[p] = float(Qc);
            }
}

}  // namespace

extern "C" {

int orc_version(void) { return 1; }

void orc_init_tgv_f32(float* f, int N, int MB, double u0) { init_tgv<float>(f, N, MB, u0); }
void orc_init_tgv_f64(double* f, int N, int MB, double u0) { init_tgv<double>(f, N, MB, u0); }
void orc_step_f32(const float* fa, float* fb, int N, int MB, float omega) { step<float>(fa, fb, N, MB, omega); }
void orc_step_f64(const double* fa, double* fb, int N, int MB, double omega) { step<double>(fa, fb, N, MB, omega); }
void orc_macro_f32(const float* f, int N, int MB, float* out) { macro<float>(f, N, MB, out); }
void orc_macro_f64(const double* f, int N, int MB, double* out) { macro<double>(f, N, MB, out); }
void orc_diag_f32(const float* F, int N, double out[3]) { diag<float>(F, N, out); }
void orc_diag_f64(const double* F, int N, double out[3]) { diag<double>(F, N, out); }
void orc_qspeed_f32(const float* F, int N, float* Q, float* speed, float* vel) { qspeed(F, N, Q, speed, vel); }

// nsteps FP32 steps in place (ping-pong through a scratch buffer of the same size); returns the
// buffer that holds the final state (0 = f, 1 = scratch).
int orc_run_f32(float* f, float* scratch, int N, int MB, float omega, long nsteps) {
    float* a = f;
    float* b = scratch;
    for (long s = 0; s < nsteps; ++s) {
        step<float>(a, b, N, MB, omega);
        float* t = a;
        a = b;
        b = t;
    }
    return a == f ? 0 : 1;
}

}  // extern "C"
