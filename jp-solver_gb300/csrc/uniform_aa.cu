// In-place streaming of the uniform cube (the AA pattern): one population array instead of two.
//
// The reference double-buffers (src/tgv3d_uniform.cu:158 allocates fa and fb, :194 swaps them every
// step), as does the pull step of uniform.cu.  The AA pattern (P. Bailey, J. Myre, S. Walsh, D. Lilja,
// M. Saar, "Accelerating lattice Boltzmann fluid flow simulations using graphics processors",
// ICPP 2009) alternates two steps over one array A[q][z][y][x]:
//   local step  (taken when the step count is even): every cell reads its own 19 slots A[q][x] as its
//               collision inputs and writes relaxed population q to A[opp q][x];
//   stream step (step count odd): every cell x reads population q from A[opp q][x - c_q], relaxes,
//               and writes it to A[q][x + c_q].
// The slots a thread writes are exactly the slots it read, so no thread overwrites a value another
// thread still needs, in either step.  With P_t the populations of the two-array pull step after t
// steps (post-collision, as the pull step stores them) the array holds
//   t even: A[q][x + c_q] = P_t[q][x]   (every population already moved to where the next step reads it)
//   t odd:  A[opp q][x]   = P_t[q][x]
// so every collision sees the same inputs as in the pull step, and the CellBgk relaxation it shares
// with that step makes the two runs agree bit for bit.  HBM traffic per lattice update is unchanged
// (every population read once and written once): the gain is the footprint, 19 n^3 elements instead
// of 38 n^3 (N=512 FP32: 10.2 GB instead of 20.4 GB).
//
// Stream step mapping: a thread owns V consecutive cells of one x-row and, for each q, reads and
// writes whole aligned V-vectors; the value that crosses the vector edge along x comes from the
// thread of the neighbouring vector in the same row (a warp shuffle, or shared memory when that
// thread sits in another warp), once for the gathered inputs and once for the relaxed outputs.  A
// CUDA block therefore holds whole rows (periodic in x), so every exchange stays inside it.
#include "kernels.h"
#include "lattice.cuh"
#include "uniform_common.cuh"

namespace jp {

// index among the ten populations with c_x != 0, for the edge exchange buffers
__host__ __device__ constexpr int xslot(int q) {
    constexpr int t[Q] = {-1, 0, 1, -1, -1, -1, -1, 2, 3, 4, 5, 6, 7, 8, 9, -1, -1, -1, -1};
    return t[q];
}

// Occupancy floor of the in-place steps: one array means the compiler cannot sink a load past a store
// (they may alias), so all 19 row vectors stay live through the collision; 384 threads per SM still
// keep ~115 KB of loads in flight per SM (FP32), far above what HBM latency needs.
template <class ST, int V, int TPB>
constexpr int aa_min_blocks() {
    return (sizeof(typename ST::raw) * V >= 8 && sizeof(typename ST::raw) <= 4) ? (384 / TPB > 0 ? 384 / TPB : 1) : 1;
}

// The stream step in 16-bit storage moves half the bytes per access of FP32 (8-byte vectors), so it
// needs more warps in flight: 512 threads per SM (128 registers at 128 threads per CTA).
// With the relaxation on packed pairs of cells the 16-bit local step also runs best at 512 threads
// per SM (N=512 FP16 in place 77.6 -> 78.3 GLUPS; 384 threads for the stream step: 75.6).
template <class ST, int V, int TPB>
constexpr int aa_stream_min_blocks() {
    return sizeof(typename ST::raw) == 2 && V == 4 ? (512 / TPB > 0 ? 512 / TPB : 1) : aa_min_blocks<ST, V, TPB>();
}
template <class ST, int V, int TPB>
constexpr int aa_local_min_blocks() { return aa_stream_min_blocks<ST, V, TPB>(); }

__device__ __forceinline__ int solve_of(const UniBatch& b) {
    int si = 0;
#pragma unroll 1
    for (int i = 1; i < b.count; ++i) si = (b.s[i].blk_begin <= (long long)blockIdx.x) ? i : si;
    return si;
}

// Local step: each thread reads its V cells' 19 slots, relaxes, writes population q to slot opp(q).
template <class ST, int V, int TPB>
__global__ void __launch_bounds__(TPB, (aa_local_min_blocks<ST, V, TPB>())) k_aa_local(const __grid_constant__ UniBatch b) {
    using raw = typename ST::raw;
    using R = typename ST::real;
    constexpr bool SH = ST::shifted;
    constexpr bool SA = SH || sizeof(raw) == 4;
    const UniSolve& d = b.s[solve_of(b)];
    const long long seg = ((long long)blockIdx.x - d.blk_begin) * TPB + threadIdx.x;
    if (seg >= d.nseg) return;
    raw* __restrict__ A = static_cast<raw*>(d.dst);
    const size_t qs = (size_t)d.n * d.n * d.n;
    const size_t o = (size_t)seg * V;

    Pack<raw, V> L[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) L[q] = ld_pack_cg<raw, V>(A + q * qs + o);
    R f[V][Q];
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int v = 0; v < V; ++v) f[v][q] = (SA && !SH) ? ST::load(L[q].v[v]) - wgt<R>(q) : ST::load(L[q].v[v]);

    const R om = sizeof(R) == 8 ? R(d.omega_d) : R(d.omega);
    CellBgk<R, V, SA, SH> c(om);
    c.moments(f);
    {
        R o0[V];
#pragma unroll
        for (int v = 0; v < V; ++v) o0[v] = c.rest(f, v);
        Pack<raw, V> p;
        put_row<ST, V, SA>(p, o0, 0);
        st_pack<raw, V>(A + o, p);
    }
#pragma unroll
    for (int q = 1; q < Q; q += 2) {
        R oa[V], ob[V];
        c.pair(f, q, oa, ob);
        Pack<raw, V> pa, pb;
        put_row<ST, V, SA>(pa, oa, q);
        put_row<ST, V, SA>(pb, ob, q + 1);
        st_pack<raw, V>(A + (q + 1) * qs + o, pa);  // population q into slot opp(q) = q + 1
        st_pack<raw, V>(A + q * qs + o, pb);
    }
}

// Stream step: gather population q from A[opp q][x - c_q], relax, scatter to A[q][x + c_q].
template <class ST, int V, int TPB>
__global__ void __launch_bounds__(TPB, (aa_stream_min_blocks<ST, V, TPB>())) k_aa_stream(const __grid_constant__ UniBatch b) {
    using raw = typename ST::raw;
    using R = typename ST::real;
    constexpr bool SH = ST::shifted;
    constexpr bool SA = SH || sizeof(raw) == 4;
    __shared__ raw x_in[10][TPB];  // vector-edge values of the gathered rows, for a neighbour in another warp
    __shared__ R x_out[10][TPB];   // the same for the relaxed values

    const UniSolve& d = b.s[solve_of(b)];
    const int n = d.n;
    const int nr = d.nxs;      // threads per x-row (n / V)
    const int rpb = TPB / nr;  // whole rows per CUDA block (>= 1, checked at launch)
    const int t = threadIdx.x;
    const int lr = t / nr;
    const int X = t - lr * nr;
    const long long row = ((long long)blockIdx.x - d.blk_begin) * rpb + lr;
    const bool in_block = lr < rpb;
    const bool active = in_block && row < (long long)n * n;
    // the threads holding the neighbouring vectors of the row (periodic); spare threads pair with themselves
    const int tl = in_block ? t - X + (X == 0 ? nr - 1 : X - 1) : t;
    const int tr = in_block ? t - X + (X == nr - 1 ? 0 : X + 1) : t;
    const bool l_warp = (tl >> 5) == (t >> 5);
    const bool r_warp = (tr >> 5) == (t >> 5);
    const int y = active ? int(row % n) : 0;
    const int z = active ? int(row / n) : 0;
    const int x0 = X * V;
    raw* __restrict__ A = static_cast<raw*>(d.dst);
    const size_t qs = (size_t)n * n * n;
    // the nine x-rows around (y, z) (periodic), this thread's x range: offsets within a population
    // plane, 32-bit (n^3 < 2^32, checked at launch); row (dy, dz) at roff[(dz + 1) * 3 + dy + 1]
    unsigned roff[9];
    {
        const int ys[3] = {y == 0 ? n - 1 : y - 1, y, y == n - 1 ? 0 : y + 1};
        const int zs[3] = {z == 0 ? n - 1 : z - 1, z, z == n - 1 ? 0 : z + 1};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) roff[a * 3 + c] = ((unsigned)zs[a] * n + ys[c]) * n + x0;
    }

    // 1. gather: the vector of slot opp(q) in the row at (y, z) - c_(y,z), covering this thread's x range
    Pack<raw, V> L[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (active) L[q] = ld_pack_cg<raw, V>(A + opp(q) * qs + roff[(1 - cz(q)) * 3 + 1 - cy(q)]);
        else zero_pack(L[q]);
    }
    // 2. the value from across the vector edge: the left vector's last (c_x > 0) or the right one's first
    raw E[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        E[q] = raw(0);
        if (cx(q) > 0) {
            if (!r_warp) x_in[xslot(q)][t] = L[q].v[V - 1];
            E[q] = shfl_from(L[q].v[V - 1], tl & 31);
        } else if (cx(q) < 0) {
            if (!l_warp) x_in[xslot(q)][t] = L[q].v[0];
            E[q] = shfl_from(L[q].v[0], tr & 31);
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (cx(q) > 0 && !l_warp) E[q] = x_in[xslot(q)][tl];
        if (cx(q) < 0 && !r_warp) E[q] = x_in[xslot(q)][tr];
    }
    // 3. collision inputs of every cell in the collision type
    R f[V][Q];
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int v = 0; v < V; ++v) {
            raw e;
            if (cx(q) > 0) e = (v == 0) ? E[q] : L[q].v[v - 1];
            else if (cx(q) < 0) e = (v == V - 1) ? E[q] : L[q].v[v + 1];
            else e = L[q].v[v];
            f[v][q] = (SA && !SH) ? ST::load(e) - wgt<R>(q) : ST::load(e);
        }
    // 4. relax in place
    const R om = sizeof(R) == 8 ? R(d.omega_d) : R(d.omega);
    CellBgk<R, V, SA, SH> c(om);
    c.moments(f);
#pragma unroll
    for (int v = 0; v < V; ++v) f[v][0] = c.rest(f, v);
#pragma unroll
    for (int q = 1; q < Q; q += 2) {
        R oa[V], ob[V];
        c.pair(f, q, oa, ob);
#pragma unroll
        for (int v = 0; v < V; ++v) {
            f[v][q] = oa[v];
            f[v][q + 1] = ob[v];
        }
    }
    // 5. scatter: the vector of slot q in the row at (y, z) + c_(y,z) over this thread's x range takes
    //    population q of the cells at x - c_x: its own shifted by one, and one from the neighbour
    R G[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        G[q] = R(0);
        if (cx(q) > 0) {
            if (!r_warp) x_out[xslot(q)][t] = f[V - 1][q];
            G[q] = shfl_from(f[V - 1][q], tl & 31);
        } else if (cx(q) < 0) {
            if (!l_warp) x_out[xslot(q)][t] = f[0][q];
            G[q] = shfl_from(f[0][q], tr & 31);
        }
    }
    __syncthreads();
    if (!active) return;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (cx(q) > 0 && !l_warp) G[q] = x_out[xslot(q)][tl];
        if (cx(q) < 0 && !r_warp) G[q] = x_out[xslot(q)][tr];
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        R e[V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
            if (cx(q) > 0) e[v] = (v == 0) ? G[q] : f[v - 1][q];
            else if (cx(q) < 0) e[v] = (v == V - 1) ? G[q] : f[v + 1][q];
            else e[v] = f[v][q];
        }
        Pack<raw, V> p;
        put_row<ST, V, SA>(p, e, q);
        st_pack<raw, V>(A + q * qs + roff[(1 + cz(q)) * 3 + 1 + cy(q)], p);
    }
}

// shared memory of the stream step at TPB threads (static, so at most 48 KB)
template <class ST, int TPB>
constexpr size_t aa_smem() {
    return (size_t)10 * TPB * (sizeof(typename ST::raw) + sizeof(typename ST::real));
}

template <class ST, int V, int TPB>
static cudaError_t launch_aa(const UniSolve* solves, int count, int parity, cudaStream_t st) {
    UniBatch b;
    b.count = count;
    b.pad = 0;
    long long blocks = 0;
    for (int i = 0; i < count; ++i) {
        UniSolve& u = b.s[i];
        u = solves[i];
        const int n = u.n;
        u.nxs = n / V;
        u.blk_begin = blocks;
        if (parity == 0) {
            u.nseg = (long long)n * n * n / V;
            blocks += (u.nseg + TPB - 1) / TPB;
        } else {
            const int rpb = TPB / u.nxs;
            u.nseg = (long long)n * n;  // rows
            blocks += (u.nseg + rpb - 1) / rpb;
        }
    }
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    if (parity == 0) {
        k_aa_local<ST, V, TPB><<<(unsigned)blocks, TPB, 0, st>>>(b);
    } else {
        if constexpr (aa_smem<ST, TPB>() <= 48 * 1024) k_aa_stream<ST, V, TPB><<<(unsigned)blocks, TPB, 0, st>>>(b);
        else return cudaErrorInvalidConfiguration;
    }
    note_launch();
    return cudaGetLastError();
}

template <class ST, int V>
static cudaError_t launch_aa_tpb(int tpb, const UniSolve* s, int c, int parity, cudaStream_t st) {
    switch (tpb) {
        case 128: return launch_aa<ST, V, 128>(s, c, parity, st);
        case 256: return launch_aa<ST, V, 256>(s, c, parity, st);
        case 512: return launch_aa<ST, V, 512>(s, c, parity, st);
    }
    return cudaErrorInvalidValue;
}

// The smallest CTA of 128, 256 or 512 threads that holds an x-row: larger CTAs run fewer resident
// threads per SM (their occupancy floor allows more registers) and measured slower (N=512: 128
// threads FP16 72.7 GLUPS, 256 threads 51.5), so a larger request is not followed.
int inplace_tpb(int storage, int vec, int /*tpb*/, int max_n) {
    if (vec == 0) vec = default_vec(storage);
    if (vec <= 0 || max_n % vec) return 0;
    const int nr = max_n / vec;
    const int cap = storage == 3 ? 256 : 512;  // FP64: the exchange buffers of 512 threads exceed 48 KB
    for (int b = 128; b <= cap; b *= 2)
        if (b >= nr) return b;
    return 0;
}

cudaError_t launch_stream_collide_inplace(int storage, const UniSolve* solves, int count, int parity, int vec,
                                          int tpb, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if (count > kMaxBatch || (parity != 0 && parity != 1)) return cudaErrorInvalidValue;
    if (vec == 0) vec = default_vec(storage);
    if (vec != default_vec(storage)) return cudaErrorInvalidValue;
    int max_n = 0;
    for (int i = 0; i < count; ++i) {
        if (solves[i].n <= 0 || solves[i].n % vec != 0 || solves[i].src != solves[i].dst) return cudaErrorInvalidValue;
        if ((long long)solves[i].n * solves[i].n * solves[i].n >= (1LL << 32)) return cudaErrorInvalidValue;
        max_n = solves[i].n > max_n ? solves[i].n : max_n;
    }
    // the stream step needs whole rows per block; the local step runs at the same width
    const int b = inplace_tpb(storage, vec, tpb, max_n);
    if (b == 0) return cudaErrorInvalidValue;
    switch (storage) {
        case 0: return launch_aa_tpb<StF32, 4>(b, solves, count, parity, st);
        case 1: return launch_aa_tpb<StF16, 4>(b, solves, count, parity, st);
        case 2: return launch_aa_tpb<StBF16, 4>(b, solves, count, parity, st);
        case 3: return launch_aa_tpb<StF64, 2>(b, solves, count, parity, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace jp
