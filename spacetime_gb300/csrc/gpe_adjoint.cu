// gpe_adjoint.cu -- reverse-mode (adjoint) derivative of the parabolic leapfrog
// run with respect to the per-step magnetic fields, with sqrt(N) checkpointing.
//
// Forward run of N steps from u_0 (the reference's time loop, Spin1GpeBCC.cu:1428-1603):
//     u_1     = u_0 + (1/2) F_0(u_0)                    forwardEuler, :667-791
//     u_{j+1} = u_{j-1} + F_j(u_j),   j = 1..N-1         leapfrog,     :793-917
// with F_j(u) = 2 dt (-i) H(u; B_j, t_j) u and t_j = t0 + j dt.  For a loss L(u_N)
// the discrete adjoint lambda_j = dL/du_j obeys the same leapfrog backwards,
//     lambda_j = lambda_{j+2} + (dF_j/du)^T lambda_{j+1},   lambda_{N+1} = 0,
// and dL/dB_j = (dF_j/dB)^T lambda_{j+1} (dt instead of 2 dt for j = 0).  With
// b = i lambda_{j+1} (i times a vector is the transpose of -i times one):
//     (dF_j/du)^T lambda = 2 dt [ L^T b + (dh/du)^T b ],
// L the DEC Laplacian (L^T takes each entry's weight from its reverse entry) and
// h(u) the local part of H(u) u (trap, interaction, Zeeman, loss).  Without the
// loss term h is the Wirtinger gradient dE/d(conj u) of a real local energy, so
// its real Jacobian is symmetric and (dh/du)^T b = (dh/du) b: one evaluation of
// the step kernels' own local_terms template on forward-mode dual numbers along
// b.  The three-body loss term -i alpha n^2 u is not Hermitian; its transpose is
// added in closed form.  The field gradients use dh/dBb_k = F_k u (Zeeman) and
// dB/dBq from mag_field.
//
// Checkpointing: the forward run keeps (u_{kS}, u_{kS+1}) for every segment k of
// S steps; the reverse run recomputes one segment at a time from its pair with the
// forward step kernel itself (bit-identical states; with the gather kernel out of
// place, u_{j+1} = u_{j-1} + F(u_j) into a fresh buffer) and walks it backwards.
// Memory: 2 ceil(N/S) + S - 2 state buffers; S = ceil(sqrt(N)) by default.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "gpe_handle.h"
#include "gpe_kernels.cuh"

namespace gpe {

// ------------------------------------------------------------- dual numbers

template <typename R>
struct Dual {
    R v, d;
    __device__ __forceinline__ Dual() {}
    __device__ __forceinline__ Dual(double x) : v((R)x), d((R)0) {}
    __device__ __forceinline__ Dual(R x, R dx) : v(x), d(dx) {}
};
template <typename R>
__device__ __forceinline__ Dual<R> operator+(Dual<R> a, Dual<R> b) { return Dual<R>(a.v + b.v, a.d + b.d); }
template <typename R>
__device__ __forceinline__ Dual<R> operator-(Dual<R> a, Dual<R> b) { return Dual<R>(a.v - b.v, a.d - b.d); }
template <typename R>
__device__ __forceinline__ Dual<R> operator-(Dual<R> a) { return Dual<R>(-a.v, -a.d); }
template <typename R>
__device__ __forceinline__ Dual<R> operator*(Dual<R> a, Dual<R> b) { return Dual<R>(a.v * b.v, a.d * b.v + a.v * b.d); }
template <typename R>
__device__ __forceinline__ Dual<R>& operator+=(Dual<R>& a, Dual<R> b) {
    a.v += b.v;
    a.d += b.d;
    return a;
}

template <typename R>
__device__ __forceinline__ Dual<R> cd(R v) { return Dual<R>(v, (R)0); }

template <typename R>
__device__ __forceinline__ PhysR<Dual<R>> dual_phys(const PhysR<R>& P) {
    PhysR<Dual<R>> Q;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        Q.p0[i] = cd<R>(P.p0[i]);
        Q.bw[i] = cd<R>(P.bw[i]);
        Q.lambda[i] = cd<R>(P.lambda[i]);
        Q.qc[i] = cd<R>(P.qc[i]);
        Q.bb[i] = cd<R>(P.bb[i]);
        Q.bbq[i] = cd<R>(P.bbq[i]);
    }
    Q.bs = cd<R>(P.bs);
    Q.trap_offset = cd<R>(P.trap_offset);
    Q.c0 = cd<R>(P.c0);
    Q.c2 = cd<R>(P.c2);
    Q.c4 = cd<R>(P.c4);
    Q.alpha = cd<R>(P.alpha);
    Q.sigma = cd<R>(P.sigma);
    Q.bq = cd<R>(P.bq);
    Q.bqq = cd<R>(P.bqq);
    Q.dt = cd<R>(P.dt);
    Q.dts = cd<R>(P.dts);
    Q.trap_on = P.trap_on;
    Q.flags = P.flags;
    return Q;
}

// Local spin density <F> (unnormalised), the quantity gpe_observe integrates.
template <typename R, int C>
__device__ __forceinline__ void local_mag(const Cx<R>* ps, R M[3]) {
    if constexpr (C == 3) {
        const Cx<R> m = (R)GPE_REF_SQRT_2 * (conj(ps[0]) * ps[1] + conj(ps[1]) * ps[2]);
        M[0] = m.x;
        M[1] = m.y;
        M[2] = (ps[0].x * ps[0].x + ps[0].y * ps[0].y) - (ps[2].x * ps[2].x + ps[2].y * ps[2].y);
    } else if constexpr (C == 5) {
        const Cx<R> fp = (R)2 * (conj(ps[0]) * ps[1] + conj(ps[3]) * ps[4]) +
                         (R)2.449489742783178098 * (conj(ps[1]) * ps[2] + conj(ps[2]) * ps[3]);
        R n[5];
#pragma unroll
        for (int s = 0; s < 5; ++s) n[s] = ps[s].x * ps[s].x + ps[s].y * ps[s].y;
        M[0] = fp.x;
        M[1] = fp.y;
        M[2] = (R)2 * n[0] + n[1] - n[3] - (R)2 * n[4];
    } else {
        M[0] = M[1] = M[2] = (R)0;
    }
}

// Re(b^H (e_k . F) u) for k = x, y, z: the spin-1 Zeeman term of local_spin1
// (Spin1GpeBCC.cu:884-896: H0 += Bz u0 + conj(Bxy) u1, H1 += Bxy u0 + conj(Bxy) u2,
// H2 += Bxy u1 - Bz u2 with Bxy = (Bx + i By)/sqrt2) for a unit field along each
// axis and every other coefficient zero, projected on b.  The generic form runs
// local_terms three times on mostly zero coefficients.
template <typename R>
__device__ __forceinline__ void zeeman_proj_spin1(const Cx<R>* b, const Cx<R>* u, R s3[3]) {
    const R h = (R)GPE_REF_INV_SQRT_2;
    // Bx = 1: H = (u1, u0 + u2, u1) / sqrt2
    s3[0] = h * (b[0].x * u[1].x + b[0].y * u[1].y + b[1].x * (u[0].x + u[2].x) + b[1].y * (u[0].y + u[2].y) +
                 b[2].x * u[1].x + b[2].y * u[1].y);
    // By = 1: H = (-i u1, i (u0 - u2), i u1) / sqrt2
    s3[1] = h * (b[0].x * u[1].y - b[0].y * u[1].x + b[1].x * (u[2].y - u[0].y) + b[1].y * (u[0].x - u[2].x) -
                 b[2].x * u[1].y + b[2].y * u[1].x);
    // Bz = 1: H = (u0, 0, -u2)
    s3[2] = b[0].x * u[0].x + b[0].y * u[0].y - (b[2].x * u[2].x + b[2].y * u[2].y);
}

// J b for the spin-1 local terms of local_spin1 (external fields, quadratic Zeeman,
// no loss; Spin1GpeBCC.cu:867-912): the directional derivative along b of
//   h0 = T u0 + Bz u0 + conj(Bxy) u1,  h1 = T u1 + Bxy u0 + conj(Bxy) u2,
//   h2 = T u2 + Bxy u1 - Bz u2  (+ the quadratic Zeeman matrix times u),
// T = pot + c0 n, B = B_ext + c2 (Re m, Im m, n1 - n_-1), m = sqrt2 (u0* u1 + u1* u2),
// Bxy = (Bx + i By) / sqrt2.  The same values as a dual-number evaluation of
// local_terms along b, without the arithmetic on the constants' zero derivatives.
template <typename R>
__device__ __forceinline__ void jvp_spin1(const PhysR<R>& P, const R r[3], R pot, const Cx<R>* u, const Cx<R>* b,
                                          Cx<R>* g) {
    const R n1 = u[0].x * u[0].x + u[0].y * u[0].y;
    const R n_1 = u[2].x * u[2].x + u[2].y * u[2].y;
    const R n = n1 + (u[1].x * u[1].x + u[1].y * u[1].y) + n_1;
    const R d1 = (R)2 * (u[0].x * b[0].x + u[0].y * b[0].y);
    const R d_1 = (R)2 * (u[2].x * b[2].x + u[2].y * b[2].y);
    const R dn = d1 + (R)2 * (u[1].x * b[1].x + u[1].y * b[1].y) + d_1;
    const R T = pot + P.c0 * n, dT = P.c0 * dn;
    const Cx<R> m = (R)GPE_REF_SQRT_2 * (conj(u[0]) * u[1] + conj(u[1]) * u[2]);
    const Cx<R> dm = (R)GPE_REF_SQRT_2 * (conj(b[0]) * u[1] + conj(u[0]) * b[1] + conj(b[1]) * u[2] + conj(u[1]) * b[2]);
    R B[3];
    mag_field(P, r, P.bq, P.bb, B);
    B[0] += P.c2 * m.x;
    B[1] += P.c2 * m.y;
    B[2] += P.c2 * (n1 - n_1);
    const R dBz = P.c2 * (d1 - d_1);
    const Cx<R> Bxy = (R)GPE_REF_INV_SQRT_2 * cx<R>(B[0], B[1]);
    const Cx<R> dBxy = ((R)GPE_REF_INV_SQRT_2 * P.c2) * dm;
    g[0] = (dT + dBz) * u[0] + (T + B[2]) * b[0] + conj(dBxy) * u[1] + conj(Bxy) * b[1];
    g[1] = dT * u[1] + T * b[1] + dBxy * u[0] + Bxy * b[0] + conj(dBxy) * u[2] + conj(Bxy) * b[2];
    g[2] = (dT - dBz) * u[2] + (T - B[2]) * b[2] + dBxy * u[1] + Bxy * b[1];
    if (P.flags & GPE_FLAG_QUADRATIC_ZEEMAN) {
        // linear in u: the same matrix applied to b
        R Q[3];
        mag_field(P, r, P.bqq, P.bbq, Q);
        const Cx<R> qxy = (R)GPE_REF_INV_SQRT_2 * cx<R>(Q[0], Q[1]);
        const Cx<R> qc = conj(qxy);
        const R nsq = (qc * qxy).x;
        const R bz2 = Q[2] * Q[2];
        g[0] += (bz2 + nsq) * b[0] + (Q[2] * qc) * b[1] + (qc * qc) * b[2];
        g[1] += (Q[2] * qxy) * b[0] + ((R)2 * nsq) * b[1] - (Q[2] * qc) * b[2];
        g[2] += (qxy * qxy) * b[0] - (Q[2] * qxy) * b[1] + (bz2 + nsq) * b[2];
    }
}

struct AdjArgs {
    const char* a_prev;     // lambda_{j+1}: neighbours read
    char* a_next;           // lambda_{j+2} -> lambda_j: read-modify-write
    const char* psi;        // forward state u_j (own node only)
    const double* wT64;     // per entry: weight of the reverse entry (0 for repeated entries)
    const float* wT32;
    double factor;          // 2 dt (leapfrog) or dt (Euler start)
    float factor32;         // the same, for the FP32 kernel
    int update;             // 0: field gradients only (the start step)
};

constexpr int kGradCount = 4;  // dL/dBq, dL/dBb.x, dL/dBb.y, dL/dBb.z

__device__ __forceinline__ void node_coords(const StepArgs& a, uint32_t i, uint32_t& x, uint32_t& y, uint32_t& z,
                                            uint32_t& l) {
    const uint32_t row = fdiv(i, a.divRow);
    const uint32_t within = i - row * a.row_items;
    x = fdiv(within, a.divV);
    l = within - x * a.g.V;
    z = fdiv(row, a.divY);
    y = row - z * a.g.Y;
}

// Block sum of K values per thread into partials[blockIdx.x * K + k] * scale
// (blockDim 256): warp and block sums in the thread's type T, one conversion to
// FP64 per block and value (FP64 and conversions share GB300's narrow FP64 pipe).
template <int K, typename T>
__device__ __forceinline__ void block_partials(T (&v)[K], double scale, double* partials) {
    __shared__ T red[8][K];
#pragma unroll
    for (int k = 0; k < K; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) red[threadIdx.x >> 5][k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x < K) {
        T s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
        partials[(size_t)blockIdx.x * K + threadIdx.x] = (double)s * scale;
    }
}

// One reverse step: lambda_j = lambda_{j+2} + factor [L^T b + (dh/du)^T b] and the
// field gradients factor (dh/dB)^T b, b = i lambda_{j+1}.  Grid-stride over the
// nodes on one wave of blocks: the tables are staged, and the gradient sums
// reduced, once per block rather than once per 256 nodes.
template <typename R, int C>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 && C <= 3) ? 4 : 1) adjoint_step_kernel(StepArgs a, AdjArgs j) {
    __shared__ SmemTables<R> st;
    __shared__ R wT[kMaxEntries];
    load_tables<R>(st, a);
    for (int i = threadIdx.x; i < a.tab.entries; i += blockDim.x) {
        if constexpr (sizeof(R) == 4) wT[i] = j.wT32[i];
        else wT[i] = j.wT64[i];
    }
    __syncthreads();
    R gsum[kGradCount] = {(R)0, (R)0, (R)0, (R)0};
    for (uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < a.total;
         gid += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x, y, z, l;
        node_coords(a, (uint32_t)gid, x, y, z, l);
        const size_t cell_off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes;
        const uint32_t node_bytes = C * 2 * sizeof(R);
        const char* abase = j.a_prev + cell_off;
        Cx<R> b[C], u[C];
        ld_node<R, C, true>(abase + l * node_bytes, b);  // whole records: (C+1)/2 loads in FP32
        ld_node<R, C, true>(j.psi + cell_off + l * node_bytes, u);
#pragma unroll
        for (int c = 0; c < C; ++c) b[c] = cx<R>(-b[c].y, b[c].x);
        const PhysR<R>& P = make_phys<R>(a);
        R r[3];
        r[0] = P.p0[0] + P.bs * ((R)x * P.bw[0] + st.pos[3 * l + 0]);
        r[1] = P.p0[1] + P.bs * ((R)y * P.bw[1] + st.pos[3 * l + 1]);
        r[2] = P.p0[2] + P.bs * ((R)z * P.bw[2] + st.pos[3 * l + 2]);
        const R pot = trap<R>(P, r);
        if (j.update) {
            // L^T b = sum_f wT_f b_nb(f) - (sum_f w_f) b
            Cx<R> K[C];
#pragma unroll
            for (int c = 0; c < C; ++c) K[c] = cx<R>((R)0, (R)0);
            R diag = 0;
            const int f0 = st.row_ptr[l], f1 = st.row_ptr[l + 1];
            if (a.tab.uniform_deg == 4 && C <= 3) {
                // 4 entries: the 4 neighbour records are loaded before they are used
                Cx<R> v[4][C];
#pragma unroll
                for (int k = 0; k < 4; ++k) ld_node<R, C, true>(abase + st.nb_off[f0 + k], v[k]);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    diag += st.w[f0 + k];
                    const R wt = wT[f0 + k];
#pragma unroll
                    for (int c = 0; c < C; ++c) K[c] += wt * cx<R>(-v[k][c].y, v[k][c].x);
                }
            } else {
                for (int f = f0; f < f1; ++f) {
                    Cx<R> av[C];
                    ld_node<R, C, true>(abase + st.nb_off[f], av);
                    diag += st.w[f];
                    const R wt = wT[f];
#pragma unroll
                    for (int c = 0; c < C; ++c) K[c] += wt * cx<R>(-av[c].y, av[c].x);
                }
            }
            // (dh/du)^T b.  Apart from three-body loss, h = dE/d(conj u) for a real
            // energy E (trap, c0 n^2/2, Zeeman B.<F>, c2 <F>^2/2, quadratic Zeeman,
            // spin-2 singlet |A00|^2), so its real Jacobian is half the Hessian of E,
            // symmetric: J^T b = J b, one dual evaluation along b.
            Cx<R> g[C];
            if constexpr (C == 3) {
                jvp_spin1<R>(P, r, pot, u, b, g);
            } else {
                PhysR<Dual<R>> PD = dual_phys<R>(P);
                PD.flags &= ~GPE_FLAG_THREE_BODY_LOSS;
                const Dual<R> rD[3] = {cd<R>(r[0]), cd<R>(r[1]), cd<R>(r[2])};
                Cx<Dual<R>> psD[C], H[C];
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    psD[c] = cx<Dual<R>>(Dual<R>(u[c].x, b[c].x), Dual<R>(u[c].y, b[c].y));
                    H[c] = cx<Dual<R>>(cd<R>((R)0), cd<R>((R)0));
                }
                local_terms<Dual<R>, C>(PD, rD, cd<R>(pot), GPE_MODE_LEAPFROG, false, psD, H);
#pragma unroll
                for (int c = 0; c < C; ++c) g[c] = cx<R>(H[c].x.d, H[c].y.d);
            }
            if (P.flags & GPE_FLAG_THREE_BODY_LOSS) {
                // h_loss = -i alpha n^2 u: J^T b = i alpha n^2 b + 4 alpha n Im(b^H u) u
                R n = 0, im = 0;
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    n += u[c].x * u[c].x + u[c].y * u[c].y;
                    im += b[c].x * u[c].y - b[c].y * u[c].x;
                }
                const R an2 = P.alpha * n * n, k4 = (R)4 * P.alpha * n * im;
#pragma unroll
                for (int c = 0; c < C; ++c) g[c] += cx<R>(-an2 * b[c].y + k4 * u[c].x, an2 * b[c].x + k4 * u[c].y);
            }
            char* o = j.a_next + cell_off + l * node_bytes;
            R fac;
            if constexpr (sizeof(R) == 4) fac = j.factor32;
            else fac = j.factor;
            Cx<R> v[C];
            ld_node<R, C, false>(o, v);
#pragma unroll
            for (int c = 0; c < C; ++c) {
                v[c].x += fac * (K[c].x - diag * b[c].x + g[c].x);
                v[c].y += fac * (K[c].y - diag * b[c].y + g[c].y);
            }
            st_node<R, C>(o, v);
        }
        // field parameters.  h depends on Bb only through the Zeeman term (B.F) u,
        // so dh/dBb_k = F_k u: the local terms with every coefficient zero except
        // Bb = e_k.  dB/dBq is mag_field's B at Bq = 1, Bb = 0.
        if constexpr (C > 1) {
            R s3[3];
            if constexpr (C == 3) {
                zeeman_proj_spin1<R>(b, u, s3);
            } else {
            PhysR<R> Z = P;
            Z.c0 = Z.c2 = Z.c4 = Z.alpha = Z.bq = Z.bqq = (R)0;
            Z.flags = 0;
            Z.trap_on = 0;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
#pragma unroll
                for (int i = 0; i < 3; ++i) Z.bb[i] = (R)(i == k);
                Cx<R> H[C];
#pragma unroll
                for (int c = 0; c < C; ++c) H[c] = cx<R>((R)0, (R)0);
                local_terms<R, C>(Z, r, (R)0, GPE_MODE_LEAPFROG, false, u, H);
                R d = 0;
#pragma unroll
                for (int c = 0; c < C; ++c) d += b[c].x * H[c].x + b[c].y * H[c].y;
                s3[k] = d;
            }
            }
            const R zero3[3] = {(R)0, (R)0, (R)0};
            R w[3];
            mag_field<R>(P, r, (R)1, zero3, w);
            gsum[0] += w[0] * s3[0] + w[1] * s3[1] + w[2] * s3[2];
            gsum[1] += s3[0];
            gsum[2] += s3[1];
            gsum[3] += s3[2];
        }
    }
    block_partials<kGradCount, R>(gsum, j.factor, a.partials);
}

// Block g adds the nblocks x K partials at partials + g * nblocks * K into
// out[g * K + k] * scale in a fixed order: thread t sums partial blocks t,
// t + kSumThreads, ... for all K values at once, then a tree over the threads.
// One launch reduces the partials of every step of a checkpoint segment.
constexpr int kSumThreads = 1024;
template <int K>
__global__ void __launch_bounds__(kSumThreads) adjoint_sum_kernel(const double* partials, uint32_t nblocks, double scale,
                                                                  double* out) {
    __shared__ double red[K][kSumThreads];
    const double* src = partials + (size_t)blockIdx.x * nblocks * K;
    double s[K];
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] = 0.0;
#pragma unroll 4
    for (uint32_t b = threadIdx.x; b < nblocks; b += kSumThreads) {
#pragma unroll
        for (int k = 0; k < K; ++k) s[k] += src[(size_t)b * K + k];
    }
#pragma unroll
    for (int k = 0; k < K; ++k) red[k][threadIdx.x] = s[k];
    __syncthreads();
    for (int w = kSumThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < K; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x < K) out[(size_t)blockIdx.x * K + threadIdx.x] = red[threadIdx.x][0] * scale;
}

constexpr int kFinalCount = 5;  // Re <T|u>, Im <T|u>, Mx, My, Mz

// Final-state quantities: the overlap sum conj(T) u and the spin density sums.
// a.prev = target T, a.next = u_N.
template <typename R, int C>
__global__ void __launch_bounds__(256) adjoint_final_kernel(StepArgs a) {
    double v[kFinalCount] = {0, 0, 0, 0, 0};
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid < a.total) {
        uint32_t x, y, z, l;
        node_coords(a, (uint32_t)gid, x, y, z, l);
        const size_t off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes +
                           l * (C * 2 * sizeof(R));
        Cx<double> u[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const Cx<R> t = ldc<R>(a.prev + off + c * 2 * sizeof(R));
            const Cx<R> p = ldc<R>(a.next + off + c * 2 * sizeof(R));
            u[c] = cx<double>((double)p.x, (double)p.y);
            v[0] += (double)t.x * p.x + (double)t.y * p.y;
            v[1] += (double)t.x * p.y - (double)t.y * p.x;
        }
        double M[3];
        local_mag<double, C>(u, M);
        v[2] = M[0];
        v[3] = M[1];
        v[4] = M[2];
    }
    block_partials<kFinalCount, double>(v, 1.0, a.partials);
}

// lambda_N = dv [ (s0 + i s1) T + sum_m s_{2+m} grad M_m(u_N) ].
// a.prev = target T, a.next = lambda buffer, psi = u_N.
template <typename R, int C>
__global__ void __launch_bounds__(256) adjoint_seed_kernel(StepArgs a, const char* psi, double s0, double s1, double sx,
                                                           double sy, double sz, double dv) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= a.total) return;
    uint32_t x, y, z, l;
    node_coords(a, (uint32_t)gid, x, y, z, l);
    const size_t off = (size_t)z * a.g.slice + (size_t)y * a.g.pitch + (size_t)x * a.g.cell_bytes +
                       l * (C * 2 * sizeof(R));
    Cx<double> u[C], g[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const Cx<R> t = ldc<R>(a.prev + off + c * 2 * sizeof(R));
        const Cx<R> p = ldc<R>(psi + off + c * 2 * sizeof(R));
        u[c] = cx<double>((double)p.x, (double)p.y);
        g[c] = cx<double>(s0 * t.x - s1 * t.y, s0 * t.y + s1 * t.x);
    }
    if (C > 1 && (sx != 0.0 || sy != 0.0 || sz != 0.0)) {
#pragma unroll
        for (int k = 0; k < 2 * C; ++k) {
            Cx<Dual<double>> uD[C];
#pragma unroll
            for (int c = 0; c < C; ++c)
                uD[c] = cx<Dual<double>>(Dual<double>(u[c].x, (double)(k == 2 * c)),
                                         Dual<double>(u[c].y, (double)(k == 2 * c + 1)));
            Dual<double> M[3];
            local_mag<Dual<double>, C>(uD, M);
            const double d = sx * M[0].d + sy * M[1].d + sz * M[2].d;
            if (k & 1) g[k >> 1].y += d;
            else g[k >> 1].x += d;
        }
    }
#pragma unroll
    for (int c = 0; c < C; ++c) stc<R>(a.next + off + c * 2 * sizeof(R), cx<R>((R)(dv * g[c].x), (R)(dv * g[c].y)));
}

// Blocks of a reverse step: one wave (the kernel's occupancy x SMs), fewer for
// small grids.  Its partials are that many blocks x kGradCount.
template <typename R, int C>
static unsigned adjoint_step_blocks(uint64_t total) {
    static int occ = 0;
    if (occ == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adjoint_step_kernel<R, C>, 256, 0);
        if (occ < 1) occ = 1;
    }
    return std::min<unsigned>(nblocks(total, 256), (unsigned)occ * (unsigned)device_sm_count());
}

// One reverse step on nb blocks (adjoint_step_blocks); its block partials go to
// a.partials (nb x kGradCount).
template <typename R, int C>
static cudaError_t launch_adjoint_step(const StepArgs& a, const AdjArgs& j, unsigned nb, cudaStream_t s) {
    adjoint_step_kernel<R, C><<<nb, 256, 0, s>>>(a, j);
    return cudaGetLastError();
}

template <typename R, int C>
static cudaError_t launch_adjoint_final(const StepArgs& a, double dv, double* out, cudaStream_t s) {
    const unsigned nb = nblocks(a.total, 256);
    adjoint_final_kernel<R, C><<<nb, 256, 0, s>>>(a);
    adjoint_sum_kernel<kFinalCount><<<1, kSumThreads, 0, s>>>(a.partials, nb, dv, out);
    return cudaGetLastError();
}

template <typename R, int C>
static cudaError_t launch_adjoint_seed(const StepArgs& a, const char* psi, const double* sd, double dv, cudaStream_t s) {
    adjoint_seed_kernel<R, C><<<nblocks(a.total, 256), 256, 0, s>>>(a, psi, sd[0], sd[1], sd[2], sd[3], sd[4], dv);
    return cudaGetLastError();
}

// Instantiates FN for the handle's precision and component count.
#define GPE_ADJ_DISPATCH(FN, H, ...)                                                               \
    ((H)->real_bytes == 8 ? ((H)->g.C == 1   ? FN<double, 1>(__VA_ARGS__)                         \
                             : (H)->g.C == 3 ? FN<double, 3>(__VA_ARGS__)                         \
                                             : FN<double, 5>(__VA_ARGS__))                        \
                          : ((H)->g.C == 1   ? FN<float, 1>(__VA_ARGS__)                          \
                             : (H)->g.C == 3 ? FN<float, 3>(__VA_ARGS__)                          \
                                             : FN<float, 5>(__VA_ARGS__)))

// ------------------------------------------------------------------ host side

void adjoint_release(gpe_handle* h) {
    AdjointStore& A = h->adj;
    for (void* p : A.ckpt) cudaFree(p);
    for (void* p : A.seg) cudaFree(p);
    A.ckpt.clear();
    A.seg.clear();
    for (void*& p : A.adj) {
        if (p) cudaFree(p);
        p = nullptr;
    }
    if (A.target) cudaFree(A.target);
    if (A.grad) cudaFree(A.grad);
    if (A.out) cudaFree(A.out);
    if (A.part) cudaFree(A.part);
    A.part = nullptr;
    A.part_count = 0;
    if (A.wT64) cudaFree(A.wT64);
    if (A.wT32) cudaFree(A.wT32);
    A.target = nullptr;
    A.grad = A.out = A.wT64 = nullptr;
    A.wT32 = nullptr;
    A.valid = false;
    A.n = A.stride = A.segments = 0;
}

static char* interior_of(const gpe_handle* h, void* base) {
    return static_cast<char*>(base) + h->g.slice + h->g.pitch + h->g.cell_bytes;
}

// Transposed Laplacian weights: entry f of row j (j -> node i at offset d) gets the
// sum of the weights of row i's entries (i -> j at offset -d); a repeated (d, i)
// in row j gets 0 so that the sum is counted once.  Every entry must have a
// reverse entry, or L^T would need entries that row j does not hold.
static gpe_status build_transpose(gpe_handle* h) {
    const gpe_lattice& L = h->lat;
    const double bs2 = h->p.block_scale * h->p.block_scale;
    const int n = (int)L.stencil.size();
    auto same = [](const gpe_stencil_entry& a, int dx, int dy, int dz, int node) {
        return a.dx == dx && a.dy == dy && a.dz == dz && a.node == node;
    };
    std::vector<double> wT(n, 0.0);
    for (int jn = 0; jn < L.V; ++jn) {
        for (int f = L.row_ptr[jn]; f < L.row_ptr[jn + 1]; ++f) {
            const gpe_stencil_entry& e = L.stencil[f];
            bool repeated = false;
            for (int f2 = L.row_ptr[jn]; f2 < f && !repeated; ++f2) repeated = same(L.stencil[f2], e.dx, e.dy, e.dz, e.node);
            if (repeated) continue;
            double s = 0;
            bool found = false;
            for (int g = L.row_ptr[e.node]; g < L.row_ptr[e.node + 1]; ++g)
                if (same(L.stencil[g], -e.dx, -e.dy, -e.dz, jn)) {
                    s += (-0.5 * L.stencil[g].hodge) / bs2;
                    found = true;
                }
            if (!found) return fail(GPE_ERR_UNSUPPORTED, "adjoint: a stencil entry has no reverse entry");
            wT[f] = s;
        }
    }
    std::vector<float> wT32(wT.begin(), wT.end());
    AdjointStore& A = h->adj;
    if (cudaMalloc(&A.wT64, n * sizeof(double)) != cudaSuccess || cudaMalloc(&A.wT32, n * sizeof(float)) != cudaSuccess)
        return fail(GPE_ERR_OOM, "cudaMalloc (adjoint tables)");
    cudaError_t e = cudaMemcpy(A.wT64, wT.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(A.wT32, wT32.data(), n * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy (adjoint tables)");
    return GPE_OK;
}

static gpe_status ensure_adjoint_buffers(gpe_handle* h, int n, int stride) {
    AdjointStore& A = h->adj;
    const int segments = (n + stride - 1) / stride;
    const size_t bytes = h->alloc_bytes[GPE_PSI_EVEN];
    const size_t want_ckpt = (size_t)2 * segments, want_seg = stride > 2 ? (size_t)(stride - 2) : 0;
    auto resize = [&](std::vector<void*>& v, size_t want) -> bool {
        while (v.size() > want) {
            cudaFree(v.back());
            v.pop_back();
        }
        while (v.size() < want) {
            void* p = nullptr;
            if (cudaMalloc(&p, bytes) != cudaSuccess) return false;
            v.push_back(p);
            // zero halos: the out-of-place recomputation writes only the interior
            if (cudaMemset(p, 0, bytes) != cudaSuccess) return false;
        }
        return true;
    };
    if (!resize(A.ckpt, want_ckpt) || !resize(A.seg, want_seg)) {
        adjoint_release(h);
        return fail(GPE_ERR_OOM, "cudaMalloc (adjoint checkpoints)");
    }
    // recompute and adjoint buffers keep zero halos: they are zeroed when
    // allocated, checkpoint copies carry the (zero) halo of a handle buffer, and
    // every kernel writes the interior only
    for (void*& p : A.adj)
        if (!p && cudaMalloc(&p, bytes) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (adjoint state)");
    if (!A.target) {
        if (cudaMalloc(&A.target, bytes) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (target)");
        if (cudaMemset(A.target, 0, bytes) != cudaSuccess) return fail(GPE_ERR_CUDA, "cudaMemset (target)");
    }
    if (A.grad && A.n < n) {
        cudaFree(A.grad);
        A.grad = nullptr;
    }
    if (!A.grad && cudaMalloc(&A.grad, (size_t)n * kGradCount * sizeof(double)) != cudaSuccess)
        return fail(GPE_ERR_OOM, "cudaMalloc (gradients)");
    if (!A.out && cudaMalloc(&A.out, 8 * sizeof(double)) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (adjoint out)");
    const size_t part = (size_t)stride * h->partial_blocks * kGradCount;
    if (A.part && A.part_count < part) {
        cudaFree(A.part);
        A.part = nullptr;
    }
    if (!A.part) {
        if (cudaMalloc(&A.part, part * sizeof(double)) != cudaSuccess) return fail(GPE_ERR_OOM, "cudaMalloc (adjoint partials)");
        A.part_count = part;
    }
    if (!A.wT64) {
        gpe_status st = build_transpose(h);
        if (st) return st;
    }
    A.buf_bytes = bytes;
    A.segments = segments;
    return GPE_OK;
}

static gpe_status copy_state(gpe_handle* h, void* dst, const void* src, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(dst, src, h->alloc_bytes[GPE_PSI_EVEN], cudaMemcpyDeviceToDevice, s);
    return e == cudaSuccess ? GPE_OK : cuda_fail(e, "checkpoint copy");
}

}  // namespace gpe

using namespace gpe;

extern "C" gpe_status gpe_adjoint_forward(gpe_handle* h, int32_t n_steps, const gpe_fields* fields, int32_t stride,
                                          const double* target, size_t count, double* out, void* stream) {
    if (!h || !fields || !target || !out) return fail(GPE_ERR_INVALID_ARG, "null argument");
    if (h->p.scheme != GPE_SCHEME_PARABOLIC) return fail(GPE_ERR_UNSUPPORTED, "the adjoint is built for the parabolic scheme");
    if (h->exp_rate != 0) return fail(GPE_ERR_UNSUPPORTED, "the adjoint does not follow condensate expansion");
    if (n_steps < 1) return fail(GPE_ERR_INVALID_ARG, "n_steps must be at least 1");
    if (count != host_count(h, false)) return fail(GPE_ERR_INVALID_ARG, "target size does not match the grid");
    if (stride <= 0) stride = (int32_t)std::ceil(std::sqrt((double)n_steps));
    if (stride > n_steps) stride = n_steps;
    AdjointStore& A = h->adj;
    A.valid = false;
    gpe_status st = ensure_adjoint_buffers(h, n_steps, stride);
    if (st) return st;
    cudaStream_t s = (cudaStream_t)stream;
    // target: host FP64 file layout -> device buffer in the handle's precision
    if ((st = ensure_stage(h, count))) return st;
    const Grid& g = h->g;
    cudaError_t e = cudaMemcpyAsync(h->stage, target, count * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = launch_pack_any(h->p.precision, h->stage, static_cast<char*>(A.target), g.X, g.Y, g.Z,
                            (uint32_t)(g.cell_bytes / h->real_bytes), g.pitch, g.slice, true, s);
    if (e != cudaSuccess) return cuda_fail(e, "target upload");
    h->launches += 1;
    A.n = n_steps;
    A.stride = stride;
    A.t0 = h->t0;
    A.fields.assign(fields, fields + n_steps);
    const double dt = h->p.dt;
    // u_j lives in PSI_ODD for even j and in PSI_EVEN for odd j
    auto slot_of = [](int j) { return (j & 1) ? GPE_PSI_EVEN : GPE_PSI_ODD; };
    if ((st = step_buffers(h, h->interior[GPE_PSI_EVEN], h->interior[GPE_PSI_ODD], fields[0], A.t0, GPE_MODE_EULER, s)))
        return st;
    if ((st = copy_state(h, A.ckpt[0], h->alloc[GPE_PSI_ODD], s))) return st;
    if ((st = copy_state(h, A.ckpt[1], h->alloc[GPE_PSI_EVEN], s))) return st;
    // steps j .. je up to the next checkpoint (after a step j that is a multiple of
    // the stride), in the interleaved layout where that is the handle's kernel for a
    // call of that length (the same states as step_buffers', bit for bit, so the
    // recomputation in the handle's layout reproduces them)
    for (int j = 1; j < n_steps;) {
        int je = (j + stride - 1) / stride * stride;
        if (je > n_steps - 1) je = n_steps - 1;
        const int32_t cnt = je - j + 1;
        if (il_leapfrog_applies(h, cnt)) {
            if ((st = il_leapfrog_explicit(h, slot_of(j), cnt, fields + j, A.t0 + j * dt, dt, s))) return st;
        } else {
            for (int jj = j; jj <= je; ++jj)
                if ((st = step_buffers(h, h->interior[slot_of(jj + 1)], h->interior[slot_of(jj)], fields[jj],
                                       A.t0 + jj * dt, GPE_MODE_LEAPFROG, s)))
                    return st;
        }
        if (je % stride == 0) {
            const int k = je / stride;
            if ((st = copy_state(h, A.ckpt[2 * k], h->alloc[slot_of(je)], s))) return st;
            if ((st = copy_state(h, A.ckpt[2 * k + 1], h->alloc[slot_of(je + 1)], s))) return st;
        }
        j = je + 1;
    }
    h->cur = slot_of(n_steps);
    h->nstep = (uint64_t)(n_steps - 1);
    StepArgs a = make_args(h, fields[n_steps - 1], A.t0 + n_steps * dt);
    a.prev = interior_of(h, A.target);
    a.next = h->interior[h->cur];
    e = GPE_ADJ_DISPATCH(launch_adjoint_final, h, a, cell_dv(h), A.out, s);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint final kernel");
    h->launches += 2;
    double r[kFinalCount];
    e = cudaMemcpyAsync(r, A.out, sizeof r, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint forward");
    if ((st = check_device_error(h, s))) return st;
    for (int k = 0; k < kFinalCount; ++k) out[k] = r[k];
    A.valid = true;
    A.epoch = h->epoch;
    return GPE_OK;
}

extern "C" gpe_status gpe_adjoint_backward(gpe_handle* h, const double* seed, double* grad, void* stream) {
    if (!h || !seed || !grad) return fail(GPE_ERR_INVALID_ARG, "null argument");
    AdjointStore& A = h->adj;
    if (!A.valid || A.epoch != h->epoch)
        return fail(GPE_ERR_INVALID_ARG, "no recorded forward run (or the state changed since gpe_adjoint_forward)");
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t epoch = h->epoch;
    const int n = A.n, S = A.stride;
    const double dt = h->p.dt;
    gpe_status st;
    cudaError_t e = cudaMemsetAsync(A.adj[0], 0, A.buf_bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(A.adj[1], 0, A.buf_bytes, s);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint clear");
    {
        StepArgs a = make_args(h, A.fields[n - 1], A.t0 + n * dt);
        a.prev = interior_of(h, A.target);
        a.next = interior_of(h, A.adj[0]);
        e = GPE_ADJ_DISPATCH(launch_adjoint_seed, h, a, h->interior[h->cur], seed, cell_dv(h), s);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint seed kernel");
        h->launches += 1;
    }
    char* P = interior_of(h, A.adj[0]);  // lambda_{j+1}
    char* Q = interior_of(h, A.adj[1]);  // lambda_{j+2} -> lambda_j
    std::vector<void*> state((size_t)S, nullptr);
    // the gather kernel recomputes a segment out of place; the tile kernels (which
    // the forward run then used) in place after a state copy, so that the states
    // stay bit-identical to the forward run's
    const bool oop = leapfrog_from_supported(h);
    for (int k = A.segments - 1; k >= 0; --k) {
        const int lo = k * S, hi = std::min(lo + S, n), len = hi - lo;
        state[0] = A.ckpt[2 * k];
        if (len > 1) state[1] = A.ckpt[2 * k + 1];
        for (int m = 2; m < len; ++m) {
            state[m] = A.seg[m - 2];
            const int jj = lo + m - 1;
            if (oop) {
                // u_{jj+1} = u_{jj-1} + F(u_jj) into a fresh buffer: no state copy
                if ((st = leapfrog_from(h, interior_of(h, state[m]), interior_of(h, state[m - 1]),
                                        interior_of(h, state[m - 2]), A.fields[jj], A.t0 + jj * dt, s)))
                    return st;
                continue;
            }
            if ((st = copy_state(h, state[m], state[m - 2], s))) return st;
            if ((st = step_buffers(h, interior_of(h, state[m]), interior_of(h, state[m - 1]), A.fields[jj],
                                   A.t0 + jj * dt, GPE_MODE_LEAPFROG, s)))
                return st;
        }
        const unsigned nb = GPE_ADJ_DISPATCH(adjoint_step_blocks, h, h->g.X * (uint64_t)h->g.Y * h->g.Z * h->g.V);
        for (int j = hi - 1; j >= lo; --j) {
            StepArgs a = make_args(h, A.fields[j], A.t0 + j * dt);
            a.partials = A.part + (size_t)(j - lo) * nb * kGradCount;
            AdjArgs aj;
            aj.a_prev = P;
            aj.a_next = Q;
            aj.psi = interior_of(h, state[j - lo]);
            aj.wT64 = A.wT64;
            aj.wT32 = A.wT32;
            aj.factor = j >= 1 ? 2.0 * dt : dt;
            aj.factor32 = (float)aj.factor;
            aj.update = j >= 1 ? 1 : 0;
            e = GPE_ADJ_DISPATCH(launch_adjoint_step, h, a, aj, nb, s);
            if (e != cudaSuccess) return cuda_fail(e, "adjoint step kernel");
            h->launches += 1;
            if (j >= 1) std::swap(P, Q);
        }
        // the field gradients of the segment's steps, one block per step
        adjoint_sum_kernel<kGradCount><<<len, kSumThreads, 0, s>>>(A.part, nb, 1.0, A.grad + (size_t)lo * kGradCount);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "adjoint gradient sums");
        h->launches += 1;
    }
    e = cudaMemcpyAsync(grad, A.grad, (size_t)n * kGradCount * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    // the recomputation ran the step kernel on the adjoint's own buffers only
    h->epoch = epoch;
    if (e != cudaSuccess) return cuda_fail(e, "adjoint backward");
    return check_device_error(h, s);
}
