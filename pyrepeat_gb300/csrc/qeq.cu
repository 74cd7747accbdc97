// QEq charges (repeat.py:2539-2634, ChargeCalculator.compute_qeq_charges) on the device.
//
// J, the atoms' Coulomb matrix under the fit's Ewald object (repeat.py:2575-2595):
//   J_ii = j_self[i]  (the idempotential, 2 x hardness)
//   J_ij = sum over the FULL shift list (2 nmax + 1)^3 of erfc(sqrt(alpha) r) / r for every
//          image with r > 1e-10 (repeat.py:2615-2626: no cutoff, unlike the fit's
//          real-space sum)
//        + sum_k w_k cos(k . (r_i - r_j))                       (repeat.py:2628-2632)
// The k-sum factorises into per-atom tables, sum_k w_k (cos_i cos_j + sin_i sin_j): one FP64
// product of [w cos | w sin] (N x 2K) with [cos | sin] (N x 2K), one triangle of it (cuBLAS
// DSYRKX).  The pair kernel adds the real-space sum of pair (i < j) to that term and writes
// J_ij and J_ji, so J is exactly symmetric like the reference's.  With KMAX 0 (the non-periodic fit) alpha is 0, the shift
// list is the zero shift alone and there are no k-vectors, so J_ij = 1/r_ij (repeat.py:
// 2588-2595).
//
// The charges: repeat.py:2597-2613 solves sum q = Q together with the rows
// (J q)_{i-1} - (J q)_i = chi_i - chi_{i-1}, i.e. (J q)_i + chi_i is the same for every
// atom.  That is the bordered system [J 1; 1^T 0] [q; mu] = [-chi; Q], the form of the fit's
// total-charge system, so it runs through the same solve (FP32 LU with FP64 refinement, FP64
// LU fallback).  Both systems have the same solution set in q.
#include <vector>

#include "common.cuh"

namespace rp {
namespace {

__global__ void qeq_tables_kernel(const double *__restrict__ kvec, const double *__restrict__ kcoef, int K,
                                  const double *__restrict__ atoms, int N, double *__restrict__ W,
                                  double *__restrict__ U) {
    // W[a] = [w_k cos(k.r_a) | w_k sin(k.r_a)], U[a] = [cos(k.r_a) | sin(k.r_a)], rows of 2K
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * K) return;
    const int a = (int)(t / K), k = (int)(t - (long long)a * K);
    const double kr =
        (atoms[3 * a] * kvec[3 * k] + atoms[3 * a + 1] * kvec[3 * k + 1]) + atoms[3 * a + 2] * kvec[3 * k + 2];
    double s, c;
    sincos(kr, &s, &c);
    const size_t row = (size_t)a * 2 * K;
    W[row + k] = kcoef[k] * c;
    W[row + K + k] = kcoef[k] * s;
    U[row + k] = c;
    U[row + K + k] = s;
}

__global__ void qeq_pairs_kernel(const double *__restrict__ atoms, int N, const double *__restrict__ shifts, int S,
                                 double sa, const double *__restrict__ R, const double *__restrict__ j_self,
                                 double *__restrict__ J) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * N) return;
    const int i = (int)(t / N), j = (int)(t - (long long)i * N);
    if (j < i) return;
    if (j == i) {
        J[t] = j_self[i];
        return;
    }
    const double dx = atoms[3 * i] - atoms[3 * j], dy = atoms[3 * i + 1] - atoms[3 * j + 1],
                 dz = atoms[3 * i + 2] - atoms[3 * j + 2];
    // images with sqrt(alpha) r > 7 are skipped: each would add erfc(7)/r < 1e-24, against
    // entries of order 1e-2..1 whose ulp is above 1e-18 (KMAX 0: alpha 0, nothing is skipped)
    const double r_far2 = sa > 0.0 ? (7.0 / sa) * (7.0 / sa) : 1e300;
    double acc = 0.0;
    for (int s = 0; s < S; ++s) {
        const double x = dx + shifts[3 * s], y = dy + shifts[3 * s + 1], z = dz + shifts[3 * s + 2];
        const double r2 = x * x + y * y + z * z;
        if (r2 > r_far2) continue;
        const double r = sqrt(r2);
        if (r > 1e-10) acc += erfc(sa * r) / r;
    }
    const double v = R ? acc + R[t] : acc;
    J[t] = v;
    J[(size_t)j * N + i] = v;
}

}  // namespace

void qeq_run(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const double *chi, const double *j_self,
             double qtot, double *q_out, double *J_out, double *info, cudaStream_t stream) {
    RP_REQUIRE(N > 0 && atoms && chi && j_self && q_out, "rp_qeq: need N > 0 and non-null atoms, chi, j_self, q");
    const int K = ew->K, K2 = 2 * ew->K;
    const int S = (int)(ew->shifts.size() / 3);
    RP_REQUIRE(S > 0, "rp_qeq: ewald object has no shifts");
    double *d_atoms = ctx->buf_t<double>("qeq_atoms", 3 * (size_t)N);
    double *d_sh = ctx->buf_t<double>("qeq_shifts", 3 * (size_t)S);
    double *d_js = ctx->buf_t<double>("qeq_jself", (size_t)N);
    double *d_b = ctx->buf_t<double>("qeq_b", (size_t)N);
    double *d_J = ctx->buf_t<double>("qeq_J", (size_t)N * N);
    double *d_q = ctx->buf_t<double>("qeq_q", (size_t)N);
    std::vector<double> nb((size_t)N);
    for (int i = 0; i < N; ++i) nb[i] = -chi[i];
    RP_CUDA(cudaMemcpyAsync(d_atoms, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_sh, ew->shifts.data(), sizeof(double) * 3 * S, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_js, j_self, sizeof(double) * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_b, nb.data(), sizeof(double) * N, cudaMemcpyHostToDevice, stream));

    const double *R = nullptr;
    if (K > 0) {
        double *W = ctx->buf_t<double>("qeq_W", (size_t)N * K2);
        double *U = ctx->buf_t<double>("qeq_U", (size_t)N * K2);
        double *dR = ctx->buf_t<double>("qeq_R", (size_t)N * N);
        {
            StageTimer tt(ctx, "qeq_tables", stream);
            const long long n = (long long)N * K;
            qeq_tables_kernel<<<ceil_div(n, 256), 256, 0, stream>>>(ew->d_kvec, ew->d_kcoef, K, d_atoms, N, W, U);
            RP_LAUNCH_CHECK();
        }
        // row-major W, U (N x 2K) are column-major 2K x N.  W U^T is symmetric, so only one
        // triangle is formed (DSYRKX, half the flops of a GEMM): column-major (j, i), j >= i,
        // i.e. R[i*N + j] = sum_k W[j][k] U[i][k] for the pairs i <= j the pair kernel reads
        StageTimer tt(ctx, "qeq_recip_dgemm", stream);
        cublasHandle_t h = ctx->blas();
        RP_CUBLAS(cublasSetStream(h, stream));
        const double one = 1.0, zero = 0.0;
        RP_CUBLAS(cublasDsyrkx(h, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, N, K2, &one, W, K2, U, K2, &zero, dR, N));
        R = dR;
    }
    {
        StageTimer tt(ctx, "qeq_pairs", stream);
        const long long n = (long long)N * N;
        qeq_pairs_kernel<<<ceil_div(n, 128), 128, 0, stream>>>(d_atoms, N, d_sh, S, ew->sqrt_alpha, R, d_js, d_J);
        RP_LAUNCH_CHECK();
    }
    {
        StageTimer tt(ctx, "qeq_solve", stream);
        static const int no_group[1] = {0};
        solve_run(ctx, d_J, d_b, N, 0, no_group, no_group, nullptr, nullptr, qtot, d_q, info, stream);
    }
    RP_CUDA(cudaMemcpyAsync(q_out, d_q, sizeof(double) * N, cudaMemcpyDeviceToHost, stream));
    if (J_out) RP_CUDA(cudaMemcpyAsync(J_out, d_J, sizeof(double) * N * N, cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaStreamSynchronize(stream));
}

}  // namespace rp
