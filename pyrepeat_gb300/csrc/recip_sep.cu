// Reciprocal-space Ewald sum by separable lattice phases (double-float, FP32 pipe).
//
// The k-sum of the reference (repeat.py:968-981; per point and atom
// sum_k w_k cos(k.(g - r_a)), w_k = kcoef) is evaluated for grid points, and a
// grid point g = i a0 + j a1 + l a2 of an n_x x n_y x n_z grid that spans the cell
// has k.g = 2 pi (n1 i/n_x + n2 j/n_y + n3 l/n_z) exactly for every reciprocal
// vector k = (n1, n2, n3).  With W_a(n) = w_k e^{-i k.r_a} (zero outside the k-set)
//
//   phi_recip(g, a) = Re sum_n1 ex[n1][i] sum_n2 ey[n2][j] sum_n3 ez[n3][l] W_a(n)
//
// is a three-stage separable transform, evaluated as
//   stage A   F[l][n2][a][n1] = sum_n3 ez[n3][l] W[a][n2][n3][n1]       (every grid plane l)
//   stage B   E[r][a][n1]     = sum_n2 ey[n2][j] F[l][n2][a][n1]         (every grid row r = j + l n_y)
//   stage C   phi_recip(m, a) = Re sum_n1 ex[n1][i_m] E[r_m][a][n1]      (per kept point, fused into
//                                                                        the real-space kernel)
// Stage C costs 2 (KMAX) multiply-adds per point-atom instead of the 4 K of a dense
// point x k table contraction (K = 754 at KMAX 7): ~50x fewer operations, so the
// whole sum runs on the FP32 pipe in double-float arithmetic (about 44 bits,
// more than the fit needs) instead of as a low-precision tensor-core GEMM.
// Indices n1 in [0, P], n2, n3 in [-P, P] with P = KMAX - 1 (the k-set keeps
// n1^2 + n2^2 + n3^2 < KMAX^2); stored with offset P on n2 and n3.
#include <cmath>

#include "common.cuh"
#include "df.cuh"

namespace rp {
namespace {

// W[col][n2'][n3'][n1]: col = atom (q == nullptr) or the single charge-weighted column
__global__ void build_w_kernel(const int *__restrict__ kidx, const double *__restrict__ kvec,
                               const double *__restrict__ kcoef, int K, int P, const double *__restrict__ atoms,
                               const double *__restrict__ q, int N, int ncols, float4 *__restrict__ W) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ncols * K) return;
    const int col = (int)(t / K), k = (int)(t - (long long)col * K);
    const int n1c = P + 1, nw = 2 * P + 1;
    double re = 0.0, im = 0.0;
    const double kx = kvec[3 * k], ky = kvec[3 * k + 1], kz = kvec[3 * k + 2];
    if (q == nullptr) {
        const double *p = atoms + 3 * col;
        const double kr = (p[0] * kx + p[1] * ky) + p[2] * kz;
        double s, c;
        sincos(kr, &s, &c);
        re = c;
        im = -s;
    } else {
        for (int a = 0; a < N; ++a) {
            const double *p = atoms + 3 * a;
            const double kr = (p[0] * kx + p[1] * ky) + p[2] * kz;
            double s, c;
            sincos(kr, &s, &c);
            re += q[a] * c;
            im -= q[a] * s;
        }
    }
    const double w = kcoef[k];
    const int n1 = kidx[3 * k], n2 = kidx[3 * k + 1] + P, n3 = kidx[3 * k + 2] + P;
    W[(((long long)col * nw + n2) * nw + n3) * n1c + n1] = dfa::split(w * re, w * im);
}

__global__ void recip_stage_a_kernel(const float4 *__restrict__ W, const float4 *__restrict__ EZ, int ncols, int P,
                                     int nz, float4 *__restrict__ F) {
    const int n1c = P + 1, nw = 2 * P + 1;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nz * nw * ncols * n1c) return;
    const int n1 = (int)(t % n1c);
    t /= n1c;
    const int a = (int)(t % ncols);
    t /= ncols;
    const int n2 = (int)(t % nw);
    const int l = (int)(t / nw);
    dfa::acc re{0.f, 0.f}, im{0.f, 0.f};
    const float4 *w = W + ((long long)a * nw + n2) * nw * n1c + n1;
    for (int n3 = 0; n3 < nw; ++n3) dfa::cmac(re, im, EZ[(long long)n3 * nz + l], w[(long long)n3 * n1c]);
    F[(((long long)l * nw + n2) * ncols + a) * n1c + n1] = dfa::pack(re, im);
}

__global__ void recip_stage_b_kernel(const float4 *__restrict__ F, const float4 *__restrict__ EY, int ncols, int P,
                                     int ny, long long nrows, float4 *__restrict__ E) {
    const int n1c = P + 1, nw = 2 * P + 1;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrows * ncols * n1c) return;
    const int n1 = (int)(t % n1c);
    long long u = t / n1c;
    const int a = (int)(u % ncols);
    const long long r = u / ncols;
    const int j = (int)(r % ny), l = (int)(r / ny);
    dfa::acc re{0.f, 0.f}, im{0.f, 0.f};
    const float4 *f = F + ((long long)l * nw * ncols + a) * n1c + n1;
    for (int n2 = 0; n2 < nw; ++n2) dfa::cmac(re, im, EY[(long long)n2 * ny + j], f[(long long)n2 * ncols * n1c]);
    E[t] = dfa::pack(re, im);
}

}  // namespace

size_t recip_rows_bytes(const rp_ewald *ew, int ncols) {
    const int P = ew->kmax - 1, n1c = P + 1;
    const long long nrows = (long long)ew->grid.n_grid[1] * ew->grid.n_grid[2];
    return sizeof(float4) * (size_t)nrows * ncols * n1c;
}

void recip_rows(rp_ctx *ctx, const rp_ewald *ew, const double *d_atoms, const double *d_q, int N, float4 *E,
                cudaStream_t stream) {
    const int P = ew->kmax - 1, n1c = P + 1, nw = 2 * P + 1;
    const int ny = ew->grid.n_grid[1], nz = ew->grid.n_grid[2];
    const int ncols = d_q ? 1 : N;
    const long long nrows = (long long)ny * nz;
    if (ew->K == 0) {
        RP_CUDA(cudaMemsetAsync(E, 0, recip_rows_bytes(ew, ncols), stream));
        return;
    }
    const size_t nW = (size_t)ncols * nw * nw * n1c, nF = (size_t)nz * nw * ncols * n1c;
    float4 *W = ctx->buf_t<float4>("rs_W", nW);
    float4 *F = ctx->buf_t<float4>("rs_F", nF);
    RP_CUDA(cudaMemsetAsync(W, 0, sizeof(float4) * nW, stream));
    const long long nk = (long long)ncols * ew->K;
    build_w_kernel<<<ceil_div(nk, 128), 128, 0, stream>>>(ew->d_kidx, ew->d_kvec, ew->d_kcoef, ew->K, P, d_atoms, d_q,
                                                         N, ncols, W);
    RP_LAUNCH_CHECK();
    recip_stage_a_kernel<<<ceil_div((long long)nF, 256), 256, 0, stream>>>(W, ew->d_ezf, ncols, P, nz, F);
    RP_LAUNCH_CHECK();
    const long long nE = nrows * ncols * n1c;
    recip_stage_b_kernel<<<ceil_div(nE, 256), 256, 0, stream>>>(F, ew->d_eyf, ncols, P, ny, nrows, E);
    RP_LAUNCH_CHECK();
}

}  // namespace rp
