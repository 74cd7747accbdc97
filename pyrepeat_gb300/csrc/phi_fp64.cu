// Plain FP64 Phi -> normal equations: the "plain FP64 GPU fit" comparator.
//
// Per chunk of kept points (Phi is held for one chunk only):
//   T[m][:]  = [cos(k.g_m) | sin(k.g_m)]            (FP64, exact per-axis phases)
//   B[a][:]  = [w_k cos(k.r_a) | w_k sin(k.r_a)]    (FP64, once per fit)
//   Phi      = T B^T                                 (cuBLAS DGEMM, native FP64)
//   Phi     += sum_s [r <= Rc] erfc(sqrt(alpha) r)/r (FP64 kernel, repeat.py:944-966)
//   Phi_c    = Phi - c  (c = column means of the first chunk: a per-column shift,
//              exactly corrected afterwards, so A needs no large cancellation)
//   G += Phi_c^T Phi_c, r += Phi_c^T Vc              (cuBLAS DGEMM / DGEMV)
// Finally A = G - s s^T / M, b = r - s sum(Vc) / M with s = sum_m Phi_c[m,:]
// (= sum_phi - M c); this is repeat.py:2266-2276's mean correction written for
// the shifted columns.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace rp {
namespace {

__global__ void realspace_fp64_kernel(const int32_t *__restrict__ kept, long long m0, long long rows,
                                      const double *__restrict__ axis, int nx, int ny,
                                      const double *__restrict__ atoms, int N, const double *__restrict__ shifts,
                                      int S, int zero_idx, double rc, double sa, double *__restrict__ phi) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * N) return;
    long long m = t / N;
    int a = (int)(t - m * N);
    int f = kept[m0 + m];
    int layer = nx * ny;
    int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
    double g[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) g[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)l * axis[6 + d];
    double acc = 0.0;
    for (int s = 0; s < S; ++s) {
        double ex = g[0] - (atoms[3 * a] + shifts[3 * s]);
        double ey = g[1] - (atoms[3 * a + 1] + shifts[3 * s + 1]);
        double ez = g[2] - (atoms[3 * a + 2] + shifts[3 * s + 2]);
        double r = sqrt(ex * ex + ey * ey + ez * ez);
        if (!(r <= rc)) continue;
        if (s == zero_idx && !(r > 1e-10)) continue;
        acc += erfc(sa * r) / r;
    }
    phi[t] += acc;
}

// Column sums of a row-major rows x cols block (ld), FP64, deterministic:
// stage 1 sums fixed row slabs per column; stage 2 adds the slabs in order.
constexpr int kSlab = 256;
__global__ void colsum_stage1(const double *__restrict__ X, long long rows, int cols, int ld,
                              double *__restrict__ part) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    long long r0 = (long long)blockIdx.y * kSlab;
    if (c >= cols) return;
    long long r1 = min(r0 + kSlab, rows);
    double s = 0.0;
    for (long long r = r0; r < r1; ++r) s += X[r * ld + c];
    part[(size_t)blockIdx.y * cols + c] = s;
}
__global__ void colsum_stage2(const double *__restrict__ part, int nslab, int cols, double *__restrict__ out,
                              int accumulate) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    double s = 0.0;
    for (int k = 0; k < nslab; ++k) s += part[(size_t)k * cols + c];
    out[c] = accumulate ? out[c] + s : s;
}

__global__ void shift_columns_kernel(double *__restrict__ X, long long rows, int cols,
                                     const double *__restrict__ c) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * cols) return;
    X[t] -= c[t % cols];
}

__global__ void set_mean_kernel(const double *__restrict__ sums, int n, double inv, double *__restrict__ c) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) c[t] = sums[t] * inv;
}

__global__ void finish_kernel(const double *__restrict__ G, const double *__restrict__ r,
                              const double *__restrict__ s, const double *__restrict__ sumV, long long M, int N,
                              double *__restrict__ A, double *__restrict__ b) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double invM = 1.0 / (double)M;
    if (t < (long long)N * N) {
        int i = (int)(t / N), j = (int)(t - (long long)i * N);
        A[t] = G[t] - s[i] * s[j] * invM;
    }
    if (t < N) b[t] = r[t] - s[t] * (*sumV) * invM;
}

__global__ void shifted_sums_kernel(const double *__restrict__ sphi, const double *__restrict__ c, long long M,
                                    int N, double *__restrict__ s) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < N) s[t] = sphi[t] - (double)M * c[t];
}

}  // namespace

void column_sums_fp64(const double *X, int64_t rows, int cols, int ld, double *out, bool accumulate, rp_ctx *ctx,
                      cudaStream_t s) {
    int nslab = (int)((rows + kSlab - 1) / kSlab);
    if (nslab == 0) {
        if (!accumulate) RP_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * cols, s));
        return;
    }
    double *part = ctx->buf_t<double>("colsum_part", (size_t)nslab * cols);
    dim3 g1(ceil_div(cols, 128), nslab);
    colsum_stage1<<<g1, 128, 0, s>>>(X, rows, cols, ld, part);
    RP_LAUNCH_CHECK();
    colsum_stage2<<<ceil_div(cols, 128), 128, 0, s>>>(part, nslab, cols, out, accumulate ? 1 : 0);
    RP_LAUNCH_CHECK();
}

void finish_normal_equations(const double *G, const double *r, const double *s_c, double *sumV_dev, int64_t M, int N,
                             double *A, double *b, cudaStream_t s) {
    long long n = std::max<long long>((long long)N * N, N);
    finish_kernel<<<ceil_div(n, 256), 256, 0, s>>>(G, r, s_c, sumV_dev, M, N, A, b);
    RP_LAUNCH_CHECK();
}

void gram_fp64(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
               const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
               cudaStream_t stream) {
    RP_REQUIRE(N > 0 && M > 0, "rp_gram: need N > 0 and M > 0");
    const int K = ew->K, K2 = 2 * ew->K;
    std::vector<double> sh;
    int zero_idx = -1;
    prune_shifts(ew, atoms, N, sh, zero_idx);
    const int S = (int)(sh.size() / 3);
    double *d_atoms = ctx->buf_t<double>("g_atoms", 3 * (size_t)N);
    double *d_shifts = ctx->buf_t<double>("g_shifts", sh.size());
    double *d_axis = ctx->buf_t<double>("g_axis", 9);
    RP_CUDA(cudaMemcpyAsync(d_atoms, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_shifts, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_axis, ew->grid.axis, sizeof(double) * 9, cudaMemcpyHostToDevice, stream));

    double *B = ctx->buf_t<double>("g64_B", (size_t)N * K2);
    if (K > 0) atom_tables_fp64(ew, d_atoms, N, B, K2, stream);

    // chunk rows so T and Phi stay within ~2 GB together
    const size_t row_bytes = sizeof(double) * ((size_t)K2 + N);
    int64_t chunk = std::max<int64_t>(256, (int64_t)((size_t)2 << 30) / (int64_t)row_bytes);
    chunk = std::min<int64_t>(chunk, M);
    double *T = ctx->buf_t<double>("g64_T", (size_t)chunk * K2);
    double *P = ctx->buf_t<double>("g64_P", (size_t)chunk * N);
    double *G = ctx->buf_t<double>("g64_G", (size_t)N * N);
    double *r = ctx->buf_t<double>("g64_r", (size_t)N);
    double *sphi = sum_phi_dev ? sum_phi_dev : ctx->buf_t<double>("g64_sphi", (size_t)N);
    double *csum = ctx->buf_t<double>("g64_csum", (size_t)N);
    double *c = ctx->buf_t<double>("g64_c", (size_t)N);
    double *s_c = ctx->buf_t<double>("g64_sc", (size_t)N);
    double *sumV = ctx->buf_t<double>("g64_sumV", 1);
    RP_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * N * N, stream));
    RP_CUDA(cudaMemsetAsync(r, 0, sizeof(double) * N, stream));
    RP_CUDA(cudaMemsetAsync(sphi, 0, sizeof(double) * N, stream));

    cublasHandle_t h = ctx->blas();
    RP_CUBLAS(cublasSetStream(h, stream));
    const double one = 1.0, zero = 0.0;
    for (int64_t m0 = 0; m0 < M; m0 += chunk) {
        const int64_t rows = std::min<int64_t>(chunk, M - m0);
        if (K > 0) {
            {
                StageTimer tt(ctx, "fp64_tables", stream);
                grid_tables_fp64(ew, kept_idx_dev, m0, rows, T, K2, stream);
            }
            StageTimer tt(ctx, "fp64_recip_dgemm", stream);
            RP_CUBLAS(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, N, (int)rows, K2, &one, B, K2, T, K2, &zero, P, N));
        } else {  // the non-periodic basis has no reciprocal part
            RP_CUDA(cudaMemsetAsync(P, 0, sizeof(double) * (size_t)rows * N, stream));
        }
        StageTimer t_r(ctx, "fp64_realspace", stream);
        realspace_fp64_kernel<<<ceil_div(rows * N, 128), 128, 0, stream>>>(
            kept_idx_dev, m0, rows, d_axis, ew->grid.n_grid[0], ew->grid.n_grid[1], d_atoms, N, d_shifts, S,
            zero_idx, ew->cutoff, ew->sqrt_alpha, P);
        RP_LAUNCH_CHECK();
        column_sums_fp64(P, rows, N, N, csum, false, ctx, stream);
        // sphi += csum (accumulating stage-2 output keeps the order fixed)
        {
            const double *cs = csum;
            RP_CUBLAS(cublasDaxpy(h, N, &one, cs, 1, sphi, 1));
        }
        if (m0 == 0) {
            set_mean_kernel<<<ceil_div(N, 128), 128, 0, stream>>>(csum, N, 1.0 / (double)rows, c);
            RP_LAUNCH_CHECK();
        }
        shift_columns_kernel<<<ceil_div(rows * N, 256), 256, 0, stream>>>(P, rows, N, c);
        RP_LAUNCH_CHECK();
        // column-major view: X = P^T is N x rows with ld N;  G += X X^T,  r += X Vc
        StageTimer t_g(ctx, "fp64_gram_dgemm", stream);
        RP_CUBLAS(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, N, N, (int)rows, &one, P, N, P, N, &one, G, N));
        RP_CUBLAS(cublasDgemv(h, CUBLAS_OP_N, N, (int)rows, &one, P, N, Vc_dev + m0, 1, &one, r, 1));
    }
    column_sums_fp64(Vc_dev, M, 1, 1, sumV, false, ctx, stream);
    shifted_sums_kernel<<<ceil_div(N, 128), 128, 0, stream>>>(sphi, c, M, N, s_c);
    RP_LAUNCH_CHECK();
    finish_normal_equations(G, r, s_c, sumV, M, N, A_dev, b_dev, stream);
    (void)K;
}

}  // namespace rp
