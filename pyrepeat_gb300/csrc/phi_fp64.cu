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

// Real-space sum in FP64 (repeat.py:944-966) over tiles of kRsPts kept points x kRsAtoms
// atoms.  For each chunk of up to kRsShiftChunk shifts, the CTA first drops, per atom,
// every shift whose image lies farther than Rc + 1e-3 Bohr from the bounding box of its
// points (an FP32 test: FP32 rounding of the coordinates moves a distance by < 1e-4
// Bohr here, so no image within Rc is dropped); each thread then tests the remaining
// images of each atom against its point in FP32 with the same margin and evaluates the
// survivors in FP64 with the reference's expressions.  Every image within Rc is summed,
// in shift order, exactly as by a loop over all shifts, while the FP64 pipe (a small
// fraction of the FP32 rate on this part) only sees the few images near each point.
// The sums are accumulated in a shared-memory tile and added into phi[m][a] (row-major,
// ld N) with coalesced stores.
constexpr int kRsPts = 128;
constexpr int kRsAtoms = 16;
constexpr int kRsShiftChunk = 128;
__global__ void __launch_bounds__(kRsPts) realspace_fp64_kernel(
    const int32_t *__restrict__ kept, long long m0, long long rows, const double *__restrict__ axis, int nx, int ny,
    const double *__restrict__ atoms, int N, const double *__restrict__ shifts, int S, int zero_idx, double rc,
    double sa, double *__restrict__ phi) {
    extern __shared__ float4 rs_cand[];  // [kRsAtoms][kRsShiftChunk] image (x, y, z) in FP32, shift index
    __shared__ double tile[kRsAtoms][kRsPts + 1];
    __shared__ int ncand[kRsAtoms];
    __shared__ float bb[2][3][kRsPts / 32];
    const long long mb = (long long)blockIdx.x * kRsPts;
    const int a0 = blockIdx.y * kRsAtoms, na = min(kRsAtoms, N - a0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long m = mb + threadIdx.x;
    const bool valid = m < rows;
    const int f = kept[m0 + (valid ? m : mb)];  // a lane past the end repeats the tile's first point
    const int layer = nx * ny;
    const int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
    double g[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) g[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)l * axis[6 + d];
    const float gf[3] = {(float)g[0], (float)g[1], (float)g[2]};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float mn = gf[d], mx = gf[d];
        for (int o = 16; o > 0; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (lane == 0) {
            bb[0][d][warp] = mn;
            bb[1][d][warp] = mx;
        }
    }
    for (int a = 0; a < kRsAtoms; ++a) tile[a][threadIdx.x] = 0.0;
    __syncthreads();
    float bmin[3], bmax[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        bmin[d] = bb[0][d][0];
        bmax[d] = bb[1][d][0];
        for (int w = 1; w < kRsPts / 32; ++w) {
            bmin[d] = fminf(bmin[d], bb[0][d][w]);
            bmax[d] = fmaxf(bmax[d], bb[1][d][w]);
        }
    }
    const float reach = (float)rc + 1e-3f, reach2 = reach * reach;
    for (int s_lo = 0; s_lo < S; s_lo += kRsShiftChunk) {
        const int s_hi = min(S, s_lo + kRsShiftChunk);
        for (int a = warp; a < na; a += kRsPts / 32) {
            int base = 0;
            const double *pa = atoms + 3 * (size_t)(a0 + a);
            for (int s0 = s_lo; s0 < s_hi; s0 += 32) {
                const int s = s0 + lane;
                bool keep = false;
                float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                if (s < s_hi) {
                    q = make_float4((float)(pa[0] + shifts[3 * s]), (float)(pa[1] + shifts[3 * s + 1]),
                                    (float)(pa[2] + shifts[3 * s + 2]), __int_as_float(s));
                    const float dx = fmaxf(fmaxf(bmin[0] - q.x, q.x - bmax[0]), 0.f);
                    const float dy = fmaxf(fmaxf(bmin[1] - q.y, q.y - bmax[1]), 0.f);
                    const float dz = fmaxf(fmaxf(bmin[2] - q.z, q.z - bmax[2]), 0.f);
                    keep = dx * dx + dy * dy + dz * dz <= reach2;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) rs_cand[a * kRsShiftChunk + base + __popc(bal & ((1u << lane) - 1u))] = q;
                base += __popc(bal);
            }
            if (lane == 0) ncand[a] = base;
        }
        __syncthreads();
        for (int a = 0; a < na; ++a) {
            const double *pa = atoms + 3 * (size_t)(a0 + a);
            double acc = tile[a][threadIdx.x];
            const int nc = ncand[a];
            for (int c = 0; c < nc; ++c) {
                const float4 h = rs_cand[a * kRsShiftChunk + c];
                const float fx = gf[0] - h.x, fy = gf[1] - h.y, fz = gf[2] - h.z;
                if (fx * fx + fy * fy + fz * fz > reach2) continue;
                const int s = __float_as_int(h.w);
                const double ex = g[0] - (pa[0] + shifts[3 * s]);
                const double ey = g[1] - (pa[1] + shifts[3 * s + 1]);
                const double ez = g[2] - (pa[2] + shifts[3 * s + 2]);
                const double r = sqrt(ex * ex + ey * ey + ez * ez);
                if (!(r <= rc)) continue;
                if (s == zero_idx && !(r > 1e-10)) continue;
                acc += erfc(sa * r) / r;
            }
            tile[a][threadIdx.x] = acc;
        }
        __syncthreads();
    }
    // tile[a][t] -> phi[(mb + t) * N + a0 + a]: kRsAtoms consecutive doubles per point
    for (int e = threadIdx.x; e < kRsPts * kRsAtoms; e += kRsPts) {
        const int t = e / kRsAtoms, a = e - t * kRsAtoms;
        if (mb + t < rows && a < na) phi[(mb + t) * N + a0 + a] += tile[a][t];
    }
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

// G (N x N, column-major) holds its upper triangle (row <= column): copy it to the lower
__global__ void mirror_upper_kernel(double *__restrict__ G, int N) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * N) return;
    const int c = (int)(t / N), r = (int)(t - (long long)c * N);
    if (r > c) G[t] = G[(size_t)r * N + c];
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
        {
            const size_t smem = sizeof(float4) * kRsAtoms * kRsShiftChunk;  // 32 KB of candidates
            // with the 16.5 KB static tile the block passes the 48 KB default: opt in
            smem_optin((const void *)realspace_fp64_kernel, 64 * 1024);
            realspace_fp64_kernel<<<dim3(ceil_div(rows, kRsPts), ceil_div(N, kRsAtoms)), kRsPts, smem, stream>>>(
                kept_idx_dev, m0, rows, d_axis, ew->grid.n_grid[0], ew->grid.n_grid[1], d_atoms, N, d_shifts, S,
                zero_idx, ew->cutoff, ew->sqrt_alpha, P);
            RP_LAUNCH_CHECK();
        }
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
        // column-major view: X = P^T is N x rows with ld N;  G += X X^T (one triangle,
        // mirrored after the last chunk),  r += X Vc
        StageTimer t_g(ctx, "fp64_gram_dsyrk", stream);
        RP_CUBLAS(cublasDsyrk(h, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, N, (int)rows, &one, P, N, &one, G, N));
        RP_CUBLAS(cublasDgemv(h, CUBLAS_OP_N, N, (int)rows, &one, P, N, Vc_dev + m0, 1, &one, r, 1));
    }
    mirror_upper_kernel<<<ceil_div((long long)N * N, 256), 256, 0, stream>>>(G, N);
    RP_LAUNCH_CHECK();
    column_sums_fp64(Vc_dev, M, 1, 1, sumV, false, ctx, stream);
    shifted_sums_kernel<<<ceil_div(N, 128), 128, 0, stream>>>(sphi, c, M, N, s_c);
    RP_LAUNCH_CHECK();
    finish_normal_equations(G, r, s_c, sumV, M, N, A_dev, b_dev, stream);
    (void)K;
}

}  // namespace rp
