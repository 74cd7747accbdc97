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
// Stage C costs 2 KMAX real multiply-adds per point-atom instead of the 4 K of a dense
// point x k table contraction (K = 754 at KMAX 7): ~50x fewer operations, so the
// whole sum runs on the FP32 pipe instead of as a tensor-core GEMM.  The weights W
// and stage A are double-float (exact to ~2^-44); stages B and C use FP32 products
// (unbiased rounding, ~1e-7 relative like the FP32 real-space terms), stored as
// float2 E rows.
// Indices n1 in [0, P], n2, n3 in [-P, P] with P = KMAX - 1 (the k-set keeps
// n1^2 + n2^2 + n3^2 < KMAX^2); stored with offset P on n2 and n3.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "df.cuh"

namespace rp {
namespace {

struct Rec9 {
    double b[9];
};

// U[a][d][n + P] = e^{-i n (b_d . r_a)} for n in [-P, P]: the per-axis atom phases, so that
// e^{-i k.r_a} = U[a][0][n1] U[a][1][n2] U[a][2][n3] needs 3 (2P+1) sincos per atom instead of K.
__global__ void atom_phases_kernel(const double *__restrict__ atoms, int N, Rec9 rb, int P,
                                   double2 *__restrict__ U) {
    const int nw = 2 * P + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * 3 * nw) return;
    const int n = t % nw - P, d = (t / nw) % 3, a = t / (3 * nw);
    const double *p = atoms + 3 * a;
    const double th = (p[0] * rb.b[3 * d] + p[1] * rb.b[3 * d + 1]) + p[2] * rb.b[3 * d + 2];
    double s, c;
    sincos((double)n * th, &s, &c);
    U[t] = make_double2(c, -s);
}

__device__ __forceinline__ double2 cmul(double2 x, double2 y) {
    return make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

// W[col][n2'][n3'][n1] = w_k e^{-i k.r} (col = atom), or sum_a q_a w_k e^{-i k.r_a} (one
// charge-weighted column when q != nullptr); FP64, stored as double-float
__global__ void build_w_kernel(const int *__restrict__ kidx, const double *__restrict__ kcoef, int K, int P,
                               const double2 *__restrict__ U, const double *__restrict__ q, int N, int ncols,
                               float4 *__restrict__ W) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ncols * K) return;
    const int col = (int)(t / K), k = (int)(t - (long long)col * K);
    const int n1c = P + 1, nw = 2 * P + 1;
    const int n1 = kidx[3 * k], n2 = kidx[3 * k + 1] + P, n3 = kidx[3 * k + 2] + P;
    double2 z;
    if (q == nullptr) {
        const double2 *u = U + (size_t)col * 3 * nw;
        z = cmul(cmul(u[n1 + P], u[nw + n2]), u[2 * nw + n3]);
    } else {
        z = make_double2(0.0, 0.0);
        for (int a = 0; a < N; ++a) {
            const double2 *u = U + (size_t)a * 3 * nw;
            const double2 v = cmul(cmul(u[n1 + P], u[nw + n2]), u[2 * nw + n3]);
            z.x += q[a] * v.x;
            z.y += q[a] * v.y;
        }
    }
    const double w = kcoef[k];
    W[(((long long)col * nw + n2) * nw + n3) * n1c + n1] = dfa::split(w * z.x, w * z.y);
}

// Each thread produces up to kN1B consecutive n1 outputs of one (plane, n2, column) or
// (row, column): kN1B independent accumulator chains, and the shared phase factor is
// loaded once per term.
constexpr int kN1B = 8;

// Stage A, one thread per (n2, column, n1 block, plane l) with l fastest: a warp reads
// one W row (broadcast) and consecutive ez phases (coalesced).
__global__ void recip_stage_a_kernel(const float4 *__restrict__ W, const float4 *__restrict__ EZ, int ncols, int P,
                                     int nz, float4 *__restrict__ F) {
    extern __shared__ float4 ezs[];  // the whole ez table [nw][nz], read once per CTA
    const int n1c = P + 1, nw = 2 * P + 1, nb = (n1c + kN1B - 1) / kN1B;
    for (int q = threadIdx.x; q < nw * nz; q += blockDim.x) ezs[q] = EZ[q];
    __syncthreads();
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nz * nw * ncols * nb) return;
    const int l = (int)(t % nz);
    t /= nz;
    const int b = (int)(t % nb);
    t /= nb;
    const int a = (int)(t % ncols);
    const int n2 = (int)(t / ncols);
    const int n10 = b * kN1B, cnt = min(kN1B, n1c - n10);
    dfa::acc re[kN1B], im[kN1B];
#pragma unroll
    for (int u = 0; u < kN1B; ++u) re[u] = im[u] = dfa::acc{0.f, 0.f};
    const float4 *w = W + ((long long)a * nw + n2) * nw * n1c + n10;
    for (int n3 = 0; n3 < nw; ++n3) {
        const float4 z = ezs[n3 * nz + l];
        const float4 *wr = w + (long long)n3 * n1c;
#pragma unroll
        for (int u = 0; u < kN1B; ++u)
            if (u < cnt) dfa::cmac(re[u], im[u], z, wr[u]);
    }
    float4 *o = F + (((long long)l * nw + n2) * ncols + a) * n1c + n10;
#pragma unroll
    for (int u = 0; u < kN1B; ++u)
        if (u < cnt) o[u] = dfa::pack(re[u], im[u]);
}

// Stage B, one CTA per (plane l, block of `ab` columns): the plane's F slab for those
// columns is staged in shared memory once and reused by every row j of the plane.
__global__ void __launch_bounds__(128) recip_stage_b_kernel(const float4 *__restrict__ F,
                                                            const float4 *__restrict__ EY, int ncols, int P, int ny,
                                                            int ab, float2 *__restrict__ E) {
    extern __shared__ float4 fs[];  // [nw][ab][n1c] F slab, then the ey table [nw][ny]
    const int n1c = P + 1, nw = 2 * P + 1;
    const int l = blockIdx.y, a0 = blockIdx.x * ab, na = min(ab, ncols - a0);
    const int slab = nw * ab * n1c;
    float4 *eys = fs + slab;
    for (int t = threadIdx.x; t < slab; t += blockDim.x) {
        const int n1 = t % n1c, u = t / n1c, a = u % ab, n2 = u / ab;
        fs[t] = (a < na) ? F[(((long long)l * nw + n2) * ncols + a0 + a) * n1c + n1] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int q = threadIdx.x; q < nw * ny; q += blockDim.x) eys[q] = EY[q];
    __syncthreads();
    const int items = na * ny;  // (a, j), j fastest: a warp reads one column's slab (broadcast)
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int a = it / ny, j = it - a * ny;
        float2 *o = E + (((long long)l * ny + j) * ncols + a0 + a) * n1c;
        for (int n10 = 0; n10 < n1c; n10 += kN1B) {
            const int cnt = min(kN1B, n1c - n10);
            float re[kN1B], im[kN1B];
#pragma unroll
            for (int u = 0; u < kN1B; ++u) re[u] = im[u] = 0.f;
            for (int n2 = 0; n2 < nw; ++n2) {
                const float4 y = eys[n2 * ny + j];
                const float4 *fr = fs + ((size_t)n2 * ab + a) * n1c + n10;
#pragma unroll
                for (int u = 0; u < kN1B; ++u)
                    if (u < cnt) dfa::cmac32(re[u], im[u], y, fr[u]);
            }
#pragma unroll
            for (int u = 0; u < kN1B; ++u)
                if (u < cnt) o[n10 + u] = make_float2(re[u], im[u]);
        }
    }
}

}  // namespace

size_t recip_rows_bytes(const rp_ewald *ew, int ncols) {
    const int P = ew->kmax - 1, n1c = P + 1;
    const long long nrows = (long long)ew->grid.n_grid[1] * ew->grid.n_grid[2];
    return sizeof(float2) * (size_t)nrows * ncols * n1c;
}

void recip_rows(rp_ctx *ctx, const rp_ewald *ew, const double *d_atoms, const double *d_q, int N, float2 *E,
                cudaStream_t stream, const std::string &slot) {
    const int P = ew->kmax - 1, n1c = P + 1, nw = 2 * P + 1;
    const int ny = ew->grid.n_grid[1], nz = ew->grid.n_grid[2];
    const int ncols = d_q ? 1 : N;
    const long long nrows = (long long)ny * nz;
    if (ew->K == 0) {
        RP_CUDA(cudaMemsetAsync(E, 0, recip_rows_bytes(ew, ncols), stream));
        return;
    }
    const size_t nW = (size_t)ncols * nw * nw * n1c, nF = (size_t)nz * nw * ncols * n1c;
    float4 *W = ctx->buf_t<float4>("rs_W" + slot, nW);
    float4 *F = ctx->buf_t<float4>("rs_F" + slot, nF);
    double2 *U = ctx->buf_t<double2>("rs_U" + slot, (size_t)N * 3 * nw);
    RP_CUDA(cudaMemsetAsync(W, 0, sizeof(float4) * nW, stream));
    Rec9 rb;
    for (int q = 0; q < 9; ++q) rb.b[q] = ew->rec[q];
    atom_phases_kernel<<<ceil_div((long long)N * 3 * nw, 128), 128, 0, stream>>>(d_atoms, N, rb, P, U);
    RP_LAUNCH_CHECK();
    const long long nk = (long long)ncols * ew->K;
    build_w_kernel<<<ceil_div(nk, 128), 128, 0, stream>>>(ew->d_kidx, ew->d_kcoef, ew->K, P, U, d_q, N, ncols, W);
    RP_LAUNCH_CHECK();
    const int nb = (n1c + kN1B - 1) / kN1B;
    const size_t smem_a = sizeof(float4) * (size_t)nw * nz;
    RP_REQUIRE(smem_a <= (200u << 10), "recip_rows: grid too large along z for KMAX");
    static size_t attr_a = 0;
    if (smem_a > (48u << 10) && smem_a > attr_a) {
        RP_CUDA(cudaFuncSetAttribute(recip_stage_a_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_a));
        attr_a = smem_a;
    }
    recip_stage_a_kernel<<<ceil_div((long long)nz * nw * ncols * nb, 128), 128, smem_a, stream>>>(W, ew->d_ezf, ncols,
                                                                                                  P, nz, F);
    RP_LAUNCH_CHECK();
    // stage B: as many columns per CTA as fit 96 KB of shared memory (at most 16)
    const size_t col_bytes = sizeof(float4) * (size_t)nw * n1c;
    const int ab = (int)std::max<size_t>(1, std::min<size_t>(16, (96u << 10) / col_bytes));
    const size_t smem = col_bytes * ab + sizeof(float4) * (size_t)nw * ny;
    RP_REQUIRE(smem <= (200u << 10), "recip_rows: KMAX too large");
    static size_t attr = 0;
    if (smem > (48u << 10) && smem > attr) {
        RP_CUDA(cudaFuncSetAttribute(recip_stage_b_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = smem;
    }
    recip_stage_b_kernel<<<dim3(ceil_div(ncols, ab), nz), 128, smem, stream>>>(F, ew->d_eyf, ncols, P, ny, ab, E);
    RP_LAUNCH_CHECK();
}

}  // namespace rp
