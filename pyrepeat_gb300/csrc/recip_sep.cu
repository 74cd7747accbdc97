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
// are computed in double-float (~2^-44) and stored rounded to FP32; stages A, B and C
// use FP32 products (unbiased rounding, ~1e-7 relative like the FP32 real-space terms;
// measured 2.6-3.1e-7 of max|Phi| against FP64), with F and E stored as float2.
// Indices n1 in [0, P], n2, n3 in [-P, P] with P = KMAX - 1 (the k-set keeps
// n1^2 + n2^2 + n3^2 < KMAX^2); stored with offset P on n2 and n3.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "df.cuh"

namespace rp {
namespace {

// One fit's reciprocal rows: its tables, scratch and output.  A launch carries up to
// kRecipJobs of them by value; every kernel below runs the blocks of all its jobs, job j
// owning blocks [blk[k][j], blk[k][j+1]) of kernel k, so a pipeline group of cubes costs one
// launch per stage instead of one per cube.
struct RecipJob {
    const double *atoms;   // [3N]
    const double *q;       // [N] charges (one weighted column) or nullptr (a column per atom)
    const int *kidx;       // [3K]
    const double *kcoef;   // [K]
    const float4 *EY, *EZ; // double-float phases of the grid rows / planes
    double2 *U;
    float4 *Udf;
    float2 *kdf;           // [K] the weights w_k as double-float (hi, lo), split once per fit
    float2 *W, *F, *E;
    double rb[9];          // reciprocal basis (rows)
    int N, ncols, K, P, ny, nz, ab;
};
constexpr int kRecipJobs = 64;
struct RecipLaunch {
    int n;
    int blk[kRecipJobs + 1];  // block offsets of the jobs in this kernel's grid
    RecipJob job[kRecipJobs];
};

// the job that owns block b (binary search over the offsets)
__device__ __forceinline__ int recip_job_of(const RecipLaunch &L, int b) {
    int lo = 0, hi = L.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.blk[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// U[a][d][n + P] = e^{-i n (b_d . r_a)} for n in [-P, P]: the per-axis atom phases, so that
// e^{-i k.r_a} = U[a][0][n1] U[a][1][n2] U[a][2][n3] needs 3 (2P+1) sincos per atom instead of K.
__global__ void atom_phases_kernel(const __grid_constant__ RecipLaunch L) {
    const int jb = recip_job_of(L, blockIdx.x);
    const RecipJob &J = L.job[jb];
    const int P = J.P, nw = 2 * P + 1;
    const int t = (blockIdx.x - L.blk[jb]) * blockDim.x + threadIdx.x;
    // the weights' double-float split for build_w_kernel, whose threads would otherwise each
    // run the FP64 conversions (the FP64 pipe is a small fraction of the FP32 rate here)
    const int nthreads = (L.blk[jb + 1] - L.blk[jb]) * blockDim.x;
    for (int k = t; k < J.K; k += nthreads) {
        const double w = J.kcoef[k];
        const float wh = (float)w;
        J.kdf[k] = make_float2(wh, (float)(w - (double)wh));
    }
    if (t >= J.N * 3 * nw) return;
    const int n = t % nw - P, d = (t / nw) % 3, a = t / (3 * nw);
    const double *p = J.atoms + 3 * a;
    const double th = (p[0] * J.rb[3 * d] + p[1] * J.rb[3 * d + 1]) + p[2] * J.rb[3 * d + 2];
    double s, c;
    sincos((double)n * th, &s, &c);
    J.U[t] = make_double2(c, -s);
    J.Udf[t] = dfa::split(c, -s);
}

__device__ __forceinline__ double2 cmul(double2 x, double2 y) {
    return make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

// W[col][n2'][n3'][n1] = w_k e^{-i k.r} (col = atom), or sum_a q_a w_k e^{-i k.r_a} (one
// charge-weighted column when q != nullptr), stored rounded to FP32.  Per atom the two
// phase products and the weight are double-float products on the FP32 pipe (~2^-44
// relative); the charge-weighted sum stays FP64.  (W is zero outside the k-set: the host
// clears it before this launch.)
__global__ void build_w_kernel(const __grid_constant__ RecipLaunch L) {
    const int jb = recip_job_of(L, blockIdx.x);
    const RecipJob &J = L.job[jb];
    const long long t = (long long)(blockIdx.x - L.blk[jb]) * blockDim.x + threadIdx.x;
    const int K = J.K, P = J.P;
    if (t >= (long long)J.ncols * K) return;
    const int col = (int)(t / K), k = (int)(t - (long long)col * K);
    const int n1c = P + 1, nw = 2 * P + 1;
    const int n1 = J.kidx[3 * k], n2 = J.kidx[3 * k + 1] + P, n3 = J.kidx[3 * k + 2] + P;
    float2 *out = J.W + (((long long)col * nw + n2) * nw + n3) * n1c + n1;
    if (J.q == nullptr) {
        const float4 *u = J.Udf + (size_t)col * 3 * nw;
        dfa::acc re{0.f, 0.f}, im{0.f, 0.f};
        dfa::cmac(re, im, u[n1 + P], u[nw + n2]);
        const float4 z12 = dfa::pack(re, im);
        re = im = dfa::acc{0.f, 0.f};
        dfa::cmac(re, im, z12, u[2 * nw + n3]);
        const float4 z3 = dfa::pack(re, im);
        const float2 wk = J.kdf[k];
        const float wh = wk.x, wl = wk.y;
        re = im = dfa::acc{0.f, 0.f};
        dfa::mac(re, wh, wl, z3.x, z3.y);
        dfa::mac(im, wh, wl, z3.z, z3.w);
        *out = make_float2(dfa::norm(re).x, dfa::norm(im).x);
        return;
    }
    double2 z = make_double2(0.0, 0.0);
    for (int a = 0; a < J.N; ++a) {
        const double2 *u = J.U + (size_t)a * 3 * nw;
        const double2 v = cmul(cmul(u[n1 + P], u[nw + n2]), u[2 * nw + n3]);
        z.x += J.q[a] * v.x;
        z.y += J.q[a] * v.y;
    }
    const double w = J.kcoef[k];
    *out = make_float2((float)(w * z.x), (float)(w * z.y));
}

// Each stage-A thread produces up to kN1B consecutive n1 outputs of one (plane, n2,
// column): kN1B independent accumulator chains, and the shared phase factor is
// loaded once per term.
constexpr int kN1B = 8;

// Stage A, one thread per (n2, column, n1 block, plane l) with l fastest: a warp reads
// one W row (broadcast) and consecutive ez phases (coalesced); FP32 products.
__global__ void recip_stage_a_kernel(const __grid_constant__ RecipLaunch L) {
    extern __shared__ float2 ezs[];  // the job's ez table [nw][nz] (FP32), read once per CTA
    const int jb = recip_job_of(L, blockIdx.x);
    const RecipJob &J = L.job[jb];
    const int P = J.P, nz = J.nz, ncols = J.ncols;
    const int n1c = P + 1, nw = 2 * P + 1, nb = (n1c + kN1B - 1) / kN1B;
    for (int q = threadIdx.x; q < nw * nz; q += blockDim.x) {
        const float4 e = J.EZ[q];
        ezs[q] = make_float2(e.x, e.z);
    }
    __syncthreads();
    long long t = (long long)(blockIdx.x - L.blk[jb]) * blockDim.x + threadIdx.x;
    if (t >= (long long)nz * nw * ncols * nb) return;
    const int l = (int)(t % nz);
    t /= nz;
    const int b = (int)(t % nb);
    t /= nb;
    const int a = (int)(t % ncols);
    const int n2 = (int)(t / ncols);
    const int n10 = b * kN1B, cnt = min(kN1B, n1c - n10);
    float re[kN1B], im[kN1B];
#pragma unroll
    for (int u = 0; u < kN1B; ++u) re[u] = im[u] = 0.f;
    const float2 *w = J.W + ((long long)a * nw + n2) * nw * n1c + n10;
    for (int n3 = 0; n3 < nw; ++n3) {
        const float2 z = ezs[n3 * nz + l];
        const float2 *wr = w + (long long)n3 * n1c;
#pragma unroll
        for (int u = 0; u < kN1B; ++u)
            if (u < cnt) {
                const float2 v = wr[u];
                re[u] = fmaf(z.x, v.x, re[u]);
                re[u] = fmaf(-z.y, v.y, re[u]);
                im[u] = fmaf(z.x, v.y, im[u]);
                im[u] = fmaf(z.y, v.x, im[u]);
            }
    }
    float2 *o = J.F + (((long long)l * nw + n2) * ncols + a) * n1c + n10;
#pragma unroll
    for (int u = 0; u < kN1B; ++u)
        if (u < cnt) o[u] = make_float2(re[u], im[u]);
}

// Stage B, one CTA per (plane l, block of `ab` columns) of a job.  The plane's F slab for
// those columns ([n2][a][n1], FP32) and the ey phases ([n2][j], rows padded to kJB) sit in
// shared memory.  A thread owns one (column, n1) and kJB consecutive rows j: its F value is
// one load per n2, the ey values are warp broadcasts read two rows at a time, and a warp's
// stores of E land on consecutive (column, n1) of one row, contiguous in memory.
constexpr int kJB = 8;
__global__ void __launch_bounds__(128) recip_stage_b_kernel(const __grid_constant__ RecipLaunch L) {
    extern __shared__ float4 smem_b[];
    const int jb = recip_job_of(L, blockIdx.x);
    const RecipJob &J = L.job[jb];
    const int P = J.P, ncols = J.ncols, ny = J.ny, ab = J.ab;
    const int n1c = P + 1, nw = 2 * P + 1;
    const int nbx = (ncols + ab - 1) / ab, bloc = blockIdx.x - L.blk[jb];
    const int l = bloc / nbx, a0 = (bloc - l * nbx) * ab, na = min(ab, ncols - a0);
    const int an = na * n1c;                                  // (column, n1) pairs of the CTA
    const int nyp = (ny + kJB - 1) / kJB * kJB;
    float2 *fs = reinterpret_cast<float2 *>(smem_b);          // [nw][an]
    float2 *eys = fs + ((nw * ab * n1c + 1) & ~1);           // [nw][nyp], 16-byte aligned rows
    for (int t = threadIdx.x; t < nw * an; t += blockDim.x) {
        const int n2 = t / an, r = t - n2 * an;
        fs[t] = J.F[(((long long)l * nw + n2) * ncols + a0) * n1c + r];
    }
    for (int q = threadIdx.x; q < nw * nyp; q += blockDim.x) {
        const int n2 = q / nyp, j = q - n2 * nyp;
        const float4 y = j < ny ? J.EY[n2 * ny + j] : make_float4(0.f, 0.f, 0.f, 0.f);
        eys[q] = make_float2(y.x, y.z);
    }
    __syncthreads();
    const int tasks = an * (nyp / kJB);
    for (int task = threadIdx.x; task < tasks; task += blockDim.x) {
        const int jj = task / an, r = task - jj * an;  // r = a n1c + n1
        float re[kJB], im[kJB];
#pragma unroll
        for (int u = 0; u < kJB; ++u) re[u] = im[u] = 0.f;
        for (int n2 = 0; n2 < nw; ++n2) {
            const float2 f = fs[n2 * an + r];
            const float4 *yp = reinterpret_cast<const float4 *>(eys + n2 * nyp + jj * kJB);
#pragma unroll
            for (int u = 0; u < kJB / 2; ++u) {
                const float4 y = yp[u];  // rows 2u and 2u+1: (re, im, re, im)
                re[2 * u] = fmaf(y.x, f.x, re[2 * u]);
                re[2 * u] = fmaf(-y.y, f.y, re[2 * u]);
                im[2 * u] = fmaf(y.x, f.y, im[2 * u]);
                im[2 * u] = fmaf(y.y, f.x, im[2 * u]);
                re[2 * u + 1] = fmaf(y.z, f.x, re[2 * u + 1]);
                re[2 * u + 1] = fmaf(-y.w, f.y, re[2 * u + 1]);
                im[2 * u + 1] = fmaf(y.z, f.y, im[2 * u + 1]);
                im[2 * u + 1] = fmaf(y.w, f.x, im[2 * u + 1]);
            }
        }
        float2 *o = J.E + (((long long)l * ny + jj * kJB) * ncols + a0) * n1c + r;
        const long long row_stride = (long long)ncols * n1c;
#pragma unroll
        for (int u = 0; u < kJB; ++u)
            if (jj * kJB + u < ny) o[u * row_stride] = make_float2(re[u], im[u]);
    }
}

// stage B's columns per CTA: as many as fit 48 KB of shared memory (at most 16)
int stage_b_columns(int P) {
    const size_t col_bytes = sizeof(float2) * (size_t)(2 * P + 1) * (P + 1);
    return (int)std::max<size_t>(1, std::min<size_t>(16, (48u << 10) / col_bytes));
}
size_t stage_b_smem(int P, int ny, int ab) {
    const size_t nw = 2 * P + 1, n1c = P + 1, nyp = (size_t)(ny + kJB - 1) / kJB * kJB;
    return sizeof(float2) * (((size_t)nw * ab * n1c + 1) & ~(size_t)1) + sizeof(float2) * nw * nyp;
}

}  // namespace

size_t recip_rows_bytes(const rp_ewald *ew, int ncols) {
    const int P = ew->kmax - 1, n1c = P + 1;
    const long long nrows = (long long)ew->grid.n_grid[1] * ew->grid.n_grid[2];
    return sizeof(float2) * (size_t)nrows * ncols * n1c;
}

void recip_rows_group(rp_ctx *ctx, const std::vector<RecipRowsJob> &jobs, cudaStream_t stream,
                      const std::string &tag) {
    if (jobs.empty()) return;
    // scratch of every job in one arena per kind; the W arena is cleared with one memset
    std::vector<size_t> oW(jobs.size() + 1, 0), oF(jobs.size() + 1, 0), oU(jobs.size() + 1, 0),
        oK(jobs.size() + 1, 0);
    for (size_t j = 0; j < jobs.size(); ++j) {
        const rp_ewald *ew = jobs[j].ew;
        const int P = std::max(ew->kmax - 1, 0), n1c = P + 1, nw = 2 * P + 1;
        const int ncols = jobs[j].d_q ? 1 : jobs[j].N;
        const bool live = ew->K > 0;
        oW[j + 1] = oW[j] + (live ? (size_t)ncols * nw * nw * n1c : 0);
        oF[j + 1] = oF[j] + (live ? (size_t)ew->grid.n_grid[2] * nw * ncols * n1c : 0);
        oU[j + 1] = oU[j] + (live ? (size_t)jobs[j].N * 3 * nw : 0);
        oK[j + 1] = oK[j] + (live ? (size_t)ew->K : 0);
    }
    const size_t nj = jobs.size();
    float2 *W = ctx->buf_t<float2>("rs_W" + tag, std::max<size_t>(oW[nj], 1));
    float2 *F = ctx->buf_t<float2>("rs_F" + tag, std::max<size_t>(oF[nj], 1));
    double2 *U = ctx->buf_t<double2>("rs_U" + tag, std::max<size_t>(oU[nj], 1));
    float4 *Udf = ctx->buf_t<float4>("rs_Udf" + tag, std::max<size_t>(oU[nj], 1));
    float2 *kdf = ctx->buf_t<float2>("rs_kdf" + tag, std::max<size_t>(oK[nj], 1));
    if (oW[nj]) RP_CUDA(cudaMemsetAsync(W, 0, sizeof(float2) * oW[nj], stream));
    for (size_t j0 = 0; j0 < nj; j0 += kRecipJobs) {
        const size_t j1 = std::min(nj, j0 + kRecipJobs);
        RecipLaunch L{};
        int blk[4][kRecipJobs + 1] = {};
        size_t smem_a = 0, smem_b = 0;
        L.n = 0;
        for (size_t j = j0; j < j1; ++j) {
            const RecipRowsJob &rj = jobs[j];
            const rp_ewald *ew = rj.ew;
            const int ncols = rj.d_q ? 1 : rj.N;
            if (ew->K == 0) {  // no k-vectors (the non-periodic basis): E is zero
                RP_CUDA(cudaMemsetAsync(rj.E, 0, recip_rows_bytes(ew, ncols), stream));
                continue;
            }
            const int P = ew->kmax - 1, n1c = P + 1, nw = 2 * P + 1;
            const int ny = ew->grid.n_grid[1], nz = ew->grid.n_grid[2];
            RecipJob &J = L.job[L.n];
            J.atoms = rj.d_atoms; J.q = rj.d_q; J.kidx = ew->d_kidx; J.kcoef = ew->d_kcoef;
            J.EY = ew->d_eyf; J.EZ = ew->d_ezf;
            J.U = U + oU[j]; J.Udf = Udf + oU[j]; J.kdf = kdf + oK[j]; J.W = W + oW[j]; J.F = F + oF[j];
            J.E = rj.E;
            for (int q = 0; q < 9; ++q) J.rb[q] = ew->rec[q];
            J.N = rj.N; J.ncols = ncols; J.K = ew->K; J.P = P; J.ny = ny; J.nz = nz; J.ab = stage_b_columns(P);
            const int nb = (n1c + kN1B - 1) / kN1B;
            const int k = L.n;
            blk[0][k + 1] = blk[0][k] + (int)ceil_div((long long)rj.N * 3 * nw, 128);
            blk[1][k + 1] = blk[1][k] + (int)ceil_div((long long)ncols * ew->K, 128);
            blk[2][k + 1] = blk[2][k] + (int)ceil_div((long long)nz * nw * ncols * nb, 128);
            blk[3][k + 1] = blk[3][k] + (int)ceil_div(ncols, J.ab) * nz;
            smem_a = std::max(smem_a, sizeof(float2) * (size_t)nw * nz);
            smem_b = std::max(smem_b, stage_b_smem(P, ny, J.ab));
            ++L.n;
        }
        if (L.n == 0) continue;
        RP_REQUIRE(smem_a <= (200u << 10), "recip_rows: grid too large along z for KMAX");
        RP_REQUIRE(smem_b <= (200u << 10), "recip_rows: KMAX too large");
        smem_optin((const void *)recip_stage_a_kernel, smem_a);
        smem_optin((const void *)recip_stage_b_kernel, smem_b);
        auto with = [&](int k) {
            std::copy(blk[k], blk[k] + L.n + 1, L.blk);
            return blk[k][L.n];
        };
        int g = with(0);
        atom_phases_kernel<<<g, 128, 0, stream>>>(L);
        RP_LAUNCH_CHECK();
        g = with(1);
        build_w_kernel<<<g, 128, 0, stream>>>(L);
        RP_LAUNCH_CHECK();
        g = with(2);
        recip_stage_a_kernel<<<g, 128, smem_a, stream>>>(L);
        RP_LAUNCH_CHECK();
        g = with(3);
        recip_stage_b_kernel<<<g, 128, smem_b, stream>>>(L);
        RP_LAUNCH_CHECK();
    }
}

void recip_rows(rp_ctx *ctx, const rp_ewald *ew, const double *d_atoms, const double *d_q, int N, float2 *E,
                cudaStream_t stream, const std::string &slot) {
    recip_rows_group(ctx, {RecipRowsJob{ew, d_atoms, d_q, N, E}}, stream, slot);
}

}  // namespace rp
