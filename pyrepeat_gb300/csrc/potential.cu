// Ewald potential of point charges at grid points: V(g) = sum_a q_a phi_a(g).
//
// Replaces the V_coul = Phi q evaluation of ChargeCalculator.compute_stats
// (repeat.py:2326-2441, used for --stats and --output) without forming Phi:
//   reciprocal  V_r(g) = Re sum_n1 ex[n1][i] E_q[r][n1]: the separable reciprocal
//               sum of recip_sep.cu applied to the structure factor
//               S(k) = sum_a q_a w_k e^{-i k.r_a} (one charge-weighted column)
//   real space  V_s(g) = sum_a q_a sum_s [|g-r_a-s| <= Rc] erfc(sqrt(alpha) r)/r
//               over a per-CTA candidate list of images near the CTA's points.
// Cost per point is O(KMAX + images within Rc) instead of O(N K).  The real-space
// terms are FP32 with double-float accumulation and the reciprocal part FP32
// (relative error ~1e-7), which is what an RMS of the fitted ESP or a synthetic
// ESP needs.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "df.cuh"

namespace rp {
namespace {

constexpr int kPotPts = 128;
constexpr int kPotCand = 4096;  // images per candidate batch in shared memory

// one thread per point: V_r = Re sum_n1 ex[n1][i] E_q[r][n1]
__global__ void __launch_bounds__(kPotPts) potential_recip_kernel(const float4 *__restrict__ EX,
                                                                  const float2 *__restrict__ Eq, int n1c, int nx,
                                                                  const int32_t *__restrict__ idx, long long npts,
                                                                  double *__restrict__ out) {
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npts) return;
    const int f = idx ? idx[m] : (int)m;
    const int row = f / nx, i = f - row * nx;
    float rs = 0.f;
    for (int n = 0; n < n1c; ++n) {
        const float2 e = Eq[(long long)row * n1c + n];
        rs = dfa::cre32(rs, EX[(long long)n * nx + i], make_float4(e.x, 0.f, e.y, 0.f));
    }
    out[m] = (double)rs;
}

__global__ void __launch_bounds__(kPotPts) potential_real_kernel(
    const double *__restrict__ axis, int nx, int ny, const int32_t *__restrict__ idx, long long npts,
    const double *__restrict__ atoms, const double *__restrict__ q, int N, const double *__restrict__ shifts, int S,
    double rc, double sa, double *__restrict__ out) {
    __shared__ float4 cand[kPotCand];  // image position relative to the tile origin, charge
    __shared__ int ncand;
    __shared__ double origin[3];
    __shared__ float tile_r;
    const long long mb = (long long)blockIdx.x * kPotPts;
    const long long m = mb + threadIdx.x;
    const int layer = nx * ny;
    double g[3] = {0, 0, 0};
    bool valid = m < npts;
    if (valid) {
        const int f = idx ? idx[m] : (int)m;
        const int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
        for (int d = 0; d < 3; ++d) g[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)l * axis[6 + d];
    }
    if (threadIdx.x == 0) {
        for (int d = 0; d < 3; ++d) origin[d] = g[d];
        tile_r = 0.f;
    }
    __syncthreads();
    float3 gl = make_float3((float)(g[0] - origin[0]), (float)(g[1] - origin[1]), (float)(g[2] - origin[2]));
    if (valid) atomicMax(reinterpret_cast<int *>(&tile_r), __float_as_int(sqrtf(gl.x * gl.x + gl.y * gl.y + gl.z * gl.z)));
    __syncthreads();
    const float reach = (float)rc + tile_r + 1e-3f;
    const float reach2 = reach * reach, rc2 = (float)(rc * rc), saf = (float)sa;
    dfa::acc acc{0.f, 0.f};  // double-float sum of FP32 terms (no FP64 per pair)
    const int total = N * S;
    for (int base = 0; base < total; base += kPotCand) {
        if (threadIdx.x == 0) ncand = 0;
        __syncthreads();
        for (int t = base + threadIdx.x; t < min(total, base + kPotCand); t += kPotPts) {
            const int a = t / S, s = t - a * S;
            float px = (float)((atoms[3 * a] + shifts[3 * s]) - origin[0]);
            float py = (float)((atoms[3 * a + 1] + shifts[3 * s + 1]) - origin[1]);
            float pz = (float)((atoms[3 * a + 2] + shifts[3 * s + 2]) - origin[2]);
            if (px * px + py * py + pz * pz <= reach2) {
                int slot = atomicAdd(&ncand, 1);
                cand[slot] = make_float4(px, py, pz, (float)q[a]);  // slot < kPotCand: one chunk holds <= kPotCand images
            }
        }
        __syncthreads();
        const int nc = ncand;
        if (valid)
            for (int c = 0; c < nc; ++c) {
                const float4 p = cand[c];
                const float dx = gl.x - p.x, dy = gl.y - p.y, dz = gl.z - p.z;
                const float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 > rc2 || r2 <= 1e-20f) continue;
                const float rinv = rsqrtf(r2);
                float t, e;
                dfa::two_sum(acc.s, p.w * (erfcf(saf * (r2 * rinv)) * rinv), t, e);
                acc.s = t;
                acc.e = __fadd_rn(acc.e, e);
            }
        __syncthreads();
    }
    if (valid) out[m] += dfa::to_double(acc);
}

}  // namespace

void potential_run(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, const double *q, int N,
                   const int32_t *idx_dev, int64_t npts, double *out_dev, cudaStream_t stream) {
    RP_REQUIRE(atoms && q && out_dev && N > 0 && npts > 0, "rp_potential: bad arguments");
    std::vector<double> sh;
    int zero_idx = -1;
    prune_shifts(ew, atoms, N, sh, zero_idx);
    const int S = (int)(sh.size() / 3);
    RP_REQUIRE((long long)N * S < (1LL << 31), "rp_potential: too many images");
    double *d_atoms = ctx->buf_t<double>("p_atoms", 3 * (size_t)N);
    double *d_q = ctx->buf_t<double>("p_q", (size_t)N);
    double *d_shifts = ctx->buf_t<double>("p_shifts", sh.size());
    double *d_axis = ctx->buf_t<double>("p_axis", 9);
    RP_CUDA(cudaMemcpyAsync(d_atoms, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_q, q, sizeof(double) * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_shifts, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_axis, ew->grid.axis, sizeof(double) * 9, cudaMemcpyHostToDevice, stream));
    const int nx = ew->grid.n_grid[0], ny = ew->grid.n_grid[1];
    float2 *Eq = ctx->buf_t<float2>("p_Eq", recip_rows_bytes(ew, 1) / sizeof(float2));
    recip_rows(ctx, ew, d_atoms, d_q, N, Eq, stream);
    potential_recip_kernel<<<ceil_div(npts, kPotPts), kPotPts, 0, stream>>>(ew->d_exf, Eq, ew->kmax, nx, idx_dev, npts,
                                                                           out_dev);
    RP_LAUNCH_CHECK();
    potential_real_kernel<<<ceil_div(npts, kPotPts), kPotPts, 0, stream>>>(d_axis, nx, ny, idx_dev, npts, d_atoms, d_q,
                                                                          N, d_shifts, S, ew->cutoff, ew->sqrt_alpha,
                                                                          out_dev);
    RP_LAUNCH_CHECK();
}

}  // namespace rp
