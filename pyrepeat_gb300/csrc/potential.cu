// Ewald potential of point charges at grid points: V(g) = sum_a q_a phi_a(g).
//
// Replaces the V_coul = Phi q evaluation of ChargeCalculator.compute_stats
// (repeat.py:2326-2441, used for --stats and --output) without forming Phi:
//   reciprocal  V_r(g) = sum_k w_k Re(e^{i k.g} conj(S_k)),  S_k = sum_a q_a e^{i k.r_a}
//               (structure factors in FP64 once; per point the exact per-axis phases)
//   real space  V_s(g) = sum_a q_a sum_s [|g-r_a-s| <= Rc] erfc(sqrt(alpha) r)/r
//               over a per-CTA candidate list of images near the CTA's points.
// Cost per point is O(K + images within Rc) instead of O(N K).  The sums use
// FP32 terms with FP64 accumulation (relative error ~1e-7), which is what an
// RMS of the fitted ESP or a synthetic ESP needs.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace rp {
namespace {

constexpr int kPotPts = 128;
constexpr int kPotCand = 4096;  // images per candidate batch in shared memory

__global__ void structure_factors_kernel(const double *__restrict__ kvec, int K, const double *__restrict__ atoms,
                                         const double *__restrict__ q, int N, double2 *__restrict__ Sk) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    double re = 0.0, im = 0.0;
    for (int a = 0; a < N; ++a) {
        double kr = (atoms[3 * a] * kvec[3 * k] + atoms[3 * a + 1] * kvec[3 * k + 1]) + atoms[3 * a + 2] * kvec[3 * k + 2];
        double s, c;
        sincos(kr, &s, &c);
        re += q[a] * c;
        im += q[a] * s;
    }
    Sk[k] = make_double2(re, im);
}

// one thread per point; the k loop reads the (w_k S_k) table and the per-axis phases
__global__ void __launch_bounds__(kPotPts) potential_recip_kernel(
    const int *__restrict__ kidx, const double *__restrict__ kcoef, const double2 *__restrict__ Sk, int K, int kmax,
    const double2 *__restrict__ ex, const double2 *__restrict__ ey, const double2 *__restrict__ ez, int nx, int ny,
    int nz, const int32_t *__restrict__ idx, long long npts, double *__restrict__ out) {
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npts) return;
    const int f = idx ? idx[m] : (int)m;
    const int layer = nx * ny;
    const int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
    double acc = 0.0;
    for (int k = 0; k < K; ++k) {
        const int n1 = kidx[3 * k], n2 = kidx[3 * k + 1], n3 = kidx[3 * k + 2];
        const double2 a = ex[n1 * nx + i], b = ey[(n2 + kmax) * ny + j], c = ez[(n3 + kmax) * nz + l];
        const float r1 = (float)(a.x * b.x - a.y * b.y), i1 = (float)(a.x * b.y + a.y * b.x);
        const float cr = r1 * (float)c.x - i1 * (float)c.y, ci = r1 * (float)c.y + i1 * (float)c.x;
        const double2 s = Sk[k];
        acc += kcoef[k] * ((double)cr * s.x + (double)ci * s.y);
    }
    out[m] = acc;
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
    const float reach2 = reach * reach, rc2 = (float)(rc * rc);
    double acc = 0.0;
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
                const float r = sqrtf(r2);
                acc += (double)(p.w * (erfcf((float)sa * r) / r));
            }
        __syncthreads();
    }
    if (valid) out[m] += acc;
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
    double2 *Sk = ctx->buf_t<double2>("p_Sk", (size_t)ew->K);
    RP_CUDA(cudaMemcpyAsync(d_atoms, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_q, q, sizeof(double) * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_shifts, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_axis, ew->grid.axis, sizeof(double) * 9, cudaMemcpyHostToDevice, stream));
    structure_factors_kernel<<<ceil_div(ew->K, 128), 128, 0, stream>>>(ew->d_kvec_s, ew->K, d_atoms, d_q, N, Sk);
    RP_LAUNCH_CHECK();
    const int nx = ew->grid.n_grid[0], ny = ew->grid.n_grid[1], nz = ew->grid.n_grid[2];
    potential_recip_kernel<<<ceil_div(npts, kPotPts), kPotPts, 0, stream>>>(
        ew->d_kidx_s, ew->d_kcoef_s, Sk, ew->K, ew->kmax, ew->d_ex, ew->d_ey, ew->d_ez, nx, ny, nz, idx_dev, npts,
        out_dev);
    RP_LAUNCH_CHECK();
    potential_real_kernel<<<ceil_div(npts, kPotPts), kPotPts, 0, stream>>>(d_axis, nx, ny, idx_dev, npts, d_atoms, d_q,
                                                                          N, d_shifts, S, ew->cutoff, ew->sqrt_alpha,
                                                                          out_dev);
    RP_LAUNCH_CHECK();
}

}  // namespace rp
