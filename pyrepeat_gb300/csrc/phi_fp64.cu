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
#include "df.cuh"

namespace rp {
namespace {

// Real-space sum in FP64 (repeat.py:944-966) over tiles of kRsPts kept points x kRsAtoms
// atoms.  For each chunk of up to kRsShiftChunk shifts, the CTA first drops, per atom,
// every shift whose image lies farther than Rc + 1e-3 Bohr from the bounding box of its
// points (an FP32 test: FP32 rounding of the coordinates moves a distance by < 1e-4
// Bohr here, so no image within Rc is dropped).  Each thread then tests the remaining
// images of each atom against its point in FP32 with the same margin.  QUEUE false: the
// survivors are evaluated in place (the plain comparator's kept points, in grid order,
// give tiles of nearby points that reach mostly the same images).  QUEUE true (the
// escalated fit, whatever the order of its kept points): each thread queues its
// survivors (atom, image) in order, the CTA
// evaluates the queued pairs in FP64, every lane on one pair, so the FP64 pipe (a small
// fraction of the FP32 rate on this part, and as slow for one active lane as for 32)
// runs full warps instead of a warp per image that any of its points reaches, and each
// thread adds its pairs' terms in queue order (a rejected pair adds +0.0, which changes
// no sum).  Either way the FP64 expressions are the reference's.  Every image within Rc is therefore summed, in shift order, exactly as by a
// loop over all shifts.  The sums are accumulated in a shared-memory tile and added into
// phi[m][a] (row-major, ld N) with coalesced stores.
constexpr int kRsPts = 128;
constexpr int kRsAtoms = 16;
constexpr int kRsQueue = 16;  // queued pairs per point per round
// shifts per chunk: in place 128, queued 64 (its queue takes the rest of the shared memory)
template <bool QUEUE> __host__ __device__ constexpr int rs_chunk() { return QUEUE ? 64 : 128; }
size_t realspace_fp64_smem(bool queue) {
    return queue ? sizeof(float4) * kRsAtoms * rs_chunk<true>() + sizeof(double) * kRsQueue * kRsPts +
                       sizeof(unsigned short) * kRsQueue * kRsPts
                 : sizeof(float4) * kRsAtoms * rs_chunk<false>();
}
template <bool QUEUE>
__global__ void __launch_bounds__(kRsPts) realspace_fp64_kernel(
    const int32_t *__restrict__ kept, long long m0, long long rows, const double *__restrict__ axis, int nx, int ny,
    const double *__restrict__ atoms, int N, const double *__restrict__ shifts, int S, int zero_idx, double rc,
    double sa, double *__restrict__ phi) {
    constexpr int kRsShiftChunk = rs_chunk<QUEUE>();
    extern __shared__ float4 rs_cand[];  // [kRsAtoms][kRsShiftChunk] image (x, y, z) in FP32, shift index
    double *qterm = reinterpret_cast<double *>(rs_cand + kRsAtoms * kRsShiftChunk);      // [kRsQueue][kRsPts]
    unsigned short *qitem = reinterpret_cast<unsigned short *>(qterm + kRsQueue * kRsPts);  // (atom << 7) | image
    __shared__ double tile[kRsAtoms][kRsPts + 1];
    __shared__ double gs[3][kRsPts];
    __shared__ int ncand[kRsAtoms];
    __shared__ int qoff[kRsPts + 1];
    __shared__ int wsum[kRsPts / 32];
    __shared__ int more;
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
    for (int d = 0; d < 3; ++d) {
        g[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)l * axis[6 + d];
        gs[d][threadIdx.x] = g[d];
    }
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
        // Evaluated where they are found (QUEUE false), the pairs cost a warp-wide FP64 pass
        // for every image that any lane of the warp reaches, which suits tiles whose points
        // lie close together; queued, they cost their number plus the queue's bookkeeping.
        {
            if (!QUEUE) {  // evaluate in place, in order
                for (int a = 0; a < na; ++a) {
                    const double *pa = atoms + 3 * (size_t)(a0 + a);
                    double acc = tile[a][threadIdx.x];
                    for (int c = 0; c < ncand[a]; ++c) {
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
                continue;
            }
        }
        // rounds: queue up to kRsQueue pairs per point (resuming where the last round stopped),
        // evaluate them with the whole CTA, add the terms in queue order
        int ra = 0, rcnd = 0;  // this thread's resume point (atom, image)
        for (;;) {
            int cnt = 0;
            while (ra < na && cnt < kRsQueue) {
                const int nc = ncand[ra];
                while (rcnd < nc && cnt < kRsQueue) {
                    const float4 h = rs_cand[ra * kRsShiftChunk + rcnd];
                    const float fx = gf[0] - h.x, fy = gf[1] - h.y, fz = gf[2] - h.z;
                    if (fx * fx + fy * fy + fz * fz <= reach2)
                        qitem[cnt++ * kRsPts + threadIdx.x] = (unsigned short)((ra << 7) | rcnd);
                    ++rcnd;
                }
                if (rcnd >= nc) {
                    ++ra;
                    rcnd = 0;
                }
            }
            // offsets of every thread's queue (block exclusive scan of cnt)
            int incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (lane == 31) wsum[warp] = incl;
            if (threadIdx.x == 0) more = 0;
            __syncthreads();
            int wbase = 0;
            for (int w = 0; w < warp; ++w) wbase += wsum[w];
            qoff[threadIdx.x] = wbase + incl - cnt;
            if (threadIdx.x == kRsPts - 1) qoff[kRsPts] = wbase + incl;
            if (ra < na) more = 1;
            __syncthreads();
            const int total = qoff[kRsPts];
            for (int idx = threadIdx.x; idx < total; idx += kRsPts) {
                int lo = 0, hi = kRsPts - 1;  // the owner: the last thread whose offset is <= idx
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (qoff[mid] <= idx) lo = mid;
                    else hi = mid - 1;
                }
                const int k = idx - qoff[lo];
                const unsigned short it = qitem[k * kRsPts + lo];
                const int a = it >> 7, c = it & 127;
                const int s = __float_as_int(rs_cand[a * kRsShiftChunk + c].w);
                const double *pa = atoms + 3 * (size_t)(a0 + a);
                const double ex = gs[0][lo] - (pa[0] + shifts[3 * s]);
                const double ey = gs[1][lo] - (pa[1] + shifts[3 * s + 1]);
                const double ez = gs[2][lo] - (pa[2] + shifts[3 * s + 2]);
                const double r = sqrt(ex * ex + ey * ey + ez * ez);
                double term = 0.0;
                if ((r <= rc) && !(s == zero_idx && !(r > 1e-10))) term = erfc(sa * r) / r;
                qterm[k * kRsPts + lo] = term;
            }
            __syncthreads();
            for (int k = 0; k < cnt; ++k) tile[qitem[k * kRsPts + threadIdx.x] >> 7][threadIdx.x] += qterm[k * kRsPts + threadIdx.x];
            const int again = more;
            __syncthreads();  // the queue is refilled on the next pass
            if (!again) break;
        }
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

// ---- FP64 separable reciprocal sum (the escalated fit) ----
// The transform of recip_sep.cu at FP64-level accuracy: stages A and B in double-float
// (~2^-46 relative, on the FP32 pipe, whose rate is many times the FP64 pipe's here), the
// weights and stage C in FP64; with the exact per-axis lattice phases ex, ey, ez of the grid
// (tables of the Ewald object) and
// W_a(n) = w_k e^{-i k.r_a},
//   F[l][n2][a][n1] = sum_n3 ez[n3][l] W[n2][n3][a][n1]      (every grid plane l)
//   E[r][a][n1]     = sum_n2 ey[n2][j_r] F[l_r][n2][a][n1]    (the rows r that hold kept points)
//   Phi[m][a]      += Re sum_n1 ex[n1][i_m] E[r_m][a][n1]     (every kept point)
// n1 in [0, P], n2, n3 in [-P, P], P = KMAX - 1 (stored with offset P; the FP64 tables
// carry offset KMAX).  On the 2000-atom triclinic cube this is ~35 GFLOP instead of the
// flat k-table's 158 (repeat.py:968-981 evaluated as one DGEMM).
struct RecBasis {
    double rb[9];
};

// U[a][d][n + P] = e^{-i n (b_d . r_a)}
__global__ void atom_phases64_kernel(const double *__restrict__ atoms, int N, RecBasis B, int P,
                                     double2 *__restrict__ U) {
    const int nw = 2 * P + 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * 3 * nw) return;
    const int n = t % nw - P, d = (t / nw) % 3, a = t / (3 * nw);
    const double *p = atoms + 3 * a;
    const double th = (p[0] * B.rb[3 * d] + p[1] * B.rb[3 * d + 1]) + p[2] * B.rb[3 * d + 2];
    double sn, cs;
    sincos((double)n * th, &sn, &cs);
    U[t] = make_double2(cs, -sn);
}

__device__ __forceinline__ double2 cmul64(double2 x, double2 y) {
    return make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
}

// W[n2'][n3'][a][n1] = w_k e^{-i k.r_a} for the k-set (zero elsewhere: cleared before), from
// FP64 phase products, stored as double-float for stage A
__global__ void build_w64_kernel(const int *__restrict__ kidx, const double *__restrict__ kcoef, int K, int N,
                                 int P, const double2 *__restrict__ U, float4 *__restrict__ W) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * K) return;
    const int a = (int)(t / K), k = (int)(t - (long long)a * K);
    const int nw = 2 * P + 1, n1c = P + 1;
    const int n1 = kidx[3 * k], n2 = kidx[3 * k + 1] + P, n3 = kidx[3 * k + 2] + P;
    const double2 *u = U + (size_t)a * 3 * nw;
    const double2 v = cmul64(cmul64(u[n1 + P], u[nw + n2]), u[2 * nw + n3]);
    const double w = kcoef[k];
    W[(((size_t)n2 * nw + n3) * N + a) * n1c + n1] = dfa::split(w * v.x, w * v.y);
}

// stage A: one thread per (l, n2, a, n1), n1 fastest, in double-float (dfa::cmac) from the
// double-float phases and W; F is stored as double-float for stage B
__global__ void stage_a64_kernel(const float4 *__restrict__ W, const float4 *__restrict__ ezf, int nz, int N,
                                 int P, float4 *__restrict__ F) {
    const int nw = 2 * P + 1, n1c = P + 1;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nz * nw * N * n1c) return;
    const long long an = (long long)N * n1c;
    const int r = (int)(t % an);           // a n1c + n1
    const int n2 = (int)((t / an) % nw), l = (int)(t / (an * nw));
    dfa::acc re{0.f, 0.f}, im{0.f, 0.f};
    for (int n3 = 0; n3 < nw; ++n3) dfa::cmac(re, im, ezf[(size_t)n3 * nz + l], W[((size_t)n2 * nw + n3) * an + r]);
    F[t] = dfa::pack(re, im);
}

// stage B over the listed rows (row = j + l ny): one thread per (row, a, n1), n1 fastest.  In
// double-float on the FP32 pipe (~2^-46 relative, dfa::cmac) from the double-float phases and F:
// the FP64 pipe is a small fraction of the FP32 rate here, and this stage is most of the sum's
// work on a sparse cube (29 GFLOP on the 2000-atom triclinic one); E is stored in FP64.
__global__ void stage_b64_kernel(const float4 *__restrict__ F, const float4 *__restrict__ eyf, int ny, int N,
                                 int P, const int *__restrict__ rows, int R, double2 *__restrict__ E) {
    const int nw = 2 * P + 1, n1c = P + 1;
    const long long an = (long long)N * n1c;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)R * an) return;
    const int ri = (int)(t / an), r = (int)(t - (long long)ri * an);
    const int row = rows[ri], l = row / ny, j = row - l * ny;
    dfa::acc re{0.f, 0.f}, im{0.f, 0.f};
    for (int n2 = 0; n2 < nw; ++n2) dfa::cmac(re, im, eyf[(size_t)n2 * ny + j], F[((size_t)l * nw + n2) * an + r]);
    E[t] = make_double2(dfa::to_double(re), dfa::to_double(im));
}

// mark the grid rows that hold kept points m0 .. m0+rows-1
__global__ void mark_rows_kernel(const int32_t *__restrict__ kept, long long m0, long long rows, int nx,
                                 unsigned char *__restrict__ mark) {
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m < rows) mark[kept[m0 + m] / nx] = 1;
}

// stage C: phi[m][a] = Re sum_n1 ex[n1][i] E[rowmap[row]][a][n1]  (one thread per (m, a), a fastest)
__global__ void stage_c64_kernel(const double2 *__restrict__ E, const double2 *__restrict__ ex, int nx, int N,
                                 int P, const int32_t *__restrict__ kept, long long m0, long long rows,
                                 const int *__restrict__ rowmap, double *__restrict__ phi) {
    const int n1c = P + 1;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= rows * N) return;
    const long long m = t / N;
    const int a = (int)(t - m * N);
    const int f = kept[m0 + m], row = f / nx, i = f - row * nx;
    const double2 *e = E + ((size_t)rowmap[row] * N + a) * n1c;
    double s = 0.0;
    for (int n1 = 0; n1 < n1c; ++n1) {
        const double2 x = ex[(size_t)n1 * nx + i], v = e[n1];
        s += x.x * v.x - x.y * v.y;
    }
    phi[t] = s;
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
               cudaStream_t stream, bool separable) {
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

    // reciprocal part: the flat k-table product (one DGEMM per chunk: the comparator), or
    // the separable transform in FP64 (the escalated fit): W and the plane stage once per fit
    const int kp = ew->kmax - 1, nw = 2 * kp + 1, n1c = kp + 1;  // the separable sum's n range
    const int nx = ew->grid.n_grid[0], ny = ew->grid.n_grid[1], nz = ew->grid.n_grid[2];
    const bool sep = separable && K > 0 && kp >= 0;
    double *B = nullptr;
    float4 *F64 = nullptr;
    if (sep) {
        StageTimer tt(ctx, "fp64_recip_sep", stream);
        double2 *U = ctx->buf_t<double2>("g64_U", (size_t)N * 3 * nw);
        float4 *W = ctx->buf_t<float4>("g64_W", (size_t)nw * nw * N * n1c);
        F64 = ctx->buf_t<float4>("g64_F", (size_t)nz * nw * N * n1c);
        RP_CUDA(cudaMemsetAsync(W, 0, sizeof(float4) * (size_t)nw * nw * N * n1c, stream));
        RecBasis rb;
        for (int q = 0; q < 9; ++q) rb.rb[q] = ew->rec[q];
        atom_phases64_kernel<<<ceil_div(N * 3 * nw, 128), 128, 0, stream>>>(d_atoms, N, rb, kp, U);
        RP_LAUNCH_CHECK();
        build_w64_kernel<<<ceil_div((long long)N * K, 128), 128, 0, stream>>>(ew->d_kidx, ew->d_kcoef, K, N, kp, U, W);
        RP_LAUNCH_CHECK();
        stage_a64_kernel<<<ceil_div((long long)nz * nw * N * n1c, 128), 128, 0, stream>>>(W, ew->d_ezf, nz, N, kp,
                                                                                          F64);
        RP_LAUNCH_CHECK();
    } else {
        B = ctx->buf_t<double>("g64_B", (size_t)N * K2);
        if (K > 0) atom_tables_fp64(ew, d_atoms, N, B, K2, stream);
    }

    // chunk rows so T and Phi stay within ~2 GB together (separable: Phi and the chunk's
    // reciprocal rows, at most one per point, within ~4 GB)
    const size_t row_bytes = sep ? sizeof(double) * N + sizeof(double2) * (size_t)N * n1c
                                 : sizeof(double) * ((size_t)K2 + N);
    int64_t chunk = std::max<int64_t>(256, (int64_t)((size_t)(sep ? 4 : 2) << 30) / (int64_t)row_bytes);
    chunk = std::min<int64_t>(chunk, M);
    double *T = sep ? nullptr : ctx->buf_t<double>("g64_T", (size_t)chunk * K2);
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

    const bool syrk = N >= 512;  // the Gram's cuBLAS call (below)
    cublasHandle_t h = ctx->blas();
    RP_CUBLAS(cublasSetStream(h, stream));
    const double one = 1.0, zero = 0.0;
    for (int64_t m0 = 0; m0 < M; m0 += chunk) {
        const int64_t rows = std::min<int64_t>(chunk, M - m0);
        if (sep) {
            StageTimer tt(ctx, "fp64_recip_sep", stream);
            // the grid rows of this chunk's points, numbered on the host
            const size_t nrows = (size_t)ny * nz;
            unsigned char *mark = ctx->buf_t<unsigned char>("g64_mark", nrows);
            RP_CUDA(cudaMemsetAsync(mark, 0, nrows, stream));
            mark_rows_kernel<<<ceil_div(rows, 256), 256, 0, stream>>>(kept_idx_dev, m0, rows, nx, mark);
            RP_LAUNCH_CHECK();
            unsigned char *hmark = static_cast<unsigned char *>(ctx->host_buf("g64_mark", nrows));
            int *hmap = static_cast<int *>(ctx->host_buf("g64_rowmap", sizeof(int) * nrows * 2));
            RP_CUDA(cudaMemcpyAsync(hmark, mark, nrows, cudaMemcpyDeviceToHost, stream));
            RP_CUDA(cudaStreamSynchronize(stream));
            int R = 0;
            int *hlist = hmap + nrows;
            for (size_t r = 0; r < nrows; ++r) {
                hmap[r] = hmark[r] ? R : -1;
                if (hmark[r]) hlist[R++] = (int)r;
            }
            int *rowmap = ctx->buf_t<int>("g64_rowmap", nrows);
            int *rowlist = ctx->buf_t<int>("g64_rowlist", (size_t)std::max(R, 1));
            RP_CUDA(cudaMemcpyAsync(rowmap, hmap, sizeof(int) * nrows, cudaMemcpyHostToDevice, stream));
            RP_CUDA(cudaMemcpyAsync(rowlist, hlist, sizeof(int) * R, cudaMemcpyHostToDevice, stream));
            double2 *E64 = ctx->buf_t<double2>("g64_E", (size_t)std::max(R, 1) * N * n1c);
            stage_b64_kernel<<<ceil_div((long long)R * N * n1c, 128), 128, 0, stream>>>(F64, ew->d_eyf, ny, N, kp,
                                                                                       rowlist, R, E64);
            RP_LAUNCH_CHECK();
            stage_c64_kernel<<<ceil_div(rows * N, 128), 128, 0, stream>>>(E64, ew->d_ex, nx, N, kp, kept_idx_dev, m0,
                                                                          rows, rowmap, P);
            RP_LAUNCH_CHECK();
            // the pinned row arrays are rewritten by the next chunk: its uploads must be done
            RP_CUDA(cudaStreamSynchronize(stream));
        } else if (K > 0) {
            {
                StageTimer tt(ctx, "fp64_tables", stream);
                grid_tables_fp64(ew, kept_idx_dev, m0, rows, T, K2, stream);
            }
            StageTimer tt(ctx, "fp64_recip_dgemm", stream);
            RP_CUBLAS(cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, N, (int)rows, K2, &one, B, K2, T, K2, &zero, P, N));
        } else {  // the non-periodic basis has no reciprocal part
            RP_CUDA(cudaMemsetAsync(P, 0, sizeof(double) * (size_t)rows * N, stream));
        }
        {
            StageTimer t_r(ctx, "fp64_realspace", stream);
            const size_t smem = realspace_fp64_smem(sep);  // candidates (and the pair queue): 32 or 36 KB
            auto kern = sep ? realspace_fp64_kernel<true> : realspace_fp64_kernel<false>;
            smem_optin((const void *)kern, smem);
            kern<<<dim3(ceil_div(rows, kRsPts), ceil_div(N, kRsAtoms)), kRsPts, smem, stream>>>(
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
        if (sep) {  // the exact two-word Gram on the tensor cores (G full, r included)
            StageTimer t_g(ctx, "fp64_gram_words", stream);
            gram_words_fp64(ctx, P, rows, N, Vc_dev + m0, G, r, stream);
        } else {
            // column-major view: X = P^T is N x rows with ld N;  G += X X^T,  r += X Vc.  DSYRK
            // (one triangle, mirrored after the last chunk) halves the work, but for few
            // columns cuBLAS's rank-k update parallelises poorly over the long k (31 ms for
            // 77 x 109,682 against ~1.5 ms as a DGEMM), so small systems take the DGEMM.
            StageTimer t_g(ctx, "fp64_gram_blas", stream);
            if (syrk)
                RP_CUBLAS(cublasDsyrk(h, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, N, (int)rows, &one, P, N, &one, G, N));
            else
                RP_CUBLAS(cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, N, N, (int)rows, &one, P, N, P, N, &one, G, N));
            RP_CUBLAS(cublasDgemv(h, CUBLAS_OP_N, N, (int)rows, &one, P, N, Vc_dev + m0, 1, &one, r, 1));
        }
    }
    if (!sep && syrk) {
        mirror_upper_kernel<<<ceil_div((long long)N * N, 256), 256, 0, stream>>>(G, N);
        RP_LAUNCH_CHECK();
    }
    column_sums_fp64(Vc_dev, M, 1, 1, sumV, false, ctx, stream);
    shifted_sums_kernel<<<ceil_div(N, 128), 128, 0, stream>>>(sphi, c, M, N, s_c);
    RP_LAUNCH_CHECK();
    finish_normal_equations(G, r, s_c, sumV, M, N, A_dev, b_dev, stream);
    (void)K;
}

}  // namespace rp
