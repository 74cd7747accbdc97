// Constraints and the bordered solve, on the device in FP64.
//
// Replaces repeat.py:2278-2313: symmetry folding (repeat.py:2445-2470: columns
// of every group into its base, then rows, linked atoms dropped), RESP
// restraints on the folded diagonal (repeat.py:2511-2520), the (n+1) bordered
// total-charge system [[A, w],[w^T, 0]] [q; l] = [b; Q] (repeat.py:2296-2304)
// solved by LU with partial pivoting (scipy.linalg.solve / repeat_cpu_omp.cpp:
// 466-495), then charges expanded to the linked atoms (repeat.py:2472-2489).
//
// For disjoint groups (each atom in at most one group) folding is the gather
//   A_red[r][c] = sum_{i in G(r)} sum_{j in G(c)} A[i][j],  b_red[r] = sum_{i in G(r)} b[i],
//   w[r] = |G(r)|
// which equals the reference's sequential column-then-row folding.  Groups
// that overlap are folded on the host with the reference's sequential rules.
//
// One CTA solves one system (so a batch of systems is one launch).  It factors the
// bordered matrix in FP32 (LU with partial pivoting) and refines x += LU32^{-1}(b - A x)
// with FP64 residuals until the backward error |b - A x| <= n eps64 |A| |x| (the
// classic mixed-precision iterative refinement; FP64 runs at a small fraction of
// the FP32 rate on this part).  If the FP32 factorisation meets a zero pivot or the
// refinement stalls (a step that does not halve the residual, or kRefineMax steps:
// cond(A) near 1/eps32), the system is factored again in FP64 with one step of FP64
// refinement.  Either way the refined residual and the pivot range are reported.
// Systems of kLUWideMin or more unknowns are factored across the whole GPU instead
// of by their CTA (lu_wide_factor), in FP32 and, when that stalls, in FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <set>

#include "common.cuh"

namespace rp {

namespace {

// Folded bordered matrices of many systems in one launch: blockIdx.y picks the system (from
// `sys`, the ones with disjoint groups), the blocks along x stride over its (n+1)^2 entries.
__global__ void build_bordered_kernel(const SolveDesc *__restrict__ descs, const int *__restrict__ sys) {
    const SolveDesc d = descs[sys[blockIdx.y]];
    const int n1 = d.n + 1;
    long long total = (long long)n1 * n1;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        int r = (int)(t / n1), c = (int)(t - (long long)r * n1);
        double v;
        if (r < d.n && c < d.n) {
            v = 0.0;
            for (int p = d.mem_ptr[r]; p < d.mem_ptr[r + 1]; ++p) {
                const double *row = d.A + (size_t)d.mem_idx[p] * d.N;
                for (int q = d.mem_ptr[c]; q < d.mem_ptr[c + 1]; ++q) v += row[d.mem_idx[q]];
            }
            if (r == c && d.resp_s) v += d.resp_s[r];
        } else if (r < d.n) {
            v = (double)(d.mem_ptr[r + 1] - d.mem_ptr[r]);
        } else if (c < d.n) {
            v = (double)(d.mem_ptr[c + 1] - d.mem_ptr[c]);
        } else {
            v = 0.0;
        }
        d.As[t] = v;
        d.A0[t] = v;
        if (c == 0) {
            double bv;
            if (r < d.n) {
                bv = 0.0;
                for (int p = d.mem_ptr[r]; p < d.mem_ptr[r + 1]; ++p) bv += d.b[d.mem_idx[p]];
                if (d.resp_s) bv += d.resp_s[r] * d.resp_t[r];
            } else {
                bv = d.qtot;
            }
            d.bs[r] = bv;
        }
    }
}

constexpr int kLU = 1024;

__device__ void block_argmax(double v, int idx, double *sv, int *si, double *out_v, int *out_i) {
    // max |v| with lowest index on ties (deterministic)
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_down_sync(0xffffffffu, v, o);
        int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sv[w] = v; si[w] = idx; }
    __syncthreads();
    if (w == 0) {
        v = (lane < kLU / 32) ? sv[lane] : -1.0;
        idx = (lane < kLU / 32) ? si[lane] : 0x7fffffff;
        for (int o = 16; o > 0; o >>= 1) {
            double ov = __shfl_down_sync(0xffffffffu, v, o);
            int oi = __shfl_down_sync(0xffffffffu, idx, o);
            if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
        }
        if (lane == 0) { *out_v = v; *out_i = idx; }
    }
    __syncthreads();
}

__device__ void lu_apply(const double *__restrict__ LU, const int *__restrict__ perm, int n1, double *__restrict__ y,
                         double *__restrict__ ysh) {
    // solve (P L U) z = y in place (y global; ysh: n1 doubles of shared memory), blocked by 32
    // columns: the diagonal block is solved by one warp with shuffles, then every thread
    // updates one remaining row with the block's 32 values (a warp instruction covers 32 rows:
    // the FP64 pipe takes as long for one lane as for 32).  The row interchanges run in
    // shared memory.  Three barriers per 32 columns.
    __shared__ double blk[32][33];
    __shared__ double yb[32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    for (int t = threadIdx.x; t < n1; t += kLU) ysh[t] = y[t];
    __syncthreads();
    if (threadIdx.x == 0) {
        int k = 0;
        for (; k + 8 <= n1; k += 8) {  // the interchanges' indices are independent loads
            int p[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) p[u] = perm[k + u];
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (p[u] != k + u) { const double t = ysh[k + u]; ysh[k + u] = ysh[p[u]]; ysh[p[u]] = t; }
        }
        for (; k < n1; ++k) {
            const int p = perm[k];
            if (p != k) { const double t = ysh[k]; ysh[k] = ysh[p]; ysh[p] = t; }
        }
    }
    __syncthreads();
    for (int c0 = 0; c0 < n1; c0 += 32) {  // forward: L, unit diagonal
        const int bs = min(32, n1 - c0);
        for (int t = threadIdx.x; t < bs * 32; t += kLU) {
            const int r = t >> 5, c = t & 31;
            blk[r][c] = c < bs ? LU[(size_t)(c0 + r) * n1 + c0 + c] : 0.0;
        }
        __syncthreads();
        if (warp == 0) {
            double yv = lane < bs ? ysh[c0 + lane] : 0.0;
            for (int c = 0; c < bs - 1; ++c) {
                const double yc = __shfl_sync(0xffffffffu, yv, c);
                if (lane > c && lane < bs) yv -= blk[lane][c] * yc;
            }
            if (lane < bs) ysh[c0 + lane] = yv;
            yb[lane] = lane < bs ? yv : 0.0;
        }
        __syncthreads();
        for (int r = c0 + bs + threadIdx.x; r < n1; r += kLU) {
            const double *row = LU + (size_t)r * n1 + c0;
            double t = 0.0;
            for (int c = 0; c < bs; ++c) t += row[c] * yb[c];
            ysh[r] -= t;
        }
        __syncthreads();
    }
    for (int c1 = n1; c1 > 0; c1 -= 32) {  // backward: U
        const int c0 = max(0, c1 - 32), bs = c1 - c0;
        for (int t = threadIdx.x; t < bs * 32; t += kLU) {
            const int r = t >> 5, c = t & 31;
            blk[r][c] = c < bs ? LU[(size_t)(c0 + r) * n1 + c0 + c] : 0.0;
        }
        __syncthreads();
        if (warp == 0) {
            double yv = lane < bs ? ysh[c0 + lane] : 0.0;
            for (int c = bs - 1; c >= 0; --c) {
                if (lane == c) yv = yv / blk[c][c];
                const double xc = __shfl_sync(0xffffffffu, yv, c);
                if (lane < c) yv -= blk[lane][c] * xc;
            }
            if (lane < bs) ysh[c0 + lane] = yv;
            yb[lane] = lane < bs ? yv : 0.0;
        }
        __syncthreads();
        for (int r = threadIdx.x; r < c0; r += kLU) {
            const double *row = LU + (size_t)r * n1 + c0;
            double t = 0.0;
            for (int c = 0; c < bs; ++c) t += row[c] * yb[c];
            ysh[r] -= t;
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n1; t += kLU) y[t] = ysh[t];
    __syncthreads();
}

// max over the block (every thread gets the result)
__device__ double block_max(double v, double *sv) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sv[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = sv[0];
    for (int w = 1; w < kLU / 32; ++w) t = fmax(t, sv[w]);
    return t;
}

// FP32 LU with partial pivoting in place (row-major n1 x n1).  Returns false on a
// zero or non-finite pivot (the same value in every thread).
// max |v| with the lowest index on ties (deterministic), FP32: the FP32 factorisation's
// pivot search stays off the FP64 pipe (a warp-wide FP64 compare holds that pipe for
// 16 cycles, and every warp of the CTA runs this at every column)
__device__ void block_argmax_f(float v, int idx, float *sv, int *si, int *out_i) {
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_down_sync(0xffffffffu, v, o);
        const int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sv[w] = v; si[w] = idx; }
    __syncthreads();
    if (w == 0) {
        v = (lane < kLU / 32) ? sv[lane] : -1.0f;
        idx = (lane < kLU / 32) ? si[lane] : 0x7fffffff;
        for (int o = 16; o > 0; o >>= 1) {
            const float ov = __shfl_down_sync(0xffffffffu, v, o);
            const int oi = __shfl_down_sync(0xffffffffu, idx, o);
            if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
        }
        if (lane == 0) *out_i = idx;
    }
    __syncthreads();
}

// FP32 LU with partial pivoting, in place; false on a zero or non-finite pivot
__device__ bool lu_factor_f32(float *A, int *perm, int n1, double *sv, int *si, double *piv_v, int *piv_i,
                              double &pmin, double &pmax) {
    float *svf = reinterpret_cast<float *>(sv);
    float fmin_p = 3.0e38f, fmax_p = 0.f;
    for (int k = 0; k < n1; ++k) {
        float best = -1.0f;
        int bi = 0x7fffffff;
        for (int r = k + threadIdx.x; r < n1; r += kLU) {
            const float v = fabsf(A[(size_t)r * n1 + k]);
            if (v > best || (v == best && r < bi)) { best = v; bi = r; }
        }
        block_argmax_f(best, bi, svf, si, piv_i);
        const int p = *piv_i;
        if (threadIdx.x == 0) perm[k] = p;
        if (p != k)
            for (int c = threadIdx.x; c < n1; c += kLU) {
                const float t = A[(size_t)k * n1 + c];
                A[(size_t)k * n1 + c] = A[(size_t)p * n1 + c];
                A[(size_t)p * n1 + c] = t;
            }
        __syncthreads();
        const float pv = A[(size_t)k * n1 + k];
        const float apv = fabsf(pv);
        if (!(apv > 0.f) || !isfinite(pv)) return false;
        fmin_p = fminf(fmin_p, apv);
        fmax_p = fmaxf(fmax_p, apv);
        const float inv = 1.0f / pv;
        for (int r = k + 1 + threadIdx.x; r < n1; r += kLU) A[(size_t)r * n1 + k] *= inv;
        __syncthreads();
        // rank-1 update: a warp per row, lanes along the row (coalesced, no index division)
        const float *prow = A + (size_t)k * n1;
        for (int rr = k + 1 + (threadIdx.x >> 5); rr < n1; rr += kLU / 32) {
            float *row = A + (size_t)rr * n1;
            const float l = row[k];
            for (int cc = k + 1 + (threadIdx.x & 31); cc < n1; cc += 32) row[cc] -= l * prow[cc];
        }
        __syncthreads();
    }
    pmin = fmin(pmin, (double)fmin_p);
    pmax = fmax(pmax, (double)fmax_p);
    (void)piv_v;
    return true;
}

// x = (P L U)^{-1} y with the FP32 factors; y (overwritten) and x in shared memory.
// One barrier per column: forward elimination updates y below the column, backward
// substitution writes x[c] and updates y above it.
// Blocked FP32 LU with partial pivoting (right-looking, panels of 32 columns), in place, for
// n1 <= kLUBlockedMax.  Per panel: the panel's rows (32 columns, stride 33 against bank
// conflicts) are factored in shared memory with the same partial pivoting; its row swaps
// are applied to the other columns (one thread per column, the swaps in order); U12 is
// solved against the panel's unit-lower block; and the trailing matrix takes one rank-32
// update per panel, staged through a 32 x 64 tile of U12, instead of 32 rank-1 updates
// that each re-read it from L2.  smem: n1 * 33 + 32 * 64 floats.  false on a zero pivot.
constexpr int kLUNB = 32;
constexpr int kLUBlockedMax = 1536;
constexpr int kLUTile = 64;
__device__ bool lu_factor_f32_blocked(float *A, int *perm, int n1, float *smem, float *svf, int *si, int *piv_i,
                                      double &pmin, double &pmax) {
    float *P = smem;                                  // [n1][33] panel rows k0..n1-1
    float *U = smem + (size_t)n1 * (kLUNB + 1);       // [32][kLUTile] tile of U12
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float fmin_p = 3.0e38f, fmax_p = 0.f;
    bool ok = true;
    for (int k0 = 0; k0 < n1; k0 += kLUNB) {
        const int nb = min(kLUNB, n1 - k0), m = n1 - k0;
        // 1. the panel into shared memory
        for (int t = threadIdx.x; t < m * kLUNB; t += kLU) {
            const int r = t >> 5, c = t & 31;
            P[r * (kLUNB + 1) + c] = c < nb ? A[(size_t)(k0 + r) * n1 + k0 + c] : 0.f;
        }
        __syncthreads();
        // 2. factor the panel (partial pivoting over all its rows)
        for (int j = 0; j < nb; ++j) {
            float best = -1.0f;
            int bi = 0x7fffffff;
            for (int r = j + threadIdx.x; r < m; r += kLU) {
                const float v = fabsf(P[r * (kLUNB + 1) + j]);
                if (v > best || (v == best && r < bi)) { best = v; bi = r; }
            }
            block_argmax_f(best, bi, svf, si, piv_i);
            const int p = *piv_i;
            if (threadIdx.x == 0) perm[k0 + j] = k0 + p;
            if (p != j && threadIdx.x < kLUNB) {
                const float t = P[j * (kLUNB + 1) + threadIdx.x];
                P[j * (kLUNB + 1) + threadIdx.x] = P[p * (kLUNB + 1) + threadIdx.x];
                P[p * (kLUNB + 1) + threadIdx.x] = t;
            }
            __syncthreads();
            const float pv = P[j * (kLUNB + 1) + j];
            const float apv = fabsf(pv);
            if (!(apv > 0.f) || !isfinite(pv)) {
                ok = false;
                break;  // uniform: every thread read the same pivot
            }
            fmin_p = fminf(fmin_p, apv);
            fmax_p = fmaxf(fmax_p, apv);
            const float inv = 1.0f / pv;
            // scale the column and update the panel's remaining columns: a thread per row, so a
            // warp instruction covers 32 rows of one column with every lane busy (stride 33:
            // no bank conflicts; the pivot row is a broadcast)
            const float *pj = P + j * (kLUNB + 1);
            for (int r = j + 1 + threadIdx.x; r < m; r += kLU) {
                float *row = P + r * (kLUNB + 1);
                const float l = row[j] * inv;
                row[j] = l;
                for (int c = j + 1; c < nb; ++c) row[c] -= l * pj[c];
            }
            __syncthreads();
        }
        if (!ok) break;
        // 3. the factored panel back to global memory
        for (int t = threadIdx.x; t < m * kLUNB; t += kLU) {
            const int r = t >> 5, c = t & 31;
            if (c < nb) A[(size_t)(k0 + r) * n1 + k0 + c] = P[r * (kLUNB + 1) + c];
        }
        // 4. the panel's row swaps on every other column (a thread per column, swaps in order)
        for (int c = threadIdx.x; c < n1; c += kLU) {
            if (c >= k0 && c < k0 + nb) continue;
            for (int j = 0; j < nb; ++j) {
                const int p = perm[k0 + j];
                if (p != k0 + j) {
                    const float t = A[(size_t)(k0 + j) * n1 + c];
                    A[(size_t)(k0 + j) * n1 + c] = A[(size_t)p * n1 + c];
                    A[(size_t)p * n1 + c] = t;
                }
            }
        }
        __syncthreads();
        const int c1 = k0 + nb;
        if (c1 >= n1) break;
        // 5. U12 = L11^-1 A12 (unit lower L11 from the panel), a thread per column
        for (int c = c1 + threadIdx.x; c < n1; c += kLU) {
            float u[kLUNB];
#pragma unroll
            for (int j = 0; j < kLUNB; ++j) u[j] = j < nb ? A[(size_t)(k0 + j) * n1 + c] : 0.f;
#pragma unroll
            for (int j = 0; j < kLUNB; ++j)
#pragma unroll
                for (int i = j + 1; i < kLUNB; ++i) u[i] -= P[i * (kLUNB + 1) + j] * u[j];
#pragma unroll
            for (int j = 0; j < kLUNB; ++j)
                if (j < nb) A[(size_t)(k0 + j) * n1 + c] = u[j];
        }
        __syncthreads();
        // 6. A22 -= L21 U12, column tiles of kLUTile staged in shared memory
        for (int t0 = c1; t0 < n1; t0 += kLUTile) {
            const int w = min(kLUTile, n1 - t0);
            for (int t = threadIdx.x; t < kLUNB * kLUTile; t += kLU) {
                const int j = t / kLUTile, c = t - j * kLUTile;
                U[t] = (j < nb && c < w) ? A[(size_t)(k0 + j) * n1 + t0 + c] : 0.f;
            }
            __syncthreads();
            const int c = threadIdx.x % kLUTile;
            if (c < w)
                for (int r = nb + threadIdx.x / kLUTile; r < m; r += kLU / kLUTile) {
                    const float *l = P + r * (kLUNB + 1);
                    float acc = A[(size_t)(k0 + r) * n1 + t0 + c];
#pragma unroll
                    for (int j = 0; j < kLUNB; ++j) acc -= l[j] * U[j * kLUTile + c];
                    A[(size_t)(k0 + r) * n1 + t0 + c] = acc;
                }
            __syncthreads();
        }
    }
    pmin = fmin(pmin, (double)fmin_p);
    pmax = fmax(pmax, (double)fmax_p);
    __syncthreads();
    return ok;
}

// Solve LU x = P y in FP32 (unit lower L, upper U, both in LU), blocked by 32 columns: the
// 32x32 diagonal block is staged in shared memory and solved by one warp (shuffles, no block
// barrier), then every warp updates the remaining rows with the block's 32 values (a warp per
// row, coalesced).  Three block barriers per 32 columns instead of one per column.
__device__ void lu_apply_f32(const float *__restrict__ LU, const int *__restrict__ perm, int n1, float *y, float *x) {
    __shared__ float blk[32][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < n1; ++k) {
            const int p = perm[k];
            if (p != k) { const float t = y[k]; y[k] = y[p]; y[p] = t; }
        }
    __syncthreads();
    // forward: L (unit diagonal)
    for (int c0 = 0; c0 < n1; c0 += 32) {
        const int bs = min(32, n1 - c0);
        for (int t = threadIdx.x; t < bs * 32; t += kLU) {
            const int r = t >> 5, c = t & 31;
            blk[r][c] = c < bs ? LU[(size_t)(c0 + r) * n1 + c0 + c] : 0.f;
        }
        __syncthreads();
        if (warp == 0) {
            float yv = lane < bs ? y[c0 + lane] : 0.f;
            for (int c = 0; c < bs - 1; ++c) {
                const float yc = __shfl_sync(0xffffffffu, yv, c);
                if (lane > c && lane < bs) yv -= blk[lane][c] * yc;
            }
            if (lane < bs) y[c0 + lane] = yv;
        }
        __syncthreads();
        for (int r = c0 + bs + warp; r < n1; r += kLU / 32) {
            float t = lane < bs ? LU[(size_t)r * n1 + c0 + lane] * y[c0 + lane] : 0.f;
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) y[r] -= t;
        }
        __syncthreads();
    }
    // backward: U
    for (int c1 = n1; c1 > 0; c1 -= 32) {
        const int c0 = max(0, c1 - 32), bs = c1 - c0;
        for (int t = threadIdx.x; t < bs * 32; t += kLU) {
            const int r = t >> 5, c = t & 31;
            blk[r][c] = c < bs ? LU[(size_t)(c0 + r) * n1 + c0 + c] : 0.f;
        }
        __syncthreads();
        if (warp == 0) {
            float yv = lane < bs ? y[c0 + lane] : 0.f;
            for (int c = bs - 1; c >= 0; --c) {
                if (lane == c) yv = yv / blk[c][c];
                const float xc = __shfl_sync(0xffffffffu, yv, c);
                if (lane < c) yv -= blk[lane][c] * xc;
            }
            if (lane < bs) {
                y[c0 + lane] = yv;
                x[c0 + lane] = yv;
            }
        }
        __syncthreads();
        for (int r = warp; r < c0; r += kLU / 32) {
            float t = lane < bs ? LU[(size_t)r * n1 + c0 + lane] * x[c0 + lane] : 0.f;
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (lane == 0) y[r] -= t;
        }
        __syncthreads();
    }
}
// sum over the block, fixed order (every thread gets the result)
__device__ double block_sum(double v, double *sv) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sv[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < kLU / 32; ++w) t += sv[w];
    return t;
}

// d.r <- K^{-1} d.r with the factors that solved the system: FP32 (in the first half of As,
// through the FP32 shared vectors ys/xs) or FP64 (in As).  Non-finite FP32 results (a system
// far beyond FP32) read as 1e300.
__device__ void apply_inverse(const SolveDesc &d, int n1, bool f32, float *ys, float *xs) {
    if (f32) {
        __syncthreads();
        for (int t = threadIdx.x; t < n1; t += kLU) ys[t] = (float)d.r[t];
        lu_apply_f32(reinterpret_cast<const float *>(d.As), d.perm, n1, ys, xs);
        for (int t = threadIdx.x; t < n1; t += kLU) {
            const float v = xs[t];
            d.r[t] = isfinite(v) ? (double)v : 1e300;
        }
        __syncthreads();
    } else {
        lu_apply(d.As, d.perm, n1, d.r, reinterpret_cast<double *>(ys));
        __syncthreads();
    }
}

// Estimate of ||K^{-1}||_1 for the symmetric bordered matrix K (so K^{-T} = K^{-1}):
// Hager's method (W. W. Hager, "Condition estimates", SIAM J. Sci. Stat. Comput. 5 (1984)
// 311-316) with Higham's extra test vector (N. J. Higham, ACM TOMS 14 (1988) 381-396),
// at most four sign iterations.  A lower bound that is almost always within a small factor.
// Uses d.r as the work vector.
__device__ double inverse_norm1_estimate(const SolveDesc &d, int n1, bool f32, float *fsh, double *sv, int *si,
                                         double *piv_v, int *piv_i) {
    float *ys = fsh, *xs = fsh + n1;
    for (int t = threadIdx.x; t < n1; t += kLU) d.r[t] = 1.0 / (double)n1;
    apply_inverse(d, n1, f32, ys, xs);
    double a = 0.0;
    for (int t = threadIdx.x; t < n1; t += kLU) a += fabs(d.r[t]);
    double est = block_sum(a, sv);
    int jprev = -1;
    for (int it = 0; it < 4; ++it) {
        for (int t = threadIdx.x; t < n1; t += kLU) d.r[t] = d.r[t] >= 0.0 ? 1.0 : -1.0;
        apply_inverse(d, n1, f32, ys, xs);  // z = K^{-T} sign(y)
        double best = -1.0, zsum = 0.0;
        int bi = 0x7fffffff;
        for (int t = threadIdx.x; t < n1; t += kLU) {
            const double v = fabs(d.r[t]);
            zsum += d.r[t];
            if (v > best || (v == best && t < bi)) { best = v; bi = t; }
        }
        zsum = block_sum(zsum, sv);
        block_argmax(best, bi, sv, si, piv_v, piv_i);
        const double zmax = *piv_v;
        const int j = *piv_i;
        const double ztx = jprev < 0 ? zsum / (double)n1 : d.r[jprev];
        __syncthreads();
        if (!(zmax > ztx)) break;  // uniform: every thread read the same values
        for (int t = threadIdx.x; t < n1; t += kLU) d.r[t] = t == j ? 1.0 : 0.0;
        apply_inverse(d, n1, f32, ys, xs);
        double b = 0.0;
        for (int t = threadIdx.x; t < n1; t += kLU) b += fabs(d.r[t]);
        b = block_sum(b, sv);
        if (!(b > est)) break;
        est = b;
        jprev = j;
    }
    for (int t = threadIdx.x; t < n1; t += kLU)
        d.r[t] = ((t & 1) ? -1.0 : 1.0) * (1.0 + (double)t / (double)max(n1 - 1, 1));
    apply_inverse(d, n1, f32, ys, xs);
    double c = 0.0;
    for (int t = threadIdx.x; t < n1; t += kLU) c += fabs(d.r[t]);
    c = 2.0 * block_sum(c, sv) / (3.0 * (double)n1);
    est = fmax(est, c);
    return est < 1e300 ? est : 1e300;
}

constexpr int kRefineMax = 30;  // and stop early once a step no longer halves the residual
// systems factored across the GPU (FP32 first by our panels, the bound being the panel rows
// that fit shared memory at 4 columns; FP64 by cuSOLVER when the FP32 refinement does not
// converge): n1 in [kLUWideMin, kLUWideMax]
constexpr int kLUWideMin = 768;
// systems of kLUHost64Min to kLUWideMin unknowns keep their FP32 factorisation in the CTA, but
// when its refinement stalls the FP64 factors come from across the GPU (cuSOLVER getrf): an
// in-CTA FP64 LU of 425 unknowns takes ~13 ms on one SM's FP64 pipe
constexpr int kLUHost64Min = 256;
constexpr int kLUWideMax = (int)((225 * 1024) / (sizeof(float) * 5));

// r = bs - A0 x in FP64: a warp per row, lanes along the row, fixed-order shuffle sum
__device__ void residual(const SolveDesc &d, int n1) {
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int rr = threadIdx.x >> 5; rr < n1; rr += kLU / 32) {
        const double *row = d.A0 + (size_t)rr * n1;
        double s = 0.0;
        for (int c = lane; c < n1; c += 32) s += row[c] * d.x[c];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) d.r[rr] = d.bs[rr] - s;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kLU) lu_solve_refine_kernel(const SolveDesc *__restrict__ descs) {
    const SolveDesc d = descs[blockIdx.x];
    if (d.wide64 || d.host32) return;  // refined on the host path (factor_refine_wide64, refine_wide32)
    const int n1 = d.n + 1;
    extern __shared__ __align__(16) float fsh[];  // [2 * n1]: right-hand side / correction in FP32 (or n1 doubles)
    float *ys = fsh, *xs = fsh + n1;
    __shared__ double sv[kLU / 32];
    __shared__ int si[kLU / 32];
    __shared__ double piv_v;
    __shared__ int piv_i;
    double pmin = 1e308, pmax = 0.0, res = 0.0;
    int singular = 0, steps = 0;
    bool done = false;

    // ---- FP32 LU + FP64-residual refinement
    if (!d.wide64) {
        float *L = reinterpret_cast<float *>(d.As);  // the first half of the FP64 work matrix
        const bool wide32 = d.pre && !d.host64;  // FP32 factors from across the GPU
        if (!wide32)
            for (long long t = threadIdx.x; t < (long long)n1 * n1; t += kLU) L[t] = (float)d.A0[t];
        for (int t = threadIdx.x; t < n1; t += kLU) {
            d.x[t] = 0.0;
            d.r[t] = d.bs[t];
        }
        __syncthreads();
        bool factored;
        if (wide32) {  // factored across the GPU before this launch (lu_wide_factor)
            factored = d.pre[0] == 0.0;
            if (factored) {
                pmin = fmin(pmin, d.pre[1]);
                pmax = fmax(pmax, d.pre[2]);
            }
        } else {
            factored = n1 <= kLUBlockedMax ? lu_factor_f32_blocked(L, d.perm, n1, fsh, reinterpret_cast<float *>(sv),
                                                                   si, &piv_i, pmin, pmax)
                                           : lu_factor_f32(L, d.perm, n1, sv, si, &piv_v, &piv_i, pmin, pmax);
        }
        if (factored) {
            double an = 0.0;  // |A| (max row sum)
            for (int rr = threadIdx.x; rr < n1; rr += kLU) {
                double s = 0.0;
                for (int c = 0; c < n1; ++c) s += fabs(d.A0[(size_t)rr * n1 + c]);
                an = fmax(an, s);
            }
            an = block_max(an, sv);
            double rprev = 1e308;
            for (int it = 0; it < kRefineMax && !done; ++it) {
                double rm = 0.0;
                for (int t = threadIdx.x; t < n1; t += kLU) rm = fmax(rm, fabs(d.r[t]));
                rm = block_max(rm, sv);
                if (rm == 0.0) {
                    done = true;
                    break;
                }
                const double inv = 1.0 / rm;
                ++steps;
                for (int t = threadIdx.x; t < n1; t += kLU) ys[t] = (float)(d.r[t] * inv);
                lu_apply_f32(L, d.perm, n1, ys, xs);
                for (int t = threadIdx.x; t < n1; t += kLU) d.x[t] += (double)xs[t] * rm;
                __syncthreads();
                double rn = 0.0, xn = 0.0;
                residual(d, n1);
                for (int rr = threadIdx.x; rr < n1; rr += kLU) {
                    rn = fmax(rn, fabs(d.r[rr]));
                    xn = fmax(xn, fabs(d.x[rr]));
                }
                rn = block_max(rn, sv);
                xn = block_max(xn, sv);
                res = rn;
                if (rn <= (double)n1 * 1.1102230246251565e-16 * an * xn) done = true;
                // stalled (cond(A) near 1/eps32 or beyond): no use refining further, FP64 takes over
                else if (it >= 2 && rn > 0.5 * rprev) break;
                rprev = rn;
            }
        }
        __syncthreads();
    }

    // A wide (or mid-size) system whose FP32 factors did not converge is factored in FP64 and
    // refined by the host path (factor_refine_wide64); nothing is written here.
    if (!done && d.pre) {
        if (threadIdx.x == 0) d.pre[0] = 2.0;
        return;
    }

    // ---- fallback: FP64 LU with one step of FP64 refinement
    const bool f32_solved = done;
    if (!done) {
        double *A = d.As;
        {
        for (long long t = threadIdx.x; t < (long long)n1 * n1; t += kLU) A[t] = d.A0[t];
        __syncthreads();
        pmin = 1e308;
        pmax = 0.0;
        for (int k = 0; k < n1; ++k) {
            double best = -1.0;
            int bi = 0x7fffffff;
            for (int r = k + threadIdx.x; r < n1; r += kLU) {
                double v = fabs(A[(size_t)r * n1 + k]);
                if (v > best || (v == best && r < bi)) { best = v; bi = r; }
            }
            block_argmax(best, bi, sv, si, &piv_v, &piv_i);
            const int p = piv_i;
            if (threadIdx.x == 0) d.perm[k] = p;
            if (p != k)
                for (int c = threadIdx.x; c < n1; c += kLU) {
                    double t = A[(size_t)k * n1 + c];
                    A[(size_t)k * n1 + c] = A[(size_t)p * n1 + c];
                    A[(size_t)p * n1 + c] = t;
                }
            __syncthreads();
            double pv = A[(size_t)k * n1 + k];
            double apv = fabs(pv);
            pmin = fmin(pmin, apv);
            pmax = fmax(pmax, apv);
            if (!(apv > 1e-300)) {  // exactly singular: keep going with a tiny pivot, flag it
                singular = 1;
                pv = (pv < 0 ? -1e-300 : 1e-300);
                if (threadIdx.x == 0) A[(size_t)k * n1 + k] = pv;
            }
            __syncthreads();
            const double inv = 1.0 / pv;
            for (int r = k + 1 + threadIdx.x; r < n1; r += kLU) A[(size_t)r * n1 + k] *= inv;
            __syncthreads();
            const double *prow = A + (size_t)k * n1;
            for (int rr = k + 1 + (threadIdx.x >> 5); rr < n1; rr += kLU / 32) {
                double *row = A + (size_t)rr * n1;
                const double l = row[k];
                for (int cc = k + 1 + (threadIdx.x & 31); cc < n1; cc += 32) row[cc] -= l * prow[cc];
            }
            __syncthreads();
        }
        }
        for (int t = threadIdx.x; t < n1; t += kLU) d.x[t] = d.bs[t];
        lu_apply(A, d.perm, n1, d.x, reinterpret_cast<double *>(fsh));
        for (int rr = threadIdx.x; rr < n1; rr += kLU) {
            double s = d.bs[rr];
            const double *row = d.A0 + (size_t)rr * n1;
            for (int c = 0; c < n1; ++c) s -= row[c] * d.x[c];
            d.r[rr] = s;
        }
        lu_apply(A, d.perm, n1, d.r, reinterpret_cast<double *>(fsh));
        for (int t = threadIdx.x; t < n1; t += kLU) d.x[t] += d.r[t];
        __syncthreads();
        double rmax = 0.0;
        for (int rr = threadIdx.x; rr < n1; rr += kLU) {
            double s = d.bs[rr];
            const double *row = d.A0 + (size_t)rr * n1;
            for (int c = 0; c < n1; ++c) s -= row[c] * d.x[c];
            rmax = fmax(rmax, fabs(s));
        }
        res = block_max(rmax, sv);
    }
    // ---- conditioning: kappa = ||A||_1 ||K^{-1}||_1 with A the folded normal matrix (RESP
    // included, the border excluded) and K the bordered matrix.  A relative error e in A moves
    // the solution by about e * kappa * |q| at worst, so kappa says how much of the Gram's
    // rounding reaches the charges (the fit escalates a mixed-precision cube beyond a limit).
    double anorm = 0.0;
    for (int c = threadIdx.x; c < d.n; c += kLU) {
        double sacc = 0.0;
        for (int rr = 0; rr < d.n; ++rr) sacc += fabs(d.A0[(size_t)rr * n1 + c]);
        anorm = fmax(anorm, sacc);
    }
    anorm = block_max(anorm, sv);
    const double kinv = inverse_norm1_estimate(d, n1, f32_solved, fsh, sv, si, &piv_v, &piv_i);
    if (threadIdx.x == 0) {
        d.info[0] = res;
        d.info[1] = pmin;
        d.info[2] = pmax;
        d.info[3] = singular;
        d.info[4] = fmin(anorm * kinv, 1e300);
        d.info[5] = n1;
        d.info[6] = steps;
        d.info[7] = f32_solved ? ((d.pre && !d.host64) ? 1.0 : 0.0) : 2.0;
    }
    __syncthreads();
    // expand to all atoms
    for (int i = threadIdx.x; i < d.N; i += kLU) d.q[i] = d.x[d.map[i]];
}

// ---------------------------------------------------------------------------
// Wide factorisation of one large system across the whole GPU, before lu_solve_refine_kernel
// refines it.  One CTA factoring n1^3 / 3 FMAs alone is SM-bound (20 ms at n1 = 1456 in FP32,
// and FP64 runs at 1/64 of the FP32 rate); here only the panels are serial.  A0 is copied into
// As (FP32 for the first attempt, FP64 when that does not converge), then per panel of nb
// columns (32, or 16 / 8 / 4 when the panel's rows do not fit shared memory at 32):
//   lu_panel_kernel   one CTA: the panel in shared memory, factored with the partial pivoting
//                     of the one-CTA factorisations (perm[k] = pivot row, full-row swaps; in
//                     FP64 a pivot below 1e-300 is replaced and flagged, as there), written
//                     back, its swaps applied to every other column;
//   lu_trsm_kernel    U12 = L11^-1 A12, a thread per column over many CTAs;
//   cuBLAS GEMM       A22 -= L21 U12 (SGEMM or DGEMM, plain GEMM).
// pre = {flag, min|pivot|, max|pivot|}.  FP32: flag 1 = zero or non-finite pivot (the later
// panels return at once), set to 2 by lu_solve_refine_kernel when the refinement does not
// converge.  FP64: flag 1 = a pivot was replaced (singular).
constexpr size_t kPanelSmem = 225 * 1024;

template <typename T>
int wide_panel_nb(int m) {
    for (int nb = 32; nb >= 4; nb /= 2)
        if (sizeof(T) * (size_t)m * (nb + 1) <= kPanelSmem) return nb;
    return 0;
}

template <typename T>
__global__ void lu_copy_kernel(const double *__restrict__ A0, T *__restrict__ L, long long n,
                               double *__restrict__ pre) {
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long t = t0; t < n; t += (long long)gridDim.x * blockDim.x) L[t] = (T)A0[t];
    if (t0 == 0) {
        pre[0] = 0.0;
        pre[1] = 1e308;
        pre[2] = 0.0;
    }
}

template <typename T>
__global__ void __launch_bounds__(kLU) lu_panel_kernel(T *__restrict__ A, int *__restrict__ perm, int n1, int k0,
                                                       int NB, double *__restrict__ pre) {
    constexpr bool f32 = sizeof(T) == 4;
    if (f32 && pre[0] != 0.0) return;  // an earlier panel met a zero pivot
    extern __shared__ __align__(16) unsigned char panel_raw[];
    T *P = reinterpret_cast<T *>(panel_raw);  // [m][NB + 1] panel rows k0..n1-1
    __shared__ double svd[kLU / 32];
    __shared__ int si[kLU / 32];
    __shared__ int piv_i;
    __shared__ double piv_v;
    const int m = n1 - k0, nb = min(NB, m), ld = NB + 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int t = threadIdx.x; t < m * NB; t += kLU) {
        const int r = t / NB, c = t - r * NB;
        P[r * ld + c] = c < nb ? A[(size_t)(k0 + r) * n1 + k0 + c] : T(0);
    }
    __syncthreads();
    double pmin_l = 1e308, pmax_l = 0.0;
    bool sing = false;
    for (int j = 0; j < nb; ++j) {
        T best = T(-1);
        int bi = 0x7fffffff;
        for (int r = j + threadIdx.x; r < m; r += kLU) {
            const T v = fabs(P[r * ld + j]);
            if (v > best || (v == best && r < bi)) { best = v; bi = r; }
        }
        if constexpr (f32)
            block_argmax_f(best, bi, reinterpret_cast<float *>(svd), si, &piv_i);
        else
            block_argmax(best, bi, svd, si, &piv_v, &piv_i);
        const int p = piv_i;
        if (threadIdx.x == 0) perm[k0 + j] = k0 + p;
        if (p != j && threadIdx.x < NB) {
            const T t = P[j * ld + threadIdx.x];
            P[j * ld + threadIdx.x] = P[p * ld + threadIdx.x];
            P[p * ld + threadIdx.x] = t;
        }
        __syncthreads();
        T pv = P[j * ld + j];
        const T apv = fabs(pv);
        if constexpr (f32) {
            if (!(apv > 0.f) || !isfinite(pv)) {  // uniform: every thread read the same pivot
                if (threadIdx.x == 0) pre[0] = 1.0;
                return;
            }
        } else {
            if (!(apv > 1e-300)) {  // exactly singular: a tiny pivot, flagged (as the one-CTA FP64 LU)
                sing = true;
                pv = pv < 0 ? T(-1e-300) : T(1e-300);
                if (threadIdx.x == 0) P[j * ld + j] = pv;
            }
        }
        pmin_l = fmin(pmin_l, (double)apv);
        pmax_l = fmax(pmax_l, (double)apv);
        const T inv = T(1) / pv;
        // a thread per row: one warp instruction covers 32 rows of a column, every lane busy
        // (the FP64 pipe takes the same time for a warp instruction with one lane or 32)
        const T *pj = P + j * ld;
        for (int r = j + 1 + threadIdx.x; r < m; r += kLU) {
            T *row = P + r * ld;
            const T l = row[j] * inv;
            row[j] = l;
            for (int c = j + 1; c < nb; ++c) row[c] -= l * pj[c];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < m * NB; t += kLU) {
        const int r = t / NB, c = t - r * NB;
        if (c < nb) A[(size_t)(k0 + r) * n1 + k0 + c] = P[r * ld + c];
    }
    for (int c = threadIdx.x; c < n1; c += kLU) {
        if (c >= k0 && c < k0 + nb) continue;
        for (int j = 0; j < nb; ++j) {
            const int p = perm[k0 + j];
            if (p != k0 + j) {
                const T t = A[(size_t)(k0 + j) * n1 + c];
                A[(size_t)(k0 + j) * n1 + c] = A[(size_t)p * n1 + c];
                A[(size_t)p * n1 + c] = t;
            }
        }
    }
    if (threadIdx.x == 0) {
        pre[1] = fmin(pre[1], pmin_l);
        pre[2] = fmax(pre[2], pmax_l);
        if (!f32 && sing) pre[0] = 1.0;
    }
}

template <typename T, int NB>
__global__ void __launch_bounds__(256) lu_trsm_kernel(T *__restrict__ A, int n1, int k0,
                                                      const double *__restrict__ pre) {
    if (sizeof(T) == 4 && pre[0] != 0.0) return;
    __shared__ T Ls[NB][NB + 1];
    const int nb = min(NB, n1 - k0), c1 = k0 + nb;
    for (int t = threadIdx.x; t < NB * NB; t += blockDim.x) {
        const int i = t / NB, j = t - i * NB;
        Ls[i][j] = (i < nb && j < nb) ? A[(size_t)(k0 + i) * n1 + k0 + j] : T(0);
    }
    __syncthreads();
    const int c = c1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n1) return;
    T u[NB];
#pragma unroll
    for (int j = 0; j < NB; ++j) u[j] = j < nb ? A[(size_t)(k0 + j) * n1 + c] : T(0);
#pragma unroll
    for (int j = 0; j < NB; ++j)
#pragma unroll
        for (int i = j + 1; i < NB; ++i) u[i] -= Ls[i][j] * u[j];
#pragma unroll
    for (int j = 0; j < NB; ++j)
        if (j < nb) A[(size_t)(k0 + j) * n1 + c] = u[j];
}

// dynamic shared memory of lu_solve_refine_kernel: the right-hand side and correction in
// FP32 (2 n1 floats) and, for the blocked factorisation, the panel and the U12 tile
size_t solve_smem_bytes(int n1) {
    size_t b = sizeof(float) * 2 * (size_t)n1;
    if (n1 <= kLUBlockedMax) b = std::max(b, sizeof(float) * ((size_t)n1 * (kLUNB + 1) + kLUNB * kLUTile));
    return b;
}

// the launch's shared memory opt-in, raised once to the largest the kernel can ask for
void lu_smem_optin() {
    smem_optin((const void *)lu_solve_refine_kernel,
               std::max(solve_smem_bytes(kLUBlockedMax), solve_smem_bytes(1)));
}

inline cublasStatus_t gemm_nn(cublasHandle_t h, int m, int n, int k, const float *alpha, const float *A, int lda,
                              const float *B, int ldb, const float *beta, float *C, int ldc) {
    return cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
inline cublasStatus_t gemm_nn(cublasHandle_t h, int m, int n, int k, const double *alpha, const double *A, int lda,
                              const double *B, int ldb, const double *beta, double *C, int ldc) {
    return cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// ---- FP64 wide factorisation by cuSOLVER's getrf
// The bordered matrix K is symmetric, so its row-major image is also K read column-major and
// cuSOLVER's getrf factors it in place (P K = L U, column-major), with its panels across the
// GPU instead of in one CTA each (an FP64 panel of 1851 x 32 costs ~0.25 ms on one SM's FP64
// pipe).  The refinement's residuals use A0 itself, so a Gram that is symmetric only to
// rounding costs nothing.
// pivot rows to 0-based interchanges, the pivots' range, and an exactly zero pivot replaced by
// 1e-300 and flagged (the in-CTA FP64 factorisation's rule); one CTA
__global__ void __launch_bounds__(1024) getrf_finish_kernel(double *__restrict__ LU, int n,
                                                            const int *__restrict__ ipiv, int *__restrict__ perm,
                                                            double *__restrict__ pre) {
    __shared__ double smin[32], smax[32];
    __shared__ int ssing[32];
    double mn = 1e308, mx = 0.0;
    int sing = 0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        perm[k] = ipiv[k] - 1;
        double *dk = LU + (size_t)k * n + k;
        const double a = fabs(*dk);
        if (!(a > 1e-300)) {
            sing = 1;
            *dk = (*dk < 0.0) ? -1e-300 : 1e-300;
        }
        mn = fmin(mn, a);
        mx = fmax(mx, a);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sing |= __shfl_xor_sync(0xffffffffu, sing, o);
    }
    if ((threadIdx.x & 31) == 0) {
        smin[threadIdx.x >> 5] = mn;
        smax[threadIdx.x >> 5] = mx;
        ssing[threadIdx.x >> 5] = sing;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mn = fmin(mn, smin[w]);
            mx = fmax(mx, smax[w]);
            sing |= ssing[w];
        }
        pre[0] = sing ? 1.0 : 0.0;
        pre[1] = mn;
        pre[2] = mx;
    }
}

// vectors of the refinement and of Hager's estimate: mode 0 fills 1/n, 1 takes the signs of v,
// 2 the unit vector e_j, 3 Higham's alternating vector (-1)^t (1 + t/(n-1)), 4 ones
__global__ void vec_fill_kernel(double *__restrict__ v, int n, int mode, int j) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (mode == 0) v[t] = 1.0 / (double)n;
    else if (mode == 1) v[t] = v[t] >= 0.0 ? 1.0 : -1.0;
    else if (mode == 2) v[t] = t == j ? 1.0 : 0.0;
    else if (mode == 3) v[t] = ((t & 1) ? -1.0 : 1.0) * (1.0 + (double)t / (double)max(n - 1, 1));
    else v[t] = 1.0;
}

// ||A||_1 of the folded normal matrix (the first n rows and columns of the bordered A0)
__global__ void anorm1_kernel(const double *__restrict__ A0, int n, int n1, unsigned long long *__restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    double s = 0.0;
    for (int r = 0; r < n; ++r) s += fabs(A0[(size_t)r * n1 + c]);
    atomicMax(out, (unsigned long long)__double_as_longlong(s));  // s >= 0: bits order like values
}

__global__ void expand_kernel(const double *__restrict__ x, const int *__restrict__ map, int N, double *__restrict__ q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) q[i] = x[map[i]];
}

// A system whose FP32 refinement cannot converge (or an escalated fit's, at once): FP64 factors
// from cuSOLVER's getrf (K is symmetric, so its row-major image read column-major is K itself),
// one step of FP64 refinement, the residual and Hager's estimate of ||K^-1||_1 (the same steps
// and vectors as lu_solve_refine_kernel's, with getrs solves and cuBLAS reductions across the
// GPU instead of triangular solves in one CTA), then the info words and the charges.  Waits.
void factor_refine_wide64(rp_ctx *ctx, const SolveDesc &d, int n1, cudaStream_t stream) {
    double *LU = d.As;
    const long long nn = (long long)n1 * n1;
    {
        StageTimer tt(ctx, "solve_lu_wide64", stream);
        lu_copy_kernel<double><<<(int)std::min<long long>(ceil_div(nn, 256), 4096), 256, 0, stream>>>(d.A0, LU, nn,
                                                                                                        d.pre);
        RP_LAUNCH_CHECK();
    }
    cusolverDnHandle_t hs = ctx->solver();
    if (cusolverDnSetStream(hs, stream) != CUSOLVER_STATUS_SUCCESS) fail(RP_E_CUDA, "cusolverDnSetStream failed");
    cublasHandle_t hb = ctx->blas();
    RP_CUBLAS(cublasSetStream(hb, stream));
    int lwork = 0;
    if (cusolverDnDgetrf_bufferSize(hs, n1, n1, LU, n1, &lwork) != CUSOLVER_STATUS_SUCCESS)
        fail(RP_E_CUDA, "cusolverDnDgetrf_bufferSize failed");
    double *work = ctx->buf_t<double>("s_getrf_work", (size_t)std::max(lwork, 1));
    int *ipiv = ctx->buf_t<int>("s_getrf_ipiv", (size_t)n1 + 1);  // [n1] pivots, then the info word
    unsigned long long *anorm_bits = ctx->buf_t<unsigned long long>("s_anorm", 1);
    {
        StageTimer tt(ctx, "solve_lu_wide64", stream);
        if (cusolverDnDgetrf(hs, n1, n1, LU, n1, work, ipiv, ipiv + n1) != CUSOLVER_STATUS_SUCCESS)
            fail(RP_E_CUDA, "cusolverDnDgetrf failed");
        getrf_finish_kernel<<<1, 1024, 0, stream>>>(LU, n1, ipiv, d.perm, d.pre);
        RP_LAUNCH_CHECK();
    }
    StageTimer tt(ctx, "solve_refine64", stream);
    auto solve = [&](double *v) {
        if (cusolverDnDgetrs(hs, CUBLAS_OP_N, n1, 1, LU, n1, ipiv, v, n1, ipiv + n1) != CUSOLVER_STATUS_SUCCESS)
            fail(RP_E_CUDA, "cusolverDnDgetrs failed");
    };
    const double one = 1.0, minus_one = -1.0;
    auto residual = [&]() {  // r = bs - A0 x (A0 row-major: its transpose in cuBLAS's terms)
        RP_CUDA(cudaMemcpyAsync(d.r, d.bs, sizeof(double) * n1, cudaMemcpyDeviceToDevice, stream));
        RP_CUBLAS(cublasDgemv(hb, CUBLAS_OP_T, n1, n1, &minus_one, d.A0, n1, d.x, 1, &one, d.r, 1));
    };
    const int nb = (int)ceil_div(n1, 256);
    RP_CUDA(cudaMemcpyAsync(d.x, d.bs, sizeof(double) * n1, cudaMemcpyDeviceToDevice, stream));
    solve(d.x);
    residual();
    solve(d.r);
    RP_CUBLAS(cublasDaxpy(hb, n1, &one, d.r, 1, d.x, 1));
    residual();
    int im = 0;
    RP_CUBLAS(cublasIdamax(hb, n1, d.r, 1, &im));  // 1-based
    double res = 0.0, pre[3];
    RP_CUDA(cudaMemcpyAsync(&res, d.r + (im - 1), sizeof(double), cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaMemcpyAsync(pre, d.pre, sizeof(pre), cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaMemsetAsync(anorm_bits, 0, sizeof(unsigned long long), stream));
    anorm1_kernel<<<(int)ceil_div(std::max(d.n, 1), 256), 256, 0, stream>>>(d.A0, d.n, n1, anorm_bits);
    RP_LAUNCH_CHECK();
    unsigned long long abits = 0;
    RP_CUDA(cudaMemcpyAsync(&abits, anorm_bits, sizeof(abits), cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaStreamSynchronize(stream));
    res = std::fabs(res);
    double anorm;
    std::memcpy(&anorm, &abits, sizeof(anorm));
    // Hager's estimate of ||K^-1||_1 (K symmetric: K^-T = K^-1), on d.r
    auto asum = [&]() {
        double v = 0.0;
        RP_CUBLAS(cublasDasum(hb, n1, d.r, 1, &v));
        return v;
    };
    double *ones = ctx->buf_t<double>("s_ones", (size_t)n1);
    vec_fill_kernel<<<nb, 256, 0, stream>>>(ones, n1, 4, 0);
    vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 0, 0);
    solve(d.r);
    double est = asum();
    int jprev = -1;
    for (int it = 0; it < 4; ++it) {
        vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 1, 0);
        solve(d.r);
        int jm = 0;
        RP_CUBLAS(cublasIdamax(hb, n1, d.r, 1, &jm));
        const int j = jm - 1;
        double zj = 0.0, ztx = 0.0;
        RP_CUDA(cudaMemcpyAsync(&zj, d.r + j, sizeof(double), cudaMemcpyDeviceToHost, stream));
        if (jprev >= 0) RP_CUDA(cudaMemcpyAsync(&ztx, d.r + jprev, sizeof(double), cudaMemcpyDeviceToHost, stream));
        double zsum = 0.0;
        RP_CUBLAS(cublasDdot(hb, n1, d.r, 1, ones, 1, &zsum));
        RP_CUDA(cudaStreamSynchronize(stream));
        if (jprev < 0) ztx = zsum / (double)n1;
        if (!(std::fabs(zj) > ztx)) break;
        vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 2, j);
        solve(d.r);
        const double bval = asum();
        if (!(bval > est)) break;
        est = bval;
        jprev = j;
    }
    vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 3, 0);
    solve(d.r);
    est = std::max(est, 2.0 * asum() / (3.0 * (double)n1));
    const double kinv = est < 1e300 ? est : 1e300;
    double *hinfo = static_cast<double *>(ctx->host_buf("s_info64", sizeof(double) * kSolveInfo));
    hinfo[0] = res;
    hinfo[1] = pre[1];
    hinfo[2] = pre[2];
    hinfo[3] = pre[0];
    hinfo[4] = std::fmin(anorm * kinv, 1e300);
    hinfo[5] = n1;
    hinfo[6] = 1;
    hinfo[7] = 3.0;  // FP64 factors from across the GPU
    RP_CUDA(cudaMemcpyAsync(d.info, hinfo, sizeof(double) * kSolveInfo, cudaMemcpyHostToDevice, stream));
    expand_kernel<<<(int)ceil_div(d.N, 256), 256, 0, stream>>>(d.x, d.map, d.N, d.q);
    RP_LAUNCH_CHECK();
    RP_CUDA(cudaStreamSynchronize(stream));  // the pinned info words are reused by the next system
}

// ---- host-driven refinement with wide FP32 factors
// The refinement of lu_solve_refine_kernel for a system whose FP32 factors were computed across
// the GPU (lu_wide_factor<float>): the same steps (scaled FP32 corrections, FP64 residuals, the
// backward-error stop, the stall rule) and the same condition estimate, with cuBLAS DGEMV
// residuals and STRSV solves across the GPU instead of one CTA's (whose FP64 residual alone takes
// ~1 ms on one SM's FP64 pipe at 2001 unknowns).  Returns false when the refinement stalls: the
// caller then factors the system in FP64 (factor_refine_wide64).  Waits.

// y (FP32) = v / scale, or v with non-finite values as they are (scale 0: plain conversion)
__global__ void to_f32_kernel(const double *__restrict__ v, int n, double scale, float *__restrict__ y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) y[t] = (float)(scale != 0.0 ? v[t] / scale : v[t]);
}
// mode 0: x += y * scale;  mode 1: x = finite(y) ? y : 1e300 (the estimate's solves)
__global__ void from_f32_kernel(const float *__restrict__ y, int n, double scale, int mode, double *__restrict__ x) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (mode == 0) x[t] += (double)y[t] * scale;
    else x[t] = isfinite(y[t]) ? (double)y[t] : 1e300;
}
// the factorisation's row interchanges applied to y in order (one CTA, in shared memory)
__global__ void __launch_bounds__(1024) swap_rows_kernel(float *__restrict__ y, const int *__restrict__ perm, int n) {
    extern __shared__ float ysm[];
    for (int t = threadIdx.x; t < n; t += blockDim.x) ysm[t] = y[t];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < n; ++k) {
            const int p = perm[k];
            if (p != k) { const float v = ysm[k]; ysm[k] = ysm[p]; ysm[p] = v; }
        }
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += blockDim.x) y[t] = ysm[t];
}
// max row sum |A0| (the backward-error bound's ||A||)
__global__ void rowabs_max_kernel(const double *__restrict__ A0, int n1, unsigned long long *__restrict__ out) {
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (r >= n1) return;
    double s = 0.0;
    for (int c = lane; c < n1; c += 32) s += fabs(A0[(size_t)r * n1 + c]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong(s));
}

bool refine_wide32(rp_ctx *ctx, const SolveDesc &d, int n1, cudaStream_t stream) {
    StageTimer tt(ctx, "solve_refine32", stream);
    const float *LU = reinterpret_cast<const float *>(d.As);
    cublasHandle_t hb = ctx->blas();
    RP_CUBLAS(cublasSetStream(hb, stream));
    float *ys = ctx->buf_t<float>("s_r32_y", (size_t)n1);
    unsigned long long *bits = ctx->buf_t<unsigned long long>("s_r32_bits", 2);
    const int nb = (int)ceil_div(n1, 256);
    // pivot range and zero-pivot flag of the wide FP32 factorisation, ||A0|| (rows)
    double pre[3];
    RP_CUDA(cudaMemcpyAsync(pre, d.pre, sizeof(pre), cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaMemsetAsync(bits, 0, 2 * sizeof(unsigned long long), stream));
    rowabs_max_kernel<<<(int)ceil_div(n1, 8), 256, 0, stream>>>(d.A0, n1, bits);
    RP_LAUNCH_CHECK();
    if (d.n > 0) {
        anorm1_kernel<<<(int)ceil_div(d.n, 256), 256, 0, stream>>>(d.A0, d.n, n1, bits + 1);
        RP_LAUNCH_CHECK();
    }
    unsigned long long hbits[2] = {0, 0};
    RP_CUDA(cudaMemcpyAsync(hbits, bits, sizeof(hbits), cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaStreamSynchronize(stream));
    if (pre[0] != 0.0) return false;  // a zero FP32 pivot: FP64 takes over
    double an, anorm;
    std::memcpy(&an, &hbits[0], sizeof(an));
    std::memcpy(&anorm, &hbits[1], sizeof(anorm));
    auto apply = [&]() {  // ys = (P L U)^-1 ys in FP32
        swap_rows_kernel<<<1, 1024, sizeof(float) * (size_t)n1, stream>>>(ys, d.perm, n1);
        RP_LAUNCH_CHECK();
        RP_CUBLAS(cublasStrsv(hb, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, CUBLAS_DIAG_UNIT, n1, LU, n1, ys, 1));
        RP_CUBLAS(cublasStrsv(hb, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n1, LU, n1, ys, 1));
    };
    auto absmax = [&](const double *v) {
        int im = 0;
        RP_CUBLAS(cublasIdamax(hb, n1, v, 1, &im));
        double x = 0.0;
        RP_CUDA(cudaMemcpyAsync(&x, v + (im - 1), sizeof(double), cudaMemcpyDeviceToHost, stream));
        RP_CUDA(cudaStreamSynchronize(stream));
        return std::fabs(x);
    };
    const double one = 1.0, minus_one = -1.0;
    RP_CUDA(cudaMemsetAsync(d.x, 0, sizeof(double) * n1, stream));
    RP_CUDA(cudaMemcpyAsync(d.r, d.bs, sizeof(double) * n1, cudaMemcpyDeviceToDevice, stream));
    bool done = false;
    double res = 0.0, rprev = 1e308;
    int steps = 0;
    for (int it = 0; it < kRefineMax && !done; ++it) {
        const double rm = absmax(d.r);
        if (rm == 0.0) {
            done = true;
            break;
        }
        ++steps;
        to_f32_kernel<<<nb, 256, 0, stream>>>(d.r, n1, rm, ys);
        RP_LAUNCH_CHECK();
        apply();
        from_f32_kernel<<<nb, 256, 0, stream>>>(ys, n1, rm, 0, d.x);
        RP_LAUNCH_CHECK();
        RP_CUDA(cudaMemcpyAsync(d.r, d.bs, sizeof(double) * n1, cudaMemcpyDeviceToDevice, stream));
        RP_CUBLAS(cublasDgemv(hb, CUBLAS_OP_T, n1, n1, &minus_one, d.A0, n1, d.x, 1, &one, d.r, 1));
        const double rn = absmax(d.r), xn = absmax(d.x);
        res = rn;
        if (rn <= (double)n1 * 1.1102230246251565e-16 * an * xn) done = true;
        else if (it >= 2 && rn > 0.5 * rprev) break;  // stalled: FP64 takes over
        rprev = rn;
    }
    if (!done) return false;
    // Hager's estimate of ||K^-1||_1 with the FP32 factors (lu_solve_refine_kernel's steps)
    auto solve_r = [&]() {
        to_f32_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 0.0, ys);
        RP_LAUNCH_CHECK();
        apply();
        from_f32_kernel<<<nb, 256, 0, stream>>>(ys, n1, 0.0, 1, d.r);
        RP_LAUNCH_CHECK();
    };
    auto asum = [&]() {
        double v = 0.0;
        RP_CUBLAS(cublasDasum(hb, n1, d.r, 1, &v));
        return v;
    };
    double *ones = ctx->buf_t<double>("s_ones", (size_t)n1);
    vec_fill_kernel<<<nb, 256, 0, stream>>>(ones, n1, 4, 0);
    vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 0, 0);
    solve_r();
    double est = asum();
    int jprev = -1;
    for (int it = 0; it < 4; ++it) {
        vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 1, 0);
        solve_r();
        int jm = 0;
        RP_CUBLAS(cublasIdamax(hb, n1, d.r, 1, &jm));
        const int j = jm - 1;
        double zj = 0.0, ztx = 0.0, zsum = 0.0;
        RP_CUDA(cudaMemcpyAsync(&zj, d.r + j, sizeof(double), cudaMemcpyDeviceToHost, stream));
        if (jprev >= 0) RP_CUDA(cudaMemcpyAsync(&ztx, d.r + jprev, sizeof(double), cudaMemcpyDeviceToHost, stream));
        RP_CUBLAS(cublasDdot(hb, n1, d.r, 1, ones, 1, &zsum));
        RP_CUDA(cudaStreamSynchronize(stream));
        if (jprev < 0) ztx = zsum / (double)n1;
        if (!(std::fabs(zj) > ztx)) break;
        vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 2, j);
        solve_r();
        const double bval = asum();
        if (!(bval > est)) break;
        est = bval;
        jprev = j;
    }
    vec_fill_kernel<<<nb, 256, 0, stream>>>(d.r, n1, 3, 0);
    solve_r();
    est = std::max(est, 2.0 * asum() / (3.0 * (double)n1));
    const double kinv = est < 1e300 ? est : 1e300;
    double *hinfo = static_cast<double *>(ctx->host_buf("s_info32", sizeof(double) * kSolveInfo));
    hinfo[0] = res;
    hinfo[1] = pre[1];
    hinfo[2] = pre[2];
    hinfo[3] = 0.0;
    hinfo[4] = std::fmin(anorm * kinv, 1e300);
    hinfo[5] = n1;
    hinfo[6] = steps;
    hinfo[7] = 1.0;  // FP32 factors from across the GPU
    RP_CUDA(cudaMemcpyAsync(d.info, hinfo, sizeof(double) * kSolveInfo, cudaMemcpyHostToDevice, stream));
    expand_kernel<<<(int)ceil_div(d.N, 256), 256, 0, stream>>>(d.x, d.map, d.N, d.q);
    RP_LAUNCH_CHECK();
    RP_CUDA(cudaStreamSynchronize(stream));  // the pinned info words are reused by the next system
    return true;
}

template <typename T>
void lu_wide_factor(rp_ctx *ctx, const SolveDesc &d, int n1, cudaStream_t stream) {
    smem_optin((const void *)lu_panel_kernel<T>, kPanelSmem);
    T *L = reinterpret_cast<T *>(d.As);
    const long long nn = (long long)n1 * n1;
    lu_copy_kernel<T><<<(int)std::min<long long>(ceil_div(nn, 256), 4096), 256, 0, stream>>>(d.A0, L, nn, d.pre);
    RP_LAUNCH_CHECK();
    cublasHandle_t h = ctx->blas();
    RP_CUBLAS(cublasSetStream(h, stream));
    const T minus_one = T(-1), one = T(1);
    for (int k0 = 0; k0 < n1;) {
        const int m = n1 - k0, NB = wide_panel_nb<T>(m), nb = std::min(NB, m), c1 = k0 + nb;
        lu_panel_kernel<T><<<1, kLU, sizeof(T) * (size_t)m * (NB + 1), stream>>>(L, d.perm, n1, k0, NB, d.pre);
        RP_LAUNCH_CHECK();
        if (c1 < n1) {
            const int w = n1 - c1, grid = (int)ceil_div(w, 256);
            switch (NB) {
                case 32: lu_trsm_kernel<T, 32><<<grid, 256, 0, stream>>>(L, n1, k0, d.pre); break;
                case 16: lu_trsm_kernel<T, 16><<<grid, 256, 0, stream>>>(L, n1, k0, d.pre); break;
                case 8: lu_trsm_kernel<T, 8><<<grid, 256, 0, stream>>>(L, n1, k0, d.pre); break;
                default: lu_trsm_kernel<T, 4><<<grid, 256, 0, stream>>>(L, n1, k0, d.pre); break;
            }
            RP_LAUNCH_CHECK();
            // row-major A22 (w x w) -= L21 (w x nb) U12 (nb x w), as column-major C^T -= U12^T L21^T
            RP_CUBLAS(gemm_nn(h, w, w, nb, &minus_one, L + (size_t)k0 * n1 + c1, n1, L + (size_t)c1 * n1 + k0, n1,
                              &one, L + (size_t)c1 * n1 + c1, n1));
        }
        k0 = c1;
    }
}

}  // namespace

// Host side: reduced-index maps (repeat.py:2445-2470 semantics).
struct FoldPlan {
    int n = 0;
    std::vector<int> map, mem_ptr, mem_idx, ind;
    bool disjoint = true;
};

static FoldPlan make_plan(int N, int n_groups, const int *gptr, const int *gidx) {
    FoldPlan p;
    std::vector<char> linked((size_t)N, 0);
    std::vector<int> seen((size_t)N, 0);
    for (int g = 0; g < n_groups; ++g) {
        for (int t = gptr[g]; t < gptr[g + 1]; ++t) {
            int a = gidx[t];
            RP_REQUIRE(a >= 0 && a < N, "rp_solve: group atom index out of range");
            if (seen[a]++) p.disjoint = false;
            if (t > gptr[g]) linked[a] = 1;
        }
    }
    p.map.assign((size_t)N, -1);
    for (int i = 0; i < N; ++i)
        if (!linked[i]) {
            p.map[i] = (int)p.ind.size();
            p.ind.push_back(i);
        }
    p.n = (int)p.ind.size();
    std::vector<std::vector<int>> mem((size_t)p.n);
    for (int r = 0; r < p.n; ++r) mem[r].push_back(p.ind[r]);
    for (int g = 0; g < n_groups; ++g) {
        int base = gidx[gptr[g]];
        for (int t = gptr[g] + 1; t < gptr[g + 1]; ++t) {
            int l = gidx[t];
            if (p.map[base] >= 0) {
                mem[p.map[base]].push_back(l);
                p.map[l] = p.map[base];
            }
        }
    }
    // linked atoms whose base is itself linked (chains) take the final base's value
    for (int pass = 0; pass < n_groups + 1; ++pass) {
        bool changed = false;
        for (int g = 0; g < n_groups; ++g) {
            int base = gidx[gptr[g]];
            for (int t = gptr[g] + 1; t < gptr[g + 1]; ++t)
                if (p.map[gidx[t]] != p.map[base] && p.map[base] >= 0) {
                    p.map[gidx[t]] = p.map[base];
                    changed = true;
                }
        }
        if (!changed) break;
    }
    for (int i = 0; i < N; ++i)
        RP_REQUIRE(p.map[i] >= 0 && p.map[i] < p.n, "rp_solve: symmetry groups link atoms in a cycle");
    p.mem_ptr.push_back(0);
    for (auto &m : mem) {
        p.mem_idx.insert(p.mem_idx.end(), m.begin(), m.end());
        p.mem_ptr.push_back((int)p.mem_idx.size());
    }
    return p;
}

// Exact sequential folding on the host for overlapping groups.
static void host_fold(int N, const std::vector<double> &A, const std::vector<double> &b, int n_groups, const int *gptr,
                      const int *gidx, const FoldPlan &p, std::vector<double> &Ar, std::vector<double> &br,
                      std::vector<double> &w) {
    std::vector<double> AA(A), bb(b), ww((size_t)N, 1.0);
    for (int g = 0; g < n_groups; ++g) {
        int base = gidx[gptr[g]];
        for (int t = gptr[g] + 1; t < gptr[g + 1]; ++t) {
            int l = gidx[t];
            bb[base] += bb[l];
            ww[base] += 1.0;
            for (int r = 0; r < N; ++r) AA[(size_t)r * N + base] += AA[(size_t)r * N + l];
        }
    }
    for (int g = 0; g < n_groups; ++g) {
        int base = gidx[gptr[g]];
        for (int t = gptr[g] + 1; t < gptr[g + 1]; ++t) {
            int l = gidx[t];
            for (int c = 0; c < N; ++c) AA[(size_t)base * N + c] += AA[(size_t)l * N + c];
        }
    }
    Ar.assign((size_t)p.n * p.n, 0.0);
    br.assign((size_t)p.n, 0.0);
    w.assign((size_t)p.n, 0.0);
    for (int r = 0; r < p.n; ++r) {
        for (int c = 0; c < p.n; ++c) Ar[(size_t)r * p.n + c] = AA[(size_t)p.ind[r] * N + p.ind[c]];
        br[r] = bb[p.ind[r]];
        w[r] = ww[p.ind[r]];
    }
}

const double *solve_batch_async(rp_ctx *ctx, const std::vector<SolveJob> &jobs, cudaStream_t stream,
                                const std::string &tag, SolvePending *pend, bool fp64_first) {
    const int nj = (int)jobs.size();
    if (nj == 0) return nullptr;
    std::vector<FoldPlan> plans((size_t)nj);
    size_t n_map = 0, n_mptr = 0, n_midx = 0, n_red = 0, n_sq = 0;
    for (int j = 0; j < nj; ++j) {
        const SolveJob &J = jobs[j];
        RP_REQUIRE(J.A && J.b && J.q && J.N > 0, "rp_solve: null argument or N <= 0");
        RP_REQUIRE(J.n_groups == 0 || (J.group_ptr && J.group_idx), "rp_solve: groups given without arrays");
        plans[j] = make_plan(J.N, J.n_groups, J.group_ptr, J.group_idx);
        const size_t n1 = (size_t)plans[j].n + 1;
        n_map += J.N;
        n_mptr += plans[j].mem_ptr.size();
        n_midx += std::max<size_t>(plans[j].mem_idx.size(), 1);
        n_red += n1;
        n_sq += n1 * n1;
    }
    int *d_map = ctx->buf_t<int>("s_map" + tag, n_map);
    int *d_mptr = ctx->buf_t<int>("s_mptr" + tag, n_mptr);
    int *d_midx = ctx->buf_t<int>("s_midx" + tag, n_midx);
    double *d_rs = ctx->buf_t<double>("s_rs" + tag, n_red);
    double *d_rt = ctx->buf_t<double>("s_rt" + tag, n_red);
    double *As = ctx->buf_t<double>("s_As" + tag, n_sq);
    double *A0 = ctx->buf_t<double>("s_A0" + tag, n_sq);
    double *bs = ctx->buf_t<double>("s_bs" + tag, n_red);
    double *x = ctx->buf_t<double>("s_x" + tag, n_red);
    double *r = ctx->buf_t<double>("s_r" + tag, n_red);
    int *perm = ctx->buf_t<int>("s_perm" + tag, n_red);
    double *d_info = ctx->buf_t<double>("s_info" + tag, (size_t)nj * kSolveInfo);
    double *d_pre = ctx->buf_t<double>("s_pre" + tag, (size_t)nj * 3);
    SolveDesc *d_desc = ctx->buf_t<SolveDesc>("s_desc" + tag, (size_t)nj);
    // host staging of the small per-system tables, one upload each
    std::vector<int> h_map(n_map), h_mptr(n_mptr), h_midx(n_midx, 0);
    std::vector<double> h_rs(n_red, 0.0), h_rt(n_red, 0.0);
    std::vector<SolveDesc> descs((size_t)nj);
    size_t o_map = 0, o_mptr = 0, o_midx = 0, o_red = 0, o_sq = 0;
    for (int j = 0; j < nj; ++j) {
        const SolveJob &J = jobs[j];
        const FoldPlan &p = plans[j];
        const int n1 = p.n + 1;
        std::copy(p.map.begin(), p.map.end(), h_map.begin() + o_map);
        std::copy(p.mem_ptr.begin(), p.mem_ptr.end(), h_mptr.begin() + o_mptr);
        std::copy(p.mem_idx.begin(), p.mem_idx.end(), h_midx.begin() + o_midx);
        if (J.resp_s)
            for (int rr = 0; rr < p.n; ++rr) {
                h_rs[o_red + rr] = J.resp_s[p.ind[rr]];
                h_rt[o_red + rr] = J.resp_t ? J.resp_t[p.ind[rr]] : 0.0;
            }
        SolveDesc &d = descs[j];
        d.A = J.A; d.b = J.b; d.N = J.N; d.n = p.n;
        d.mem_ptr = d_mptr + o_mptr; d.mem_idx = d_midx + o_midx;
        d.resp_s = J.resp_s ? d_rs + o_red : nullptr; d.resp_t = J.resp_s ? d_rt + o_red : nullptr;
        d.map = d_map + o_map; d.qtot = J.qtot;
        d.As = As + o_sq; d.A0 = A0 + o_sq; d.bs = bs + o_red; d.x = x + o_red; d.r = r + o_red;
        d.perm = perm + o_red; d.q = J.q; d.info = d_info + kSolveInfo * (size_t)j;
        o_map += J.N;
        o_mptr += p.mem_ptr.size();
        o_midx += std::max<size_t>(p.mem_idx.size(), 1);
        o_red += (size_t)n1;
        o_sq += (size_t)n1 * n1;
    }
    // wide systems are factored across the GPU before the refinement kernel: their flags
    std::vector<int> disjoint;
    for (int j = 0; j < nj; ++j) {
        const int n1 = plans[j].n + 1;
        if (n1 >= kLUHost64Min && n1 <= kLUWideMax) {
            descs[j].pre = d_pre + 3 * (size_t)j;
            descs[j].host64 = n1 < kLUWideMin;
            if (fp64_first) descs[j].wide64 = 1;
            else if (n1 >= kLUWideMin) descs[j].host32 = 1;
        }
        if (plans[j].disjoint) disjoint.push_back(j);
    }
    // the small tables go up from one pinned staging block per tag (asynchronous copies that
    // never wait for the stream; a later solve with another tag cannot overwrite them)
    const size_t st_bytes[7] = {sizeof(int) * n_map, sizeof(int) * n_mptr, sizeof(int) * n_midx,
                                sizeof(double) * n_red, sizeof(double) * n_red, sizeof(SolveDesc) * nj,
                                sizeof(int) * std::max<size_t>(disjoint.size(), 1)};
    size_t st_off[7], st_end = 0;
    for (int t = 0; t < 7; ++t) {
        st_off[t] = st_end;
        st_end += (st_bytes[t] + 15) / 16 * 16;
    }
    char *stage = static_cast<char *>(ctx->host_buf("s_stage" + tag, st_end));
    std::memcpy(stage + st_off[0], h_map.data(), st_bytes[0]);
    std::memcpy(stage + st_off[1], h_mptr.data(), st_bytes[1]);
    std::memcpy(stage + st_off[2], h_midx.data(), st_bytes[2]);
    std::memcpy(stage + st_off[3], h_rs.data(), st_bytes[3]);
    std::memcpy(stage + st_off[4], h_rt.data(), st_bytes[4]);
    RP_CUDA(cudaMemcpyAsync(d_map, stage + st_off[0], st_bytes[0], cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_mptr, stage + st_off[1], st_bytes[1], cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_midx, stage + st_off[2], st_bytes[2], cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_rs, stage + st_off[3], st_bytes[3], cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_rt, stage + st_off[4], st_bytes[4], cudaMemcpyHostToDevice, stream));
    std::memcpy(stage + st_off[5], descs.data(), st_bytes[5]);
    RP_CUDA(cudaMemcpyAsync(d_desc, stage + st_off[5], st_bytes[5], cudaMemcpyHostToDevice, stream));
    if (!disjoint.empty()) {  // every system with disjoint groups: one launch
        int *d_sys = ctx->buf_t<int>("s_sys" + tag, disjoint.size());
        std::memcpy(stage + st_off[6], disjoint.data(), st_bytes[6]);
        RP_CUDA(cudaMemcpyAsync(d_sys, stage + st_off[6], st_bytes[6], cudaMemcpyHostToDevice, stream));
        long long most = 1;
        for (int j : disjoint) most = std::max<long long>(most, (long long)(plans[j].n + 1) * (plans[j].n + 1));
        const dim3 grid((unsigned)std::min<long long>(ceil_div(most, 256), 1024), (unsigned)disjoint.size());
        build_bordered_kernel<<<grid, 256, 0, stream>>>(d_desc, d_sys);
        RP_LAUNCH_CHECK();
    }
    for (int j = 0; j < nj; ++j) {
        const SolveJob &J = jobs[j];
        const FoldPlan &p = plans[j];
        const int n1 = p.n + 1;
        if (!p.disjoint) {
            // overlapping groups: the reference's sequential folding on the host
            std::vector<double> hA((size_t)J.N * J.N), hb((size_t)J.N), Ar, br, w;
            RP_CUDA(cudaMemcpyAsync(hA.data(), J.A, sizeof(double) * hA.size(), cudaMemcpyDeviceToHost, stream));
            RP_CUDA(cudaMemcpyAsync(hb.data(), J.b, sizeof(double) * J.N, cudaMemcpyDeviceToHost, stream));
            RP_CUDA(cudaStreamSynchronize(stream));
            host_fold(J.N, hA, hb, J.n_groups, J.group_ptr, J.group_idx, p, Ar, br, w);
            std::vector<double> hs((size_t)n1 * n1, 0.0), hbs((size_t)n1, 0.0);
            for (int rr = 0; rr < p.n; ++rr) {
                for (int c = 0; c < p.n; ++c) hs[(size_t)rr * n1 + c] = Ar[(size_t)rr * p.n + c];
                double rsv = J.resp_s ? J.resp_s[p.ind[rr]] : 0.0;
                double rtv = (J.resp_s && J.resp_t) ? J.resp_t[p.ind[rr]] : 0.0;
                hs[(size_t)rr * n1 + rr] += rsv;
                hs[(size_t)rr * n1 + p.n] = w[rr];
                hs[(size_t)p.n * n1 + rr] = w[rr];
                hbs[rr] = br[rr] + rsv * rtv;
            }
            hbs[p.n] = J.qtot;
            RP_CUDA(cudaMemcpyAsync(descs[j].As, hs.data(), sizeof(double) * hs.size(), cudaMemcpyHostToDevice, stream));
            RP_CUDA(cudaMemcpyAsync(descs[j].A0, hs.data(), sizeof(double) * hs.size(), cudaMemcpyHostToDevice, stream));
            RP_CUDA(cudaMemcpyAsync(descs[j].bs, hbs.data(), sizeof(double) * hbs.size(), cudaMemcpyHostToDevice, stream));
            RP_CUDA(cudaStreamSynchronize(stream));
        }
    }
    // large systems: factored across the GPU first (lu_solve_refine_kernel then refines them)
    bool any_wide = false, any_pre = false;
    for (int j = 0; j < nj; ++j) any_pre |= descs[j].pre != nullptr;
    if (pend) *pend = SolvePending{};
    if (any_pre) RP_CUDA(cudaMemsetAsync(d_pre, 0, sizeof(double) * 3 * nj, stream));
    for (int j = 0; j < nj; ++j) {
        if (!descs[j].pre || descs[j].wide64) continue;  // wide64: factored and refined after the launch
        if (descs[j].host64) {
            any_wide = true;  // its flag is read after the launch, as a wide system's
        } else {
            StageTimer tt(ctx, "solve_lu_wide", stream);
            lu_wide_factor<float>(ctx, descs[j], plans[j].n + 1, stream);
            any_wide = true;
        }
    }
    {
        StageTimer tt(ctx, "solve_lu", stream);
        int n1max = 1;
        for (const FoldPlan &p : plans) n1max = std::max(n1max, p.n + 1);
        lu_smem_optin();
        lu_solve_refine_kernel<<<nj, kLU, solve_smem_bytes(n1max), stream>>>(d_desc);
        RP_LAUNCH_CHECK();
    }
    for (int j = 0; j < nj; ++j)  // systems known to need FP64 (an escalated fit): getrf, host-driven refinement
        if (descs[j].wide64) factor_refine_wide64(ctx, descs[j], plans[j].n + 1, stream);
    std::vector<int> refine32;
    for (int j = 0; j < nj; ++j)
        if (descs[j].host32) refine32.push_back(j);
    double *h_info = static_cast<double *>(ctx->host_buf("s_info" + tag, sizeof(double) * kSolveInfo * nj));
    if (any_wide) {
        // wide systems whose FP32 refinement did not converge (flag 2) are factored again in FP64:
        // their flags go to pinned memory, and solve_wide_fp64 (now, or, with `pend`, when the
        // caller's completion reaches it) reads them and redoes those systems
        double *h_pre = static_cast<double *>(ctx->host_buf("s_preh" + tag, sizeof(double) * 3 * nj));
        RP_CUDA(cudaMemcpyAsync(h_pre, d_pre, sizeof(double) * 3 * nj, cudaMemcpyDeviceToHost, stream));
        SolvePending local;
        SolvePending &pd = pend ? *pend : local;
        pd.any_wide = true;
        pd.tag = tag;
        pd.h_pre = h_pre;
        pd.h_info = h_info;
        pd.d_info = d_info;
        pd.descs = descs;
        pd.n1.resize((size_t)nj);
        for (int j = 0; j < nj; ++j) pd.n1[j] = plans[j].n + 1;
        pd.refine32 = refine32;
        if (!pend) {
            RP_CUDA(cudaStreamSynchronize(stream));
            solve_wide_fp64(ctx, pd, stream);
        }
    }
    RP_CUDA(cudaMemcpyAsync(h_info, d_info, sizeof(double) * kSolveInfo * nj, cudaMemcpyDeviceToHost, stream));
    return h_info;
}

void solve_wide_fp64(rp_ctx *ctx, SolvePending &pd, cudaStream_t stream) {
    if (!pd.any_wide) return;
    pd.any_wide = false;
    const int nj = (int)pd.descs.size();
    bool any = false;
    for (int j : pd.refine32) {  // wide FP32 factors: refined here, FP64 factors when that stalls
        if (!refine_wide32(ctx, pd.descs[j], pd.n1[j], stream)) factor_refine_wide64(ctx, pd.descs[j], pd.n1[j], stream);
        any = true;
    }
    pd.refine32.clear();
    for (int j = 0; j < nj; ++j) {
        if (!pd.descs[j].pre || pd.descs[j].host32 || pd.h_pre[3 * j] != 2.0) continue;
        factor_refine_wide64(ctx, pd.descs[j], pd.n1[j], stream);
        any = true;
    }
    if (!any) return;
    RP_CUDA(cudaMemcpyAsync(pd.h_info, pd.d_info, sizeof(double) * kSolveInfo * nj, cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaStreamSynchronize(stream));
}

void solve_batch(rp_ctx *ctx, const std::vector<SolveJob> &jobs, std::vector<double> &info, cudaStream_t stream,
                 bool fp64_first) {
    const int nj = (int)jobs.size();
    info.assign((size_t)nj * kSolveInfo, 0.0);
    if (nj == 0) return;
    const double *h = solve_batch_async(ctx, jobs, stream, "", nullptr, fp64_first);
    RP_CUDA(cudaStreamSynchronize(stream));
    std::copy(h, h + kSolveInfo * (size_t)nj, info.begin());
}

void solve_run(rp_ctx *ctx, const double *A_dev, const double *b_dev, int N, int n_groups, const int *group_ptr,
               const int *group_idx, const double *resp_s, const double *resp_t, double qtot, double *q_dev,
               double *info, cudaStream_t stream) {
    std::vector<SolveJob> jobs(1);
    jobs[0] = SolveJob{A_dev, b_dev, N, n_groups, group_ptr, group_idx, resp_s, resp_t, qtot, q_dev};
    std::vector<double> hinfo;
    solve_batch(ctx, jobs, hinfo, stream);
    if (info) {
        info[0] = hinfo[0];
        info[1] = hinfo[1];
        info[2] = hinfo[2];
        info[3] = hinfo[4];
    }
    if (hinfo[3] != 0.0) fail(RP_E_SINGULAR, "rp_solve: bordered system is singular (zero pivot)");
}

}  // namespace rp

// ---------------------------------------------------------------------------
// No-allocation variant of the constrained bordered solve.
//
// For callers that must not allocate device memory while they run: a serving
// loop that cannot afford the device-wide synchronisation cudaMalloc/cudaFree
// may cause, or an embedder whose device memory is owned entirely by its own
// allocator.  Its scratch is the file-scope array below (kNoAllocScratchBytes,
// enough for N <= kNoAllocMaxN atoms), which every GPU that loads this library
// keeps until the process exits.  Host code only sees a host-side stand-in for
// that symbol; the device address comes from cudaGetSymbolAddress, looked up once
// per device with that device current, on the first call made on it (make that
// first call before any stream capture).  With lazy module loading that first call
// may also be what loads the library's device code, and the array with it.  The
// address is kept for the life of the process: a cudaDeviceReset voids it, so do
// not call this entry point after resetting the device.  A call is synchronous: it
// returns once the solve on `stream` has finished.  All calls share the array and it
// keeps the last call's contents (every region is fully rewritten before it is read),
// so calls that overlap on the GPU race: serialise them on one stream.
namespace rp {
namespace {

constexpr int kNoAllocMaxN = 512;
constexpr size_t kNoAllocScratchBytes = 4718592;  // 4.5 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

unsigned char *noalloc_scratch_device() {
    static std::mutex mu;
    static unsigned char *addr[256] = {};
    int dev = 0;
    RP_CUDA(cudaGetDevice(&dev));
    RP_REQUIRE(dev >= 0 && dev < 256, "rp_solve_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) fail(RP_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        addr[dev] = static_cast<unsigned char *>(p);
    }
    return addr[dev];
}

// Bump allocator over the static array (256-byte aligned slices).
struct Carve {
    unsigned char *base;
    size_t off = 0;
    template <class T>
    T *take(size_t count) {
        size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        if (off + bytes > kNoAllocScratchBytes) fail(RP_E_NOMEM, "rp_solve_noalloc: static scratch exhausted");
        T *p = reinterpret_cast<T *>(base + off);
        off += bytes;
        return p;
    }
};

}  // namespace
}  // namespace rp

extern "C" int rp_solve_noalloc(const double *A_dev, const double *b_dev, int N, int n_groups, const int *group_ptr,
                                const int *group_idx, const double *resp_s, const double *resp_t, double qtot,
                                double *q_dev, double *info, rp_stream_t stream_) {
    using namespace rp;
    cudaStream_t stream = (cudaStream_t)stream_;
    try {
        RP_REQUIRE(A_dev && b_dev && q_dev, "rp_solve_noalloc: null argument");
        if (N <= 0 || N > kNoAllocMaxN) return RP_E_ARG;  // N must be in 1..512
        RP_REQUIRE(n_groups == 0 || (group_ptr && group_idx), "rp_solve_noalloc: groups given without arrays");
        FoldPlan p = make_plan(N, n_groups, group_ptr, group_idx);
        const int n1 = p.n + 1;
        Carve cv{noalloc_scratch_device()};
        int *d_map = cv.take<int>((size_t)N);
        int *d_mptr = cv.take<int>(p.mem_ptr.size());
        int *d_midx = cv.take<int>(std::max<size_t>(p.mem_idx.size(), 1));
        double *d_rs = cv.take<double>((size_t)p.n);
        double *d_rt = cv.take<double>((size_t)p.n);
        double *As = cv.take<double>((size_t)n1 * n1);
        double *A0 = cv.take<double>((size_t)n1 * n1);
        double *bs = cv.take<double>((size_t)n1);
        double *x = cv.take<double>((size_t)n1);
        double *r = cv.take<double>((size_t)n1);
        int *perm = cv.take<int>((size_t)n1);
        double *d_info = cv.take<double>(kSolveInfo);
        SolveDesc *d_desc = cv.take<SolveDesc>(1);
        int *d_sys = cv.take<int>(1);
        std::vector<double> rs((size_t)p.n, 0.0), rt((size_t)p.n, 0.0);
        if (resp_s)
            for (int k = 0; k < p.n; ++k) {
                rs[k] = resp_s[p.ind[k]];
                rt[k] = resp_t ? resp_t[p.ind[k]] : 0.0;
            }
        RP_CUDA(cudaMemcpyAsync(d_map, p.map.data(), sizeof(int) * N, cudaMemcpyHostToDevice, stream));
        RP_CUDA(cudaMemcpyAsync(d_mptr, p.mem_ptr.data(), sizeof(int) * p.mem_ptr.size(), cudaMemcpyHostToDevice, stream));
        if (!p.mem_idx.empty())
            RP_CUDA(cudaMemcpyAsync(d_midx, p.mem_idx.data(), sizeof(int) * p.mem_idx.size(), cudaMemcpyHostToDevice,
                                    stream));
        if (p.n > 0) {
            RP_CUDA(cudaMemcpyAsync(d_rs, rs.data(), sizeof(double) * p.n, cudaMemcpyHostToDevice, stream));
            RP_CUDA(cudaMemcpyAsync(d_rt, rt.data(), sizeof(double) * p.n, cudaMemcpyHostToDevice, stream));
        }
        SolveDesc d{};
        d.A = A_dev; d.b = b_dev; d.N = N; d.n = p.n; d.mem_ptr = d_mptr; d.mem_idx = d_midx;
        d.resp_s = resp_s ? d_rs : nullptr; d.resp_t = resp_s ? d_rt : nullptr; d.map = d_map; d.qtot = qtot;
        d.As = As; d.A0 = A0; d.bs = bs; d.x = x; d.r = r; d.perm = perm; d.q = q_dev; d.info = d_info;
        RP_CUDA(cudaMemcpyAsync(d_desc, &d, sizeof(SolveDesc), cudaMemcpyHostToDevice, stream));
        if (p.disjoint) {
            RP_CUDA(cudaMemsetAsync(d_sys, 0, sizeof(int), stream));  // the one system
            const dim3 grid((unsigned)std::min<long long>(ceil_div((long long)n1 * n1, 256), 1024), 1u);
            build_bordered_kernel<<<grid, 256, 0, stream>>>(d_desc, d_sys);
            RP_LAUNCH_CHECK();
        } else {
            std::vector<double> hA((size_t)N * N), hb((size_t)N), Ar, br, w;
            RP_CUDA(cudaMemcpyAsync(hA.data(), A_dev, sizeof(double) * hA.size(), cudaMemcpyDeviceToHost, stream));
            RP_CUDA(cudaMemcpyAsync(hb.data(), b_dev, sizeof(double) * N, cudaMemcpyDeviceToHost, stream));
            RP_CUDA(cudaStreamSynchronize(stream));
            host_fold(N, hA, hb, n_groups, group_ptr, group_idx, p, Ar, br, w);
            std::vector<double> hs((size_t)n1 * n1, 0.0), hbs((size_t)n1, 0.0);
            for (int k = 0; k < p.n; ++k) {
                for (int c = 0; c < p.n; ++c) hs[(size_t)k * n1 + c] = Ar[(size_t)k * p.n + c];
                hs[(size_t)k * n1 + k] += rs[k];
                hs[(size_t)k * n1 + p.n] = w[k];
                hs[(size_t)p.n * n1 + k] = w[k];
                hbs[k] = br[k] + rs[k] * rt[k];
            }
            hbs[p.n] = qtot;
            RP_CUDA(cudaMemcpyAsync(As, hs.data(), sizeof(double) * hs.size(), cudaMemcpyHostToDevice, stream));
            RP_CUDA(cudaMemcpyAsync(A0, hs.data(), sizeof(double) * hs.size(), cudaMemcpyHostToDevice, stream));
            RP_CUDA(cudaMemcpyAsync(bs, hbs.data(), sizeof(double) * hbs.size(), cudaMemcpyHostToDevice, stream));
        }
        lu_smem_optin();
        lu_solve_refine_kernel<<<1, kLU, solve_smem_bytes(n1), stream>>>(d_desc);
        RP_LAUNCH_CHECK();
        double hinfo[kSolveInfo];
        RP_CUDA(cudaMemcpyAsync(hinfo, d_info, sizeof(hinfo), cudaMemcpyDeviceToHost, stream));
        RP_CUDA(cudaStreamSynchronize(stream));
        if (info) {
            info[0] = hinfo[0];
            info[1] = hinfo[1];
            info[2] = hinfo[2];
            info[3] = hinfo[4];
        }
        return hinfo[3] != 0.0 ? RP_E_SINGULAR : RP_OK;
    } catch (const rp::Error &e) {
        return e.code;
    } catch (const std::exception &) {
        return RP_E_ARG;
    }
}
