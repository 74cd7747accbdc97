// vdW grid filter: keep mask, ordered compaction and ESP centring.
//
// Replaces ChargeCalculator._filter_grid (repeat.py:1922-2113) and its GPU
// kernel filter_bins (repeat.py:445-518).  The keep rule is the reference's
// FP64 squared-distance rule:
//     keep(g) = all_e |g-e|^2 > rmin_e^2  and  any_e |g-e|^2 <= rmax_e^2
// over the 27 lattice images e of every atom (clipped like repeat.py:1945-1969),
// with g = (i*a0 + j*a1) + k*a2 and |d|^2 = (dx*dx + dy*dy) + dz*dz evaluated in
// IEEE FP64 without contraction.
//
// GB300 design: one CTA per brick of 8 x 4 x 4 grid points.  The CTA culls the
// images of the cell-list bins around its points (bin edge >= max rmin, so no
// other image can reject a point) to those within rmin of the brick's bounding
// box, keeps them in shared memory, and classifies every point in FP32 against
// that short list.  A pair whose FP32 squared distance lies within a proven error
// band of rmin^2 is re-evaluated in FP64 exactly as above, so the mask is
// bit-identical to the FP64 rule while almost all work runs on the FP32 pipe.
// "near" is proved for the whole grid on the host when one image's rmax covers
// every grid corner (always true at the default vdw_max = 1000); otherwise it
// is tested the same way (FP32 with an FP64 recheck band) against every image.
//
// Traffic per grid point: 1 B mask write (plus the compaction pass: 1 B mask read
// + 8 B V read per point, 4 B index + 8 B V write per kept point).  The mask pass
// is bound by its FP32 distance tests, ~5 candidate images per point after the
// brick's cull.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace rp {
namespace {

constexpr int kFilterThreads = 256;


// Not inlined on purpose: the call sits in a branch that almost never runs, and as an
// inlined body the compiler may evaluate it speculatively for every candidate, which puts
// the FP64 pipe (a small fraction of the FP32 rate on this part) on the critical path.
__device__ __noinline__ double exact_d2(const double *axd, int i, int j, int k, double ex, double ey,
                                        double ez) {
    // ((i*a0 + j*a1) + k*a2) and ((dx*dx + dy*dy) + dz*dz), every op rounded (no FMA)
    double gx = __dadd_rn(__dadd_rn(__dmul_rn((double)i, axd[0]), __dmul_rn((double)j, axd[3])),
                          __dmul_rn((double)k, axd[6]));
    double gy = __dadd_rn(__dadd_rn(__dmul_rn((double)i, axd[1]), __dmul_rn((double)j, axd[4])),
                          __dmul_rn((double)k, axd[7]));
    double gz = __dadd_rn(__dadd_rn(__dmul_rn((double)i, axd[2]), __dmul_rn((double)j, axd[5])),
                          __dmul_rn((double)k, axd[8]));
    double dx = __dsub_rn(gx, ex), dy = __dsub_rn(gy, ey), dz = __dsub_rn(gz, ez);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Reject test of one grid point against the atoms of its 27 neighbouring bins (bin edge >=
// max rmin): FP32 distances, FP64 recheck inside the band.  Returns false when some image
// rejects the point.
__device__ __forceinline__ bool valid_by_bins(const FilterParams &p, int i, int j, int k, float gx, float gy,
                                              float gz, const float4 *__restrict__ eff,
                                              const D4 *__restrict__ eff64, const int *__restrict__ boff,
                                              const int *__restrict__ bidx, unsigned &nre) {
    int bc[3];
    const float g3[3] = {gx, gy, gz};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float t = (g3[d] - p.bmin[d]) * p.inv_bsize;
        t = fminf(fmaxf(t, -1.0f), (float)p.bn[d]);
        bc[d] = min(max((int)floorf(t), 0), p.bn[d] - 1);
    }
    for (int dz = -1; dz <= 1; ++dz) {
        const int z2 = bc[2] + dz;
        if (z2 < 0 || z2 >= p.bn[2]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y2 = bc[1] + dy;
            if (y2 < 0 || y2 >= p.bn[1]) continue;
            const int row = p.bn[0] * (y2 + p.bn[1] * z2);
            const int x0 = max(bc[0] - 1, 0), x1 = min(bc[0] + 1, p.bn[0] - 1);
            const int t0 = boff[row + x0], t1 = boff[row + x1 + 1];
            for (int t = t0; t < t1; ++t) {
                const int a = bidx[t];
                const float4 e = eff[a];
                const float ddx = gx - e.x, ddy = gy - e.y, ddz = gz - e.z;
                const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                if (d2 <= e.w - p.err_min) return false;
                if (d2 <= e.w + p.err_min) {
                    const D4 e8 = eff64[a];
                    ++nre;
                    if (exact_d2(p.axd, i, j, k, e8.x, e8.y, e8.z) <= e8.w) return false;
                }
            }
        }
    }
    return true;
}

// The near test (some image with |g-e|^2 <= rmax^2), needed only when the host could not
// prove it for the whole grid (vdw_max below its default): every image, FP32 with the
// FP64 recheck band.
__device__ __forceinline__ bool near_any(const FilterParams &p, int i, int j, int k, float gx, float gy, float gz,
                                         const float4 *__restrict__ eff, const D4 *__restrict__ eff64,
                                         const double *__restrict__ rmax2, const float *__restrict__ rmax2f,
                                         unsigned &nre) {
    for (int a = 0; a < p.A; ++a) {
        const float4 e = eff[a];
        const float ddx = gx - e.x, ddy = gy - e.y, ddz = gz - e.z;
        const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
        const float r2 = rmax2f[a];
        if (d2 <= r2 - p.err_max) return true;
        if (d2 <= r2 + p.err_max) {
            const D4 e8 = eff64[a];
            ++nre;
            if (exact_d2(p.axd, i, j, k, e8.x, e8.y, e8.z) <= rmax2[a]) return true;
        }
    }
    return false;
}

// Bricks of 8 x 4 x 4 grid points (one CTA of 128 threads each, x fastest), bricks in
// x-then-y-then-z order, points inside a brick in the same order: the unit of the culled
// mask kernel and of the brick-ordered compaction.
constexpr int kBrickX = 8, kBrickY = 4, kBrickZ = 4;
constexpr int kBrickPts = kBrickX * kBrickY * kBrickZ;  // 128
constexpr int kCullCap = 512;  // candidate images a brick keeps in shared memory
constexpr int kCullRows = 64;  // (y, z) bin rows a brick's cull shares out over its threads

// One cube's filter in a grouped launch: its plan, grid values, scratch and outputs.  A launch
// carries up to kFilterJobs of them by value; job j owns blocks [blk[j], blk[j+1]) of the
// kernel's grid, so a pipeline group of cubes costs one launch per stage.
struct FilterJob {
    FilterParams p;
    const float4 *e32;
    const D4 *e64;
    const double *rmax2;
    const float *rmax2f;
    const int *boff, *bidx;
    const double *V;
    uint8_t *mask;
    int *counts;          // kept points per compaction block (bricks, or flat blocks of 256)
    long long *offsets;   // their exclusive scan
    double *vsum;         // per compaction block: sum of the kept ESP values
    int ncount;           // compaction blocks
    int32_t *kept;
    double *Vc;
    long long *M;         // kept count (device)
    double *mean;
    double2 *vpart;       // kCenterParts partial (sum, max |.|) of the centred ESP
    double *vstats;       // (sum, max |.|), or nullptr
    int nbx, nby;
};
constexpr int kFilterJobs = 40;
struct FilterLaunch {
    int n;
    int blk[kFilterJobs + 1];
    FilterJob job[kFilterJobs];
};
constexpr int kCenterParts = 32;  // CTAs per cube of the centring pass

__device__ __forceinline__ int filter_job_of(const FilterLaunch &L, int b) {
    int lo = 0, hi = L.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (L.blk[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ long long brick_point(int b, int t, int nx, int ny, int nz, int nbx, int nby) {
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    const int i = bx * kBrickX + (t % kBrickX), j = by * kBrickY + ((t / kBrickX) % kBrickY),
              l = bz * kBrickZ + t / (kBrickX * kBrickY);
    if (i >= nx || j >= ny || l >= nz) return -1;
    return (long long)i + (long long)nx * (j + (long long)ny * l);
}

// The mask, one brick per CTA.  The CTA first culls the images of the bins around its points'
// bounding box to those that can reject any of them (FP32 distance from the image to the box
// within rmin^2 + the error band, with a relative margin above the FP32 rounding of both
// distances), keeping them in shared memory; each point then tests only those (about a
// quarter of its 27 bins' images).  A culled image is farther than the band from every point
// of the brick, so it could neither reject a point nor trigger its FP64 recheck: the mask is
// the one of the per-point bin test (valid_by_bins), which a brick with more than kCullCap
// candidates falls back to.  Writes the mask and the brick's kept count.
__global__ void __launch_bounds__(kBrickPts) filter_brick_kernel(const __grid_constant__ FilterLaunch L,
                                                                  int write_counts) {
    __shared__ float4 cand[kCullCap];
    __shared__ int cidx[kCullCap];
    __shared__ int ncand, covered;
    __shared__ float box[6];
    __shared__ int row_t0[kCullRows], row_pre[kCullRows + 1];
    const int jb = filter_job_of(L, blockIdx.x);
    const FilterJob &J = L.job[jb];
    const FilterParams &p = J.p;
    const float4 *__restrict__ eff = J.e32;
    const D4 *__restrict__ eff64 = J.e64;
    const int *__restrict__ boff = J.boff;
    const int *__restrict__ bidx = J.bidx;
    const int nbx = J.nbx, nby = J.nby;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int b = blockIdx.x - L.blk[jb];
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    const int i = bx * kBrickX + (t % kBrickX), j = by * kBrickY + ((t / kBrickX) % kBrickY),
              k = bz * kBrickZ + t / (kBrickX * kBrickY);
    const bool inside = i < p.nx && j < p.ny && k < p.nz;
    const float gx = (i * p.ax[0] + j * p.ax[3]) + k * p.ax[6];
    const float gy = (i * p.ax[1] + j * p.ax[4]) + k * p.ax[7];
    const float gz = (i * p.ax[2] + j * p.ax[5]) + k * p.ax[8];
    // bounding box of the brick: its index box's eight corners (clipped to the grid) in FP32 by
    // the points' own expression, padded by 16 ulps of the largest coordinate, which covers the
    // rounding by which an inner point's FP32 coordinates can pass the corners' box
    if (warp == 0) {
        const int ci = (lane & 1) ? min(bx * kBrickX + kBrickX - 1, p.nx - 1) : bx * kBrickX;
        const int cj = (lane & 2) ? min(by * kBrickY + kBrickY - 1, p.ny - 1) : by * kBrickY;
        const int ck = (lane & 4) ? min(bz * kBrickZ + kBrickZ - 1, p.nz - 1) : bz * kBrickZ;
        float v[6];
        v[0] = v[3] = (ci * p.ax[0] + cj * p.ax[3]) + ck * p.ax[6];
        v[1] = v[4] = (ci * p.ax[1] + cj * p.ax[4]) + ck * p.ax[7];
        v[2] = v[5] = (ci * p.ax[2] + cj * p.ax[5]) + ck * p.ax[8];
#pragma unroll
        for (int o = 1; o < 8; o <<= 1)
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const float w = __shfl_xor_sync(0xffffffffu, v[q], o);
                v[q] = q < 3 ? fminf(v[q], w) : fmaxf(v[q], w);
            }
        if (lane == 0) {
            float big = 0.f;
#pragma unroll
            for (int q = 0; q < 6; ++q) big = fmaxf(big, fabsf(v[q]));
            const float pad = 16.f * big * 1.1920929e-7f + 1e-30f;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                box[q] = v[q] - pad;
                box[3 + q] = v[3 + q] + pad;
            }
            ncand = 0;
            covered = 0;
        }
    }
    __syncthreads();
    float lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = box[d];
        hi[d] = box[3 + d];
    }
    // bins that can hold a rejecting image: one bin beyond the box's own on every side
    int c0[3], c1[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float ta = fminf(fmaxf((lo[d] - p.bmin[d]) * p.inv_bsize, -1.0f), (float)p.bn[d]);
        const float tb = fminf(fmaxf((hi[d] - p.bmin[d]) * p.inv_bsize, -1.0f), (float)p.bn[d]);
        c0[d] = max(min(max((int)floorf(ta), 0), p.bn[d] - 1) - 1, 0);
        c1[d] = min(min(max((int)floorf(tb), 0), p.bn[d] - 1) + 1, p.bn[d] - 1);
    }
    // the images of those bins: a contiguous run of the cell list per (y, z) bin row; the rows'
    // runs are concatenated (prefix in shared memory) and shared out over the threads
    const int ry = c1[1] - c0[1] + 1, R = ry * (c1[2] - c0[2] + 1);
    // A brick whose farthest point lies strictly inside an exclusion sphere (by the FP32 rule's
    // margin, and a relative 1e-4 more for the order of the FP32 operations) loses all its
    // points to that image: every point's FP32 distance is at most the box's farthest, so the
    // per-point loop would reject each of them by the same test.
    auto cull = [&](int a) {
        const float4 e = eff[a];
        const float fx = fmaxf(fabsf(e.x - lo[0]), fabsf(e.x - hi[0]));
        const float fy = fmaxf(fabsf(e.y - lo[1]), fabsf(e.y - hi[1]));
        const float fz = fmaxf(fabsf(e.z - lo[2]), fabsf(e.z - hi[2]));
        if (fx * fx + fy * fy + fz * fz <= (e.w - p.err_min) * 0.9999f) covered = 1;
        const float dx = fmaxf(fmaxf(lo[0] - e.x, e.x - hi[0]), 0.f);
        const float dy = fmaxf(fmaxf(lo[1] - e.y, e.y - hi[1]), 0.f);
        const float dz = fmaxf(fmaxf(lo[2] - e.z, e.z - hi[2]), 0.f);
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 <= (e.w + p.err_min) * 1.0001f) {
            const int pos = atomicAdd(&ncand, 1);
            if (pos < kCullCap) {
                cand[pos] = e;
                cidx[pos] = a;
            }
        }
    };
    if (R <= kCullRows) {
        if (warp < kCullRows / 32) {  // row runs and their prefix (a warp scan per 32 rows)
            const int r = t;
            int cnt = 0;
            if (r < R) {
                const int y2 = c0[1] + r % ry, z2 = c0[2] + r / ry;
                const int row = p.bn[0] * (y2 + p.bn[1] * z2);
                const int t0 = boff[row + c0[0]];
                row_t0[r] = t0;
                cnt = boff[row + c1[0] + 1] - t0;
            }
            int inc = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int w = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += w;
            }
            row_pre[r + 1] = inc;  // inclusive within its warp; the warps are joined below
        }
        __syncthreads();
        if (t == 0) {
            row_pre[0] = 0;
            for (int w = 1; w < kCullRows / 32; ++w)
                for (int r = 32 * w + 1; r <= 32 * w + 32; ++r) row_pre[r] += row_pre[32 * w];
        }
        __syncthreads();
        const int total = row_pre[R];
        for (int u = t; u < total; u += kBrickPts) {
            int lo_r = 0, hi_r = R - 1;  // the row whose run holds u
            while (lo_r < hi_r) {
                const int mid = (lo_r + hi_r + 1) >> 1;
                if (row_pre[mid] <= u) lo_r = mid;
                else hi_r = mid - 1;
            }
            cull(bidx[row_t0[lo_r] + (u - row_pre[lo_r])]);
        }
    } else {
        for (int z2 = c0[2]; z2 <= c1[2]; ++z2)
            for (int y2 = c0[1]; y2 <= c1[1]; ++y2) {
                const int row = p.bn[0] * (y2 + p.bn[1] * z2);
                const int t0 = boff[row + c0[0]], t1 = boff[row + c1[0] + 1];
                for (int u = t0 + t; u < t1; u += kBrickPts) cull(bidx[u]);
            }
    }
    __syncthreads();
    const int nc = ncand;
    int keep = 0;
    unsigned nre = 0;
    if (inside && covered) {
        J.mask[(long long)i + (long long)p.nx * (j + (long long)p.ny * k)] = 0;
    } else if (inside) {
        bool valid = true;
        if (nc <= kCullCap) {
            for (int c = 0; c < nc; ++c) {
                const float4 e = cand[c];
                const float ddx = gx - e.x, ddy = gy - e.y, ddz = gz - e.z;
                const float d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                if (d2 <= e.w - p.err_min) { valid = false; break; }
                if (d2 <= e.w + p.err_min) {
                    const D4 e8 = eff64[cidx[c]];
                    ++nre;
                    if (exact_d2(p.axd, i, j, k, e8.x, e8.y, e8.z) <= e8.w) { valid = false; break; }
                }
            }
        } else {
            valid = valid_by_bins(p, i, j, k, gx, gy, gz, eff, eff64, boff, bidx, nre);
        }
        const bool near =
            p.near_all != 0 || (valid && near_any(p, i, j, k, gx, gy, gz, eff, eff64, J.rmax2, J.rmax2f, nre));
        keep = (valid && near) ? 1 : 0;
        J.mask[(long long)i + (long long)p.nx * (j + (long long)p.ny * k)] = (uint8_t)keep;
    }
    const int cnt = __syncthreads_count(keep);
    if (t == 0 && write_counts) J.counts[b] = cnt;
    (void)nre;
}

// Kept points per block of kFilterThreads consecutive flat indices (the flat-order compaction).
__global__ void __launch_bounds__(kFilterThreads) flat_count_kernel(const uint8_t *__restrict__ mask, long long n_total,
                                                                    int *__restrict__ counts) {
    const long long f = (long long)blockIdx.x * kFilterThreads + threadIdx.x;
    const int keep = f < n_total ? mask[f] : 0;
    const int cnt = __syncthreads_count(keep);
    if (threadIdx.x == 0) counts[blockIdx.x] = cnt;
}

// Exclusive scan of each job's per-block counts (one CTA per job; up to a few 10^5 blocks),
// and the job's kept count.
__global__ void __launch_bounds__(1024) scan_counts_kernel(const __grid_constant__ FilterLaunch L) {
    const FilterJob &J = L.job[blockIdx.x];
    const int nb = J.ncount;
    __shared__ long long part[1024];
    int t = threadIdx.x;
    int per = (nb + 1023) / 1024;
    int b0 = t * per, b1 = min(b0 + per, nb);
    long long s = 0;
    for (int b = b0; b < b1; ++b) s += J.counts[b];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive scan
        long long v = (t >= off) ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    long long run = (t == 0) ? 0 : part[t - 1];
    for (int b = b0; b < b1; ++b) {
        J.offsets[b] = run;
        run += J.counts[b];
    }
    if (t == 1023) *J.M = part[1023];
}

__global__ void __launch_bounds__(kFilterThreads) compact_kernel(
    const uint8_t *__restrict__ mask, const double *__restrict__ V, long long n_total,
    const long long *__restrict__ offsets, long long capacity, int32_t *__restrict__ kept_idx,
    double *__restrict__ Vc, double *__restrict__ block_vsum) {
    __shared__ int warp_base[kFilterThreads / 32];
    __shared__ double warp_sum[kFilterThreads / 32];
    long long f = (long long)blockIdx.x * kFilterThreads + threadIdx.x;
    int keep = (f < n_total) ? mask[f] : 0;
    double v = keep ? V[f] : 0.0;
    unsigned bal = __ballot_sync(0xffffffffu, keep);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int pos_in_warp = __popc(bal & ((1u << lane) - 1u));
    // fixed-order FP64 warp sum
    double s = v;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
        warp_base[warp] = __popc(bal);
        warp_sum[warp] = s;
    }
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; ++w) base += warp_base[w];
    if (keep) {
        long long pos = offsets[blockIdx.x] + base + pos_in_warp;
        if (pos < capacity) {
            kept_idx[pos] = (int32_t)f;
            Vc[pos] = v;
        }
    }
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kFilterThreads / 32; ++w) t += warp_sum[w];
        block_vsum[blockIdx.x] = t;
    }
}

// Brick-ordered compaction (bricks as in filter_brick_kernel, whose kept counts it uses).
// The kept points of a brick are contiguous, so any 128 consecutive kept points span a
// compact region of the cell (the real-space culling of the mixed fit keeps fewer images
// for compact tiles).  Deterministic (ballots only).
__global__ void __launch_bounds__(kBrickPts) brick_compact_kernel(const __grid_constant__ FilterLaunch L) {
    __shared__ int warp_base[kBrickPts / 32];
    __shared__ double warp_sum[kBrickPts / 32];
    const int jb = filter_job_of(L, blockIdx.x);
    const FilterJob &J = L.job[jb];
    const int b = blockIdx.x - L.blk[jb];
    const long long f = brick_point(b, threadIdx.x, J.p.nx, J.p.ny, J.p.nz, J.nbx, J.nby);
    const int keep = (f >= 0) ? J.mask[f] : 0;
    const double v = keep ? J.V[f] : 0.0;
    const unsigned bal = __ballot_sync(0xffffffffu, keep);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int pos_in_warp = __popc(bal & ((1u << lane) - 1u));
    double s = v;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
        warp_base[warp] = __popc(bal);
        warp_sum[warp] = s;
    }
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; ++w) base += warp_base[w];
    if (keep) {
        const long long pos = J.offsets[b] + base + pos_in_warp;
        if (pos < J.p.n_total) {
            J.kept[pos] = (int32_t)f;
            J.Vc[pos] = v;
        }
    }
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kBrickPts / 32; ++w) t += warp_sum[w];
        J.vsum[b] = t;
    }
}

// Mean of each job's kept V over its blocks in a fixed order (deterministic), one CTA per job.
__global__ void __launch_bounds__(1024) vmean_kernel(const __grid_constant__ FilterLaunch L) {
    const FilterJob &J = L.job[blockIdx.x];
    __shared__ double part[1024];
    int t = threadIdx.x;
    double s = 0.0;
    for (int b = t; b < J.ncount; b += 1024) s += J.vsum[b];
    part[t] = s;
    __syncthreads();
    for (int off = 512; off > 0; off >>= 1) {
        if (t < off) part[t] += part[t + off];
        __syncthreads();
    }
    if (t == 0) {
        long long M = *J.M;
        *J.mean = M > 0 ? part[0] / (double)M : 0.0;
    }
}

// Centre each job's kept ESP (Vc -= mean), kCenterParts CTAs per job, and write each CTA's
// sum of the centred values and their largest magnitude (the ESP row statistics of the mixed
// Gram), reduced in a fixed order by vstats_kernel.
constexpr int kCenterThreads = 256;
__global__ void __launch_bounds__(kCenterThreads) center_kernel(const __grid_constant__ FilterLaunch L) {
    const FilterJob &J = L.job[blockIdx.x / kCenterParts];
    const int part = blockIdx.x % kCenterParts;
    const double m = *J.mean;
    const long long M = *J.M;
    double s = 0.0, mx = 0.0;
    for (long long i = (long long)part * blockDim.x + threadIdx.x; i < M; i += (long long)kCenterParts * blockDim.x) {
        const double v = J.Vc[i] - m;
        J.Vc[i] = v;
        s += v;
        mx = fmax(mx, fabs(v));
    }
    __shared__ double ss[kCenterThreads / 32], sm[kCenterThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = s;
        sm[threadIdx.x >> 5] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, u = 0.0;
        for (int w = 0; w < kCenterThreads / 32; ++w) {
            t += ss[w];
            u = fmax(u, sm[w]);
        }
        J.vpart[part] = make_double2(t, u);
    }
}

// One warp per job: its parts in a fixed shuffle tree (deterministic).
__global__ void vstats_kernel(const __grid_constant__ FilterLaunch L) {
    const FilterJob &J = L.job[blockIdx.x];
    if (!J.vstats) return;
    double t = 0.0, u = 0.0;
    for (int b = threadIdx.x; b < kCenterParts; b += 32) {
        t += J.vpart[b].x;
        u = fmax(u, J.vpart[b].y);
    }
    for (int o = 16; o > 0; o >>= 1) {
        t += __shfl_xor_sync(0xffffffffu, t, o);
        u = fmax(u, __shfl_xor_sync(0xffffffffu, u, o));
    }
    if (threadIdx.x == 0) {
        J.vstats[0] = t;
        J.vstats[1] = u;
    }
}

}  // namespace

double radius_of(int z) {
    static const double VDW[] = {
        2.72687, 2.23177, 2.31586, 2.59365, 3.85788, 3.63867, 3.45820, 3.30702, 3.17852, 3.06419, 2.81853,
        2.85443, 4.25094, 4.05819, 3.91835, 3.81252, 3.72937, 3.65473, 3.60182, 3.21159, 3.11332, 2.99994,
        2.97065, 2.85632, 2.79774, 2.75144, 2.71365, 2.67774, 3.30230, 2.61066, 4.14133, 4.04401, 3.99677,
        3.97315, 3.95803, 3.91268, 3.88717, 3.44025, 3.16057, 2.95175, 2.99049, 2.88372, 2.83270, 2.79963,
        2.76750, 2.73916, 2.97443, 2.69097, 4.21692, 4.14984, 4.17629, 4.22354, 4.25188, 4.16118, 4.26795,
        3.49883, 3.32781, 3.35993, 3.40718, 3.37789, 3.35143, 3.32592, 3.30041, 3.18230, 3.26072, 3.23899,
        3.22104, 3.20403, 3.18797, 3.17002, 3.43930, 2.96781, 2.99522, 2.89978, 2.79113, 2.94797, 2.68341,
        2.60215, 3.11143, 2.55585, 4.10732, 4.06008, 4.12905, 4.44936, 4.48810, 4.50227, 4.62983, 3.47426,
        3.28623, 3.20875, 3.23521, 3.20781, 3.23521, 3.23521, 3.19458, 3.14261, 3.15490, 3.13033, 3.11710,
        3.10482, 3.09348, 3.06892, 3.05758, 3.04513, 3.03268, 3.02023, 3.00778};
    const int n = (int)(sizeof(VDW) / sizeof(VDW[0]));
    return (z >= 1 && z <= n) ? VDW[z - 1] : 3.0;
}

void filter_plan(const rp_grid *grid, const double *atoms, const int *Z, int N, double vdw_factor, double vdw_max,
                 FilterPlan &plan) {
    RP_REQUIRE(grid && atoms && Z, "rp_filter: null argument");
    RP_REQUIRE(N >= 0, "rp_filter: N < 0");
    const int nx = grid->n_grid[0], ny = grid->n_grid[1], nz = grid->n_grid[2];
    RP_REQUIRE(nx > 0 && ny > 0 && nz > 0, "rp_filter: grid counts must be positive");
    const long long n_total = (long long)nx * ny * nz;
    RP_REQUIRE(n_total < (1LL << 31), "rp_filter: grid larger than 2^31 points");
    RP_REQUIRE(vdw_factor >= 0.0 && vdw_max >= 0.0, "rp_filter: negative vdW factor");
    const double *ax = grid->axis;

    // ---- effective atoms (repeat.py:1933-1969), FP64, reference operation order
    double box[9];
    for (int i = 0; i < 3; ++i)
        for (int d = 0; d < 3; ++d) box[3 * i + d] = (double)grid->n_grid[i] * ax[3 * i + d];
    double gmaxr = 5.0;
    if (N > 0) {
        gmaxr = -1e300;
        for (int a = 0; a < N; ++a) gmaxr = std::max(gmaxr, vdw_max * radius_of(Z[a]));
    }
    double cmin[3] = {1e300, 1e300, 1e300}, cmax[3] = {-1e300, -1e300, -1e300};
    for (int c = 0; c < 8; ++c) {  // corners of the grid-step parallelepiped, as the reference forms them
        int fI = (c >> 2) & 1, fJ = (c >> 1) & 1, fK = c & 1;
        for (int d = 0; d < 3; ++d) {
            double v = (fI * ax[d] + fJ * ax[3 + d]) + fK * ax[6 + d];
            cmin[d] = std::min(cmin[d], v);
            cmax[d] = std::max(cmax[d], v);
        }
    }
    const double margin = gmaxr + 0.1;
    // working arrays live in the plan, so a plan reused across batches allocates nothing
    std::vector<D4> &e64 = plan.w_e64;
    std::vector<double> &rmax2 = plan.w_rmax2;
    e64.clear();
    rmax2.clear();
    e64.reserve(27 * (size_t)N);
    double max_rmin = 0.0, max_rmax = 0.0, emax = 0.0;
    for (int a = 0; a < N; ++a) {
        double raw = radius_of(Z[a]);
        double rn = vdw_factor * raw, rx = vdw_max * raw;
        for (int kz = -1; kz <= 1; ++kz)
            for (int ky = -1; ky <= 1; ++ky)
                for (int kx = -1; kx <= 1; ++kx) {
                    double p[3];
                    bool in = true;
                    for (int d = 0; d < 3; ++d) {
                        double sh = (kx * box[d] + ky * box[3 + d]) + kz * box[6 + d];
                        p[d] = atoms[3 * a + d] + sh;
                        if (!(p[d] >= cmin[d] - margin && p[d] <= cmax[d] + margin)) in = false;
                    }
                    if (!in) continue;
                    e64.push_back(D4{p[0], p[1], p[2], rn * rn});
                    rmax2.push_back(rx * rx);
                    max_rmin = std::max(max_rmin, rn);
                    max_rmax = std::max(max_rmax, rx);
                    for (int d = 0; d < 3; ++d) emax = std::max(emax, std::fabs(p[d]));
                }
    }
    const int A = (int)e64.size();

    // ---- near proved for every grid point?  (the grid hull is convex: its corners bound it)
    int near_all = 0;
    for (int a = 0; a < A && !near_all; ++a) {
        double worst = 0.0;
        for (int c = 0; c < 8; ++c) {
            int f0 = (c & 1) ? nx - 1 : 0, f1 = (c & 2) ? ny - 1 : 0, f2 = (c & 4) ? nz - 1 : 0;
            double d2 = 0.0;
            for (int d = 0; d < 3; ++d) {
                double v = (f0 * ax[d] + f1 * ax[3 + d]) + f2 * ax[6 + d];
                v -= (d == 0 ? e64[a].x : (d == 1 ? e64[a].y : e64[a].z));
                d2 += v * v;
            }
            worst = std::max(worst, d2);
        }
        if (worst * (1.0 + 1e-9) + 1e-9 < rmax2[a]) near_all = 1;
    }

    // ---- FP32 error band (see header comment): |d2_32 - d2_64| <= err
    double gs = 0.0;  // bound on |i*a0|+|j*a1|+|k*a2| per component
    for (int d = 0; d < 3; ++d)
        gs = std::max(gs, (nx - 1) * std::fabs(ax[d]) + (ny - 1) * std::fabs(ax[3 + d]) + (nz - 1) * std::fabs(ax[6 + d]));
    const double u = std::ldexp(1.0, -24);
    const double ddx = 8.0 * u * gs + 2.0 * u * emax + 2.0 * u * (gs + emax);
    auto band = [&](double r) {
        return 4.0 * (2.0 * std::sqrt(3.0) * r * 1.01 * ddx + 3.0 * ddx * ddx + 8.0 * u * r * r * 1.02) + 1e-30;
    };
    const double err_min = band(max_rmin);
    const double err_max = band(max_rmax);

    // ---- cell list for the reject test: bin edge >= max rmin + coordinate error
    double bsize = std::max(max_rmin, 1e-3) * (1.0 + 1e-4) + 16.0 * ddx + 1e-3;
    double bmin[3] = {1e300, 1e300, 1e300}, bmax[3] = {-1e300, -1e300, -1e300};
    for (auto &e : e64) {
        double p[3] = {e.x, e.y, e.z};
        for (int d = 0; d < 3; ++d) {
            bmin[d] = std::min(bmin[d], p[d]);
            bmax[d] = std::max(bmax[d], p[d]);
        }
    }
    if (A == 0)
        for (int d = 0; d < 3; ++d) bmin[d] = bmax[d] = 0.0;
    int bn[3];
    for (int d = 0; d < 3; ++d) bn[d] = std::max(1, (int)std::ceil((bmax[d] - bmin[d]) / bsize) + 1);
    while ((long long)bn[0] * bn[1] * bn[2] > (1LL << 22)) {  // keep the table small; grow bins
        bsize *= 1.25;
        for (int d = 0; d < 3; ++d) bn[d] = std::max(1, (int)std::ceil((bmax[d] - bmin[d]) / bsize) + 1);
    }
    const int nb = bn[0] * bn[1] * bn[2];
    std::vector<int> &boff = plan.boff, &bidx = plan.bidx, &binof = plan.w_binof;
    boff.assign((size_t)nb + 1, 0);
    bidx.resize((size_t)std::max(A, 1));
    binof.resize((size_t)std::max(A, 1));
    for (int a = 0; a < A; ++a) {
        double p[3] = {e64[a].x, e64[a].y, e64[a].z};
        int b = 0, m = 1;
        for (int d = 0; d < 3; ++d) {
            int c = (int)std::floor((p[d] - bmin[d]) / bsize);
            c = std::min(std::max(c, 0), bn[d] - 1);
            b += m * c;
            m *= bn[d];
        }
        binof[a] = b;
        boff[b + 1]++;
    }
    for (int b = 0; b < nb; ++b) boff[b + 1] += boff[b];
    {
        std::vector<int> &cur = plan.w_cur;
        cur.assign(boff.begin(), boff.end() - 1);
        for (int a = 0; a < A; ++a) bidx[cur[binof[a]]++] = a;
    }
    // FP32 copies, ordered by bin so a bin's atoms are contiguous in memory
    std::vector<float4> &e32 = plan.e32;
    std::vector<D4> &e64s = plan.e64;
    std::vector<double> &rmax2s = plan.rmax2;
    std::vector<float> &rmax2f = plan.rmax2f;
    e32.resize((size_t)std::max(A, 1));
    e64s.resize((size_t)std::max(A, 1));
    rmax2s.resize((size_t)std::max(A, 1));
    rmax2f.resize((size_t)std::max(A, 1));
    for (int t = 0; t < A; ++t) {
        int a = bidx[t];
        e64s[t] = e64[a];
        rmax2s[t] = rmax2[a];
        rmax2f[t] = (float)rmax2[a];
        e32[t] = make_float4((float)e64[a].x, (float)e64[a].y, (float)e64[a].z, (float)e64[a].w);
        bidx[t] = t;
    }

    // FP32 copies, ordered by bin (above); the launch parameters
    FilterParams &p = plan.p;
    p = FilterParams{};
    p.nx = nx; p.ny = ny; p.nz = nz; p.n_total = n_total;
    for (int t = 0; t < 9; ++t) { p.ax[t] = (float)ax[t]; p.axd[t] = ax[t]; }
    for (int d = 0; d < 3; ++d) { p.bmin[d] = (float)bmin[d]; p.bn[d] = bn[d]; }
    p.inv_bsize = (float)(1.0 / bsize);
    p.err_min = (float)err_min;
    p.err_max = (float)err_max;
    p.near_all = near_all;
    p.A = A;
}

namespace {
// every packed array starts on a 32-byte boundary: D4 is read with one 32-byte vector load
size_t al32(size_t n) { return (n + 31) / 32 * 32; }
}  // namespace

size_t FilterPlan::bytes() const {
    return al32(e32.size() * sizeof(float4)) + al32(e64.size() * sizeof(D4)) + al32(rmax2.size() * sizeof(double)) +
           al32(rmax2f.size() * sizeof(float)) + al32(boff.size() * sizeof(int)) + al32(bidx.size() * sizeof(int));
}

void FilterPlan::pack(char *dst) const {
    auto put = [&](const void *src, size_t n) {
        std::memcpy(dst, src, n);
        dst += al32(n);
    };
    put(e32.data(), e32.size() * sizeof(float4));
    put(e64.data(), e64.size() * sizeof(D4));
    put(rmax2.data(), rmax2.size() * sizeof(double));
    put(rmax2f.data(), rmax2f.size() * sizeof(float));
    put(boff.data(), boff.size() * sizeof(int));
    put(bidx.data(), bidx.size() * sizeof(int));
}

namespace {
// A job's plan arrays, read from its packed device image.
void job_from_plan(const FilterPlan &plan, const char *packed_dev, FilterJob &J) {
    const char *src = packed_dev;
    auto take = [&](size_t n) {
        const char *r = src;
        src += al32(n);
        return r;
    };
    J.p = plan.p;
    J.e32 = reinterpret_cast<const float4 *>(take(plan.e32.size() * sizeof(float4)));
    J.e64 = reinterpret_cast<const D4 *>(take(plan.e64.size() * sizeof(D4)));
    J.rmax2 = reinterpret_cast<const double *>(take(plan.rmax2.size() * sizeof(double)));
    J.rmax2f = reinterpret_cast<const float *>(take(plan.rmax2f.size() * sizeof(float)));
    J.boff = reinterpret_cast<const int *>(take(plan.boff.size() * sizeof(int)));
    J.bidx = reinterpret_cast<const int *>(take(plan.bidx.size() * sizeof(int)));
    J.nbx = (plan.p.nx + kBrickX - 1) / kBrickX;
    J.nby = (plan.p.ny + kBrickY - 1) / kBrickY;
}
int bricks_of(const FilterParams &p) {
    return ((p.nx + kBrickX - 1) / kBrickX) * ((p.ny + kBrickY - 1) / kBrickY) * ((p.nz + kBrickZ - 1) / kBrickZ);
}
}  // namespace

void filter_group(rp_ctx *ctx, const std::vector<FilterItem> &items, cudaStream_t stream, const std::string &tag) {
    if (items.empty()) return;
    const size_t n = items.size();
    std::vector<size_t> o_pts(n + 1, 0), o_br(n + 1, 0);
    for (size_t i = 0; i < n; ++i) {
        const FilterParams &p = items[i].plan->p;
        RP_REQUIRE(items[i].V && items[i].M && items[i].packed_dev, "rp_filter: null argument");
        o_pts[i + 1] = o_pts[i] + (size_t)p.n_total;
        o_br[i + 1] = o_br[i] + (size_t)bricks_of(p);
    }
    uint8_t *mask = ctx->buf_t<uint8_t>("flt_mask" + tag, o_pts[n]);
    int *counts = ctx->buf_t<int>("flt_bcounts" + tag, o_br[n]);
    long long *offs = ctx->buf_t<long long>("flt_boffsets" + tag, o_br[n]);
    double *vsum = ctx->buf_t<double>("flt_bvsum" + tag, o_br[n]);
    double *mean = ctx->buf_t<double>("flt_mean" + tag, n);
    double2 *vpart = ctx->buf_t<double2>("flt_vpart" + tag, n * kCenterParts);
    StageTimer t_f(ctx, "filter", stream);
    for (size_t j0 = 0; j0 < n; j0 += kFilterJobs) {
        const size_t j1 = std::min(n, j0 + kFilterJobs);
        FilterLaunch L{};
        L.n = (int)(j1 - j0);
        for (size_t i = j0; i < j1; ++i) {
            FilterJob &J = L.job[i - j0];
            job_from_plan(*items[i].plan, items[i].packed_dev, J);
            J.V = items[i].V;
            J.mask = mask + o_pts[i];
            J.counts = counts + o_br[i];
            J.offsets = offs + o_br[i];
            J.vsum = vsum + o_br[i];
            J.ncount = (int)(o_br[i + 1] - o_br[i]);
            J.kept = items[i].kept;
            J.Vc = items[i].Vc;
            J.M = items[i].M;
            J.mean = mean + i;
            J.vpart = vpart + i * kCenterParts;
            J.vstats = items[i].vstats;
            L.blk[i - j0 + 1] = L.blk[i - j0] + J.ncount;
        }
        const int nbr = L.blk[L.n];
        filter_brick_kernel<<<nbr, kBrickPts, 0, stream>>>(L, 1);
        RP_LAUNCH_CHECK();
        scan_counts_kernel<<<L.n, 1024, 0, stream>>>(L);
        RP_LAUNCH_CHECK();
        brick_compact_kernel<<<nbr, kBrickPts, 0, stream>>>(L);
        RP_LAUNCH_CHECK();
        vmean_kernel<<<L.n, 1024, 0, stream>>>(L);
        RP_LAUNCH_CHECK();
        center_kernel<<<L.n * kCenterParts, kCenterThreads, 0, stream>>>(L);
        RP_LAUNCH_CHECK();
        vstats_kernel<<<L.n, 32, 0, stream>>>(L);
        RP_LAUNCH_CHECK();
    }
}

void filter_launch(rp_ctx *ctx, const FilterPlan &plan, const char *packed_dev, const double *V_dev,
                   int32_t *kept_idx_dev, double *Vc_dev, long long *M_dev, uint8_t *mask_dev, cudaStream_t stream,
                   const std::string &tag, bool brick_order, double *vstats_dev) {
    RP_REQUIRE(V_dev && M_dev && packed_dev, "rp_filter: null argument");
    if (brick_order && !mask_dev) {
        filter_group(ctx, {FilterItem{&plan, packed_dev, V_dev, kept_idx_dev, Vc_dev, M_dev, vstats_dev}}, stream,
                     tag);
        return;
    }
    // flat order (rp_filter): the culled mask, then the compaction over flat blocks
    const long long n_total = plan.p.n_total;
    const int nblk = (int)((n_total + kFilterThreads - 1) / kFilterThreads);
    FilterLaunch L{};
    L.n = 1;
    FilterJob &J = L.job[0];
    job_from_plan(plan, packed_dev, J);
    J.V = V_dev;
    J.mask = mask_dev ? mask_dev : ctx->buf_t<uint8_t>("flt_mask" + tag, (size_t)n_total);
    J.counts = ctx->buf_t<int>("flt_counts" + tag, (size_t)nblk);
    J.offsets = ctx->buf_t<long long>("flt_offsets" + tag, (size_t)nblk);
    J.vsum = ctx->buf_t<double>("flt_vsum" + tag, (size_t)nblk);
    J.ncount = nblk;
    J.kept = kept_idx_dev;
    J.Vc = Vc_dev;
    J.M = M_dev;
    J.mean = ctx->buf_t<double>("flt_mean" + tag, 1);
    J.vpart = ctx->buf_t<double2>("flt_vpart" + tag, kCenterParts);
    J.vstats = vstats_dev;
    StageTimer t_f(ctx, "filter", stream);
    L.blk[1] = bricks_of(plan.p);
    filter_brick_kernel<<<L.blk[1], kBrickPts, 0, stream>>>(L, 0);
    RP_LAUNCH_CHECK();
    flat_count_kernel<<<nblk, kFilterThreads, 0, stream>>>(J.mask, n_total, J.counts);
    RP_LAUNCH_CHECK();
    scan_counts_kernel<<<1, 1024, 0, stream>>>(L);
    RP_LAUNCH_CHECK();
    compact_kernel<<<nblk, kFilterThreads, 0, stream>>>(J.mask, V_dev, n_total, J.offsets, n_total, kept_idx_dev,
                                                        Vc_dev, J.vsum);
    RP_LAUNCH_CHECK();
    vmean_kernel<<<1, 1024, 0, stream>>>(L);
    RP_LAUNCH_CHECK();
    center_kernel<<<kCenterParts, kCenterThreads, 0, stream>>>(L);
    RP_LAUNCH_CHECK();
    vstats_kernel<<<1, 32, 0, stream>>>(L);
    RP_LAUNCH_CHECK();
}

void filter_async(rp_ctx *ctx, const rp_grid *grid, const double *atoms, const int *Z, int N, const double *V_dev,
                  double vdw_factor, double vdw_max, int32_t *kept_idx_dev, double *Vc_dev, long long *M_dev,
                  uint8_t *mask_dev, cudaStream_t stream, const std::string &tag, bool brick_order,
                  double *vstats_dev) {
    RP_REQUIRE(grid && atoms && Z && V_dev && M_dev, "rp_filter: null argument");
    FilterPlan plan;
    filter_plan(grid, atoms, Z, N, vdw_factor, vdw_max, plan);
    std::vector<char> host(plan.bytes());
    plan.pack(host.data());
    char *dev = static_cast<char *>(ctx->buf("flt_plan" + tag, host.size()));
    RP_CUDA(cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, stream));
    filter_launch(ctx, plan, dev, V_dev, kept_idx_dev, Vc_dev, M_dev, mask_dev, stream, tag, brick_order,
                  vstats_dev);
}

void filter_run(rp_ctx *ctx, const rp_grid *grid, const double *atoms, const int *Z, int N, const double *V_dev,
                double vdw_factor, double vdw_max, int32_t *kept_idx_dev, double *Vc_dev, int64_t capacity,
                int64_t *M_out, uint8_t *mask_dev, cudaStream_t stream) {
    RP_REQUIRE(grid && M_out, "rp_filter: null argument");
    const long long npts = (long long)grid->n_grid[0] * grid->n_grid[1] * grid->n_grid[2];
    // the compaction writes every kept point, so the caller's buffers must hold the
    // whole grid unless the kept count is known to fit; stage through ctx scratch otherwise
    const bool direct = capacity >= npts;
    int32_t *kid = direct ? kept_idx_dev : ctx->buf_t<int32_t>("flt_kept_stage", (size_t)npts);
    double *vc = direct ? Vc_dev : ctx->buf_t<double>("flt_vc_stage", (size_t)npts);
    long long *d_M = ctx->buf_t<long long>("flt_total", 1);
    filter_async(ctx, grid, atoms, Z, N, V_dev, vdw_factor, vdw_max, kid, vc, d_M, mask_dev, stream, "", false,
                 nullptr);
    long long M = 0;
    RP_CUDA(cudaMemcpyAsync(&M, d_M, sizeof(long long), cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaStreamSynchronize(stream));
    *M_out = M;
    if (M > capacity)
        fail(RP_E_ARG, "rp_filter: " + std::to_string(M) + " kept points exceed capacity " + std::to_string(capacity));
    if (!direct && M > 0) {
        RP_CUDA(cudaMemcpyAsync(kept_idx_dev, kid, sizeof(int32_t) * M, cudaMemcpyDeviceToDevice, stream));
        RP_CUDA(cudaMemcpyAsync(Vc_dev, vc, sizeof(double) * M, cudaMemcpyDeviceToDevice, stream));
    }
}

}  // namespace rp
