// Mixed-precision Phi -> normal equations on the sm_103a tensor cores.
//
// Replaces, on the device, the Phi build of EwaldCalculator._compute_gpu*
// (repeat.py:1199-1435) and the Gram accumulation of fit_charges
// (repeat.py:2246-2276).  Per chunk of kept points:
//
//  1. tables  T[m][k'] = sqrt(w_k) 2^10 [cos(k.g_m) | sin(k.g_m)] and
//             B[a][k'] = sqrt(w_k) 2^10 [cos(k.r_a) | sin(k.r_a)], each split into
//             an FP16 pair hi + lo (22 significant bits; sqrt(w) on both sides keeps
//             every term inside FP16 range).  Grid phases are exact per-axis tables.
//  2. GEMM-1  Phi_recip = T B^T on tcgen05 (kind::f16, FP32 accumulator in TMEM)
//             as hi*hi + hi*lo + lo*hi, written atom-major (Phi_t[a][m]).
//  3. real    Phi_t[a][m] += sum_s [r <= Rc] erfc(sqrt(alpha) r)/r in FP32, with
//             coordinates taken relative to a per-tile origin.
//  4. split   X[a][m] = (Phi_t[a][m] - c_a) * 2^e_a as FP16 hi + lo, plus a row for
//             the centred ESP: c_a is the column mean of the first chunk (a per-
//             column shift corrected exactly later), 2^e_a a power-of-two row scale.
//  5. GEMM-2  G = X X^T on tcgen05 (upper-triangle tiles), split over points so each
//             FP32 run is short; partial tiles are summed in FP64 in a fixed order.
//  6. finish  A = G - s s^T/M, b = G[:,V] - s sum(V)/M with s = sum_m (Phi - c)
//             (FP64), i.e. repeat.py:2266-2276 for the shifted columns.
//
// Dropping lo*lo costs ~2^-22 relative per product; measured on the synthetic
// workloads the charges move by <~2e-7 e against the FP64 fit (BF16 hi+lo, with
// 16 significant bits and the atom-table error coherent across all points, moved
// them by ~5e-6 e, which is why the split type is FP16).
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "tc.cuh"

namespace rp {
namespace {

constexpr int kBM = 128;       // tile rows (TMEM lanes)
constexpr int kBN = 128;       // tile columns
constexpr int kBK = 64;        // K elements per stage (128 B of FP16 = one swizzle row)
constexpr int kStages = 3;
constexpr int kGemmThreads = 192;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2-5 epilogue
constexpr int kTileBytes = kBM * kBK * 2;  // 16 KB per operand tile
constexpr int kStageBytes = 4 * kTileBytes;
constexpr int kGemmSmem = kStages * kStageBytes + 1024 + 256;
constexpr float kTableScale = 1024.0f;   // 2^10 on each table side

struct GemmArgs {
    int mode;            // 0: Phi tiles (write D*scale atom-major); 1: Gram partial tiles
    int m_tiles, n_tiles;
    int kb_total;        // K blocks of 64 in the reduction
    int kb_per_split;    // mode 1
    int ntri;            // mode 1: number of upper-triangle tiles
    int rows_m, rows_n;  // valid extents of the A and B row ranges (mode 0)
    float out_scale;
    float *out;
    long long ld_out;
    int *status;
};

__device__ __forceinline__ void tri_decode(int t, int nt, int &ti, int &tj) {
    // upper-triangle tile t -> (ti <= tj), row-major over ti
    ti = 0;
    int rowlen = nt;
    while (t >= rowlen) {
        t -= rowlen;
        ++ti;
        --rowlen;
    }
    tj = ti + t;
}

__global__ void __launch_bounds__(kGemmThreads, 1) split_gemm_kernel(const __grid_constant__ CUtensorMap tmAh,
                                                                       const __grid_constant__ CUtensorMap tmAl,
                                                                       const __grid_constant__ CUtensorMap tmBh,
                                                                       const __grid_constant__ CUtensorMap tmBl,
                                                                       GemmArgs g) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw_s = tc::smem_u32(smem_raw);
    uint8_t *smem = smem_raw + (((raw_s + 1023u) & ~1023u) - raw_s);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kStages * kStageBytes);
    uint64_t *empty = full + kStages;
    uint64_t *accb = empty + kStages;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(accb + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int a_row0, b_row0, kb0, kb1, out_tile = 0;
    if (g.mode == 0) {
        const int mt = blockIdx.x % g.m_tiles, nt = blockIdx.x / g.m_tiles;
        a_row0 = mt * kBM;
        b_row0 = nt * kBN;
        kb0 = 0;
        kb1 = g.kb_total;
    } else {
        const int tri = blockIdx.x % g.ntri, split = blockIdx.x / g.ntri;
        int ti, tj;
        tri_decode(tri, g.m_tiles, ti, tj);
        a_row0 = ti * kBM;
        b_row0 = tj * kBN;
        kb0 = split * g.kb_per_split;
        kb1 = min(kb0 + g.kb_per_split, g.kb_total);
        out_tile = blockIdx.x;
    }
    const int nkb = kb1 - kb0;  // >= 1 by construction

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accb, 1);
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_holder, kBN);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0 && lane == 0) {
        tc::prefetch_tmap(&tmAh);
        tc::prefetch_tmap(&tmAl);
        tc::prefetch_tmap(&tmBh);
        tc::prefetch_tmap(&tmBl);
        int issued = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kStages, u = kb / kStages;
            if (u > 0 && !tc::mbar_wait(&empty[s], (u - 1) & 1, g.status)) break;
            uint8_t *st = smem + s * kStageBytes;
            tc::mbar_arrive_expect_tx(&full[s], kStageBytes);
            const int x = (kb0 + kb) * kBK;
            tc::tma_load_2d(st, &tmAh, x, a_row0, &full[s]);
            tc::tma_load_2d(st + kTileBytes, &tmAl, x, a_row0, &full[s]);
            tc::tma_load_2d(st + 2 * kTileBytes, &tmBh, x, b_row0, &full[s]);
            tc::tma_load_2d(st + 3 * kTileBytes, &tmBl, x, b_row0, &full[s]);
            issued = kb + 1;
        }
        if (*reinterpret_cast<volatile int *>(g.status) != 0) {
            // unwind: let the copies already issued land before the CTA exits
            for (int kb = max(0, issued - kStages); kb < issued; ++kb) {
                int dummy = 0;
                tc::mbar_wait(&full[kb % kStages], (kb / kStages) & 1, &dummy);
            }
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = tc::idesc_f16_f32(kBM, kBN);
        int done = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kStages, u = kb / kStages;
            if (!tc::mbar_wait(&full[s], u & 1, g.status)) break;
            tc::fence_after_sync();
            const uint32_t st = tc::smem_u32(smem + s * kStageBytes);
            const uint64_t ah = tc::sdesc_k_sw128(st), al = tc::sdesc_k_sw128(st + kTileBytes);
            const uint64_t bh = tc::sdesc_k_sw128(st + 2 * kTileBytes), bl = tc::sdesc_k_sw128(st + 3 * kTileBytes);
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const uint64_t o = (uint64_t)(kk * 2);  // 32 B per K=16 step, in 16-B units
                tc::umma_f16(tmem, ah + o, bh + o, idesc, (kb | kk) != 0);
                tc::umma_f16(tmem, ah + o, bl + o, idesc, 1u);
                tc::umma_f16(tmem, al + o, bh + o, idesc, 1u);
            }
            tc::umma_commit(&empty[s]);
            done = kb + 1;
        }
        tc::umma_commit(accb);
        (void)done;
    } else if (warp >= 2) {
        if (tc::mbar_wait(accb, 0, g.status) && *reinterpret_cast<volatile int *>(g.status) == 0) {
            tc::fence_after_sync();
            const int lane_base = (warp & 3) * 32;
            const int r = lane_base + lane;
#pragma unroll 1
            for (int c = 0; c < kBN / 32; ++c) {
                float v[32];
                tc::tmem_ld_32x32(tmem + ((uint32_t)lane_base << 16) + (uint32_t)(c * 32), v);
                if (g.mode == 0) {
                    const int m = a_row0 + r;
                    if (m < g.rows_m) {
#pragma unroll
                        for (int i = 0; i < 32; ++i) {
                            const int n = b_row0 + c * 32 + i;
                            if (n < g.rows_n) g.out[(long long)n * g.ld_out + m] = v[i] * g.out_scale;
                        }
                    }
                } else {
                    float *o = g.out + (long long)out_tile * (kBM * kBN);
#pragma unroll
                    for (int i = 0; i < 32; ++i) o[(c * 32 + i) * kBM + r] = v[i];
                }
            }
        }
    }
    // the MMA thread's last commit must have landed before TMEM is released
    if (warp == 1 && lane == 0) {
        int dummy = 0;
        tc::mbar_wait(accb, 0, &dummy);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1) tc::tmem_dealloc(tmem, kBN);
}

// ------------------------------------------------------------------ tables

__device__ __forceinline__ void split_f16(float x, __half &hi, __half &lo) {
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

__global__ void atom_tables_f16_kernel(const double *__restrict__ kvec, const double *__restrict__ kcoef, int K,
                                       int K2p, const double *__restrict__ atoms, int N, __half *__restrict__ Bh,
                                       __half *__restrict__ Bl) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * K2p) return;
    int a = (int)(t / K2p), k2 = (int)(t - (long long)a * K2p);
    float val = 0.0f;
    if (k2 < 2 * K) {
        int k = k2 < K ? k2 : k2 - K;
        double kr = (atoms[3 * a] * kvec[3 * k] + atoms[3 * a + 1] * kvec[3 * k + 1]) + atoms[3 * a + 2] * kvec[3 * k + 2];
        double s, c;
        sincos(kr, &s, &c);
        double sw = sqrt(kcoef[k]) * (double)kTableScale;
        val = (float)(sw * (k2 < K ? c : s));
    }
    __half h, l;
    split_f16(val, h, l);
    Bh[t] = h;
    Bl[t] = l;
}

__global__ void grid_tables_f16_kernel(const int *__restrict__ kidx, const float *__restrict__ swk, int K, int K2p,
                                       int kmax, const float2 *__restrict__ ex, const float2 *__restrict__ ey,
                                       const float2 *__restrict__ ez, int nx, int ny, int nz,
                                       const int32_t *__restrict__ kept, long long m0, long long rows,
                                       long long rows_pad, __half *__restrict__ Th, __half *__restrict__ Tl) {
    // one thread per (point, k): writes column k (cos) and K+k (sin) of row m
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int half = K2p / 2;  // >= K; columns [K, half) and [K+half ...) unused -> zero
    if (t >= rows_pad * half) return;
    long long m = t / half;
    int k = (int)(t - m * half);
    float re = 0.f, im = 0.f;
    if (m < rows && k < K) {
        int f = kept[m0 + m];
        int layer = nx * ny;
        int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
        int n1 = kidx[3 * k], n2 = kidx[3 * k + 1], n3 = kidx[3 * k + 2];
        float2 a = ex[n1 * nx + i], b = ey[(n2 + kmax) * ny + j], c = ez[(n3 + kmax) * nz + l];
        float r1 = a.x * b.x - a.y * b.y, i1 = a.x * b.y + a.y * b.x;
        float sw = swk[k];
        re = (r1 * c.x - i1 * c.y) * sw;
        im = (r1 * c.y + i1 * c.x) * sw;
    }
    // layout: [cos block | sin block], both of width K, then zero pad to K2p
    __half h, l;
    long long row = m * (long long)K2p;
    if (k < K) {
        split_f16(re, h, l);
        Th[row + k] = h;
        Tl[row + k] = l;
        split_f16(im, h, l);
        Th[row + K + k] = h;
        Tl[row + K + k] = l;
    } else {
        // zero padding columns 2K .. K2p-1 (k runs over [K, half))
        int c0 = 2 * K + (k - K) * 2;
        for (int c = c0; c < c0 + 2 && c < K2p; ++c) {
            Th[row + c] = __float2half_rn(0.f);
            Tl[row + c] = __float2half_rn(0.f);
        }
    }
}

// ------------------------------------------------------------------ real space (FP32)

constexpr int kRealPts = 128;   // points per CTA (one per thread)
constexpr int kRealAtoms = 32;  // atoms per CTA

// Phi_t[a][m] += sum_s erfc(sqrt(alpha) r)/r over images within Rc.  Coordinates
// are taken relative to the CTA's first point (computed in FP64 on the fly) so
// FP32 differences keep their precision.
__global__ void __launch_bounds__(kRealPts) realspace_f32_kernel(
    const int32_t *__restrict__ kept, long long m0, long long rows, const double *__restrict__ axis, int nx, int ny,
    const double *__restrict__ atoms, int N, const double *__restrict__ shifts, int S, int zero_idx, float rc2,
    float sa, float *__restrict__ phit, long long ld) {
    __shared__ float3 img[kRealAtoms * 128];   // S <= 128 images per atom (host checks)
    __shared__ double origin[3];
    const long long mb = (long long)blockIdx.x * kRealPts;
    const int a0 = blockIdx.y * kRealAtoms;
    const int na = min(kRealAtoms, N - a0);
    const int layer = nx * ny;
    if (threadIdx.x == 0) {
        int f = kept[m0 + mb];
        int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
        for (int d = 0; d < 3; ++d) origin[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)l * axis[6 + d];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < na * S; t += kRealPts) {
        int a = t / S, s = t - a * S;
        const double *p = atoms + 3 * (a0 + a);
        img[a * S + s] = make_float3((float)(p[0] + shifts[3 * s] - origin[0]), (float)(p[1] + shifts[3 * s + 1] - origin[1]),
                                     (float)(p[2] + shifts[3 * s + 2] - origin[2]));
    }
    __syncthreads();
    const long long m = mb + threadIdx.x;
    if (m >= rows) return;
    const int f = kept[m0 + m];
    const int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
    double gd[3];
    for (int d = 0; d < 3; ++d) gd[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)l * axis[6 + d] - origin[d];
    const float gx = (float)gd[0], gy = (float)gd[1], gz = (float)gd[2];
    for (int a = 0; a < na; ++a) {
        float acc = 0.f;
        const float3 *ia = img + a * S;
        for (int s = 0; s < S; ++s) {
            float dx = gx - ia[s].x, dy = gy - ia[s].y, dz = gz - ia[s].z;
            float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 <= rc2 && (s != zero_idx || r2 > 1e-20f)) {
                float r = sqrtf(r2);
                acc += erfcf(sa * r) / r;
            }
        }
        phit[(long long)(a0 + a) * ld + m] += acc;
    }
}

// ------------------------------------------------------------------ column statistics and the split

// Per-atom sums (FP64) and max |Phi| over a chunk: stage 1 per (atom, slab of points)
constexpr int kStatSlab = 4096;
__global__ void colstats_kernel(const float *__restrict__ phit, long long ld, long long rows, int N,
                                double *__restrict__ psum, float *__restrict__ pmax) {
    const int a = blockIdx.y;
    const long long r0 = (long long)blockIdx.x * kStatSlab;
    const long long r1 = min(r0 + kStatSlab, rows);
    double s = 0.0;
    float mx = 0.f;
    for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        float v = phit[(long long)a * ld + r];
        s += v;
        mx = fmaxf(mx, fabsf(v));
    }
    __shared__ double ss[256];
    __shared__ float sm[256];
    ss[threadIdx.x] = s;
    sm[threadIdx.x] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            ss[threadIdx.x] += ss[threadIdx.x + o];
            sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        psum[(size_t)a * gridDim.x + blockIdx.x] = ss[0];
        pmax[(size_t)a * gridDim.x + blockIdx.x] = sm[0];
    }
}

// Per-atom: chunk sum (into sphi), and on the first chunk the centre c and scale.
__global__ void colstats_finish_kernel(const double *__restrict__ psum, const float *__restrict__ pmax, int nslab,
                                       int N, long long rows, int first, double *__restrict__ sphi,
                                       double *__restrict__ c, float *__restrict__ cf, float *__restrict__ scale) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= N) return;
    double s = 0.0;
    float mx = 0.f;
    for (int k = 0; k < nslab; ++k) {
        s += psum[(size_t)a * nslab + k];
        mx = fmaxf(mx, pmax[(size_t)a * nslab + k]);
    }
    sphi[a] = first ? s : sphi[a] + s;
    if (first) {
        double mean = s / (double)rows;
        c[a] = mean;
        cf[a] = (float)mean;
        // |Phi - c| <= 2 max|Phi|; scale so that bound sits in [2^-4, 2^-3): FP16 headroom for later chunks
        float bound = 2.f * mx;
        int e = 0;
        if (bound > 0.f) frexpf(bound, &e);
        scale[a] = ldexpf(1.f, -e - 3);
    }
}

// X rows: a < N: (Phi_t[a][m] - c_a) * scale_a;  a == N: Vc[m] * scale_V;  rest zero
__global__ void split_rows_kernel(const float *__restrict__ phit, long long ld, long long rows, long long rows_pad,
                                  int N, int Np_pad, const float *__restrict__ cf, const float *__restrict__ scale,
                                  const double *__restrict__ Vc, long long m0, float vscale, __half *__restrict__ Xh,
                                  __half *__restrict__ Xl) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)Np_pad * rows_pad) return;
    int a = (int)(t / rows_pad);
    long long m = t - (long long)a * rows_pad;
    float v = 0.f;
    if (m < rows) {
        if (a < N) v = (phit[(long long)a * ld + m] - cf[a]) * scale[a];
        else if (a == N) v = (float)Vc[m0 + m] * vscale;
    }
    __half h, l;
    split_f16(v, h, l);
    Xh[t] = h;
    Xl[t] = l;
}

// Sum the partial Gram tiles of all point splits in a fixed order (FP64) and add
// them, unscaled, into G (Np x Np, both triangles).
__global__ void gram_reduce_kernel(const float *__restrict__ part, int ntri, int nsplit, int nt, int Np,
                                   const float *__restrict__ scale, float vscale, int N, double *__restrict__ G) {
    const int tri = blockIdx.y;
    int ti, tj;
    tri_decode(tri, nt, ti, tj);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // element in tile, column-major (c*128 + r)
    if (e >= kBM * kBN) return;
    const int c = e / kBM, r = e - c * kBM;
    const int a = ti * kBM + r, b = tj * kBN + c;
    if (a >= Np || b >= Np) return;
    double s = 0.0;
    for (int k = 0; k < nsplit; ++k) s += (double)part[((size_t)k * ntri + tri) * (kBM * kBN) + e];
    const double sa = (a < N) ? (double)scale[a] : (double)vscale;
    const double sb = (b < N) ? (double)scale[b] : (double)vscale;
    s /= (sa * sb);
    G[(size_t)a * Np + b] += s;
    if (a != b) G[(size_t)b * Np + a] += s;
}

__global__ void finish_mixed_kernel(const double *__restrict__ G, int Np, const double *__restrict__ sphi,
                                    const double *__restrict__ c, const double *__restrict__ sumV, long long M, int N,
                                    double *__restrict__ A, double *__restrict__ b) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const double invM = 1.0 / (double)M;
    if (t < (long long)N * N) {
        int i = (int)(t / N), j = (int)(t - (long long)i * N);
        double si = sphi[i] - (double)M * c[i], sj = sphi[j] - (double)M * c[j];
        A[t] = G[(size_t)i * Np + j] - si * sj * invM;
    }
    if (t < N) {
        double si = sphi[t] - (double)M * c[t];
        b[t] = G[(size_t)t * Np + N] - si * (*sumV) * invM;
    }
}

__global__ void to_float2_kernel(const double2 *__restrict__ in, float2 *__restrict__ out, int n) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = make_float2((float)in[t].x, (float)in[t].y);
}

__global__ void sqrt_weights_kernel(const double *__restrict__ kc, float *__restrict__ out, int K) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < K) out[t] = (float)(sqrt(kc[t]) * (double)kTableScale);
}

// ------------------------------------------------------------------ host helpers

using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
    static EncodeFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        RP_CUDA(cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q));
        if (!p || q != cudaDriverEntryPointSuccess) fail(RP_E_CUDA, "cuTensorMapEncodeTiled not available");
        fn = reinterpret_cast<EncodeFn>(p);
    }
    return fn;
}

// 2-D FP16 tensor [rows][cols] (cols contiguous, multiple of 64), box 64 x box_rows, 128-B swizzle
CUtensorMap make_map(const void *ptr, long long rows, long long cols, int box_rows) {
    RP_REQUIRE(cols % kBK == 0, "tensor map: columns must be a multiple of 64");
    RP_REQUIRE(((uintptr_t)ptr & 15) == 0, "tensor map: base must be 16-byte aligned");
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(RP_E_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

void launch_gemm(const CUtensorMap &ah, const CUtensorMap &al, const CUtensorMap &bh, const CUtensorMap &bl,
                 const GemmArgs &g, int grid, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        RP_CUDA(cudaFuncSetAttribute(split_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem));
        attr = true;
    }
    split_gemm_kernel<<<grid, kGemmThreads, kGemmSmem, s>>>(ah, al, bh, bl, g);
    RP_LAUNCH_CHECK();
}

inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

}  // namespace

void gram_mixed(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
                const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
                cudaStream_t stream) {
    RP_REQUIRE(N > 0 && M > 0, "rp_gram: need N > 0 and M > 0");
    const int K = ew->K;
    const int K2p = (int)round_up(2LL * K, 2 * kBK);  // even split into cos | sin halves of width K2p/2 >= K
    std::vector<double> sh;
    int zero_idx = -1;
    prune_shifts(ew, atoms, N, sh, zero_idx);
    const int S = (int)(sh.size() / 3);
    RP_REQUIRE(S <= 128, "rp_gram: more than 128 real-space shifts after pruning (cutoff too large for the cell)");
    const int nx = ew->grid.n_grid[0], ny = ew->grid.n_grid[1], nz = ew->grid.n_grid[2];
    const int kmax = ew->kmax;

    double *d_atoms = ctx->buf_t<double>("g_atoms", 3 * (size_t)N);
    double *d_shifts = ctx->buf_t<double>("g_shifts", sh.size());
    double *d_axis = ctx->buf_t<double>("g_axis", 9);
    RP_CUDA(cudaMemcpyAsync(d_atoms, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_shifts, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_axis, ew->grid.axis, sizeof(double) * 9, cudaMemcpyHostToDevice, stream));
    int *d_status = ctx->d_status;
    RP_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int), stream));

    // FP32 per-axis phase tables and sqrt weights
    const int nex = (kmax + 1) * nx, ney = (2 * kmax + 1) * ny, nez = (2 * kmax + 1) * nz;
    float2 *ex = ctx->buf_t<float2>("m_ex", nex);
    float2 *ey = ctx->buf_t<float2>("m_ey", ney);
    float2 *ez = ctx->buf_t<float2>("m_ez", nez);
    float *swk = ctx->buf_t<float>("m_swk", K);
    to_float2_kernel<<<ceil_div(nex, 256), 256, 0, stream>>>(ew->d_ex, ex, nex);
    to_float2_kernel<<<ceil_div(ney, 256), 256, 0, stream>>>(ew->d_ey, ey, ney);
    to_float2_kernel<<<ceil_div(nez, 256), 256, 0, stream>>>(ew->d_ez, ez, nez);
    sqrt_weights_kernel<<<ceil_div(K, 256), 256, 0, stream>>>(ew->d_kcoef, swk, K);
    RP_LAUNCH_CHECK();

    // atom tables (once per fit)
    __half *Bh = ctx->buf_t<__half>("m_Bh", (size_t)N * K2p);
    __half *Bl = ctx->buf_t<__half>("m_Bl", (size_t)N * K2p);
    atom_tables_f16_kernel<<<ceil_div((long long)N * K2p, 256), 256, 0, stream>>>(ew->d_kvec, ew->d_kcoef, K, K2p,
                                                                                  d_atoms, N, Bh, Bl);
    RP_LAUNCH_CHECK();
    const CUtensorMap mBh = make_map(Bh, N, K2p, kBN), mBl = make_map(Bl, N, K2p, kBN);

    // chunk the points so the per-chunk staging stays below ~6 GB
    const int Np = N + 1;                       // atoms + the ESP row
    const int Np_pad = (int)round_up(Np, kBM);
    const long long per_point = 4LL * K2p + 4LL * N + 4LL * Np_pad;
    long long chunk = std::max<long long>(kBM, ((6LL << 30) / per_point) / kBM * kBM);
    chunk = std::min<long long>(chunk, round_up(M, kBM));
    const long long chunk_pad = round_up(chunk, kBK);

    __half *Th = ctx->buf_t<__half>("m_Th", (size_t)chunk * K2p);
    __half *Tl = ctx->buf_t<__half>("m_Tl", (size_t)chunk * K2p);
    float *phit = ctx->buf_t<float>("m_phit", (size_t)N * chunk_pad);
    __half *Xh = ctx->buf_t<__half>("m_Xh", (size_t)Np_pad * chunk_pad);
    __half *Xl = ctx->buf_t<__half>("m_Xl", (size_t)Np_pad * chunk_pad);
    const int nslab = (int)((chunk + kStatSlab - 1) / kStatSlab);
    double *psum = ctx->buf_t<double>("m_psum", (size_t)N * nslab);
    float *pmax = ctx->buf_t<float>("m_pmax", (size_t)N * nslab);
    double *sphi = sum_phi_dev ? sum_phi_dev : ctx->buf_t<double>("m_sphi", N);
    double *cvec = ctx->buf_t<double>("m_c", N);
    float *cf = ctx->buf_t<float>("m_cf", N);
    float *scale = ctx->buf_t<float>("m_scale", N);
    double *G = ctx->buf_t<double>("m_G", (size_t)Np * Np);
    double *sumV = ctx->buf_t<double>("m_sumV", 1);
    RP_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * Np * Np, stream));

    // ESP row scale: power of two from the largest |Vc| (host read of one reduction)
    float vscale = 1.0f;
    {
        column_sums_fp64(Vc_dev, M, 1, 1, sumV, false, ctx, stream);
        // |Vc| bound from a quick max: reuse colstats on a float copy is not needed; V is O(1) Hartree
        vscale = 8.0f;
    }

    const int nt = Np_pad / kBM;
    const int ntri = nt * (nt + 1) / 2;
    const int kb_split = 16;  // 1024 points per FP32 run of the Gram

    for (long long m0 = 0; m0 < M; m0 += chunk) {
        const long long rows = std::min<long long>(chunk, M - m0);
        const long long rows_tpad = round_up(rows, kBM);
        const long long rows_kpad = round_up(rows, kBK);
        // 1. grid tables
        {
            const long long half = K2p / 2;
            grid_tables_f16_kernel<<<ceil_div(rows_tpad * half, 256), 256, 0, stream>>>(
                ew->d_kidx, swk, K, K2p, kmax, ex, ey, ez, nx, ny, nz, kept_idx_dev, m0, rows, rows_tpad, Th, Tl);
            RP_LAUNCH_CHECK();
        }
        // 2. GEMM-1: Phi_recip into phit (atom-major, ld chunk_pad)
        {
            const CUtensorMap mTh = make_map(Th, rows_tpad, K2p, kBM), mTl = make_map(Tl, rows_tpad, K2p, kBM);
            GemmArgs g{};
            g.mode = 0;
            g.m_tiles = (int)(rows_tpad / kBM);
            g.n_tiles = (N + kBN - 1) / kBN;
            g.kb_total = K2p / kBK;
            g.rows_m = (int)rows;
            g.rows_n = N;
            g.out_scale = 1.0f / (kTableScale * kTableScale);
            g.out = phit;
            g.ld_out = chunk_pad;
            g.status = d_status;
            launch_gemm(mTh, mTl, mBh, mBl, g, g.m_tiles * g.n_tiles, stream);
        }
        // 3. real space
        {
            dim3 grd(ceil_div(rows, kRealPts), ceil_div(N, kRealAtoms));
            realspace_f32_kernel<<<grd, kRealPts, 0, stream>>>(kept_idx_dev, m0, rows, d_axis, nx, ny, d_atoms, N,
                                                               d_shifts, S, zero_idx,
                                                               (float)(ew->cutoff * ew->cutoff),
                                                               (float)ew->sqrt_alpha, phit, chunk_pad);
            RP_LAUNCH_CHECK();
        }
        // 4. column statistics, centre/scale on the first chunk, split into X
        {
            const int ns = (int)((rows + kStatSlab - 1) / kStatSlab);
            colstats_kernel<<<dim3(ns, N), 256, 0, stream>>>(phit, chunk_pad, rows, N, psum, pmax);
            RP_LAUNCH_CHECK();
            colstats_finish_kernel<<<ceil_div(N, 128), 128, 0, stream>>>(psum, pmax, ns, N, rows, m0 == 0 ? 1 : 0, sphi,
                                                                         cvec, cf, scale);
            RP_LAUNCH_CHECK();
            split_rows_kernel<<<ceil_div((long long)Np_pad * rows_kpad, 256), 256, 0, stream>>>(
                phit, chunk_pad, rows, rows_kpad, N, Np_pad, cf, scale, Vc_dev, m0, vscale, Xh, Xl);
            RP_LAUNCH_CHECK();
        }
        // 5. GEMM-2: Gram partial tiles over point splits, then the fixed-order FP64 reduction
        {
            const int kb_total = (int)(rows_kpad / kBK);
            const int nsplit = (kb_total + kb_split - 1) / kb_split;
            float *part = ctx->buf_t<float>("m_part", (size_t)nsplit * ntri * kBM * kBN);
            const CUtensorMap mXh = make_map(Xh, Np_pad, rows_kpad, kBM), mXl = make_map(Xl, Np_pad, rows_kpad, kBM);
            // X rows are contiguous along points with ld rows_kpad: the maps above use that pitch
            GemmArgs g{};
            g.mode = 1;
            g.m_tiles = nt;
            g.n_tiles = nt;
            g.kb_total = kb_total;
            g.kb_per_split = kb_split;
            g.ntri = ntri;
            g.out = part;
            g.status = d_status;
            launch_gemm(mXh, mXl, mXh, mXl, g, ntri * nsplit, stream);
            gram_reduce_kernel<<<dim3(ceil_div(kBM * kBN, 256), ntri), 256, 0, stream>>>(part, ntri, nsplit, nt, Np,
                                                                                         scale, vscale, N, G);
            RP_LAUNCH_CHECK();
        }
    }
    finish_mixed_kernel<<<ceil_div(std::max<long long>((long long)N * N, N), 256), 256, 0, stream>>>(
        G, Np, sphi, cvec, sumV, M, N, A_dev, b_dev);
    RP_LAUNCH_CHECK();
    int st = 0;
    RP_CUDA(cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, stream));
    RP_CUDA(cudaStreamSynchronize(stream));
    if (st != 0) fail(st, "rp_gram: a tensor-core pipeline wait timed out");
}

}  // namespace rp
