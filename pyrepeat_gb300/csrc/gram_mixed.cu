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
#include <cstdlib>

#include "common.cuh"
#include "tc.cuh"

namespace rp {
namespace {

constexpr int kBM = 128;       // tile rows (TMEM lanes)
constexpr int kBN = 128;       // tile columns
constexpr int kBK = 64;        // K elements per stage (128 B of FP16 = one swizzle row)
constexpr int kTileBytes = kBM * kBK * 2;  // 16 KB per operand tile
constexpr float kTableScale = 1024.0f;     // 2^10 on each table side

// ---- GEMM-1 (k-contraction): FP16 hi+lo operands, 3 products, 4 TMEM accumulators
// Stage kb accumulates into accumulator kb % 4, so each FP32 accumulator sees a
// quarter of the additions (the tensor core's FP32 accumulation truncates; fewer
// additions per accumulator means less drift).  The epilogue adds the four.
constexpr int kRecStages = 3;
constexpr int kRecAcc = 4;
constexpr int kRecThreads = 192;  // warp 0 TMA, warp 1 MMA + TMEM owner, warps 2-5 epilogue
constexpr int kRecStageBytes = 4 * kTileBytes;
constexpr int kRecSmem = kRecStages * kRecStageBytes + 1024 + 256;

// ---- GEMM-2 (Gram): exact integer products of four 7-bit fixed-point slices
// x = 2^-6 (x0 + 2^-7 x1 + 2^-14 x2 + 2^-21 x3), x_s integers with |x0| <= 32,
// |x1..x3| <= 64 (|x| <= 1/2; 28 bits below the row maximum, because a centred
// column's typical value sits orders of magnitude below its maximum).  All 16
// slice products are kept (the low digits carry full-size rounding noise
// whatever |x| is), grouped by weight g = s+u into seven TMEM accumulators of a
// 128 x 64 tile.  Every product is an integer <= 2^12, one MMA adds <= 2^16, a
// group gets at most 16 MMAs per stage, so kGramFlush = 8 stages stay below 2^24
// and the FP32 sums are exact.  At each flush the epilogue folds the groups into
// one int64 per element (sum_g D_g 2^(7(6-g))), so the Gram carries no rounding
// bias (its diagonal is the most sensitive quantity of the fit).
constexpr int kGN = 64;          // Gram tile columns
constexpr int kGSlices = 4;
constexpr int kGroups = 2 * kGSlices - 1;
constexpr int kGramStages = 2;
constexpr int kGramFlush = 8;
constexpr int kGramEpiWarps = 8;
constexpr int kGramThreads = 64 + 32 * kGramEpiWarps;  // 320
constexpr int kBTileBytes = kGN * kBK * 2;             // 8 KB
constexpr int kGramStageBytes = kGSlices * kTileBytes + kGSlices * kBTileBytes;
constexpr int kGramSmem = kGramStages * kGramStageBytes + 1024 + 256;

struct RecArgs {
    int m_tiles, kb_total, rows_m, rows_n;
    double out_scale;
    double *out;
    long long ld_out;
    int *status;
};

struct GramArgs {
    int nt, ntri, kb_total, kb_per_split, flush;  // flush: stages per exact FP32 run (<= kGramFlush)
    double *out;  // partial tiles [split*ntri + tri][col][row], FP64 (exact integers)
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

__device__ __forceinline__ uint8_t *align1024(uint8_t *raw) {
    const uint32_t s = tc::smem_u32(raw);
    return raw + (((s + 1023u) & ~1023u) - s);
}

__global__ void __launch_bounds__(kRecThreads, 1) recip_gemm_kernel(const __grid_constant__ CUtensorMap tmAh,
                                                                      const __grid_constant__ CUtensorMap tmAl,
                                                                      const __grid_constant__ CUtensorMap tmBh,
                                                                      const __grid_constant__ CUtensorMap tmBl,
                                                                      RecArgs g) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = align1024(smem_raw);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kRecStages * kRecStageBytes);
    uint64_t *empty = full + kRecStages;
    uint64_t *accb = empty + kRecStages;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(accb + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a_row0 = (blockIdx.x % g.m_tiles) * kBM, b_row0 = (blockIdx.x / g.m_tiles) * kBN;
    const int nkb = g.kb_total;  // >= 1

    if (threadIdx.x == 0) {
        for (int s = 0; s < kRecStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accb, 1);
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_holder, kRecAcc * kBN);
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
            const int s = kb % kRecStages, u = kb / kRecStages;
            if (u > 0 && !tc::mbar_wait(&empty[s], (u - 1) & 1, g.status)) break;
            uint8_t *st = smem + s * kRecStageBytes;
            tc::mbar_arrive_expect_tx(&full[s], kRecStageBytes);
            const int x = kb * kBK;
            tc::tma_load_2d(st, &tmAh, x, a_row0, &full[s]);
            tc::tma_load_2d(st + kTileBytes, &tmAl, x, a_row0, &full[s]);
            tc::tma_load_2d(st + 2 * kTileBytes, &tmBh, x, b_row0, &full[s]);
            tc::tma_load_2d(st + 3 * kTileBytes, &tmBl, x, b_row0, &full[s]);
            issued = kb + 1;
        }
        if (*reinterpret_cast<volatile int *>(g.status) != 0)
            for (int kb = max(0, issued - kRecStages); kb < issued; ++kb)
                tc::mbar_wait(&full[kb % kRecStages], (kb / kRecStages) & 1, nullptr);
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = tc::idesc_f16_f32(kBM, kBN);
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kRecStages, u = kb / kRecStages;
            if (!tc::mbar_wait(&full[s], u & 1, g.status)) break;
            tc::fence_after_sync();
            const uint32_t st = tc::smem_u32(smem + s * kRecStageBytes);
            const uint64_t ah = tc::sdesc_k_sw128(st), al = tc::sdesc_k_sw128(st + kTileBytes);
            const uint64_t bh = tc::sdesc_k_sw128(st + 2 * kTileBytes), bl = tc::sdesc_k_sw128(st + 3 * kTileBytes);
            const uint32_t d = tmem + (uint32_t)((kb % kRecAcc) * kBN);
            const uint32_t first = (kb < kRecAcc) ? 1u : 0u;  // first use of this accumulator
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const uint64_t o = (uint64_t)(kk * 2);  // 32 B per K=16 step, in 16-B units
                tc::umma_f16(d, ah + o, bh + o, idesc, (first && kk == 0) ? 0u : 1u);
                tc::umma_f16(d, ah + o, bl + o, idesc, 1u);
                tc::umma_f16(d, al + o, bh + o, idesc, 1u);
            }
            tc::umma_commit(&empty[s]);
        }
        tc::umma_commit(accb);
    } else if (warp >= 2) {
        if (tc::mbar_wait(accb, 0, g.status) && *reinterpret_cast<volatile int *>(g.status) == 0) {
            tc::fence_after_sync();
            const int lane_base = (warp & 3) * 32;
            const int m = a_row0 + lane_base + lane;
            const int nacc = min(nkb, kRecAcc);
#pragma unroll 1
            for (int c = 0; c < kBN / 32; ++c) {
                double v[32];
                {
                    float w[32];
                    tc::tmem_ld_32x32(tmem + ((uint32_t)lane_base << 16) + (uint32_t)(c * 32), w);
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[i] = (double)w[i];
                }
                for (int q = 1; q < nacc; ++q) {
                    float w[32];
                    tc::tmem_ld_32x32(tmem + ((uint32_t)lane_base << 16) + (uint32_t)(q * kBN + c * 32), w);
#pragma unroll
                    for (int i = 0; i < 32; ++i) v[i] += (double)w[i];
                }
                if (m < g.rows_m) {
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const int n = b_row0 + c * 32 + i;
                        if (n < g.rows_n) g.out[(long long)n * g.ld_out + m] = v[i] * g.out_scale;
                    }
                }
            }
        }
    }
    if (warp == 1 && lane == 0) tc::mbar_wait(accb, 0, nullptr);  // last MMAs landed before TMEM is freed
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1) tc::tmem_dealloc(tmem, kRecAcc * kBN);
}

// Gram tile t -> (ti, tj): rows [128 ti, +128), columns [64 tj, +64), tj >= 2 ti.
__device__ __forceinline__ void gram_tile_decode(int t, int nt, int &ti, int &tj) {
    ti = 0;
    int len = 2 * nt;
    while (t >= len) {
        t -= len;
        ++ti;
        len -= 2;
    }
    tj = 2 * ti + t;
}

__global__ void __launch_bounds__(kGramThreads, 1) gram_exact_kernel(
    const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
    const __grid_constant__ CUtensorMap tm2, const __grid_constant__ CUtensorMap tm3,
    const __grid_constant__ CUtensorMap tb0, const __grid_constant__ CUtensorMap tb1,
    const __grid_constant__ CUtensorMap tb2, const __grid_constant__ CUtensorMap tb3, GramArgs g) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = align1024(smem_raw);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kGramStages * kGramStageBytes);
    uint64_t *empty = full + kGramStages;
    uint64_t *accf = empty + kGramStages;  // accumulators ready for the epilogue
    uint64_t *acce = accf + 1;             // epilogue done reading them
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(acce + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x % g.ntri, split = blockIdx.x / g.ntri;
    int ti, tj;
    gram_tile_decode(tile, g.nt, ti, tj);
    const bool inblock = (tj < 2 * ti + 2);       // columns inside the row block: B rows are part of A's tile
    const uint32_t b_in_a = (uint32_t)(tj - 2 * ti) * (kGN * 128);  // byte offset of B's rows inside A's tile
    const int a_row0 = ti * kBM, b_row0 = tj * kGN;
    const int kb0 = split * g.kb_per_split, kb1 = min(kb0 + g.kb_per_split, g.kb_total);
    const int nkb = kb1 - kb0;  // >= 1
    const int nflush = (nkb + g.flush - 1) / g.flush;
    const uint32_t stage_tx = inblock ? kGSlices * kTileBytes : kGSlices * (kTileBytes + kBTileBytes);
    const CUtensorMap *ta[kGSlices] = {&tm0, &tm1, &tm2, &tm3};
    const CUtensorMap *tb[kGSlices] = {&tb0, &tb1, &tb2, &tb3};

    if (threadIdx.x == 0) {
        for (int s = 0; s < kGramStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accf, 1);
        tc::mbar_init(acce, 32 * kGramEpiWarps);
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_holder, 512);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0 && lane == 0) {
        int issued = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kGramStages, u = kb / kGramStages;
            if (u > 0 && !tc::mbar_wait(&empty[s], (u - 1) & 1, g.status)) break;
            uint8_t *st = smem + s * kGramStageBytes;
            tc::mbar_arrive_expect_tx(&full[s], stage_tx);
            const int x = (kb0 + kb) * kBK;
#pragma unroll
            for (int q = 0; q < kGSlices; ++q) {
                tc::tma_load_2d(st + q * kTileBytes, ta[q], x, a_row0, &full[s]);
                if (!inblock)
                    tc::tma_load_2d(st + kGSlices * kTileBytes + q * kBTileBytes, tb[q], x, b_row0, &full[s]);
            }
            issued = kb + 1;
        }
        if (*reinterpret_cast<volatile int *>(g.status) != 0)
            for (int kb = max(0, issued - kGramStages); kb < issued; ++kb)
                tc::mbar_wait(&full[kb % kGramStages], (kb / kGramStages) & 1, nullptr);
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = tc::idesc_f16_f32(kBM, kGN);
        uint32_t d[kGroups];  // group accumulators, 64 TMEM columns each
#pragma unroll
        for (int q = 0; q < kGroups; ++q) d[q] = tmem + (uint32_t)(q * kGN);
        bool ok = true;
        for (int f = 0; f < nflush && ok; ++f) {
            if (f > 0 && !tc::mbar_wait(acce, (f - 1) & 1, g.status)) break;  // epilogue drained the sums
            tc::fence_after_sync();
            const int kbf0 = f * g.flush, kbf1 = min(kbf0 + g.flush, nkb);
            for (int kb = kbf0; kb < kbf1; ++kb) {
                const int s = kb % kGramStages, u = kb / kGramStages;
                if (!tc::mbar_wait(&full[s], u & 1, g.status)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t st = tc::smem_u32(smem + s * kGramStageBytes);
                uint64_t x[kGSlices], y[kGSlices];
#pragma unroll
                for (int q = 0; q < kGSlices; ++q) {
                    x[q] = tc::sdesc_k_sw128(st + q * kTileBytes);
                    y[q] = inblock ? tc::sdesc_k_sw128(st + q * kTileBytes + b_in_a)
                                   : tc::sdesc_k_sw128(st + kGSlices * kTileBytes + q * kBTileBytes);
                }
#pragma unroll
                for (int kk = 0; kk < kBK / 16; ++kk) {
                    const uint64_t o = (uint64_t)(kk * 2);
                    bool started[kGroups] = {false, false, false, false, false, false, false};
#pragma unroll
                    for (int a = 0; a < kGSlices; ++a)
#pragma unroll
                        for (int b = 0; b < kGSlices; ++b) {
                            const int grp = a + b;
                            const uint32_t acc = (kb == kbf0 && kk == 0 && !started[grp]) ? 0u : 1u;
                            started[grp] = true;
                            tc::umma_f16(d[grp], x[a] + o, y[b] + o, idesc, acc);
                        }
                }
                tc::umma_commit(&empty[s]);
            }
            tc::umma_commit(accf);
        }
    } else if (warp >= 2) {
        const int ew = warp - 2;
        const int lane_base = (warp & 3) * 32;
        const int col0 = (ew >> 2) * 32;  // this warp's 32 columns of the 64
        long long acc[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[i] = 0;
        bool ok = true;
        for (int f = 0; f < nflush; ++f) {
            if (!tc::mbar_wait(accf, f & 1, g.status)) {
                ok = false;
                break;
            }
            tc::fence_after_sync();
            const uint32_t base = tmem + ((uint32_t)lane_base << 16) + (uint32_t)col0;
#pragma unroll
            for (int q = 0; q < kGroups; ++q) {
                float v[32];
                tc::tmem_ld_32x32(base + (uint32_t)(q * kGN), v);
                const int sh = 7 * (kGroups - 1 - q);
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[i] += (long long)__float2int_rn(v[i]) << sh;
            }
            tc::fence_before_sync();
            tc::mbar_arrive(acce);
        }
        if (ok && *reinterpret_cast<volatile int *>(g.status) == 0) {
            double *o = g.out + (long long)blockIdx.x * (kBM * kGN);
            const int r = lane_base + lane;
#pragma unroll
            for (int i = 0; i < 32; ++i) o[(col0 + i) * kBM + r] = (double)acc[i];
        }
    }
    if (warp == 1 && lane == 0) tc::mbar_wait(accf, (nflush - 1) & 1, nullptr);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1) tc::tmem_dealloc(tmem, 512);
}

// ---- GEMM-1b (heaviest k columns): exact products of four 7-bit fixed-point
// slices of T (points) and B (atoms), 16 products in 7 weight groups (TMEM 448
// columns of a 128 x 64 tile).  A group gets at most 16 MMAs per stage, each
// adding <= 2^16, and the block has <= kTopMaxStages stages, so every FP32 sum is
// an exact integer; the epilogue folds the groups into an int64 and adds
// 2^-54 * I * out_scale to Phi_t (FP64).
constexpr int kTopSlices = 4;
constexpr int kTopGroups = 7;
constexpr int kTopMaxStages = 8;
constexpr int kTopStages = 2;
constexpr int kTopThreads = 64 + 32 * 8;
constexpr int kTopStageBytes = kTopSlices * kTileBytes + kTopSlices * kBTileBytes;
constexpr int kTopSmem = kTopStages * kTopStageBytes + 1024 + 256;

struct TopArgs {
    int m_tiles, kb_total, rows_m, rows_n;
    double out_scale;
    double *out;
    long long ld_out;
    int *status;
};

__global__ void __launch_bounds__(kTopThreads, 1) recip_top_kernel(
    const __grid_constant__ CUtensorMap ta0, const __grid_constant__ CUtensorMap ta1,
    const __grid_constant__ CUtensorMap ta2, const __grid_constant__ CUtensorMap ta3,
    const __grid_constant__ CUtensorMap tb0, const __grid_constant__ CUtensorMap tb1,
    const __grid_constant__ CUtensorMap tb2, const __grid_constant__ CUtensorMap tb3, TopArgs g) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = align1024(smem_raw);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kTopStages * kTopStageBytes);
    uint64_t *empty = full + kTopStages;
    uint64_t *accf = empty + kTopStages;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(accf + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int a_row0 = (blockIdx.x % g.m_tiles) * kBM, b_row0 = (blockIdx.x / g.m_tiles) * kGN;
    const int nkb = g.kb_total;  // 1..kTopMaxStages
    const CUtensorMap *ta[4] = {&ta0, &ta1, &ta2, &ta3};
    const CUtensorMap *tb[4] = {&tb0, &tb1, &tb2, &tb3};

    if (threadIdx.x == 0) {
        for (int s = 0; s < kTopStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accf, 1);
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_holder, 512);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0 && lane == 0) {
        int issued = 0;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kTopStages, u = kb / kTopStages;
            if (u > 0 && !tc::mbar_wait(&empty[s], (u - 1) & 1, g.status)) break;
            uint8_t *st = smem + s * kTopStageBytes;
            tc::mbar_arrive_expect_tx(&full[s], kTopStageBytes);
            const int x = kb * kBK;
#pragma unroll
            for (int q = 0; q < kTopSlices; ++q) {
                tc::tma_load_2d(st + q * kTileBytes, ta[q], x, a_row0, &full[s]);
                tc::tma_load_2d(st + kTopSlices * kTileBytes + q * kBTileBytes, tb[q], x, b_row0, &full[s]);
            }
            issued = kb + 1;
        }
        if (*reinterpret_cast<volatile int *>(g.status) != 0)
            for (int kb = max(0, issued - kTopStages); kb < issued; ++kb)
                tc::mbar_wait(&full[kb % kTopStages], (kb / kTopStages) & 1, nullptr);
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = tc::idesc_f16_f32(kBM, kGN);
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kTopStages, u = kb / kTopStages;
            if (!tc::mbar_wait(&full[s], u & 1, g.status)) break;
            tc::fence_after_sync();
            const uint32_t st = tc::smem_u32(smem + s * kTopStageBytes);
            uint64_t x[kTopSlices], y[kTopSlices];
#pragma unroll
            for (int q = 0; q < kTopSlices; ++q) {
                x[q] = tc::sdesc_k_sw128(st + q * kTileBytes);
                y[q] = tc::sdesc_k_sw128(st + kTopSlices * kTileBytes + q * kBTileBytes);
            }
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const uint64_t o = (uint64_t)(kk * 2);
                bool started[kTopGroups] = {false, false, false, false, false, false, false};
#pragma unroll
                for (int a = 0; a < kTopSlices; ++a)
#pragma unroll
                    for (int b = 0; b < kTopSlices; ++b) {
                        const int grp = a + b;
                        const uint32_t acc = (kb == 0 && kk == 0 && !started[grp]) ? 0u : 1u;
                        started[grp] = true;
                        tc::umma_f16(tmem + (uint32_t)(grp * kGN), x[a] + o, y[b] + o, idesc, acc);
                    }
            }
            tc::umma_commit(&empty[s]);
        }
        tc::umma_commit(accf);
    } else if (warp >= 2) {
        const int ew = warp - 2;
        const int lane_base = (warp & 3) * 32;
        const int col0 = (ew >> 2) * 32;
        if (tc::mbar_wait(accf, 0, g.status) && *reinterpret_cast<volatile int *>(g.status) == 0) {
            tc::fence_after_sync();
            long long acc[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) acc[i] = 0;
            const uint32_t base = tmem + ((uint32_t)lane_base << 16) + (uint32_t)col0;
#pragma unroll
            for (int q = 0; q < kTopGroups; ++q) {
                float v[32];
                tc::tmem_ld_32x32(base + (uint32_t)(q * kGN), v);
                const int sh = 7 * (kTopGroups - 1 - q);
#pragma unroll
                for (int i = 0; i < 32; ++i) acc[i] += (long long)__float2int_rn(v[i]) << sh;
            }
            const int m = a_row0 + lane_base + lane;
            if (m < g.rows_m) {
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int n = b_row0 + col0 + i;
                    if (n < g.rows_n) g.out[(long long)n * g.ld_out + m] += ldexp((double)acc[i], -54) * g.out_scale;
                }
            }
        }
    }
    if (warp == 1 && lane == 0) tc::mbar_wait(accf, 0, nullptr);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1) tc::tmem_dealloc(tmem, 512);
}

// ------------------------------------------------------------------ tables

__device__ __forceinline__ void split_f16(float x, __half &hi, __half &lo) {
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}

// k columns: the sorted (ascending kcoef) k-set is split into a "float" block
// (all but the ntop heaviest k) and a "top" block (the ntop heaviest).  Within a
// block, sorted k index q occupies columns cos, sin at (width - 2*count + 2*(q-q0)),
// so the block ends with its heaviest k and starts with zero padding.
struct KBlock {
    int q0, count, width;  // sorted k range [q0, q0+count), width columns (multiple of 64)
};

__device__ __forceinline__ int kcol_to_q(const KBlock &b, int c, int &is_sin) {
    const int off = c - (b.width - 2 * b.count);
    if (off < 0) return -1;
    is_sin = off & 1;
    return b.q0 + (off >> 1);
}

// FP16 hi + lo atom table of the float block
__global__ void atom_tables_f16_kernel(const double *__restrict__ kvec, const double *__restrict__ kcoef, KBlock blk,
                                       const double *__restrict__ atoms, int N, __half *__restrict__ Bh,
                                       __half *__restrict__ Bl) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * blk.width) return;
    int a = (int)(t / blk.width), c = (int)(t - (long long)a * blk.width);
    int is_sin = 0;
    int q = kcol_to_q(blk, c, is_sin);
    float val = 0.0f;
    if (q >= 0) {
        double kr = (atoms[3 * a] * kvec[3 * q] + atoms[3 * a + 1] * kvec[3 * q + 1]) + atoms[3 * a + 2] * kvec[3 * q + 2];
        double sn, cs;
        sincos(kr, &sn, &cs);
        val = (float)(sqrt(kcoef[q]) * (double)kTableScale * (is_sin ? sn : cs));
    }
    __half h, l;
    split_f16(val, h, l);
    Bh[t] = h;
    Bl[t] = l;
}

// FP16 hi + lo grid table of the float block (FP32 phase products)
__global__ void grid_tables_f16_kernel(const int *__restrict__ kidx, const float *__restrict__ swk, KBlock blk,
                                       int kmax, const float2 *__restrict__ ex, const float2 *__restrict__ ey,
                                       const float2 *__restrict__ ez, int nx, int ny, int nz,
                                       const int32_t *__restrict__ kept, long long m0, long long rows,
                                       long long rows_pad, __half *__restrict__ Th, __half *__restrict__ Tl) {
    // one thread per (point, column pair)
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int pairs = blk.width / 2;
    if (t >= rows_pad * pairs) return;
    long long m = t / pairs;
    int cp = (int)(t - m * pairs);
    int is_sin = 0;
    int q = kcol_to_q(blk, 2 * cp, is_sin);
    float re = 0.f, im = 0.f;
    if (m < rows && q >= 0) {
        int f = kept[m0 + m];
        int layer = nx * ny;
        int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
        int n1 = kidx[3 * q], n2 = kidx[3 * q + 1], n3 = kidx[3 * q + 2];
        float2 a = ex[n1 * nx + i], b = ey[(n2 + kmax) * ny + j], c = ez[(n3 + kmax) * nz + l];
        float r1 = a.x * b.x - a.y * b.y, i1 = a.x * b.y + a.y * b.x;
        float sw = swk[q];
        re = (r1 * c.x - i1 * c.y) * sw;
        im = (r1 * c.y + i1 * c.x) * sw;
    }
    __half h, l;
    const long long base = m * (long long)blk.width + 2 * cp;
    split_f16(re, h, l);
    Th[base] = h;
    Tl[base] = l;
    split_f16(im, h, l);
    Th[base + 1] = h;
    Tl[base + 1] = l;
}

// Four 7-bit fixed-point slices of x (|x| <= 1): x = 2^-6 (s0 + 2^-7 s1 + 2^-14 s2 + 2^-21 s3)
// up to 2^-28.  One FP64 multiply and one rounding conversion give the 27-bit
// integer round(x 2^27); the signed digits (round-half-up per digit, so
// |s0| <= 64, |s1..s3| <= 64) then come from integer shifts.
__device__ __forceinline__ void slice4(double x, __half *o0, __half *o1, __half *o2, __half *o3, long long idx) {
    long long v = __double2ll_rn(x * 134217728.0);  // 2^27
    long long s0 = (v + (1LL << 20)) >> 21;
    long long r = v - (s0 << 21);                   // [-2^20, 2^20)
    long long s1 = (r + (1LL << 13)) >> 14;
    r -= s1 << 14;                                  // [-2^13, 2^13)
    long long s2 = (r + (1LL << 6)) >> 7;
    long long s3 = r - (s2 << 7);                   // [-64, 64)
    o0[idx] = __int2half_rn((int)s0);
    o1[idx] = __int2half_rn((int)s1);
    o2[idx] = __int2half_rn((int)s2);
    o3[idx] = __int2half_rn((int)s3);
}

// Fixed-point slices of the top block, atom side (FP64 values, scaled by sB)
__global__ void atom_tables_top_kernel(const double *__restrict__ kvec, const double *__restrict__ kcoef, KBlock blk,
                                       const double *__restrict__ atoms, int N, double sB, __half *__restrict__ B0,
                                       __half *__restrict__ B1, __half *__restrict__ B2, __half *__restrict__ B3) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * blk.width) return;
    int a = (int)(t / blk.width), c = (int)(t - (long long)a * blk.width);
    int is_sin = 0;
    int q = kcol_to_q(blk, c, is_sin);
    double val = 0.0;
    if (q >= 0) {
        double kr = (atoms[3 * a] * kvec[3 * q] + atoms[3 * a + 1] * kvec[3 * q + 1]) + atoms[3 * a + 2] * kvec[3 * q + 2];
        double sn, cs;
        sincos(kr, &sn, &cs);
        val = sqrt(kcoef[q]) * (double)kTableScale * (is_sin ? sn : cs) * sB;
    }
    slice4(val, B0, B1, B2, B3, t);
}

// Fixed-point slices of the top block, grid side (FP64 phase products, scaled by sT)
__global__ void grid_tables_top_kernel(const int *__restrict__ kidx, const double *__restrict__ wtop, KBlock blk,
                                       int kmax, const double2 *__restrict__ ex, const double2 *__restrict__ ey,
                                       const double2 *__restrict__ ez, int nx, int ny, int nz,
                                       const int32_t *__restrict__ kept, long long m0, long long rows,
                                       long long rows_pad, double sT, __half *__restrict__ T0, __half *__restrict__ T1,
                                       __half *__restrict__ T2, __half *__restrict__ T3) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int pairs = blk.width / 2;
    if (t >= rows_pad * pairs) return;
    long long m = t / pairs;
    int cp = (int)(t - m * pairs);
    int is_sin = 0;
    int q = kcol_to_q(blk, 2 * cp, is_sin);
    double re = 0.0, im = 0.0;
    if (m < rows && q >= 0) {
        int f = kept[m0 + m];
        int layer = nx * ny;
        int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
        int n1 = kidx[3 * q], n2 = kidx[3 * q + 1], n3 = kidx[3 * q + 2];
        double2 a = ex[n1 * nx + i], b = ey[(n2 + kmax) * ny + j], c = ez[(n3 + kmax) * nz + l];
        double r1 = a.x * b.x - a.y * b.y, i1 = a.x * b.y + a.y * b.x;
        double sw = wtop[q - blk.q0];  // sqrt(kcoef) 2^10 sT
        re = (r1 * c.x - i1 * c.y) * sw;
        im = (r1 * c.y + i1 * c.x) * sw;
    }
    const long long base = m * (long long)blk.width + 2 * cp;
    slice4(re, T0, T1, T2, T3, base);
    slice4(im, T0, T1, T2, T3, base + 1);
}

// ------------------------------------------------------------------ real space (FP32)

constexpr int kRealPts = 128;   // points per CTA (one per thread)
constexpr int kRealAtoms = 16;  // atoms per CTA

// Phi_t[a][m] += sum_s erfc(sqrt(alpha) r)/r over images within Rc.  Distances
// are formed in FP32 from double-float image coordinates taken relative to the
// CTA's first point, so no coordinate rounding enters; pairs closer than
// kNearR (where the term is large) are re-evaluated entirely in FP64, the rest
// use FP32 erfcf.  The sum per (point, atom) is kept in FP64.

__global__ void __launch_bounds__(kRealPts) realspace_kernel(
    const int32_t *__restrict__ kept, long long m0, long long rows, const double *__restrict__ axis, int nx, int ny,
    const double *__restrict__ atoms, int N, const double *__restrict__ shifts, int S, int zero_idx, double rc,
    double sa, float near2, double *__restrict__ phit, long long ld) {
    __shared__ float3 img_hi[kRealAtoms * 128];   // S <= 128 images per atom (host checks)
    __shared__ float3 img_lo[kRealAtoms * 128];
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
        double q[3];
        for (int d = 0; d < 3; ++d) q[d] = (p[d] + shifts[3 * s + d]) - origin[d];
        float3 h = make_float3((float)q[0], (float)q[1], (float)q[2]);
        img_hi[a * S + s] = h;
        img_lo[a * S + s] = make_float3((float)(q[0] - h.x), (float)(q[1] - h.y), (float)(q[2] - h.z));
    }
    __syncthreads();
    const long long m = mb + threadIdx.x;
    if (m >= rows) return;
    const int f = kept[m0 + m];
    const int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
    double gabs[3], gd[3];
    for (int d = 0; d < 3; ++d) {
        gabs[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)l * axis[6 + d];
        gd[d] = gabs[d] - origin[d];
    }
    const float gx = (float)gd[0], gy = (float)gd[1], gz = (float)gd[2];
    const float gxl = (float)(gd[0] - gx), gyl = (float)(gd[1] - gy), gzl = (float)(gd[2] - gz);
    const float rc2 = (float)(rc * rc) * 1.0001f, saf = (float)sa;
    for (int a = 0; a < na; ++a) {
        double acc = 0.0;
        float acc32 = 0.f;
        const float3 *ih = img_hi + a * S, *il = img_lo + a * S;
        const double *p = atoms + 3 * (a0 + a);
        for (int s = 0; s < S; ++s) {
            float dx = (gx - ih[s].x) + (gxl - il[s].x), dy = (gy - ih[s].y) + (gyl - il[s].y),
                  dz = (gz - ih[s].z) + (gzl - il[s].z);
            float r2 = dx * dx + dy * dy + dz * dz;
            if (r2 > rc2) continue;
            if (r2 < near2 || fabsf(r2 - (float)(rc * rc)) < 1e-3f * (float)(rc * rc)) {
                double ex = gabs[0] - (p[0] + shifts[3 * s]), ey = gabs[1] - (p[1] + shifts[3 * s + 1]),
                       ez = gabs[2] - (p[2] + shifts[3 * s + 2]);
                double r = sqrt(ex * ex + ey * ey + ez * ez);
                if (r <= rc && (s != zero_idx || r > 1e-10)) acc += erfc(sa * r) / r;
            } else {
                float r = sqrtf(r2);
                if ((double)r <= rc) acc32 += erfcf(saf * r) / r;
            }
        }
        phit[(long long)(a0 + a) * ld + m] += acc + (double)acc32;
    }
}

// ------------------------------------------------------------------ column statistics and the split

// Per-atom sums (FP64) and max |Phi| over a chunk: stage 1 per (atom, slab of points)
constexpr int kStatSlab = 4096;
__global__ void colstats_kernel(const double *__restrict__ phit, long long ld, long long rows, int N,
                                double *__restrict__ psum, float *__restrict__ pmax) {
    const int a = blockIdx.y;
    const long long r0 = (long long)blockIdx.x * kStatSlab;
    const long long r1 = min(r0 + kStatSlab, rows);
    double s = 0.0;
    float mx = 0.f;
    for (long long r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        double v = phit[(long long)a * ld + r];
        s += v;
        mx = fmaxf(mx, (float)fabs(v));
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
        // |Phi - c| <= 2 max|Phi| =: bound in [2^(e-1), 2^e); scale 2^(-e-1) puts |x| below 1/2,
        // so the fixed-point slices stay within |x_s| <= 64 even if a later chunk doubles the range
        float bound = 2.f * mx;
        int e = 0;
        if (bound > 0.f) frexpf(bound, &e);
        scale[a] = ldexpf(1.f, -e - 1);
    }
}

// X rows: a < N: (Phi_t[a][m] - c_a) * scale_a;  a == N: Vc[m] * scale_V;  rest zero.
// Each value x (|x| <= 1) is cut into four 7-bit fixed-point slices
// x = 2^-6 (x0 + 2^-7 x1 + 2^-14 x2 + 2^-21 x3), x_s integers in [-64, 64], exact in FP16.
__global__ void slice_rows_kernel(const double *__restrict__ phit, long long ld, long long rows, long long rows_pad,
                                  int N, int Np_pad, const double *__restrict__ c, const float *__restrict__ scale,
                                  const double *__restrict__ Vc, long long m0, const float *__restrict__ vscale_p,
                                  __half *__restrict__ X0, __half *__restrict__ X1, __half *__restrict__ X2,
                                  __half *__restrict__ X3, int *__restrict__ clamped) {
    const float vscale = *vscale_p;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)Np_pad * rows_pad) return;
    int a = (int)(t / rows_pad);
    long long m = t - (long long)a * rows_pad;
    double v = 0.0;
    if (m < rows) {
        if (a < N) v = (phit[(long long)a * ld + m] - c[a]) * (double)scale[a];
        else if (a == N) v = Vc[m0 + m] * (double)vscale;
    }
    if (fabs(v) > 1.0) {
        atomicAdd(clamped, 1);
        v = fmin(fmax(v, -1.0), 1.0);
    }
    slice4(v, X0, X1, X2, X3, t);
}

// Sum the partial Gram tiles of all point splits in a fixed order (FP64; each
// partial is an exact integer) and add them, unscaled, into G (Np x Np).  Tiles
// inside a 128-row block already hold both (a,b) and (b,a); the others are mirrored.
__global__ void gram_reduce_kernel(const double *__restrict__ part, int ntiles, int nsplit, int nt, int Np,
                                   const float *__restrict__ scale, const float *__restrict__ vscale_p, int N,
                                   double *__restrict__ G) {
    const float vscale = *vscale_p;
    const int tile = blockIdx.y;
    int ti, tj;
    gram_tile_decode(tile, nt, ti, tj);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // element in tile, column-major (c*128 + r)
    if (e >= kBM * kGN) return;
    const int c = e / kBM, r = e - c * kBM;
    const int a = ti * kBM + r, b = tj * kGN + c;
    if (a >= Np || b >= Np) return;
    double s = 0.0;
    for (int k = 0; k < nsplit; ++k) s += part[((size_t)k * ntiles + tile) * (kBM * kGN) + e];
    const double sa = (a < N) ? (double)scale[a] : (double)vscale;
    const double sb = (b < N) ? (double)scale[b] : (double)vscale;
    s = ldexp(s, -54) / (sa * sb);
    G[(size_t)a * Np + b] += s;
    if (tj >= 2 * ti + 2) G[(size_t)b * Np + a] += s;
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

__global__ void __launch_bounds__(1024) absmax_kernel(const double *__restrict__ x, long long n,
                                                     double *__restrict__ out) {
    __shared__ double sm[1024];
    double m = 0.0;
    for (long long i = threadIdx.x; i < n; i += 1024) m = fmax(m, fabs(x[i]));
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int o = 512; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

// ESP row scale 2^(-e-1) with max|Vc| in [2^(e-1), 2^e), so |V * scale| < 1/2
__global__ void vscale_kernel(const double *__restrict__ vmax, float *__restrict__ vscale) {
    int e = 0;
    if (*vmax > 0.0) frexp(*vmax, &e);
    *vscale = ldexpf(1.0f, -e - 1);
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
        RP_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
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

void launch_recip(const CUtensorMap &ah, const CUtensorMap &al, const CUtensorMap &bh, const CUtensorMap &bl,
                  const RecArgs &g, int grid, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        RP_CUDA(cudaFuncSetAttribute(recip_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kRecSmem));
        attr = true;
    }
    recip_gemm_kernel<<<grid, kRecThreads, kRecSmem, s>>>(ah, al, bh, bl, g);
    RP_LAUNCH_CHECK();
}

void launch_gram(const __half *const *X, int Np_pad, long long cols, const GramArgs &g, int grid, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        RP_CUDA(cudaFuncSetAttribute(gram_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGramSmem));
        attr = true;
    }
    CUtensorMap a[kGSlices], b[kGSlices];
    for (int q = 0; q < kGSlices; ++q) {
        a[q] = make_map(X[q], Np_pad, cols, kBM);
        b[q] = make_map(X[q], Np_pad, cols, kGN);
    }
    gram_exact_kernel<<<grid, kGramThreads, kGramSmem, s>>>(a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3], g);
    RP_LAUNCH_CHECK();
}

void launch_top(const __half *const *T, long long rows_pad, const __half *const *B, int N, int width, const TopArgs &g,
                int grid, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        RP_CUDA(cudaFuncSetAttribute(recip_top_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTopSmem));
        attr = true;
    }
    CUtensorMap a[4], b[4];
    for (int q = 0; q < 4; ++q) {
        a[q] = make_map(T[q], rows_pad, width, kBM);
        b[q] = make_map(B[q], N, width, kGN);
    }
    recip_top_kernel<<<grid, kTopThreads, kTopSmem, s>>>(a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3], g);
    RP_LAUNCH_CHECK();
}

inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

}  // namespace

// Pairs closer than this radius (Bohr) get the FP64 real-space term; tunable with
// RP_REAL_FP64_R.  Default 0: with double-float image coordinates the FP32 terms
// keep the fitted charges within ~3e-7 e of the FP64 fit on the synthetic
// workloads, so FP64 is used only to decide images that sit at the cutoff.
float real_near2() {
    static float v = [] {
        const char *e = getenv("RP_REAL_FP64_R");
        double r = e ? atof(e) : 0.0;
        return (float)(r * r);
    }();
    return v;
}

// Split the sorted k-set into the float block and the exact top block: the top
// block takes every k with kcoef >= kTopRel * max kcoef (at least 32, at most
// kTopMaxStages*32 k), so the terms that carry the sum are accumulated exactly.
constexpr double kTopRel = 1e-5;

void plan_kblocks(const rp_ewald *ew, KBlock &fl, KBlock &top) {
    const int K = ew->K;
    double wmax = 0.0;
    for (double w : ew->kcoef) wmax = std::max(wmax, w);
    int heavy = 0;
    for (double w : ew->kcoef) heavy += (w >= kTopRel * wmax) ? 1 : 0;
    int ntop = std::min(K, std::max(32, (int)round_up(heavy, 32)));
    ntop = std::min(ntop, kTopMaxStages * kBK / 2);
    top.q0 = K - ntop;
    top.count = ntop;
    top.width = (int)round_up(2LL * ntop, kBK);
    fl.q0 = 0;
    fl.count = K - ntop;
    fl.width = std::max<int>((int)round_up(2LL * fl.count, kBK), kBK);
}

void gram_mixed(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
                const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
                cudaStream_t stream) {
    RP_REQUIRE(N > 0 && M > 0, "rp_gram: need N > 0 and M > 0");
    const int K = ew->K;
    KBlock fl, top;
    plan_kblocks(ew, fl, top);
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
    int *d_status = ctx->d_status;  // cleared by the caller (rp_gram / the batch driver)

    // FP32 per-axis phase tables and sqrt weights for the float block
    const int nex = (kmax + 1) * nx, ney = (2 * kmax + 1) * ny, nez = (2 * kmax + 1) * nz;
    float2 *ex = ctx->buf_t<float2>("m_ex", nex);
    float2 *ey = ctx->buf_t<float2>("m_ey", ney);
    float2 *ez = ctx->buf_t<float2>("m_ez", nez);
    float *swk = ctx->buf_t<float>("m_swk", K);
    to_float2_kernel<<<ceil_div(nex, 256), 256, 0, stream>>>(ew->d_ex, ex, nex);
    RP_LAUNCH_CHECK();
    to_float2_kernel<<<ceil_div(ney, 256), 256, 0, stream>>>(ew->d_ey, ey, ney);
    RP_LAUNCH_CHECK();
    to_float2_kernel<<<ceil_div(nez, 256), 256, 0, stream>>>(ew->d_ez, ez, nez);
    RP_LAUNCH_CHECK();
    sqrt_weights_kernel<<<ceil_div(K, 256), 256, 0, stream>>>(ew->d_kcoef_s, swk, K);
    RP_LAUNCH_CHECK();

    // table scales of the exact block: |sqrt(w) 2^10 cos| * s <= 1/2
    double wmax = 0.0;
    for (double w : ew->kcoef) wmax = std::max(wmax, w);
    int et = 0;
    std::frexp(std::sqrt(wmax) * (double)kTableScale, &et);
    const double sTop = std::ldexp(1.0, -et - 1);
    double *wtop = ctx->buf_t<double>("m_wtop", (size_t)top.count);
    {
        std::vector<double> kc(ew->kcoef);
        std::sort(kc.begin(), kc.end());  // the device tables use the ascending order
        std::vector<double> w((size_t)top.count);
        for (int q = 0; q < top.count; ++q) w[q] = std::sqrt(kc[top.q0 + q]) * (double)kTableScale * sTop;
        RP_CUDA(cudaMemcpyAsync(wtop, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, stream));
    }

    // atom tables (once per fit)
    __half *Bh = ctx->buf_t<__half>("m_Bh", (size_t)N * fl.width);
    __half *Bl = ctx->buf_t<__half>("m_Bl", (size_t)N * fl.width);
    atom_tables_f16_kernel<<<ceil_div((long long)N * fl.width, 256), 256, 0, stream>>>(ew->d_kvec_s, ew->d_kcoef_s, fl,
                                                                                       d_atoms, N, Bh, Bl);
    RP_LAUNCH_CHECK();
    __half *Bt[4];
    for (int q = 0; q < 4; ++q) Bt[q] = ctx->buf_t<__half>("m_Bt" + std::to_string(q), (size_t)N * top.width);
    atom_tables_top_kernel<<<ceil_div((long long)N * top.width, 256), 256, 0, stream>>>(
        ew->d_kvec_s, ew->d_kcoef_s, top, d_atoms, N, sTop, Bt[0], Bt[1], Bt[2], Bt[3]);
    RP_LAUNCH_CHECK();
    const CUtensorMap mBh = make_map(Bh, N, fl.width, kBN), mBl = make_map(Bl, N, fl.width, kBN);

    // chunk the points so the per-chunk staging stays below ~6 GB
    const int Np = N + 1;                       // atoms + the ESP row
    const int Np_pad = (int)round_up(Np, kBM);
    const long long per_point = 4LL * fl.width + 8LL * top.width + 8LL * N + 8LL * Np_pad;
    long long chunk = std::max<long long>(kBM, ((6LL << 30) / per_point) / kBM * kBM);
    chunk = std::min<long long>(chunk, round_up(M, kBM));
    const long long chunk_pad = round_up(chunk, kBK);

    __half *Th = ctx->buf_t<__half>("m_Th", (size_t)chunk * fl.width);
    __half *Tl = ctx->buf_t<__half>("m_Tl", (size_t)chunk * fl.width);
    __half *Tt[4];
    for (int q = 0; q < 4; ++q) Tt[q] = ctx->buf_t<__half>("m_Tt" + std::to_string(q), (size_t)chunk * top.width);
    double *phit = ctx->buf_t<double>("m_phit", (size_t)N * chunk_pad);
    __half *X[kGSlices];
    for (int q = 0; q < kGSlices; ++q) X[q] = ctx->buf_t<__half>("m_X" + std::to_string(q), (size_t)Np_pad * chunk_pad);
    int *d_clamped = ctx->d_status + 1;  // second status word: fixed-point range overflows
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

    // ESP row scale: power of two from the largest |Vc|, computed on the device
    float *vscale = ctx->buf_t<float>("m_vscale", 1);
    {
        column_sums_fp64(Vc_dev, M, 1, 1, sumV, false, ctx, stream);
        double *d_vmax = ctx->buf_t<double>("m_vmax", 1);
        absmax_kernel<<<1, 1024, 0, stream>>>(Vc_dev, M, d_vmax);
        RP_LAUNCH_CHECK();
        vscale_kernel<<<1, 1, 0, stream>>>(d_vmax, vscale);
        RP_LAUNCH_CHECK();
    }

    const int nt = Np_pad / kBM;
    const int ntri = nt * (nt + 1);  // 128 x 64 Gram tiles with columns at or right of the row block
    const int kb_split = 2 * kGramFlush;  // 1024 points per CTA (int64 headroom), exact sums flushed every 512

    for (long long m0 = 0; m0 < M; m0 += chunk) {
        const long long rows = std::min<long long>(chunk, M - m0);
        const long long rows_tpad = round_up(rows, kBM);
        const long long rows_kpad = round_up(rows, kBK);
        // 1. grid tables of both blocks
        {
        StageTimer t_tab(ctx, "grid_tables", stream);
        grid_tables_f16_kernel<<<ceil_div(rows_tpad * (fl.width / 2), 256), 256, 0, stream>>>(
            ew->d_kidx_s, swk, fl, kmax, ex, ey, ez, nx, ny, nz, kept_idx_dev, m0, rows, rows_tpad, Th, Tl);
        RP_LAUNCH_CHECK();
        grid_tables_top_kernel<<<ceil_div(rows_tpad * (top.width / 2), 256), 256, 0, stream>>>(
            ew->d_kidx_s, wtop, top, kmax, ew->d_ex, ew->d_ey, ew->d_ez, nx, ny, nz, kept_idx_dev, m0, rows,
            rows_tpad, sTop, Tt[0], Tt[1], Tt[2], Tt[3]);
        RP_LAUNCH_CHECK();
        }
        // 2a. GEMM-1 over the float block: Phi_t = T B^T (atom-major, ld chunk_pad)
        {
            StageTimer tt(ctx, "recip_gemm_f16x3", stream);
            const CUtensorMap mTh = make_map(Th, rows_tpad, fl.width, kBM), mTl = make_map(Tl, rows_tpad, fl.width, kBM);
            RecArgs g{};
            g.m_tiles = (int)(rows_tpad / kBM);
            g.kb_total = fl.width / kBK;
            g.rows_m = (int)rows;
            g.rows_n = N;
            g.out_scale = 1.0 / ((double)kTableScale * (double)kTableScale);
            g.out = phit;
            g.ld_out = chunk_pad;
            g.status = d_status;
            launch_recip(mTh, mTl, mBh, mBl, g, g.m_tiles * ((N + kBN - 1) / kBN), stream);
        }
        // 2b. exact GEMM over the heaviest k: Phi_t += T_top B_top^T
        {
            StageTimer tt(ctx, "recip_gemm_exact_top", stream);
            TopArgs g{};
            g.m_tiles = (int)(rows_tpad / kBM);
            g.kb_total = top.width / kBK;
            g.rows_m = (int)rows;
            g.rows_n = N;
            g.out_scale = 1.0 / ((double)kTableScale * (double)kTableScale * sTop * sTop);
            g.out = phit;
            g.ld_out = chunk_pad;
            g.status = d_status;
            const __half *Tq[4] = {Tt[0], Tt[1], Tt[2], Tt[3]};
            const __half *Bq[4] = {Bt[0], Bt[1], Bt[2], Bt[3]};
            launch_top(Tq, rows_tpad, Bq, N, top.width, g, g.m_tiles * ((N + kGN - 1) / kGN), stream);
        }
        // 3. real space
        {
            StageTimer tt(ctx, "realspace", stream);
            dim3 grd(ceil_div(rows, kRealPts), ceil_div(N, kRealAtoms));
            realspace_kernel<<<grd, kRealPts, 0, stream>>>(kept_idx_dev, m0, rows, d_axis, nx, ny, d_atoms, N,
                                                           d_shifts, S, zero_idx, ew->cutoff, ew->sqrt_alpha,
                                                           real_near2(), phit, chunk_pad);
            RP_LAUNCH_CHECK();
        }
        // 4. column statistics, centre/scale on the first chunk, fixed-point slices of X
        {
            StageTimer tt(ctx, "center_slice", stream);
            const int ns = (int)((rows + kStatSlab - 1) / kStatSlab);
            colstats_kernel<<<dim3(ns, N), 256, 0, stream>>>(phit, chunk_pad, rows, N, psum, pmax);
            RP_LAUNCH_CHECK();
            colstats_finish_kernel<<<ceil_div(N, 128), 128, 0, stream>>>(psum, pmax, ns, N, rows, m0 == 0 ? 1 : 0, sphi,
                                                                         cvec, cf, scale);
            RP_LAUNCH_CHECK();
            slice_rows_kernel<<<ceil_div((long long)Np_pad * rows_kpad, 256), 256, 0, stream>>>(
                phit, chunk_pad, rows, rows_kpad, N, Np_pad, cvec, scale, Vc_dev, m0, vscale, X[0], X[1], X[2], X[3], d_clamped);
            RP_LAUNCH_CHECK();
        }
        // 5. GEMM-2: exact Gram partial tiles over point splits, then the fixed-order FP64 reduction
        {
            const int kb_total = (int)(rows_kpad / kBK);
            const int nsplit = (kb_total + kb_split - 1) / kb_split;
            double *part = ctx->buf_t<double>("m_part", (size_t)nsplit * ntri * kBM * kGN);
            GramArgs g{};
            g.nt = nt;
            g.ntri = ntri;
            g.kb_total = kb_total;
            g.kb_per_split = kb_split;
            g.flush = kGramFlush;
            g.out = part;
            g.status = d_status;
            const __half *Xq[kGSlices] = {X[0], X[1], X[2], X[3]};
            {
                StageTimer tt(ctx, "gram_exact", stream);
                launch_gram(Xq, Np_pad, rows_kpad, g, ntri * nsplit, stream);
            }
            StageTimer tr(ctx, "gram_reduce_fp64", stream);
            gram_reduce_kernel<<<dim3(ceil_div(kBM * kGN, 256), ntri), 256, 0, stream>>>(part, ntri, nsplit, nt, Np,
                                                                                         scale, vscale, N, G);
            RP_LAUNCH_CHECK();
        }
    }
    finish_mixed_kernel<<<ceil_div(std::max<long long>((long long)N * N, N), 256), 256, 0, stream>>>(
        G, Np, sphi, cvec, sumV, M, N, A_dev, b_dev);
    RP_LAUNCH_CHECK();
}

}  // namespace rp

// Diagnostics (not part of the public ABI): the two FP32 Phi parts of the mixed
// path for the first `rows` kept points, atom-major [N][rows].  Used to check the
// tensor-core k-contraction and the FP32 real-space sum against FP64 separately.
extern "C" int rp_debug_mixed_phi_parts(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N,
                                        const int32_t *kept_idx_dev, int64_t rows, double *recip_dev,
                                        double *real_dev) {
    using namespace rp;
    try {
        RP_CUDA(cudaSetDevice(ctx->device));
        RP_REQUIRE(rows > 0 && rows <= (1LL << 30), "bad rows");
        // run the real pipeline pieces through gram_mixed's staging by calling it on a
        // zero ESP would also solve; instead reuse its stages directly on one chunk
        const int K = ew->K;
        KBlock fl, top;
        plan_kblocks(ew, fl, top);
        std::vector<double> sh;
        int zero_idx = -1;
        prune_shifts(ew, atoms, N, sh, zero_idx);
        const int S = (int)(sh.size() / 3);
        const int nx = ew->grid.n_grid[0], ny = ew->grid.n_grid[1], nz = ew->grid.n_grid[2], kmax = ew->kmax;
        double *d_atoms = ctx->buf_t<double>("g_atoms", 3 * (size_t)N);
        double *d_shifts = ctx->buf_t<double>("g_shifts", sh.size());
        double *d_axis = ctx->buf_t<double>("g_axis", 9);
        RP_CUDA(cudaMemcpy(d_atoms, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice));
        RP_CUDA(cudaMemcpy(d_shifts, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice));
        RP_CUDA(cudaMemcpy(d_axis, ew->grid.axis, sizeof(double) * 9, cudaMemcpyHostToDevice));
        RP_CUDA(cudaMemset(ctx->d_status, 0, sizeof(int)));
        const int nex = (kmax + 1) * nx, ney = (2 * kmax + 1) * ny, nez = (2 * kmax + 1) * nz;
        float2 *ex = ctx->buf_t<float2>("m_ex", nex), *ey = ctx->buf_t<float2>("m_ey", ney),
               *ez = ctx->buf_t<float2>("m_ez", nez);
        float *swk = ctx->buf_t<float>("m_swk", K);
        to_float2_kernel<<<ceil_div(nex, 256), 256>>>(ew->d_ex, ex, nex);
        RP_LAUNCH_CHECK();
        to_float2_kernel<<<ceil_div(ney, 256), 256>>>(ew->d_ey, ey, ney);
        RP_LAUNCH_CHECK();
        to_float2_kernel<<<ceil_div(nez, 256), 256>>>(ew->d_ez, ez, nez);
        RP_LAUNCH_CHECK();
        sqrt_weights_kernel<<<ceil_div(K, 256), 256>>>(ew->d_kcoef_s, swk, K);
        RP_LAUNCH_CHECK();
        double wmax = 0.0;
        for (double w : ew->kcoef) wmax = std::max(wmax, w);
        int et = 0;
        std::frexp(std::sqrt(wmax) * (double)kTableScale, &et);
        const double sTop = std::ldexp(1.0, -et - 1);
        double *wtop = ctx->buf_t<double>("m_wtop", (size_t)top.count);
        {
            std::vector<double> kc(ew->kcoef);
            std::sort(kc.begin(), kc.end());
            std::vector<double> w((size_t)top.count);
            for (int q = 0; q < top.count; ++q) w[q] = std::sqrt(kc[top.q0 + q]) * (double)kTableScale * sTop;
            RP_CUDA(cudaMemcpy(wtop, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice));
        }
        __half *Bh = ctx->buf_t<__half>("m_Bh", (size_t)N * fl.width), *Bl = ctx->buf_t<__half>("m_Bl", (size_t)N * fl.width);
        atom_tables_f16_kernel<<<ceil_div((long long)N * fl.width, 256), 256>>>(ew->d_kvec_s, ew->d_kcoef_s, fl, d_atoms,
                                                                                N, Bh, Bl);
        RP_LAUNCH_CHECK();
        __half *Bt[4], *Tt[4];
        const long long rows_tpad = round_up(rows, kBM);
        for (int q = 0; q < 4; ++q) {
            Bt[q] = ctx->buf_t<__half>("m_Bt" + std::to_string(q), (size_t)N * top.width);
            Tt[q] = ctx->buf_t<__half>("m_Tt" + std::to_string(q), (size_t)rows_tpad * top.width);
        }
        atom_tables_top_kernel<<<ceil_div((long long)N * top.width, 256), 256>>>(ew->d_kvec_s, ew->d_kcoef_s, top,
                                                                                 d_atoms, N, sTop, Bt[0], Bt[1], Bt[2], Bt[3]);
        RP_LAUNCH_CHECK();
        __half *Th = ctx->buf_t<__half>("m_Th", (size_t)rows_tpad * fl.width),
               *Tl = ctx->buf_t<__half>("m_Tl", (size_t)rows_tpad * fl.width);
        grid_tables_f16_kernel<<<ceil_div(rows_tpad * (fl.width / 2), 256), 256>>>(
            ew->d_kidx_s, swk, fl, kmax, ex, ey, ez, nx, ny, nz, kept_idx_dev, 0, rows, rows_tpad, Th, Tl);
        RP_LAUNCH_CHECK();
        grid_tables_top_kernel<<<ceil_div(rows_tpad * (top.width / 2), 256), 256>>>(
            ew->d_kidx_s, wtop, top, kmax, ew->d_ex, ew->d_ey, ew->d_ez, nx, ny, nz, kept_idx_dev, 0, rows,
            rows_tpad, sTop, Tt[0], Tt[1], Tt[2], Tt[3]);
        RP_LAUNCH_CHECK();
        RecArgs g{};
        g.m_tiles = (int)(rows_tpad / kBM);
        g.kb_total = fl.width / kBK;
        g.rows_m = (int)rows;
        g.rows_n = N;
        g.out_scale = 1.0 / ((double)kTableScale * (double)kTableScale);
        g.out = recip_dev;
        g.ld_out = rows;
        g.status = ctx->d_status;
        launch_recip(make_map(Th, rows_tpad, fl.width, kBM), make_map(Tl, rows_tpad, fl.width, kBM),
                     make_map(Bh, N, fl.width, kBN), make_map(Bl, N, fl.width, kBN), g, g.m_tiles * ((N + kBN - 1) / kBN), 0);
        TopArgs tg{};
        tg.m_tiles = (int)(rows_tpad / kBM);
        tg.kb_total = top.width / kBK;
        tg.rows_m = (int)rows;
        tg.rows_n = N;
        tg.out_scale = 1.0 / ((double)kTableScale * (double)kTableScale * sTop * sTop);
        tg.out = recip_dev;
        tg.ld_out = rows;
        tg.status = ctx->d_status;
        const __half *Tq[4] = {Tt[0], Tt[1], Tt[2], Tt[3]};
        const __half *Bq[4] = {Bt[0], Bt[1], Bt[2], Bt[3]};
        launch_top(Tq, rows_tpad, Bq, N, top.width, tg, tg.m_tiles * ((N + kGN - 1) / kGN), 0);
        RP_CUDA(cudaMemset(real_dev, 0, sizeof(double) * (size_t)N * rows));
        realspace_kernel<<<dim3(ceil_div(rows, kRealPts), ceil_div(N, kRealAtoms)), kRealPts>>>(
            kept_idx_dev, 0, rows, d_axis, nx, ny, d_atoms, N, d_shifts, S, zero_idx, ew->cutoff, ew->sqrt_alpha,
            real_near2(), real_dev, rows);
        RP_LAUNCH_CHECK();
        RP_CUDA(cudaDeviceSynchronize());
        int st = 0;
        RP_CUDA(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        if (st) fail(st, "pipeline wait timed out");
        return RP_OK;
    } catch (const rp::Error &e) {
        ctx->last_error = e.msg;
        return e.code;
    }
}

// Diagnostics: the exact-Gram kernel on caller-provided FP16 slices X0, X1, X2
// ([Np_pad][cols], cols a multiple of 64) -> 2^-40 * sum over points and all nine
// slice products of x_s y_u 2^(7(4-s-u)) (FP64, Np x Np).
extern "C" int rp_debug_gram_slices(rp_ctx *ctx, const void *X0, const void *X1, const void *X2, const void *X3,
                                    int Np, long long cols, int flush, int kb_split, double *I_dev) {
    using namespace rp;
    try {
        RP_CUDA(cudaSetDevice(ctx->device));
        const int Np_pad = (int)round_up(Np, kBM);
        const int nt = Np_pad / kBM, ntri = nt * (nt + 1);
        const int kb_total = (int)(cols / kBK);
        const int nsplit = (kb_total + kb_split - 1) / kb_split;
        double *part = ctx->buf_t<double>("dbg_part", (size_t)nsplit * ntri * kBM * kGN);
        RP_CUDA(cudaMemset(ctx->d_status, 0, sizeof(int)));
        GramArgs g{};
        g.nt = nt; g.ntri = ntri; g.kb_total = kb_total; g.kb_per_split = kb_split;
        g.flush = std::min(std::max(flush, 1), kGramFlush);
        g.out = part; g.status = ctx->d_status;
        const __half *Xq[kGSlices] = {(const __half *)X0, (const __half *)X1, (const __half *)X2, (const __half *)X3};
        launch_gram(Xq, Np_pad, cols, g, ntri * nsplit, 0);
        float *ones = ctx->buf_t<float>("dbg_ones", Np);
        std::vector<float> h((size_t)Np, 1.0f);
        RP_CUDA(cudaMemcpy(ones, h.data(), sizeof(float) * Np, cudaMemcpyHostToDevice));
        RP_CUDA(cudaMemset(I_dev, 0, sizeof(double) * Np * Np));
        gram_reduce_kernel<<<dim3(ceil_div(kBM * kGN, 256), ntri), 256>>>(part, ntri, nsplit, nt, Np, ones, ones, Np, I_dev);
        RP_LAUNCH_CHECK();
        RP_CUDA(cudaDeviceSynchronize());
        int st = 0;
        RP_CUDA(cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        if (st) fail(st, "gram kernel wait timed out");
        return RP_OK;
    } catch (const rp::Error &e) {
        ctx->last_error = e.msg;
        return e.code;
    }
}
