// Mixed-precision Phi -> normal equations on GB300.
//
// Replaces, on the device, the Phi build of EwaldCalculator._compute_gpu*
// (repeat.py:1199-1435) and the Gram accumulation of fit_charges
// (repeat.py:2246-2276).  Once per fit:
//
//  0. recip   E[r][a][n1] for every grid row r (separable reciprocal sum, stages A
//             and B in recip_sep.cu, on the FP32 pipe).
//
// Then per chunk of kept points (Phi exists for one chunk only):
//
//  1. Phi     Phi_t[a][m] = real-space erfc sum (FP32 terms from double-float
//             coordinates, FP64 at the cutoff, double-float per-pair sums)
//             + Re sum_n1 ex[n1][i_m] E[r_m][a][n1] (FP32), written once,
//             atom-major (phi_chunk_kernel).
//  2. split   X[a][m] = (Phi_t[a][m] - c_a) * 2^e_a cut into four 7-bit fixed-point
//             digits, plus a row for the centred ESP: c_a is the column mean of the
//             first chunk (a per-column shift corrected exactly later), 2^e_a a
//             power-of-two row scale.
//  3. Gram    G = X X^T on tcgen05 (kind::f16, FP32 accumulators in TMEM) with all
//             16 digit products kept: every partial sum is an integer below 2^24,
//             so the Gram of the staged Phi is exact; a persistent kernel (one CTA
//             per SM) takes work units (one point split of one tile) from a counter
//             and adds each unit's int64 sums to the tile's exact 64-bit totals with
//             atomics, which are rounded to FP64 once.
//  4. finish  A = G - s s^T/M, b = G[:,V] - s sum(V)/M with s = sum_m (Phi - c)
//             (FP64), i.e. repeat.py:2266-2276 for the shifted columns.
//
// Error budget: Phi carries the FP32 real-space terms and the FP32 reciprocal
// stages B and C (~1e-7 relative each, unbiased rounding) and the 28-bit digit
// quantisation of the Gram input (~2^-29 of each row's range, unbiased).  The
// tensor cores' FP32 accumulation truncates, which is why the Gram is done in
// exact integer digits instead of as an FP16/BF16 hi+lo product.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>

#include "common.cuh"
#include "df.cuh"
#include "tc.cuh"

namespace rp {
namespace {

constexpr int kBM = 128;       // Gram tile rows (TMEM lanes)
constexpr int kKPad = 64;      // digit rows are padded to a multiple of 64 points (the tensor maps' unit)
constexpr int kBK = 32;        // points (K elements) per stage: 64 B of FP16 = one 64-byte swizzle row
constexpr int kTileBytes = kBM * kBK * 2;  // 8 KB per operand tile

// ---- GEMM-2 (Gram): exact integer products of four 7-bit fixed-point slices
// x = 2^-6 (x0 + 2^-7 x1 + 2^-14 x2 + 2^-21 x3), x_s integers with |x0| <= 32,
// |x1..x3| <= 64 (|x| <= 1/2; 28 bits below the row maximum, because a centred
// column's typical value sits orders of magnitude below its maximum).  All 16
// slice products are kept: for the many values far below their row's maximum the
// low digits carry the signal, not rounding noise (leaving out the three products of
// weight 5 and 6 moved the batch's charges from 4e-7 to 4e-6 e of FP64).  They are
// grouped by weight g = s+u into seven TMEM accumulators of a 128 x 64 tile.  Per
// point, a group's products sum to at most 12288 in magnitude (weight 3: x0 x3 +
// x3 x0 <= 2 * 32 * 64, x1 x2 + x2 x1 <= 2 * 64 * 64; weight 4: three products
// <= 64 * 64; the others less), so a stage of 32 points adds at most 393,216 =
// 3 * 2^17 to a group and kGramFlush = 32 stages (1024 points) stay below 2^24 (12.6 M):
// the FP32 sums are exact, and a work unit of kGramSplit = 32 stages drains them once, at
// its end.
// (A row whose |x| passed 1/2 is clamped, counted and its cube refitted from the
// staged Phi, whose own scale keeps |x| < 1/2.)  At each flush the epilogue folds the
// groups into one int64 per element (sum_g D_g 2^(7(6-g))), so the Gram carries no
// rounding bias (its diagonal is the most sensitive quantity of the fit).
constexpr int kGN = 64;          // Gram tile columns
constexpr int kGSlices = 4;
constexpr int kGroups = 2 * kGSlices - 1;
constexpr int kGramStages = 3;   // 3 x 48 KB: two stages in flight while one is multiplied
constexpr int kGramFlush = 32;
constexpr int kGramSplit = 32;   // stages per work unit: 1024 points, the int64 fold's headroom (2^52 per point)
constexpr int kStagesPer64 = kKPad / kBK;  // the autotuner's and the diagnostics' 64-point blocks, in stages
constexpr int kGramEpiWarps = 8;
constexpr int kEpiCols = kGN * 4 / kGramEpiWarps;  // Gram tile columns per epilogue warp (TMEM lane quarter)
constexpr int kGramThreads = 64 + 32 * kGramEpiWarps;  // 320
constexpr int kBTileBytes = kGN * kBK * 2;             // 4 KB
constexpr int kGramStageBytes = kGSlices * kTileBytes + kGSlices * kBTileBytes;
constexpr int kGramSmem = kGramStages * kGramStageBytes + 1024 + 256;

constexpr int kSched = 4;         // work-unit ring entries (producer -> MMA thread and epilogue)
// the barriers, the ring and the TMEM address after the stages, in the last 256 bytes
static_assert((2 * kGramStages + 3 + 2 * kSched) * 8 + kSched * 4 + 4 <= 256, "gram smem tail");

struct GramArgs {
    int nt, ntj, ntri, kb_total, kb_per_split, flush;  // flush: stages per exact FP32 run (<= kGramFlush)
    int unit0, nunits;  // this launch's work units unit0 .. unit0 + nunits - 1 of the ntri Gram
                        // tiles x ceil(kb_total / kb_per_split) point splits
    int *next_unit;     // this launch's work counter, zero at launch
    // exact tile sums [tri][col][row] as two's complement 64-bit halves: every unit adds the
    // high (acc >> 32) and low (acc & (2^32 - 1)) parts of its int64 partial (|acc| < 2^62)
    unsigned long long *out_hi, *out_lo;
    int *status;
    long long budget;  // clock budget of the pipeline's waits (tc::kWaitBudgetCycles; <= 0: give up at once)
};

__device__ __forceinline__ uint8_t *align1024(uint8_t *raw) {
    const uint32_t s = tc::smem_u32(raw);
    return raw + (((s + 1023u) & ~1023u) - s);
}

// Gram tile t -> (ti, tj): rows [128 ti, +128), columns [64 tj, +64), 2 ti <= tj < ntj,
// ntj = ceil(rows / 64): tiles wholly beyond the last row are never computed, and rows
// past the end of the digit arrays read as zeros (the tensor maps' out-of-bounds fill).
__device__ __forceinline__ void gram_tile_decode(int t, int ntj, int &ti, int &tj) {
    ti = 0;
    int len = ntj;
    while (t >= len) {
        t -= len;
        ++ti;
        len -= 2;
    }
    tj = 2 * ti + t;
}

// Work unit u = (tile u % ntri, point split u / ntri): consecutive units share their points,
// so the CTAs working at one time read the same digit columns through L2.
struct GramUnit {
    int tile, a_row0, b_row0, kb0, nkb;
};
__device__ __forceinline__ GramUnit gram_unit(const GramArgs &g, int unit) {
    GramUnit w;
    w.tile = unit % g.ntri;
    int ti, tj;
    gram_tile_decode(w.tile, g.ntj, ti, tj);
    w.a_row0 = ti * kBM;
    w.b_row0 = tj * kGN;
    w.kb0 = (unit / g.ntri) * g.kb_per_split;
    w.nkb = min(w.kb0 + g.kb_per_split, g.kb_total) - w.kb0;  // >= 1
    return w;
}

// Persistent: one CTA per SM takes work units from the launch's counter until none are left.
// Warp 0 (one thread) takes the units, posts each in a shared ring and streams its digit
// tiles by TMA through the stages, running ahead across unit boundaries; warp 1 (one
// thread) issues the MMAs; warps 2..9 drain the seven group accumulators from TMEM into
// int64 sums once per flush, 16 columns at a time, and add them to the tile's totals with
// 64-bit atomics (the last columns' while the MMAs of the next unit already run).
// At most 96 registers and 3 x 48 KB of stages: the SM keeps room for CTAs of other kernels
// (the Phi kernel of other cubes, bound by instruction issue, which this kernel barely uses).
__global__ void __maxnreg__(96) gram_exact_kernel(
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
    uint64_t *sfull = acce + 1;            // work unit posted in the ring
    uint64_t *sempty = sfull + kSched;     // ring entry read by the MMA thread and every epilogue warp
    uint64_t *fin = sempty + kSched;       // every MMA the CTA issued is complete
    volatile int *sched = reinterpret_cast<volatile int *>(fin + 1);
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(const_cast<int *>(sched + kSched));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // B is loaded for every tile (also where its rows lie inside A's tile): the four B slices
    // then sit back to back and form one 256-row operand
    const uint32_t stage_tx = kGSlices * (kTileBytes + kBTileBytes);
    const CUtensorMap *ta[kGSlices] = {&tm0, &tm1, &tm2, &tm3};
    const CUtensorMap *tb[kGSlices] = {&tb0, &tb1, &tb2, &tb3};

    if (threadIdx.x == 0) {
        for (int s = 0; s < kGramStages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(accf, 1);
        tc::mbar_init(acce, 32 * kGramEpiWarps);
        for (int r = 0; r < kSched; ++r) {
            tc::mbar_init(&sfull[r], 1);
            tc::mbar_init(&sempty[r], 1 + kGramEpiWarps);
        }
        tc::mbar_init(fin, 1);
        tc::fence_mbar_init();
    }
    if (warp == 1) tc::tmem_alloc(tmem_holder, 512);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0 && lane == 0) {
        int it = 0;  // stages issued
        bool ok = true;
        for (int j = 0; ok; ++j) {
            const int r = j % kSched;
            if (j >= kSched && !tc::mbar_wait(&sempty[r], ((j / kSched) - 1) & 1, g.status, g.budget)) break;
            const int k = atomicAdd(g.next_unit, 1);
            const int unit = k < g.nunits ? g.unit0 + k : -1;
            sched[r] = unit;
            tc::mbar_arrive(&sfull[r]);  // release: the entry is visible to the waiters
            if (unit < 0) break;
            const GramUnit w = gram_unit(g, unit);
            for (int kb = 0; kb < w.nkb; ++kb, ++it) {
                const int s = it % kGramStages, u = it / kGramStages;
                if (u > 0 && !tc::mbar_wait(&empty[s], (u - 1) & 1, g.status, g.budget)) {
                    ok = false;
                    break;
                }
                uint8_t *st = smem + s * kGramStageBytes;
                tc::mbar_arrive_expect_tx(&full[s], stage_tx);
                const int x = (w.kb0 + kb) * kBK;
#pragma unroll
                for (int q = 0; q < kGSlices; ++q) {
                    tc::tma_load_2d(st + q * kTileBytes, ta[q], x, w.a_row0, &full[s]);
                    tc::tma_load_2d(st + kGSlices * kTileBytes + q * kBTileBytes, tb[q], x, w.b_row0, &full[s]);
                }
            }
        }
        // after a timeout, the copies still in flight land before the CTA exits
        if (*reinterpret_cast<volatile int *>(g.status) != 0)
            for (int k = max(0, it - kGramStages); k < it; ++k)
                tc::mbar_wait(&full[k % kGramStages], (k / kGramStages) & 1, nullptr);
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = tc::idesc_f16_f32(kBM, kGN);
        const uint32_t idesc4 = tc::idesc_f16_f32(kBM, 4 * kGN);  // all four B slices, four adjacent groups
        uint32_t d[kGroups];  // group accumulators, 64 TMEM columns each
#pragma unroll
        for (int q = 0; q < kGroups; ++q) d[q] = tmem + (uint32_t)(q * kGN);
        int it = 0, fc = 0;  // stages consumed, flushes committed
        bool ok = true;
        for (int j = 0; ok; ++j) {
            const int r = j % kSched;
            if (!tc::mbar_wait(&sfull[r], (j / kSched) & 1, g.status, g.budget)) break;
            const int unit = sched[r];
            tc::mbar_arrive(&sempty[r]);
            if (unit < 0) break;
            const GramUnit w = gram_unit(g, unit);
            const int nflush = (w.nkb + g.flush - 1) / g.flush;
            for (int f = 0; f < nflush; ++f) {
                if (fc > 0 && !tc::mbar_wait(acce, (fc - 1) & 1, g.status, g.budget)) {  // sums drained
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const int kbf0 = f * g.flush, kbf1 = min(kbf0 + g.flush, w.nkb);
                for (int kb = kbf0; kb < kbf1; ++kb, ++it) {
                    const int s = it % kGramStages, u = it / kGramStages;
                    if (!tc::mbar_wait(&full[s], u & 1, g.status, g.budget)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t st = tc::smem_u32(smem + s * kGramStageBytes);
                    uint64_t x[kGSlices], y[kGSlices];
#pragma unroll
                    for (int q = 0; q < kGSlices; ++q) {
                        x[q] = tc::sdesc_k_sw64(st + q * kTileBytes);
                        y[q] = tc::sdesc_k_sw64(st + kGSlices * kTileBytes + q * kBTileBytes);
                    }
#pragma unroll
                    for (int kk = 0; kk < kBK / 16; ++kk) {
                        const uint64_t o = (uint64_t)(kk * 2);
                        if (kb == kbf0 && kk == 0) {
                            // the first products of a flush start each group's sum: one MMA per
                            // (slice a, slice b), the first into a group overwriting it
                            bool started[kGroups] = {false, false, false, false, false, false, false};
#pragma unroll
                            for (int a = 0; a < kGSlices; ++a)
#pragma unroll
                                for (int b = 0; b < kGSlices; ++b) {
                                    const int grp = a + b;
                                    const uint32_t acc = started[grp] ? 1u : 0u;
                                    started[grp] = true;
                                    tc::umma_f16(d[grp], x[a] + o, y[b] + o, idesc, acc);
                                }
                        } else {
                            // then N = 256: slice a against the four B slices back to back (a 256-row
                            // operand) writes the products of weights a .. a+3 into the four adjacent
                            // groups from d[a] (the same products, in the same order per group, as the
                            // pairs above), reading A once instead of four times
#pragma unroll
                            for (int a = 0; a < kGSlices; ++a) tc::umma_f16(d[a], x[a] + o, y[0] + o, idesc4, 1u);
                        }
                    }
                    tc::umma_commit(&empty[s]);
                }
                if (!ok) break;
                tc::umma_commit(accf);
                ++fc;
            }
        }
        tc::umma_commit(fin);  // tracks every MMA issued above
    } else if (warp >= 2) {
        const int ew = warp - 2;
        const int lane_base = (warp & 3) * 32;
        const int col0 = (ew >> 2) * kEpiCols;  // this warp's columns of the 64
        const uint32_t base = tmem + ((uint32_t)lane_base << 16) + (uint32_t)col0;
        int fc = 0;  // flushes drained
        bool ok = true;
        // every wait's outcome is made warp-uniform by a vote before the warp-wide
        // TMEM loads and the __syncwarp below
        for (int j = 0; ok; ++j) {
            const int r = j % kSched;
            if (!__all_sync(0xffffffffu, tc::mbar_wait(&sfull[r], (j / kSched) & 1, g.status, g.budget))) break;
            const int unit = sched[r];
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&sempty[r]);
            if (unit < 0) break;
            const GramUnit w = gram_unit(g, unit);
            const int nflush = (w.nkb + g.flush - 1) / g.flush;
            const long long t0 = (long long)w.tile * (kBM * kGN);
            const int rr = lane_base + lane;
            for (int f = 0; f < nflush; ++f, ++fc) {
                if (!__all_sync(0xffffffffu, tc::mbar_wait(accf, fc & 1, g.status, g.budget)) ||
                    __any_sync(0xffffffffu, *reinterpret_cast<volatile int *>(g.status) != 0)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                // the warp's columns 16 at a time (fewer live registers): the flush's int64 sums
                // of 16 columns go to the tile totals before the next 16 are loaded
#pragma unroll
                for (int h = 0; h < kEpiCols / 16; ++h) {
                    long long acc[16];
#pragma unroll
                    for (int i = 0; i < 16; ++i) acc[i] = 0;
#pragma unroll
                    for (int q = 0; q < kGroups; ++q) {
                        float v[16];
                        tc::tmem_ld_32x16(base + (uint32_t)(q * kGN + 16 * h), v);
                        const int sh = 7 * (kGroups - 1 - q);
#pragma unroll
                        for (int i = 0; i < 16; ++i) acc[i] += (long long)__float2int_rn(v[i]) << sh;
                    }
                    if (h == kEpiCols / 16 - 1) {
                        tc::fence_before_sync();
                        tc::mbar_arrive(acce);
                    }
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const long long e = t0 + (col0 + 16 * h + i) * kBM + rr;
                        atomicAdd(g.out_hi + e, (unsigned long long)(acc[i] >> 32));
                        atomicAdd(g.out_lo + e, (unsigned long long)(acc[i] & 0xffffffffLL));
                    }
                }
            }
        }
    }
    // TMEM is freed only after every MMA of the CTA has completed (also after a timeout)
    if (warp == 1 && lane == 0) tc::mbar_wait(fin, 0, nullptr);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 1) tc::tmem_dealloc(tmem, 512);
}

// ESP row scale 2^(-e-1) with max|Vc| in [2^(e-1), 2^e), so |V * scale| < 1/2
__device__ __forceinline__ float vscale_of(double vmax) {
    int e = 0;
    if (vmax > 0.0) frexp(vmax, &e);
    return ldexpf(1.0f, -e - 1);
}

// Four 7-bit signed digits of an integer I = round(x 2^27), |x| <= 1:
// x ~ 2^-6 (s0 + 2^-7 s1 + 2^-14 s2 + 2^-21 s3), digits rounded half up so |s| <= 64,
// each exact in FP16.  Integer shifts only (no FP64 on the per-element path).
// Exact warp sum of fixed-point values |I| <= 2^27: two 32-bit warp reductions of the
// 14-bit halves (each sum stays below 2^19), recombined in 64 bits.
__device__ __forceinline__ long long warp_sum_fixed(int I) {
    const int hi = I >> 14, lo = I - (hi << 14);  // I = hi 2^14 + lo, lo in [0, 2^14)
    const int shi = __reduce_add_sync(0xffffffffu, hi);
    const int slo = __reduce_add_sync(0xffffffffu, lo);
    return (long long)shi * 16384 + slo;
}

__device__ __forceinline__ void split4(int v, int &s0, int &s1, int &s2, int &s3) {
    s0 = (v + (1 << 20)) >> 21;
    int r = v - (s0 << 21);  // [-2^20, 2^20)
    s1 = (r + (1 << 13)) >> 14;
    r -= s1 << 14;           // [-2^13, 2^13)
    s2 = (r + (1 << 6)) >> 7;
    s3 = r - (s2 << 7);      // [-64, 64)
}

__device__ __forceinline__ void digits4(int v, __half *o0, __half *o1, __half *o2, __half *o3, long long idx) {
    int s0, s1, s2, s3;
    split4(v, s0, s1, s2, s3);
    o0[idx] = __int2half_rn(s0);
    o1[idx] = __int2half_rn(s1);
    o2[idx] = __int2half_rn(s2);
    o3[idx] = __int2half_rn(s3);
}

// round((h + l) * sc) for a double-float (h, l) and a power of two sc, |(h + l) sc| <= 2^27:
// rint of the high part is exact, the remainder (h sc - I1) is exact (Sterbenz), and the
// low part decides the last unit.
__device__ __forceinline__ int round_df(float h, float l, float sc) {
    const float H = h * sc, L = l * sc;
    const float I1 = rintf(H);
    const float I2 = rintf(__fadd_rn(__fadd_rn(H, -I1), L));
    return (int)I1 + (int)I2;
}

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

// I = round(x 2^27) of one element of X (x = (Phi - c) scale, or the scaled ESP), |x| <= 1
__device__ __forceinline__ int x_fixed(float h, float l, float sc, int *clamped) {
    sc *= 134217728.0f;  // 2^27
    if (fabsf(h * sc) > 134217728.0f) {  // |x| beyond 1: clamp (counted; the fit reports it)
        atomicAdd(clamped, 1);
        return h > 0.f ? (1 << 27) : -(1 << 27);
    }
    return round_df(h, l, sc);
}

// ------------------------------------------------------------------ Phi of one chunk

// The approximate reciprocal, reciprocal square root and base-2 exponential of the
// multi-function unit, flushing subnormals (the arguments here are normal numbers), so
// that each is one instruction with no subnormal fix-up around it.
__device__ __forceinline__ float rcp_ftz(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_ftz(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// erfc(x), x >= 0, in FP32 by the Chebyshev fit "erfcc" of Press, Teukolsky, Vetterling
// and Flannery, Numerical Recipes in C (2nd ed., section 6.2): erfc(x) = t exp(-x^2 + P(t)),
// t = 1/(1 + x/2), fractional error below 1.2e-7.  It is evaluated in base 2: the argument
// comes pre-scaled, xs = sqrt(log2 e) x, and log2(e) is folded into the coefficients, so
//   erfc(x) = t 2^(-xs^2 + log2(e) P(t)),   t = 1 / (1 + xs / (2 sqrt(log2 e))),
// 14 instructions (one reciprocal, one exponential).  In FP32 the rounding of the exponent
// -xs^2 + p and of the reciprocal and exponential instructions dominates the error
// (measured against FP64 erfc and against CUDA's erfcf in the tests).  A degree-7 fit for
// the bounded range x <= pi (two FMAs fewer) was measured and dropped: its coefficients,
// up to 15 with alternating signs, lose bits in FP32 Horner evaluation (1.3e-6 for
// x < 1.5) and moved the batch's charges from 3.9e-7 to 4.6e-7 e of FP64.
constexpr double kLog2e = 1.4426950408889634074;
constexpr double kSqrtLog2e = 1.2011224087864498;  // sqrt(log2 e)
__device__ __forceinline__ float erfc_nr2(float xs) {
    const float t = rcp_ftz(fmaf((float)(0.5 / kSqrtLog2e), xs, 1.0f));
    float p = (float)(kLog2e * 0.17087277);
    p = fmaf(t, p, (float)(kLog2e * -0.82215223));
    p = fmaf(t, p, (float)(kLog2e * 1.48851587));
    p = fmaf(t, p, (float)(kLog2e * -1.13520398));
    p = fmaf(t, p, (float)(kLog2e * 0.27886807));
    p = fmaf(t, p, (float)(kLog2e * -0.18628806));
    p = fmaf(t, p, (float)(kLog2e * 0.09678418));
    p = fmaf(t, p, (float)(kLog2e * 0.37409196));
    p = fmaf(t, p, (float)(kLog2e * 1.00002368));
    p = fmaf(t, p, (float)(kLog2e * -1.26551223));
    return t * ex2_ftz(fmaf(-xs, xs, p));
}

constexpr int kPhiPts = 128;     // points per CTA (one per thread)
constexpr int kPhiAtoms = 16;    // atoms per CTA by default (8 and 32 are the other tile shapes)
constexpr int kMaxShifts = 128;  // pruned real-space shifts (checked on the host)

// The reference's FP64 cutoff decision for one (point, image) pair (repeat.py:944-966:
// r = |g - (a + s)| with g = (i a0 + j a1) + k a2, r <= Rc, the self image skipped at
// r <= 1e-10).  Returns 0 (outside), 1 (inside: the caller adds the FP32 term) or, with
// full = true, 2 and the FP64 term as a double-float (th, tl).  Not inlined on purpose:
// it runs for a few pairs in a million, and inlined the compiler may evaluate it
// speculatively for every pair on the slow FP64 pipe.
__device__ __noinline__ int fp64_pair(const double *axis, int i, int j, int k, const double *p,
                                      const double *shifts, int s, int zero_idx, double rc, double sa, bool full,
                                      float &th, float &tl) {
    double g[3];
    for (int d = 0; d < 3; ++d) g[d] = ((double)i * axis[d] + (double)j * axis[3 + d]) + (double)k * axis[6 + d];
    const double ex = g[0] - (p[0] + shifts[3 * s]), ey = g[1] - (p[1] + shifts[3 * s + 1]),
                 ez = g[2] - (p[2] + shifts[3 * s + 2]);
    const double r = sqrt(ex * ex + ey * ey + ez * ez);
    if (!(r <= rc) || (s == zero_idx && !(r > 1e-10))) return 0;
    if (!full) return 1;
    const double t = erfc(sa * r) / r;
    th = (float)t;
    tl = (float)(t - (double)th);
    return 2;
}

// Image positions atom + shift as double-float, [N][S] x {hi (x, y, z, shift index), lo}
__global__ void images_df_kernel(const double *__restrict__ atoms, int N, const double *__restrict__ shifts, int S,
                                 float4 *__restrict__ img) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N * S) return;
    const int a = t / S, s = t - a * S;
    double q[3];
    for (int d = 0; d < 3; ++d) q[d] = atoms[3 * a + d] + shifts[3 * s + d];
    const float hx = (float)q[0], hy = (float)q[1], hz = (float)q[2];
    img[2 * t] = make_float4(hx, hy, hz, __int_as_float(s));
    img[2 * t + 1] = make_float4((float)(q[0] - (double)hx), (float)(q[1] - (double)hy), (float)(q[2] - (double)hz), 0.f);
}

// (ah + al) - (bh + bl) as a normalised double-float
__device__ __forceinline__ float2 df_sub(float ah, float al, float bh, float bl) {
    float s, e;
    dfa::two_sum(ah, -bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, -bl));
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fadd_rn(e, -__fadd_rn(h, -s)));
}

// Phi_t[a][m] = sum over the images of atom a within Rc of erfc(sqrt(alpha) r)/r
//             + Re sum_n1 ex[n1][i_m] E[r_m][a][n1],   stored as double-float (hi, lo).
// Real space (repeat.py:944-966): the CTA first culls the images of its atoms to
// those within Rc + 1e-3 Bohr of the bounding box of its points, in shift order
// (warp-ballot compaction, so the summation order is fixed).  Distances are formed
// in FP32 from double-float coordinates relative to the CTA's first point; images
// within 2e-6 of Rc are decided in FP64 with the reference's expressions (the term
// is the FP32 one), pairs closer than sqrt(near2) are evaluated entirely in FP64,
// the rest with FP32 erfcf.  Reciprocal part: stage C of the
// separable sum in FP32.  `parts`: bit 0 real space, bit 1 reciprocal.
// With psum/pmax given, the CTA also writes each atom's sum and max |Phi| over its
// points (fixed-order reductions), the column statistics of the centring step.
// The grid step vectors as double-float (a[d] = h[d] + l[d]), passed by value.
struct AxisDF {
    float h[9], l[9];
};

// k * (ah + al) for a small integer k, as an unevaluated pair (p, e)
__device__ __forceinline__ void int_times_df(float k, float ah, float al, float &p, float &e) {
    p = __fmul_rn(k, ah);
    e = __fmaf_rn(k, ah, -p);
    e = __fmaf_rn(k, al, e);
}

// Digit output of the Phi kernel (single pass): instead of Phi_t, the kernel writes the
// four fixed-point digit slices of X rows a0..a0+na-1 (x = Phi * scale_a, centre 0) and,
// from the CTAs of the first atom block, the ESP row N (x = Vc * scale_V); columns
// rows..rows_kpad-1 get zero digits.  Exact row sums go to rowsum (one atomic per CTA
// and row), values beyond |x| = 1 are clamped and counted in *clamped.
struct PhiDigits {
    __half *X0, *X1, *X2, *X3;
    long long ldx;        // row stride of the slices
    long long rows_kpad;  // columns written (the chunk padded to the Gram's K step)
    const float *scale;   // per atom, a power of two
    const double *Vc;     // the chunk's centred ESP
    const double *vmax_p; // max |Vc| (the ESP row scale)
    unsigned long long *rowsum;
    int *clamped;
    int N;
};

// NC > 0: the number of n1 terms is the compile-time constant NC (KMAX = NC, the
// reference's default 7): an atom's NC E values are loaded at the top of its iteration
// and used after the real-space loop, which hides their L2 latency; stage C is unrolled.
// NC = 0: any KMAX, loads in the loop.  The register cap keeps 7 CTAs per SM.
template <int NC, bool DIG, int AT>
__global__ void __launch_bounds__(kPhiPts, 7) phi_chunk_kernel(
    const int32_t *__restrict__ kept, long long m0, long long rows, const double *__restrict__ axis, AxisDF adf,
    int nx, int ny,
    const double *__restrict__ atoms, int N, const double *__restrict__ shifts, int S, int scap, int zero_idx,
    double rc, double sa, float rcf, float saf_in, float near2, const float4 *__restrict__ img,
    const float4 *__restrict__ EX,
    const float2 *__restrict__ E, int n1c, int parts, float2 *__restrict__ phit, long long ld,
    double *__restrict__ psum, float *__restrict__ pmax, PhiDigits dg) {
    extern __shared__ float4 dsm[];
    float4 *img_hi = dsm;                                 // [AT][scap] (x, y, z, shift index)
    float4 *img_lo = img_hi + (size_t)AT * scap;   // [AT][scap]
    float2 *exs = reinterpret_cast<float2 *>(img_lo + (size_t)AT * scap);  // [n1c][kPhiPts] ex[n1][i]
    __shared__ int ncand[AT];
    __shared__ float bb[2][3][kPhiPts / 32];
    __shared__ float wsum[kPhiPts / 32][AT];
    __shared__ float wmax[kPhiPts / 32][AT];
    __shared__ long long wrow[kPhiPts / 32][AT + 1];  // digit-row partial sums (DIG)
    const long long mb = (long long)blockIdx.x * kPhiPts;
    const int a0 = blockIdx.y * AT;
    const int na = min(AT, N - a0);
    const int layer = nx * ny;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long m = mb + threadIdx.x;
    const bool valid = m < rows;

    // CTA origin: the first point of the tile (FP64 once, shared as a double-float)
    __shared__ float org[6];
    __shared__ int org_idx[3];
    if (threadIdx.x == 0) {
        const int f0 = kept[m0 + mb];
        const int l0 = f0 / layer, r0 = f0 - l0 * layer, j0 = r0 / nx, i0 = r0 - j0 * nx;
        for (int d = 0; d < 3; ++d) {
            const double o = ((double)i0 * axis[d] + (double)j0 * axis[3 + d]) + (double)l0 * axis[6 + d];
            org[d] = (float)o;
            org[3 + d] = (float)(o - (double)org[d]);
        }
        org_idx[0] = i0;
        org_idx[1] = j0;
        org_idx[2] = l0;
    }
    __syncthreads();
    const int f = kept[m0 + (valid ? m : mb)];
    const int l = f / layer, rem = f - l * layer, j = rem / nx, i = rem - j * nx;
    // point - origin = di a0 + dj a1 + dl a2 with small integers: double-float on the FP32 pipe
    float gh[3], gl[3], oh[3], ol[3];
    {
        const float di = (float)(i - org_idx[0]), dj = (float)(j - org_idx[1]), dl = (float)(l - org_idx[2]);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            float p0, e0, p1, e1, p2, e2, s, t;
            int_times_df(di, adf.h[d], adf.l[d], p0, e0);
            int_times_df(dj, adf.h[3 + d], adf.l[3 + d], p1, e1);
            int_times_df(dl, adf.h[6 + d], adf.l[6 + d], p2, e2);
            dfa::two_sum(p0, p1, s, t);
            float s2, t2;
            dfa::two_sum(s, p2, s2, t2);
            const float e = __fadd_rn(__fadd_rn(__fadd_rn(e0, e1), e2), __fadd_rn(t, t2));
            gh[d] = __fadd_rn(s2, e);
            gl[d] = __fadd_rn(e, -__fadd_rn(gh[d], -s2));
            oh[d] = org[d];
            ol[d] = org[3 + d];
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float mn = gh[d], mx = gh[d];
        for (int o = 16; o > 0; o >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
        if (lane == 0) {
            bb[0][d][warp] = mn;
            bb[1][d][warp] = mx;
        }
    }
    if (parts & 2)
        for (int n = 0; n < n1c; ++n) {
            const float4 x = EX[(long long)n * nx + i];
            exs[n * kPhiPts + threadIdx.x] = make_float2(x.x, x.z);
        }
    __syncthreads();

    if (parts & 1) {
        float bmin[3], bmax[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            bmin[d] = bb[0][d][0];
            bmax[d] = bb[1][d][0];
            for (int w = 1; w < kPhiPts / 32; ++w) {
                bmin[d] = fminf(bmin[d], bb[0][d][w]);
                bmax[d] = fmaxf(bmax[d], bb[1][d][w]);
            }
        }
        const float reach = rcf + 1e-3f, reach2 = reach * reach;
        for (int a = warp; a < AT; a += kPhiPts / 32) {
            int base = 0;
            if (a < na) {
                const float4 *src = img + 2 * (size_t)(a0 + a) * S;
                for (int s0 = 0; s0 < S; s0 += 32) {
                    const int s = s0 + lane;
                    bool keep = false;
                    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), lo = h;
                    if (s < S) {
                        const float4 ph = src[2 * s], pl = src[2 * s + 1];
                        const float2 qx = df_sub(ph.x, pl.x, oh[0], ol[0]), qy = df_sub(ph.y, pl.y, oh[1], ol[1]),
                                     qz = df_sub(ph.z, pl.z, oh[2], ol[2]);
                        h = make_float4(qx.x, qy.x, qz.x, ph.w);
                        lo = make_float4(qx.y, qy.y, qz.y, 0.f);
                        const float dx = fmaxf(fmaxf(bmin[0] - h.x, h.x - bmax[0]), 0.f);
                        const float dy = fmaxf(fmaxf(bmin[1] - h.y, h.y - bmax[1]), 0.f);
                        const float dz = fmaxf(fmaxf(bmin[2] - h.z, h.z - bmax[2]), 0.f);
                        keep = dx * dx + dy * dy + dz * dz <= reach2;
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, keep);
                    if (keep) {
                        const int pos = base + __popc(bal & ((1u << lane) - 1u));
                        img_hi[a * scap + pos] = h;
                        img_lo[a * scap + pos] = lo;
                    }
                    base += __popc(bal);
                }
            }
            if (lane == 0) ncand[a] = base;
        }
    }
    __syncthreads();

    // FP64 decides every image whose FP32 squared distance lies within +-4e-6 Rc^2 of the
    // cutoff: with coordinates exact to ~2^-48, dx carries <= 2^-23 relative error and
    // r2 <= 2^-21 (4.8e-7), so the band covers the FP32 error 8-fold.  Only the decision
    // r <= Rc is made in FP64 (the reference's expressions); the term itself, ~erfc(pi)/Rc
    // there, is the FP32 one.  FP64 runs at 1/64 of the FP32 rate per lane on this part,
    // and one lane in the band makes its whole warp run the FP64 code, so it stays short.
    const float rcc = rcf * rcf, band = 4e-6f * rcc, saf = saf_in;  // sqrt(alpha log2 e), the argument scale of erfc_nr2
    const float fp64_below = fmaxf(near2, 1e-6f);
    const long long row = f / nx;  // j + l * ny
    const float2 *erow = E + (row * N + a0) * (NC > 0 ? NC : n1c);
    float2 *prow = phit + (long long)a0 * ld + m;
    for (int a = 0; a < na; ++a, erow += (NC > 0 ? NC : n1c), prow += ld) {
        dfa::acc v{0.f, 0.f};
        float2 ey[NC > 0 ? NC : 1];  // this atom's E values, in flight during the real-space loop
        if (NC > 0 && valid && (parts & 2)) {
#pragma unroll
            for (int n = 0; n < (NC > 0 ? NC : 1); ++n) ey[n] = erow[n];
        }
        if (parts & 1) {  // every lane runs the loop (a lane past the end repeats the tile's first point)
            const float4 *ih = img_hi + a * scap, *il = img_lo + a * scap;
            const int nc = ncand[a];
            float acc32 = 0.f;
            // Branch-free over the candidates: most of them are inside the cutoff for some lane of
            // the warp, so the term is computed for all and selected.  Images whose decision needs
            // FP64 (within the band around Rc, or on top of the point) are skipped here and taken
            // in a second pass, which a warp runs only when one of its lanes met one.  (A per-warp
            // ballot mask over the tile's candidates, which skips images out of the warp's reach,
            // measured 3 % more instructions: the mask costs more than the images it drops.)
            bool spec_any = false;
            for (int c = 0; c < nc; ++c) {
                const float4 h = ih[c], lo = il[c];
                const float hx = gh[0] - h.x, hy = gh[1] - h.y, hz = gh[2] - h.z;
                const float dx = hx + (gl[0] - lo.x), dy = hy + (gl[1] - lo.y), dz = hz + (gl[2] - lo.z);
                const float r2 = dx * dx + dy * dy + dz * dz;
                const bool ok = r2 >= fp64_below && r2 <= rcc - band;
                spec_any |= !ok && r2 <= rcc + band;
                const float rinv = rsqrt_ftz(r2);
                const float t = fmaf(erfc_nr2(saf * (r2 * rinv)), rinv, acc32);
                acc32 = ok ? t : acc32;
            }
            if (__any_sync(0xffffffffu, spec_any)) {
                float x64h = 0.f, x64l = 0.f;  // rare FP64 terms, folded in as double-float pairs
                for (int c = 0; c < nc; ++c) {
                    const float4 h = ih[c], lo = il[c];
                    const float hx = gh[0] - h.x, hy = gh[1] - h.y, hz = gh[2] - h.z;
                    const float dx = hx + (gl[0] - lo.x), dy = hy + (gl[1] - lo.y), dz = hz + (gl[2] - lo.z);
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (!(r2 < fp64_below || (r2 > rcc - band && r2 <= rcc + band))) continue;
                    float th, tl;
                    const int dec = fp64_pair(axis, i, j, l, atoms + 3 * (a0 + a), shifts, __float_as_int(h.w),
                                              zero_idx, rc, sa, r2 < fp64_below, th, tl);
                    if (dec == 1) {  // inside the cutoff: the FP32 term
                        const float rinv = rsqrt_ftz(r2);
                        acc32 = fmaf(erfc_nr2(saf * (r2 * rinv)), rinv, acc32);
                    } else if (dec == 2) {  // a point on top of an image: the large term in FP64
                        float s2, e2;
                        dfa::two_sum(x64h, th, s2, e2);
                        x64h = s2;
                        x64l = __fadd_rn(x64l, __fadd_rn(e2, tl));
                    }
                }
                float s_, e_;
                dfa::two_sum(acc32, x64h, s_, e_);
                v.s = s_;
                v.e = __fadd_rn(e_, x64l);
            } else {
                v.s = acc32;
            }
        }
        if (valid && (parts & 2)) {  // stage C: Re sum_n1 ex[n1][i] E[row][a][n1]
            float rs = 0.f;
            if (NC > 0) {
#pragma unroll
                for (int n = 0; n < (NC > 0 ? NC : 1); ++n) {
                    const float2 x = exs[n * kPhiPts + threadIdx.x];
                    rs = fmaf(x.x, ey[n].x, rs);
                    rs = fmaf(-x.y, ey[n].y, rs);
                }
            } else {
                for (int n = 0; n < n1c; ++n) {
                    const float2 x = exs[n * kPhiPts + threadIdx.x], y = erow[n];
                    rs = fmaf(x.x, y.x, rs);
                    rs = fmaf(-x.y, y.y, rs);
                }
            }
            float s_, e_;
            dfa::two_sum(v.s, rs, s_, e_);
            v.s = s_;
            v.e = __fadd_rn(v.e, e_);
        }
        const float2 out = dfa::norm(v);
        if (DIG) {
            int I = 0;
            if (valid) I = x_fixed(out.x, out.y, dg.scale[a0 + a], dg.clamped);
            const long long rs = warp_sum_fixed(I);
            if (lane == 0) wrow[warp][a] = rs;
            if (m < dg.rows_kpad) digits4(I, dg.X0, dg.X1, dg.X2, dg.X3, (long long)(a0 + a) * dg.ldx + m);
        } else if (valid) {
            *prow = out;
        }
        if (!DIG && psum) {  // column statistics for the centre and the scale: FP32 is enough (any
                     // centre is corrected exactly; the max is exact)
            float sh = valid ? out.x : 0.f, mx = valid ? fabsf(out.x) : 0.f;
            for (int o = 16; o > 0; o >>= 1) {
                sh += __shfl_xor_sync(0xffffffffu, sh, o);
                mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            }
            if (lane == 0) {
                wsum[warp][a] = sh;
                wmax[warp][a] = mx;
            }
        }
    }
    if (DIG) {
        // the ESP row, from the CTAs of the first atom block
        if (blockIdx.y == 0) {
            int I = 0;
            if (valid) {
                const double v = dg.Vc[m];
                const float h = (float)v;
                I = x_fixed(h, (float)(v - (double)h), vscale_of(*dg.vmax_p), dg.clamped);
            }
            const long long rs = warp_sum_fixed(I);
            if (lane == 0) wrow[warp][AT] = rs;
            if (m < dg.rows_kpad) digits4(I, dg.X0, dg.X1, dg.X2, dg.X3, (long long)dg.N * dg.ldx + m);
        }
        __syncthreads();
        // exact row sums (two's complement int64 atomics: order-independent), one per CTA and row
        if (threadIdx.x < na || (blockIdx.y == 0 && threadIdx.x == AT)) {
            const int a = threadIdx.x;
            long long t = 0;
            for (int w = 0; w < kPhiPts / 32; ++w) t += wrow[w][a];
            if (t != 0) atomicAdd(dg.rowsum + (a == AT ? dg.N : a0 + a), (unsigned long long)t);
        }
    } else if (psum) {
        __syncthreads();
        if (threadIdx.x < na) {
            const int a = threadIdx.x;
            double s = 0.0;
            float mx = 0.f;
            for (int w = 0; w < kPhiPts / 32; ++w) {
                s += (double)wsum[w][a];
                mx = fmaxf(mx, wmax[w][a]);
            }
            psum[(size_t)(a0 + a) * gridDim.x + blockIdx.x] = s;
            pmax[(size_t)(a0 + a) * gridDim.x + blockIdx.x] = mx;
        }
    }
}

size_t phi_smem_bytes(int n1c, int scap, int at) {
    return sizeof(float4) * 2 * (size_t)at * scap + sizeof(float2) * (size_t)n1c * kPhiPts;
}

// The instantiation for (KMAX 7 or any, digits or staged Phi, atoms per CTA)
using PhiKernel = decltype(&phi_chunk_kernel<7, false, 16>);
template <int AT>
PhiKernel phi_kernel_for(bool regs, bool dig) {
    return dig ? (regs ? phi_chunk_kernel<7, true, AT> : phi_chunk_kernel<0, true, AT>)
               : (regs ? phi_chunk_kernel<7, false, AT> : phi_chunk_kernel<0, false, AT>);
}
PhiKernel phi_kernel(bool regs, bool dig, int at) {
    switch (at) {
        case 8: return phi_kernel_for<8>(regs, dig);
        case 32: return phi_kernel_for<32>(regs, dig);
        default: return phi_kernel_for<16>(regs, dig);
    }
}

void launch_phi(const int32_t *kept, long long m0, long long rows, const double *d_axis, const double *h_axis, int nx, int ny,
                const double *d_atoms, int N, const double *d_shifts, int S, int zero_idx, double rc, double sa,
                const float4 *img, const float4 *EX, const float2 *E, int n1c, int parts, float2 *phit, long long ld,
                double *psum, float *pmax, const PhiDigits *dig, cudaStream_t s, int at) {
    if (at != 8 && at != 32) at = 16;
    RP_REQUIRE(S >= 1 && S <= kMaxShifts, "more than 128 real-space shifts after pruning (cutoff too large for the cell)");
    const int scap = (S + 31) / 32 * 32;
    const bool regs = (n1c == 7);  // KMAX 7: the specialised kernel
    const size_t smem = phi_smem_bytes(n1c, scap, at);
    // the static shared memory (the statistics and row-sum tiles, ~1.3 KB) counts against
    // the same 48 KB default, so the opt-in is raised whenever the dynamic part could cross it
    RP_REQUIRE(smem <= 192 * 1024, "phi kernel: KMAX too large for shared memory");
    auto kern = phi_kernel(regs, dig != nullptr, at);
    smem_optin((const void *)kern, std::max<size_t>(smem, 96 * 1024));
    AxisDF adf;
    for (int q = 0; q < 9; ++q) {
        adf.h[q] = (float)h_axis[q];
        adf.l[q] = (float)(h_axis[q] - (double)adf.h[q]);
    }
    dim3 grd(ceil_div(rows, kPhiPts), ceil_div(N, at));
    const PhiDigits dg = dig ? *dig : PhiDigits{};
    kern<<<grd, kPhiPts, smem, s>>>(kept, m0, rows, d_axis, adf, nx, ny, d_atoms, N, d_shifts, S, scap, zero_idx, rc,
                                    sa, (float)rc, (float)(sa * kSqrtLog2e), real_near2(), img, EX, E, n1c, parts,
                                    phit, ld, psum, pmax, dg);
    RP_LAUNCH_CHECK();
}

// ------------------------------------------------------------------ column statistics and the split

// Per atom (one warp each), on the first chunk: the centre c (the chunk mean, as a
// double-float; cvec holds its exact FP64 value) and the power-of-two scale, from the
// phi kernel's per-CTA partial sums and maxima.  Any centre works: the mean correction
// uses the exact sums of the fixed-point rows (slice_rows_kernel).
__global__ void colstats_finish_kernel(const double *__restrict__ psum, const float *__restrict__ pmax, int nblk,
                                       int N, long long rows, double *__restrict__ c, float2 *__restrict__ cdf,
                                       float *__restrict__ scale) {
    const int a = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (a >= N) return;  // whole warp
    double s = 0.0;
    float mx = 0.f;
    for (int k = lane; k < nblk; k += 32) {
        s += psum[(size_t)a * nblk + k];
        mx = fmaxf(mx, pmax[(size_t)a * nblk + k]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane != 0) return;
    const double mean = s / (double)rows;
    const float ch = (float)mean, cl = (float)(mean - (double)ch);
    cdf[a] = make_float2(ch, cl);
    c[a] = (double)ch + (double)cl;  // the shift actually applied, exactly
    // |Phi - c| <= 2 max|Phi| =: bound in [2^(e-1), 2^e); scale 2^(-e-1) puts |x| below 1/2,
    // so the fixed-point slices stay within |x_s| <= 64 (later chunks: colstats_scale_kernel)
    float bound = 2.f * mx;
    int e = 0;
    if (bound > 0.f) frexpf(bound, &e);
    scale[a] = ldexpf(1.f, -e - 1);
}

// Later chunks of a two-pass fit keep the first chunk's centre c and take a scale of their
// own: |Phi - c| <= 2 max(max|Phi|, |c|) =: bound in [2^(e-1), 2^e), scale 2^(-e-1).  Each
// chunk's Gram tiles and row sums are converted to Phi units with that chunk's scale
// (gram_finish_tiles_kernel, rowsum_flush_kernel), so chunks need not share one.
__global__ void colstats_scale_kernel(const float *__restrict__ pmax, int nblk, int N, const double *__restrict__ c,
                                      float *__restrict__ scale) {
    const int a = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (a >= N) return;  // whole warp
    float mx = 0.f;
    for (int k = lane; k < nblk; k += 32) mx = fmaxf(mx, pmax[(size_t)a * nblk + k]);
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane != 0) return;
    float bound = 2.f * fmaxf(mx, (float)fabs(c[a]) * 1.0001f);
    int e = 0;
    if (bound > 0.f) frexpf(bound, &e);
    scale[a] = ldexpf(1.f, -e - 1);
}

// After each chunk: its exact fixed-point row sums, converted to Phi units with the chunk's
// scales (exact: an int64 below 2^53 times a power of two), are added to sums[Np] and
// the integer sums are cleared for the next chunk.
__global__ void rowsum_flush_kernel(unsigned long long *__restrict__ rowsum, const float *__restrict__ scale,
                                    const double *__restrict__ vmax_p, int N, double *__restrict__ sums) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a > N) return;
    const double sc = a < N ? (double)scale[a] : (double)vscale_of(*vmax_p);
    sums[a] += ldexp((double)(long long)rowsum[a], -27) / sc;
    rowsum[a] = 0ull;
}

constexpr int kSliceThreads = 256;

// X rows: a < N: (Phi_t[a][m] - c_a) * scale_a;  a == N: Vc[m] * scale_V;  rest zero.
// Each value x (|x| <= 1) becomes I = round(x 2^27) and four 7-bit digits
// x ~ 2^-6 (x0 + 2^-7 x1 + 2^-14 x2 + 2^-21 x3), x_s integers in [-64, 64], exact in FP16.
// One thread per two consecutive points of one row (16-B loads, 4-B stores).
__global__ void __launch_bounds__(kSliceThreads) slice_rows_kernel(const float2 *__restrict__ phit, long long ld, long long rows, long long rows_pad,
                                  int N, const float2 *__restrict__ cdf, const float *__restrict__ scale,
                                  const double *__restrict__ Vc, long long m0, const double *__restrict__ vmax_p,
                                  __half *__restrict__ X0, __half *__restrict__ X1, __half *__restrict__ X2,
                                  __half *__restrict__ X3, int *__restrict__ clamped,
                                  unsigned long long *__restrict__ rowsum) {
    const int a = blockIdx.y;  // uniform per CTA: the ESP row and the padding rows branch as a whole
    const long long m = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    int I[2] = {0, 0};
    if (m >= rows_pad) {
        // lanes past the row end only join the shuffle
    } else if (a == N) {
        const float sc = vscale_of(*vmax_p);
        for (int u = 0; u < 2; ++u)
            if (m + u < rows) {
                const double v = Vc[m0 + m + u];
                const float h = (float)v;
                I[u] = x_fixed(h, (float)(v - (double)h), sc, clamped);
            }
    } else if (a < N) {
        const float2 c = cdf[a];
        const float sc = scale[a];
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (m + 1 < rows) v = *reinterpret_cast<const float4 *>(phit + (long long)a * ld + m);
        else if (m < rows) {
            const float2 v0 = phit[(long long)a * ld + m];
            v.x = v0.x;
            v.y = v0.y;
        }
        if (m < rows) {
            const float2 d = df_sub(v.x, v.y, c.x, c.y);
            I[0] = x_fixed(d.x, d.y, sc, clamped);
        }
        if (m + 1 < rows) {
            const float2 d = df_sub(v.z, v.w, c.x, c.y);
            I[1] = x_fixed(d.x, d.y, sc, clamped);
        }
    }
    // exact sum of the row's fixed-point values (two's complement int64 atomics: exact and
    // order-independent, so the mean correction sees exactly the values the Gram sees)
    __shared__ long long wpart[kSliceThreads / 32];
    long long rs = (long long)I[0] + (long long)I[1];
    for (int o = 16; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o);
    if ((threadIdx.x & 31) == 0) wpart[threadIdx.x >> 5] = rs;
    __syncthreads();
    if (threadIdx.x == 0 && a <= N) {
        long long t = 0;
        for (int w = 0; w < kSliceThreads / 32; ++w) t += wpart[w];
        if (t != 0) atomicAdd(rowsum + a, (unsigned long long)t);  // one per CTA and row
    }
    if (m >= rows_pad) return;
    __half d0[2], d1[2], d2[2], d3[2];
    for (int u = 0; u < 2; ++u) digits4(I[u], d0, d1, d2, d3, u);
    const long long idx = (long long)a * rows_pad + m;
    *reinterpret_cast<__half2 *>(X0 + idx) = __halves2half2(d0[0], d0[1]);
    *reinterpret_cast<__half2 *>(X1 + idx) = __halves2half2(d1[0], d1[1]);
    *reinterpret_cast<__half2 *>(X2 + idx) = __halves2half2(d2[0], d2[1]);
    *reinterpret_cast<__half2 *>(X3 + idx) = __halves2half2(d3[0], d3[1]);
}

// The Gram tiles' exact sums (high and low 64-bit halves accumulated by the Gram kernel's
// work units, whatever the points per unit) rounded to FP64 once, (hi 2^32 exactly) + lo after
// normalising lo to [0, 2^32), and added, unscaled, into G (Np x Np).  Tiles inside a
// 128-row block already hold both (a,b) and (b,a); the others are mirrored.
__global__ void gram_finish_tiles_kernel(const unsigned long long *__restrict__ th,
                                         const unsigned long long *__restrict__ tl, int ntj, int Np,
                                         const float *__restrict__ scale, const double *__restrict__ vmax_p, int N,
                                         double *__restrict__ G) {
    const float vscale = vscale_of(*vmax_p);
    const int tile = blockIdx.y;
    int ti, tj;
    gram_tile_decode(tile, ntj, ti, tj);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;  // element in tile, column-major (c*128 + r)
    if (e >= kBM * kGN) return;
    const int c = e / kBM, r = e - c * kBM;
    const int a = ti * kBM + r, b = tj * kGN + c;
    if (a >= Np || b >= Np) return;
    const size_t k = (size_t)tile * (kBM * kGN) + e;
    long long hi = (long long)th[k], lo = (long long)tl[k];
    hi += lo >> 32;  // lo in [0, 2^32), |hi| < 2^53 (the total is below 2^85)
    lo &= 0xffffffffLL;
    double s = (double)hi * 4294967296.0 + (double)lo;
    const double sa = (a < N) ? (double)scale[a] : (double)vscale;
    const double sb = (b < N) ? (double)scale[b] : (double)vscale;
    s = ldexp(s, -54) / (sa * sb);
    G[(size_t)a * Np + b] += s;
    if (tj >= 2 * ti + 2) G[(size_t)b * Np + a] += s;
}

// A = G - s s^T / M, b = G[:, V] - s s_V / M with s the exact column sums of the
// fixed-point rows in Phi units (rowsum_flush_kernel), i.e. repeat.py:2266-2276 for the
// shifted, quantised columns; optionally sum_phi = s + M c.
__global__ void finish_mixed_kernel(const double *__restrict__ G, int Np, const double *__restrict__ sums,
                                    const double *__restrict__ c, long long M, int N, double *__restrict__ A,
                                    double *__restrict__ b, double *__restrict__ sum_phi) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const double invM = 1.0 / (double)M;
    const double sv = sums[N];
    if (t < (long long)N * N) {
        const int i = (int)(t / N), j = (int)(t - (long long)i * N);
        A[t] = G[(size_t)i * Np + j] - sums[i] * sums[j] * invM;
    }
    if (t < N) {
        const double si = sums[t];
        b[t] = G[(size_t)t * Np + N] - si * sv * invM;
        if (sum_phi) sum_phi[t] = si + (double)M * c[t];
    }
}

__global__ void df_to_double_kernel(const float2 *__restrict__ x, long long n, double *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = (double)x[t].x + (double)x[t].y;
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

// 2-D FP16 tensor [rows][cols] (cols contiguous, multiple of 64), box 32 x box_rows, 64-B swizzle
CUtensorMap make_map(const void *ptr, long long rows, long long cols, int box_rows) {
    RP_REQUIRE(cols % kKPad == 0, "tensor map: columns must be a multiple of 64");
    RP_REQUIRE(((uintptr_t)ptr & 15) == 0, "tensor map: base must be 16-byte aligned");
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(RP_E_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

// Work units of a Gram: ntri tiles x ceil(kb_total / kb_per_split) point splits.
int gram_units_total(const GramArgs &g) {
    RP_REQUIRE(g.kb_per_split >= 1 && g.kb_per_split <= kGramSplit && g.flush >= 1 && g.flush <= kGramFlush,
               "gram: bad split");
    const long long u = (long long)g.ntri * ceil_div(g.kb_total, g.kb_per_split);
    RP_REQUIRE(u < (1LL << 30), "gram: too many work units");
    return (int)u;
}
// Units per launch: kGramRounds rounds of one unit per SM.  A larger Gram is cut into launches
// of that size, so that it holds the SMs for well under a millisecond at a time: between two
// launches the block scheduler hands whole SMs to the waiting CTAs of streams of higher
// priority (the small fits of a served stream), which a single persistent launch over a large
// cube's ~10^5 units would keep to the room left beside its CTAs for tens of milliseconds.
constexpr int kGramRounds = 16;
int gram_units_per_launch(const rp_ctx *ctx) { return std::max(1, ctx->sm_count) * kGramRounds; }

// Zeroed tile totals (high and low halves, 2 x ntri x 128 x 64 words) with one work counter
// per launch after them, in one buffer cleared by one memset on the stream
void gram_totals_init(rp_ctx *ctx, const std::string &name, GramArgs &g, cudaStream_t s) {
    const size_t n = (size_t)g.ntri * kBM * kGN;
    const size_t nl = (size_t)ceil_div(gram_units_total(g), gram_units_per_launch(ctx));
    const size_t words = 2 * n + (nl + 1) / 2 + 1;
    unsigned long long *t = ctx->buf_t<unsigned long long>(name, words);
    RP_CUDA(cudaMemsetAsync(t, 0, sizeof(unsigned long long) * words, s));
    g.out_hi = t;
    g.out_lo = t + n;
    g.next_unit = reinterpret_cast<int *>(t + 2 * n);
}

// One CTA per SM (the stages fill most of its shared memory), at most one per work unit;
// launches of at most gram_units_per_launch units, each with its own counter
void launch_gram(rp_ctx *ctx, const __half *const *X, int rows, long long cols, GramArgs g, cudaStream_t s) {
    smem_optin((const void *)gram_exact_kernel, kGramSmem);
    {
        // the SM's whole shared memory as such, so that CTAs of other kernels fit beside this one
        static std::atomic<unsigned long long> carved{0};
        const int dev = ctx->device;
        if (dev >= 0 && dev < 64 && !(carved.load() & (1ULL << dev))) {
            RP_CUDA(cudaFuncSetAttribute((const void *)gram_exact_kernel,
                                         cudaFuncAttributePreferredSharedMemoryCarveout,
                                         (int)cudaSharedmemCarveoutMaxShared));
            carved.fetch_or(1ULL << dev);
        }
    }
    const int total = gram_units_total(g), per = gram_units_per_launch(ctx);
    CUtensorMap a[kGSlices], b[kGSlices];
    for (int q = 0; q < kGSlices; ++q) {
        a[q] = make_map(X[q], rows, cols, kBM);   // rows past `rows` read as zeros
        b[q] = make_map(X[q], rows, cols, kGN);
    }
    int *const counters = g.next_unit;
    for (int k = 0, u0 = 0; u0 < total; ++k, u0 += per) {
        g.unit0 = u0;
        g.nunits = std::min(per, total - u0);
        g.next_unit = counters + k;
        const int grid = std::min(g.nunits, ctx->sm_count > 0 ? ctx->sm_count : 1);
        gram_exact_kernel<<<grid, kGramThreads, kGramSmem, s>>>(a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3], g);
        RP_LAUNCH_CHECK();
    }
}


inline long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

}  // namespace

// Upper bound B_a on |Phi[a][m]| over the kept points, which sets the digit scale of the
// single-pass path (false: an exclusion radius below 0.5 Bohr makes the bound useless).
//   Real space: the filter keeps no point within rn_a (the scaled vdW radius) of an image
//   of atom a, and two images are a lattice vector apart, at least the smallest
//   interplanar spacing d, so at most one image is nearer than d/2; hence
//   sum <= erfc(s rn)/rn + (S - 1) erfc(s d/2)/(d/2), erfc(s x)/x decreasing.
//   Reciprocal space: |sum_k c_k cos(k.r)| <= sum_k |c_k|.
// Should a cell defeat the argument (an image outside the filter's 27 nearest to a
// point), the kernel counts the clamped values and the caller redoes the fit in two passes.
static bool phi_bounds(const rp_ewald *ew, int S, const double *rn, int N, double bound_scale,
                       std::vector<float> &scale) {
    const double *b = ew->box;
    double d = 1e300;
    for (int q = 0; q < 3; ++q) {
        const double *u = b + 3 * ((q + 1) % 3), *v = b + 3 * ((q + 2) % 3), *w = b + 3 * q;
        const double cx = u[1] * v[2] - u[2] * v[1], cy = u[2] * v[0] - u[0] * v[2], cz = u[0] * v[1] - u[1] * v[0];
        const double area = std::sqrt(cx * cx + cy * cy + cz * cz);
        const double vol = std::fabs(w[0] * cx + w[1] * cy + w[2] * cz);
        if (area > 0.0) d = std::min(d, vol / area);
    }
    double rec = 0.0;
    for (double c : ew->kcoef) rec += std::fabs(c);
    const double sa = ew->sqrt_alpha, h = 0.5 * d;
    const double tail = (S > 1 && h > 0.0) ? (S - 1) * std::erfc(sa * h) / h : 0.0;
    scale.resize((size_t)N);
    for (int a = 0; a < N; ++a) {
        if (!(rn[a] >= 0.5)) return false;
        const double B = (std::erfc(sa * rn[a]) / rn[a] + tail + rec) * bound_scale;
        int e = 0;
        std::frexp(B, &e);  // B in [2^(e-1), 2^e): |x| = |Phi| 2^(-e-1) < 1/2
        scale[a] = std::ldexp(1.0f, -e - 1);
    }
    return true;
}

void gram_mixed(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
                const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
                cudaStream_t stream, const double *vstats_dev, const std::string &slot, const double *rn,
                int *clamp_dev, const double *d_atoms_pre, const float2 *E_pre, TileConfig tiles) {
    RP_REQUIRE(N > 0 && M > 0, "rp_gram: need N > 0 and M > 0");
    std::vector<double> sh;
    int zero_idx = -1;
    prune_shifts(ew, atoms, N, sh, zero_idx);
    const int S = (int)(sh.size() / 3);
    RP_REQUIRE(S <= kMaxShifts, "rp_gram: more than 128 real-space shifts after pruning (cutoff too large for the cell)");
    const int nx = ew->grid.n_grid[0], ny = ew->grid.n_grid[1];
    const int n1c = ew->kmax;

    const double *d_atoms = d_atoms_pre;
    if (!d_atoms) {
        double *a = ctx->buf_t<double>("g_atoms" + slot, 3 * (size_t)N);
        RP_CUDA(cudaMemcpyAsync(a, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, stream));
        d_atoms = a;
    }
    double *d_shifts = ctx->buf_t<double>("g_shifts" + slot, sh.size());
    double *d_axis = ctx->buf_t<double>("g_axis" + slot, 9);
    RP_CUDA(cudaMemcpyAsync(d_shifts, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice, stream));
    RP_CUDA(cudaMemcpyAsync(d_axis, ew->grid.axis, sizeof(double) * 9, cudaMemcpyHostToDevice, stream));
    int *d_status = ctx->status_words();  // cleared by the caller (rp_gram / the batch driver)

    // reciprocal rows of every atom (stages A and B; or the caller's, computed for a whole
    // pipeline group) and the double-float images, once per fit
    const float2 *E = E_pre;
    float4 *img = ctx->buf_t<float4>("m_img" + slot, 2 * (size_t)N * S);
    {
        StageTimer tt(ctx, "recip_rows", stream);
        if (!E) {
            float2 *e = ctx->buf_t<float2>("m_E" + slot, recip_rows_bytes(ew, N) / sizeof(float2));
            recip_rows(ctx, ew, d_atoms, nullptr, N, e, stream, slot);
            E = e;
        }
        images_df_kernel<<<ceil_div((long long)N * S, 128), 128, 0, stream>>>(d_atoms, N, d_shifts, S, img);
        RP_LAUNCH_CHECK();
    }

    // chunk the points so the per-chunk staging stays below ~6 GB
    const int Np = N + 1;                       // atoms + the ESP row
    const long long per_point = 8LL * N + 8LL * Np;  // Phi (double-float, two-pass) + four FP16 digits
    long long chunk = std::max<long long>(kBM, ((6LL << 30) / per_point) / kBM * kBM);
    if (ctx->chunk_cap > 0) chunk = std::max<long long>(kBM, std::min<long long>(chunk, ctx->chunk_cap / kBM * kBM));
    chunk = std::min<long long>(chunk, round_up(M, kBM));
    const long long chunk_pad = round_up(chunk, kKPad);

    // single pass: Phi goes straight to digits, scaled by the a-priori bounds, centre 0
    std::vector<float> hscale;
    const bool single = rn && clamp_dev && phi_bounds(ew, S, rn, N, ctx->bound_scale, hscale);
    float2 *phit = single ? nullptr : ctx->buf_t<float2>("m_phit" + slot, (size_t)N * chunk_pad);
    __half *X[kGSlices];
    for (int q = 0; q < kGSlices; ++q) X[q] = ctx->buf_t<__half>("m_X" + slot + std::to_string(q), (size_t)Np * chunk_pad);
    int *d_clamped = ctx->status_words() + 1;  // second status word: fixed-point range overflows
    const int nblk = (int)ceil_div(chunk, kPhiPts);
    double *psum = single ? nullptr : ctx->buf_t<double>("m_psum" + slot, (size_t)N * nblk);
    float *pmax = single ? nullptr : ctx->buf_t<float>("m_pmax" + slot, (size_t)N * nblk);
    unsigned long long *rowsum = ctx->buf_t<unsigned long long>("m_rowsum" + slot, (size_t)Np);
    double *sums = ctx->buf_t<double>("m_sums" + slot, (size_t)Np);
    double *cvec = ctx->buf_t<double>("m_c" + slot, N);
    float2 *cdf = ctx->buf_t<float2>("m_cdf" + slot, N);
    float *scale = ctx->buf_t<float>("m_scale" + slot, N);
    double *G = ctx->buf_t<double>("m_G" + slot, (size_t)Np * Np);
    RP_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * Np * Np, stream));
    RP_CUDA(cudaMemsetAsync(rowsum, 0, sizeof(unsigned long long) * Np, stream));
    RP_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * Np, stream));

    // ESP row scale from max |Vc| (the filter's, or computed here)
    const double *vmax = vstats_dev ? vstats_dev + 1 : nullptr;
    if (!vstats_dev) {
        double *st = ctx->buf_t<double>("m_vmax" + slot, 1);
        absmax_kernel<<<1, 1024, 0, stream>>>(Vc_dev, M, st);
        RP_LAUNCH_CHECK();
        vmax = st;
    }

    if (single) {
        RP_CUDA(cudaMemcpyAsync(scale, hscale.data(), sizeof(float) * N, cudaMemcpyHostToDevice, stream));
        RP_CUDA(cudaMemsetAsync(cvec, 0, sizeof(double) * N, stream));
    }

    const int nt = (int)ceil_div(Np, kBM), ntj = (int)ceil_div(Np, kGN);
    int ntri = 0;  // 128 x 64 Gram tiles with columns at or right of the row block, up to the last row
    for (int ti = 0; ti < nt; ++ti) ntri += ntj - 2 * ti;
    // points per CTA: kGramSplit stages (1024 points, the int64 headroom, exact sums drained
    // once) or fewer, for more CTAs on cubes with few Gram tiles (the autotuner's choice)
    const int kb_split = kStagesPer64 * std::min(std::max(tiles.gram_split, 1), kGramSplit / kStagesPer64);

    for (long long m0 = 0; m0 < M; m0 += chunk) {
        const long long rows = std::min<long long>(chunk, M - m0);
        const long long rows_kpad = round_up(rows, kKPad);
        // 1. Phi of the chunk (real space + reciprocal stage C) and its column statistics
        const int nb = (int)ceil_div(rows, kPhiPts);
        if (single) {  // Phi of the chunk straight to the digits of X
            StageTimer tt(ctx, "phi", stream);
            // the slices' row stride is the chunk's padded length, as the Gram's tensor maps read them
            const PhiDigits dg{X[0], X[1], X[2], X[3], rows_kpad, rows_kpad, scale, Vc_dev + m0, vmax,
                               rowsum, clamp_dev, N};
            launch_phi(kept_idx_dev, m0, rows, d_axis, ew->grid.axis, nx, ny, d_atoms, N, d_shifts, S, zero_idx,
                       ew->cutoff, ew->sqrt_alpha, img, ew->d_exf, E, n1c, 3, nullptr, chunk_pad, nullptr, nullptr,
                       &dg, stream, tiles.phi_atoms);
        } else {
            StageTimer tt(ctx, "phi", stream);
            launch_phi(kept_idx_dev, m0, rows, d_axis, ew->grid.axis, nx, ny, d_atoms, N, d_shifts, S, zero_idx, ew->cutoff,
                       ew->sqrt_alpha, img, ew->d_exf, E, n1c, 3, phit, chunk_pad, psum, pmax, nullptr, stream,
                       tiles.phi_atoms);
        }
        // 2. centre on the first chunk, a scale per chunk, fixed-point digits of X
        if (!single) {
            StageTimer tt(ctx, "center_slice", stream);
            if (m0 == 0) {
                colstats_finish_kernel<<<ceil_div(N, 4), 128, 0, stream>>>(psum, pmax, nb, N, rows, cvec, cdf, scale);
            } else {
                colstats_scale_kernel<<<ceil_div(N, 4), 128, 0, stream>>>(pmax, nb, N, cvec, scale);
            }
            RP_LAUNCH_CHECK();
            slice_rows_kernel<<<dim3(ceil_div(rows_kpad / 2, kSliceThreads), Np), kSliceThreads, 0, stream>>>(
                phit, chunk_pad, rows, rows_kpad, N, cdf, scale, Vc_dev, m0, vmax, X[0], X[1], X[2], X[3], d_clamped,
                rowsum);
            RP_LAUNCH_CHECK();
        }
        // 3. exact Gram tiles (work units over point splits add exactly into the tiles' 64-bit
        //    totals), then the totals rounded once into G
        {
            const int kb_total = (int)(rows_kpad / kBK);
            GramArgs g{};
            g.nt = nt;
            g.ntj = ntj;
            g.ntri = ntri;
            g.kb_total = kb_total;
            g.kb_per_split = kb_split;
            g.flush = kGramFlush;
            g.status = d_status;
            g.budget = ctx->wait_budget;
            gram_totals_init(ctx, "m_tsum" + slot, g, stream);
            const __half *Xq[kGSlices] = {X[0], X[1], X[2], X[3]};
            {
                StageTimer tt(ctx, "gram_exact", stream);
                launch_gram(ctx, Xq, Np, rows_kpad, g, stream);
            }
            StageTimer tr(ctx, "gram_totals", stream);
            gram_finish_tiles_kernel<<<dim3(ceil_div(kBM * kGN, 256), ntri), 256, 0, stream>>>(
                g.out_hi, g.out_lo, ntj, Np, scale, vmax, N, G);
            RP_LAUNCH_CHECK();
            rowsum_flush_kernel<<<ceil_div(Np, 128), 128, 0, stream>>>(rowsum, scale, vmax, N, sums);
            RP_LAUNCH_CHECK();
        }
    }
    finish_mixed_kernel<<<ceil_div(std::max<long long>((long long)N * N, N), 256), 256, 0, stream>>>(
        G, Np, sums, cvec, M, N, A_dev, b_dev, sum_phi_dev);
    RP_LAUNCH_CHECK();
}

// ---------------------------------------------------------------- exact Gram of FP64 columns
// For the escalated (FP64) fit: the columns of a chunk of Phi (rows x N, row-major, ld N,
// centred) and the centred ESP are scaled by powers of two to |x| < 1/2 and cut into two
// 28-bit words, x = 2^-27 (I1 + 2^-27 I2) + O(2^-55); the 2(N+1) rows [I1 of every column;
// I2 of every column] go through the exact digit Gram (every digit product exact, tile
// totals exact, one FP64 rounding), and
//   G[a][b] += (G11 + 2^-27 (G12 + G21) + 2^-54 G22)[a][b] / (s_a s_b)
// with the ESP as column N (G[a][N] = (Phi^T V)[a]).  An FP64-accurate Gram from the
// tensor cores: 4x the work of the mixed path's Gram, instead of DSYRK at the FP64 rate.
namespace {

// max |x| of each column (N of Phi, then the ESP as column N), as order-preserving bits
__global__ void colmax_fp64_kernel(const double *__restrict__ P, long long rows, int N, const double *__restrict__ V,
                                   unsigned long long *__restrict__ mx) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > N) return;
    const long long r0 = (long long)blockIdx.y * 256, r1 = min(rows, r0 + 256);
    double m = 0.0;
    for (long long r = r0; r < r1; ++r) m = fmax(m, fabs(c < N ? P[r * N + c] : V[r]));
    atomicMax(mx + c, (unsigned long long)__double_as_longlong(m));  // m >= 0: bits order like values
}

__device__ __forceinline__ double pow2_scale(unsigned long long mbits) {
    const double m = __longlong_as_double((long long)mbits);
    int e = 0;
    if (m > 0.0) frexp(m, &e);  // m in [2^(e-1), 2^e): m 2^(-e-1) < 1/2
    return ldexp(1.0, -e - 1);
}

// two 28-bit words of each value, as four 7-bit digits each: column c < N and the ESP
// (c = N) to rows c and c + N + 1 of the slices; a 32 x 32 tile per CTA through shared
// memory, so both the reads of Phi and the writes of the slices coalesce
__global__ void split_words_kernel(const double *__restrict__ P, long long rows, long long cols_pad, int N,
                                   const double *__restrict__ V, const unsigned long long *__restrict__ mx,
                                   __half *__restrict__ X0, __half *__restrict__ X1, __half *__restrict__ X2,
                                   __half *__restrict__ X3) {
    __shared__ double t[32][33];
    const long long m0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {  // t[point][column]
        const long long m = m0 + k;
        const int c = c0 + threadIdx.x;
        double v = 0.0;
        if (m < rows && c <= N) v = c < N ? P[m * N + c] : V[m];
        t[k][threadIdx.x] = v;
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {  // column c0 + k, point m0 + x
        const int c = c0 + k;
        const long long m = m0 + threadIdx.x;
        if (c > N || m >= cols_pad) continue;
        const double x = t[threadIdx.x][k] * pow2_scale(mx[c]) * 134217728.0;  // |x| < 2^26
        const double i1 = rint(x);
        const double i2 = rint((x - i1) * 134217728.0);                          // |x - i1| <= 1/2
        digits4((int)i1, X0, X1, X2, X3, (long long)c * cols_pad + m);
        digits4((int)i2, X0, X1, X2, X3, (long long)(c + N + 1) * cols_pad + m);
    }
}

// G2 (2(N+1) square, row-major) = 2^-54 x the exact tile totals: Gram of the word rows
__global__ void words_gram_kernel(const unsigned long long *__restrict__ th, const unsigned long long *__restrict__ tl,
                                  int ntj, int Np2, double *__restrict__ G2) {
    const int tile = blockIdx.y;
    int ti, tj;
    gram_tile_decode(tile, ntj, ti, tj);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= kBM * kGN) return;
    const int c = e / kBM, r = e - c * kBM;
    const int a = ti * kBM + r, b = tj * kGN + c;
    if (a >= Np2 || b >= Np2) return;
    const size_t k = (size_t)tile * (kBM * kGN) + e;
    long long hi = (long long)th[k], lo = (long long)tl[k];
    hi += lo >> 32;
    lo &= 0xffffffffLL;
    const double s = ldexp((double)hi * 4294967296.0 + (double)lo, -54);
    G2[(size_t)a * Np2 + b] = s;
    G2[(size_t)b * Np2 + a] = s;
}

// G[a][b] (N x N, either order: symmetric) and r[a] (b = N) += the combined words / (s_a s_b)
__global__ void combine_words_kernel(const double *__restrict__ G2, int N, const unsigned long long *__restrict__ mx,
                                     double *__restrict__ G, double *__restrict__ r) {
    const int Np = N + 1, Np2 = 2 * Np;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * Np) return;
    const int a = (int)(t / Np), b = (int)(t - (long long)a * Np);
    const double g11 = G2[(size_t)a * Np2 + b], g12 = G2[(size_t)a * Np2 + Np + b];
    const double g21 = G2[(size_t)(Np + a) * Np2 + b], g22 = G2[(size_t)(Np + a) * Np2 + Np + b];
    const double v = (g11 + 7.450580596923828125e-9 * (g12 + g21) + 5.5511151231257827e-17 * g22) /
                     (pow2_scale(mx[a]) * pow2_scale(mx[b]));
    if (b < N) G[(size_t)a * N + b] += v;
    else r[a] += v;
}

}  // namespace

void gram_words_fp64(rp_ctx *ctx, const double *P, long long rows, int N, const double *V, double *G, double *r,
                     cudaStream_t stream) {
    const int Np = N + 1, Np2 = 2 * Np;
    const long long cols_pad = round_up(rows, kKPad);
    unsigned long long *mx = ctx->buf_t<unsigned long long>("w64_mx", (size_t)Np);
    RP_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * Np, stream));
    colmax_fp64_kernel<<<dim3(ceil_div(Np, 256), ceil_div(rows, 256)), 256, 0, stream>>>(P, rows, N, V, mx);
    RP_LAUNCH_CHECK();
    __half *X[kGSlices];
    for (int q = 0; q < kGSlices; ++q) X[q] = ctx->buf_t<__half>("w64_X" + std::to_string(q), (size_t)Np2 * cols_pad);
    split_words_kernel<<<dim3(ceil_div(cols_pad, 32), ceil_div(Np, 32)), dim3(32, 8), 0, stream>>>(
        P, rows, cols_pad, N, V, mx, X[0], X[1], X[2], X[3]);
    RP_LAUNCH_CHECK();
    const int nt = (int)ceil_div(Np2, kBM), ntj = (int)ceil_div(Np2, kGN);
    int ntri = 0;
    for (int ti = 0; ti < nt; ++ti) ntri += ntj - 2 * ti;
    const int kb_total = (int)(cols_pad / kBK);
    RP_CUDA(cudaMemsetAsync(ctx->status_words(), 0, sizeof(int), stream));
    GramArgs g{};
    g.nt = nt;
    g.ntj = ntj;
    g.ntri = ntri;
    g.kb_total = kb_total;
    g.kb_per_split = kGramSplit;
    g.flush = kGramFlush;
    g.status = ctx->status_words();
    g.budget = ctx->wait_budget;
    gram_totals_init(ctx, "w64_tsum", g, stream);
    const __half *Xq[kGSlices] = {X[0], X[1], X[2], X[3]};
    launch_gram(ctx, Xq, Np2, cols_pad, g, stream);
    double *G2 = ctx->buf_t<double>("w64_G2", (size_t)Np2 * Np2);
    words_gram_kernel<<<dim3(ceil_div(kBM * kGN, 256), ntri), 256, 0, stream>>>(g.out_hi, g.out_lo, ntj, Np2, G2);
    RP_LAUNCH_CHECK();
    combine_words_kernel<<<ceil_div((long long)N * Np, 256), 256, 0, stream>>>(G2, N, mx, G, r);
    RP_LAUNCH_CHECK();
    status_check(ctx, stream);
}

}  // namespace rp

// Diagnostics (not part of the public ABI): a factor on the single-pass Phi bounds of
// the batched fit (1 = the analytic bounds).  A factor far below 1 makes every cube clamp
// and fall back to the two-pass fit, which a test compares with the normal path.
extern "C" int rp_debug_bound_scale(rp_ctx *ctx, double factor) {
    if (!ctx || !(factor > 0.0)) return RP_E_ARG;
    ctx->bound_scale = factor;
    return RP_OK;
}

// Diagnostics (not part of the public ABI): the clock budget of the Gram pipeline's waits
// (cycles < 0: the default, ~2 s; 0: every wait gives up at once, which exercises the
// timeout path: RP_E_TIMEOUT, the kernel unwinds, the ctx stays usable).
extern "C" int rp_debug_wait_budget(rp_ctx *ctx, long long cycles) {
    if (!ctx) return RP_E_ARG;
    ctx->wait_budget = cycles < 0 ? rp::tc::kWaitBudgetCycles : cycles;
    return RP_OK;
}

// Diagnostics (not part of the public ABI): an upper bound on the kept points per chunk of
// the staged mixed Gram (0 = the memory-based size), so tests can run many chunks on a
// small cube.
extern "C" int rp_debug_chunk_cap(rp_ctx *ctx, long long points) {
    if (!ctx || points < 0) return RP_E_ARG;
    ctx->chunk_cap = points;
    return RP_OK;
}

// Diagnostics: how many cubes of the last batched fit were redone in two passes.
extern "C" int rp_debug_last_fallbacks(const rp_ctx *ctx) { return ctx ? ctx->last_fallbacks : RP_E_ARG; }

namespace rp {
namespace {
__global__ void erfc_kernel(const float *__restrict__ x, long long n, float *__restrict__ out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = erfc_nr2((float)kSqrtLog2e * x[t]);
}
}  // namespace
}  // namespace rp

// Diagnostics (not part of the public ABI): the real-space kernels' FP32 erfc at n
// arguments x (device arrays), for the test against FP64 erfc and CUDA's erfcf.
extern "C" int rp_debug_erfc(const float *x_dev, long long n, float *out_dev) {
    using namespace rp;
    if (!x_dev || !out_dev || n < 0) return RP_E_ARG;
    if (n == 0) return RP_OK;
    erfc_kernel<<<(unsigned)((n + 255) / 256), 256>>>(x_dev, n, out_dev);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return RP_E_CUDA;
    return RP_OK;
}

// Diagnostics (not part of the public ABI): the mixed path's Phi for the first
// `rows` kept points, atom-major [N][rows]; parts = 1 real space, 2 reciprocal,
// 3 both.  Used to check each part against FP64 separately.
extern "C" int rp_debug_mixed_phi(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N,
                                  const int32_t *kept_idx_dev, int64_t rows, int parts, double *phi_dev) {
    using namespace rp;
    try {
        RP_CUDA(cudaSetDevice(ctx->device));
        RP_REQUIRE(N > 0 && rows > 0 && rows <= (1LL << 30) && parts >= 1 && parts <= 3, "bad arguments");
        std::vector<double> sh;
        int zero_idx = -1;
        prune_shifts(ew, atoms, N, sh, zero_idx);
        const int S = (int)(sh.size() / 3);
        double *d_atoms = ctx->buf_t<double>("g_atoms", 3 * (size_t)N);
        double *d_shifts = ctx->buf_t<double>("g_shifts", sh.size());
        double *d_axis = ctx->buf_t<double>("g_axis", 9);
        RP_CUDA(cudaMemcpy(d_atoms, atoms, sizeof(double) * 3 * N, cudaMemcpyHostToDevice));
        RP_CUDA(cudaMemcpy(d_shifts, sh.data(), sizeof(double) * sh.size(), cudaMemcpyHostToDevice));
        RP_CUDA(cudaMemcpy(d_axis, ew->grid.axis, sizeof(double) * 9, cudaMemcpyHostToDevice));
        float2 *E = ctx->buf_t<float2>("m_E", recip_rows_bytes(ew, N) / sizeof(float2));
        float4 *img = ctx->buf_t<float4>("m_img", 2 * (size_t)N * S);
        recip_rows(ctx, ew, d_atoms, nullptr, N, E, 0);
        images_df_kernel<<<ceil_div((long long)N * S, 128), 128>>>(d_atoms, N, d_shifts, S, img);
        RP_LAUNCH_CHECK();
        float2 *ph = ctx->buf_t<float2>("dbg_phi", (size_t)N * rows);
        launch_phi(kept_idx_dev, 0, rows, d_axis, ew->grid.axis, ew->grid.n_grid[0], ew->grid.n_grid[1], d_atoms, N, d_shifts, S,
                   zero_idx, ew->cutoff, ew->sqrt_alpha, img, ew->d_exf, E, ew->kmax, parts, ph, rows, nullptr,
                   nullptr, nullptr, 0, kPhiAtoms);
        df_to_double_kernel<<<ceil_div((long long)N * rows, 256), 256>>>(ph, (long long)N * rows, phi_dev);
        RP_LAUNCH_CHECK();
        RP_CUDA(cudaDeviceSynchronize());
        return RP_OK;
    } catch (const rp::Error &e) {
        ctx->last_error = e.msg;
        return e.code;
    }
}

// Diagnostics: the exact-Gram kernel on caller-provided FP16 slices X0 .. X3
// ([Np_pad][cols], cols a multiple of 64) -> 2^-54 * sum over points and all sixteen
// slice products of x_s y_u 2^(7(6-s-u)) (FP64, Np x Np).
extern "C" int rp_debug_gram_slices(rp_ctx *ctx, const void *X0, const void *X1, const void *X2, const void *X3,
                                    int Np, long long cols, int flush, int kb_split, double *I_dev) {
    using namespace rp;
    try {
        RP_CUDA(cudaSetDevice(ctx->device));
        const int nt = (int)ceil_div(Np, kBM), ntj = (int)ceil_div(Np, kGN);
        int ntri = 0;
        for (int ti = 0; ti < nt; ++ti) ntri += ntj - 2 * ti;
        const int kb_total = (int)(cols / kBK);
        // flush and kb_split count 64-point blocks (the padding unit): two stages each
        RP_REQUIRE(kb_split >= 1 && kb_split * kStagesPer64 <= kGramSplit, "kb_split must lie in [1, 16]");
        RP_CUDA(cudaMemset(ctx->d_status, 0, sizeof(int)));
        GramArgs g{};
        g.nt = nt; g.ntj = ntj; g.ntri = ntri; g.kb_total = kb_total; g.kb_per_split = kb_split * kStagesPer64;
        g.flush = kStagesPer64 * std::min(std::max(flush, 1), kGramFlush / kStagesPer64);
        g.status = ctx->d_status; g.budget = ctx->wait_budget;
        gram_totals_init(ctx, "dbg_tsum", g, 0);
        const __half *Xq[kGSlices] = {(const __half *)X0, (const __half *)X1, (const __half *)X2, (const __half *)X3};
        launch_gram(ctx, Xq, Np, cols, g, 0);
        float *ones = ctx->buf_t<float>("dbg_ones", Np);
        std::vector<float> h((size_t)Np, 1.0f);
        RP_CUDA(cudaMemcpy(ones, h.data(), sizeof(float) * Np, cudaMemcpyHostToDevice));
        RP_CUDA(cudaMemset(I_dev, 0, sizeof(double) * Np * Np));
        double *vmax = ctx->buf_t<double>("dbg_vmax", 1);  // unused: every row is an atom row (N = Np)
        RP_CUDA(cudaMemset(vmax, 0, sizeof(double)));
        gram_finish_tiles_kernel<<<dim3(ceil_div(kBM * kGN, 256), ntri), 256>>>(g.out_hi, g.out_lo, ntj, Np, ones,
                                                                               vmax, Np, I_dev);
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

