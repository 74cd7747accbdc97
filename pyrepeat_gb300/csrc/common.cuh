// Internal definitions shared by the translation units of librepeat_gb300.
#pragma once

#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <condition_variable>
#include <deque>
#include <exception>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "repeat_gb300.h"

namespace rp {

// Thrown inside the library and turned into a status code at the C boundary.
struct Error {
    int code;
    std::string msg;
};

[[noreturn]] inline void fail(int code, const std::string &msg) { throw Error{code, msg}; }

#define RP_CUDA(call)                                                                       \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            ::rp::fail(RP_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

#define RP_CUBLAS(call)                                                                     \
    do {                                                                                    \
        cublasStatus_t s_ = (call);                                                         \
        if (s_ != CUBLAS_STATUS_SUCCESS)                                                    \
            ::rp::fail(RP_E_CUDA, std::string(#call) + ": cublas status " + std::to_string((int)s_)); \
    } while (0)

#define RP_REQUIRE(cond, msg)                                                               \
    do {                                                                                    \
        if (!(cond)) ::rp::fail(RP_E_ARG, msg);                                             \
    } while (0)

// Kernel launches issued by the library (read with rp_launch_count).
extern std::atomic<long long> g_launches;

// Check a kernel launch (configuration errors surface here, not later) and count it.
#define RP_LAUNCH_CHECK()                     \
    do {                                      \
        ::rp::g_launches.fetch_add(1);        \
        RP_CUDA(cudaGetLastError());          \
    } while (0)

struct Buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace rp

// Host worker threads owned by a context, started on first use: run(n, f) calls f(i) for
// i in [0, n) on the workers and the calling thread (the cubes of a batch are independent)
// and returns when all are done, rethrowing the first exception.  No thread is created per
// batch, and the per-cube host work (filter plans, Ewald tables) is spread over the cores.
namespace rp {
struct FilterPlan;

// Queue and worker thread of the asynchronous batches (rp_batch_submit / poll / wait).
struct BatchServer {
    struct Job {
        long long ticket = 0;
        std::vector<rp_fit_desc> descs;
        std::vector<const double *> vdev;
        bool has_vdev = false;
        double *q_out = nullptr;
        int64_t *M_out = nullptr;
        double *info_out = nullptr;
    };
    std::thread th;
    std::mutex mu;
    std::condition_variable cv, finished;
    std::deque<Job> queue;
    std::set<long long> pending;                                   // submitted, not yet retired
    std::unordered_map<long long, std::pair<int, std::string>> done;  // ticket -> status, message
    long long next = 1;
    bool stop = false;
};

class HostPool {
  public:
    explicit HostPool(int workers) {
        for (int t = 0; t < workers; ++t) th_.emplace_back([this] { loop(); });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &t : th_) t.join();
    }
    void run(int n, const std::function<void(int)> &f) {
        if (n <= 0) return;
        if (th_.empty() || n == 1) {
            for (int i = 0; i < n; ++i) f(i);
            return;
        }
        {
            std::lock_guard<std::mutex> g(mu_);
            job_ = &f;
            count_ = n;
            next_.store(0);
            err_ = nullptr;
            pending_ = (int)th_.size();
            ++gen_;
        }
        cv_.notify_all();
        drain();
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return pending_ == 0; });  // every worker is past this job
        job_ = nullptr;
        if (err_) {
            std::exception_ptr e = err_;
            err_ = nullptr;
            lk.unlock();
            std::rethrow_exception(e);
        }
    }

  private:
    void loop() {
        long long seen = 0;
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
            if (stop_) return;
            seen = gen_;
            lk.unlock();
            drain();
            lk.lock();
            if (--pending_ == 0) done_.notify_all();
        }
    }
    void drain() {
        for (int i = next_.fetch_add(1); i < count_; i = next_.fetch_add(1)) {
            try {
                (*job_)(i);
            } catch (...) {
                std::lock_guard<std::mutex> g(mu_);
                if (!err_) err_ = std::current_exception();
            }
        }
    }
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int)> *job_ = nullptr;
    std::atomic<int> next_{0};
    int count_ = 0, pending_ = 0;
    long long gen_ = 0;
    bool stop_ = false;
    std::exception_ptr err_;
};

}  // namespace rp

// Default limit on kappa / (n+1), kappa = ||A||_1 ||K^-1||_1 of the bordered system of n+1
// unknowns, above which a mixed-precision fit is redone in FP64.  The mixed Gram's relative
// error is ~1e-7, and on 30 seeded cubes of 9 to 2000 atoms the mixed charges moved from the
// FP64 ones by about 2e-11 kappa/(n+1) e (kappa/(n+1) from 1e3 to 3e6, within 3x): the limit
// keeps that below ~4e-6 e.  (Beyond ~1e8 the error saturates near 0.1-1 e.)
constexpr double kDefaultKappaLimit = 2e5;

namespace rp {
// Tile shapes of the mixed-precision normal equations: atoms per CTA of the Phi kernel (8, 16
// or 32) and Gram points per work unit, in blocks of 64 (up to 16).  Neither changes a result: every
// Phi value and every exact digit sum is the same whatever the tiling.
struct TileConfig {
    int phi_atoms = 16;
    int gram_split = 16;
};
// The autotuner's bucket of a fit: atoms, kept points, KMAX.
inline long long tile_key(int N, long long M, int kmax) {
    const int nb = N < 32 ? 0 : N < 64 ? 1 : N < 128 ? 2 : N < 256 ? 3 : N < 512 ? 4 : 5;
    const int mb = M < 32768 ? 0 : M < 131072 ? 1 : M < 524288 ? 2 : 3;
    return ((long long)nb * 4 + mb) * 64 + std::min(std::max(kmax, 0), 63);
}
// Batches of the asynchronous server in flight at once.  Each runs in a slot of the ctx with
// its own scratch (names carry the slot), pinned staging, streams, status words, cuBLAS
// handle and host object pools; slot 0 is also what rp_fit_batch and the staged calls use.
constexpr int kBatchSlots = 3;
// streams of a slot: 4 for normal equations, 4 for filters, uploads, the pipeline groups'
// reciprocal rows, and the batch's own stream (the server's)
constexpr int kLaneFilter0 = 4, kLaneCopy = 8, kLaneRecip = 9, kLaneBatch = 10;
constexpr int kSlotLanes = 11;
// A served batch whose largest cube has at least this many grid points x atoms runs on
// streams of the default (lowest) priority, every other served batch on streams of the
// device's greatest priority: the block scheduler then hands free SMs to a small request's
// kernels before the pending blocks of a large cube's, so small requests are not held
// behind large ones.
constexpr double kLowPriorityWork = 1e9;
}  // namespace rp

struct rp_ctx {
    int device = 0;
    int sm_count = 0;
    size_t budget = 0;
    size_t used = 0;
    std::string last_error;
    cublasHandle_t cublas[rp::kBatchSlots] = {};
    cusolverDnHandle_t cusolver[rp::kBatchSlots] = {};  // FP64 factorisations of wide systems
    std::unordered_map<std::string, rp::Buffer> scratch;
    int *d_status = nullptr;  // device status words (two per slot) for bounded waits / clamps
    // The slot the calling code runs in.  Set by the one thread that uses the ctx at a time
    // (the caller, or the batch server's worker while tickets are outstanding); scratch,
    // staging, streams, status words and the cuBLAS handle below all follow it.
    int cur_slot = 0;
    int cur_prio = 0;  // streams of the current batch: 0 default priority, 1 the greatest
    std::string slot_key(const std::string &name) const {
        return cur_slot == 0 ? name : name + "@" + std::to_string(cur_slot);
    }
    int *status_words() const { return d_status + 2 * cur_slot; }
    // optional per-stage CUDA-event timing (rp_set_timing / rp_stage_times)
    bool timing = false;
    struct Mark {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Mark> marks;

    // Grow-only named scratch buffer owned by the ctx (one per name and slot).
    void *buf(const std::string &name_in, size_t bytes) {
        const std::string name = slot_key(name_in);
        bytes = (bytes + 255) & ~size_t(255);
        if (bytes == 0) bytes = 256;
        auto &b = scratch[name];
        if (b.bytes >= bytes) return b.ptr;
        if (b.ptr) {
            cudaDeviceSynchronize();  // queued work may still read the old buffer
            cudaFree(b.ptr);
            used -= b.bytes;
            b.ptr = nullptr;
            b.bytes = 0;
        }
        if (used + bytes > budget)
            rp::fail(RP_E_NOMEM, "scratch '" + name + "' of " + std::to_string(bytes) +
                                     " B exceeds the ctx HBM budget (" + std::to_string(budget - used) +
                                     " B left)");
        cudaError_t e = cudaMalloc(&b.ptr, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            rp::fail(RP_E_NOMEM, "cudaMalloc(" + std::to_string(bytes) + ") failed: " + cudaGetErrorString(e));
        }
        b.bytes = bytes;
        used += bytes;
        return b.ptr;
    }
    template <class T>
    T *buf_t(const std::string &name, size_t count) {
        return static_cast<T *>(buf(name, count * sizeof(T)));
    }
    // Grow-only pinned host staging buffer (one H2D copy per batch instead of many
    // small pageable ones); callers synchronise their stream before it is reused.
    std::unordered_map<std::string, rp::Buffer> host_scratch;
    double bound_scale = 1.0;  // factor on the single-pass Phi bounds (tests shrink it to force clamps)
    long long chunk_cap = 0;   // cap on the staged mixed Gram's points per chunk (tests; 0 = none)
    long long wait_budget = 4000000000LL;  // clock budget of the Gram pipeline's waits (tests shorten it)
    std::unique_ptr<rp::HostPool> pool;  // host workers (created on first use)
    std::unique_ptr<rp::BatchServer> server;  // asynchronous batches (created on first submit)
    // per-cube host objects of the batched fit, kept across batches for their capacity (per slot)
    std::vector<std::unique_ptr<rp_ewald>> ew_pool[rp::kBatchSlots];
    std::vector<std::unique_ptr<rp::FilterPlan>> plan_pool[rp::kBatchSlots];
    void parallel(int n, const std::function<void(int)> &f) {
        if (!pool) {
            const int hw = std::max(1, (int)std::thread::hardware_concurrency());
            pool.reset(new rp::HostPool(std::min(16, hw) - 1));
        }
        pool->run(n, f);
    }
    // host-side timeline of the batched fit (rp_debug_trace): phase labels and host times,
    // for finding where the host waits; off by default
    bool trace = false;
    std::vector<std::pair<std::string, double>> trace_log;
    void trace_mark(const std::string &label) {
        if (!trace) return;
        const double t = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
        std::lock_guard<std::mutex> lk(trace_mu);
        trace_log.emplace_back(label, t);
    }
    std::mutex trace_mu;
    int last_fallbacks = 0;    // cubes of the last batch redone in two passes after a clamp
    int last_escalations = 0;  // mixed-precision cubes of the last batch refitted in FP64
    // mixed-precision fits whose kappa / (n+1) (the solve's ||A||_1 ||K^-1||_1 over the
    // bordered system's unknowns) exceeds this are refitted in plain FP64
    // (rp_set_kappa_limit; 0 = never)
    double kappa_limit = kDefaultKappaLimit;
    // tile shapes per autotuner bucket (rp_autotune / rp_load_tiles); absent: the defaults
    std::map<long long, rp::TileConfig> tiles;
    rp::TileConfig tiles_for(int N, long long M, int kmax) const {
        auto it = tiles.find(rp::tile_key(N, M, kmax));
        return it == tiles.end() ? rp::TileConfig{} : it->second;
    }
    void *host_buf(const std::string &name_in, size_t bytes) {
        const std::string name = slot_key(name_in);
        bytes = std::max<size_t>(256, (bytes + 255) & ~size_t(255));
        auto &b = host_scratch[name];
        if (b.bytes >= bytes) return b.ptr;
        if (b.ptr) cudaFreeHost(b.ptr);
        b.ptr = nullptr;
        b.bytes = 0;
        cudaError_t e = cudaMallocHost(&b.ptr, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            rp::fail(RP_E_NOMEM, "cudaMallocHost(" + std::to_string(bytes) + ") failed: " + cudaGetErrorString(e));
        }
        b.bytes = bytes;
        return b.ptr;
    }
    cublasHandle_t blas();  // the current slot's handle
    cusolverDnHandle_t solver();  // the current slot's cuSOLVER handle
    // Worker streams for fits that run concurrently inside one batch (created on first use,
    // non-blocking, destroyed with the ctx): lane i of the current slot.
    std::vector<cudaStream_t> lanes;
    cudaStream_t lane(int i_in) {
        const int i = i_in + rp::kSlotLanes * (cur_slot + rp::kBatchSlots * cur_prio);
        while ((int)lanes.size() <= i) {
            const bool high = (int)lanes.size() >= rp::kSlotLanes * rp::kBatchSlots;
            int least = 0, greatest = 0;
            if (high) cudaDeviceGetStreamPriorityRange(&least, &greatest);
            cudaStream_t st = nullptr;
            cudaError_t e = cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, high ? greatest : 0);
            if (e != cudaSuccess) rp::fail(RP_E_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
            lanes.push_back(st);
        }
        return lanes[i];
    }
};

struct rp_ewald {
    int device = 0;
    rp_grid grid{};
    double cutoff = 20.0, alpha = 0.0, sqrt_alpha = 0.0, volume = 0.0;
    double box[9]{};
    double rec[9]{};  // reciprocal basis b1, b2, b3 (rows), b_i . box_j = 2 pi delta_ij
    int kmax = 7;
    int K = 0;
    std::vector<double> kvec;    // 3K
    std::vector<double> kcoef;   // K
    std::vector<int> kidx;       // 3K integer indices (n1, n2, n3)
    std::vector<double> shifts;  // 3S full list (repeat.py:815-822 order)
    int S = 0;
    // device copies
    int *d_kidx = nullptr;        // 3K
    double *d_kcoef = nullptr;    // K
    double *d_kvec = nullptr;     // 3K
    double2 *d_ex = nullptr;      // (kmax+1) * nx   e^{2 pi i n1 i / nx}
    double2 *d_ey = nullptr;      // (2kmax+1) * ny  e^{2 pi i n2 j / ny}, n2 offset by kmax
    double2 *d_ez = nullptr;      // (2kmax+1) * nz
    // the same phases as double-float float4 (re_h, re_l, im_h, im_l) over the index
    // range the k-set uses, n in [-(kmax-1), kmax-1] (offset kmax-1; n1 >= 0 only)
    float4 *d_exf = nullptr;      // kmax * nx
    float4 *d_eyf = nullptr;      // (2kmax-1) * ny
    float4 *d_ezf = nullptr;      // (2kmax-1) * nz
    // every device table above lives in one block: `image` is its host copy, `off` the
    // table offsets; d_block is owned (rp_ewald_setup) or borrowed from a ctx arena (batches)
    std::vector<char> image;  // empty when the image was written into a caller's arena
    size_t image_bytes = 0;
    size_t off[9]{};
    void *d_block = nullptr;
    bool owns = false;
};

namespace rp {

// Raise a kernel's dynamic shared-memory limit to at least `bytes` on the current device.
// The limit belongs to the device context, and the batch server's worker and a caller's
// thread may launch the same kernel, so raised limits are recorded per (kernel, device)
// under a lock.  Sizes within the 48 KB default need nothing.
void smem_optin(const void *kernel, size_t bytes);

// Ewald tables (ewald_tables.cu): host part, device image size, placement in a device block.
// dst (optional, ewald_layout bytes): where the device image is written; else ew->image
void ewald_build_host(rp_ewald *ew, const rp_grid *grid, double cutoff, int kmax, char *dst = nullptr);
// offsets of the device tables in one image for this grid and KMAX, and its size
size_t ewald_layout(const rp_grid *grid, int kmax, size_t off[9], int *K_out = nullptr);
size_t ewald_device_bytes(const rp_ewald *ew);
void ewald_place(rp_ewald *ew, void *dev);
void ewald_build(rp_ewald *ew, const rp_grid *grid, double cutoff, int kmax);  // owns one cudaMalloc block
void ewald_free(rp_ewald *ew);

// Stops the ctx's asynchronous batch worker (rp_capi.cu): the running batch finishes.
void batch_server_stop(rp_ctx *ctx);

// Cutoff of the non-periodic basis (KMAX 0): beyond every distance, finite in FP32 squared.
constexpr double kNonPeriodicCutoff = 1e15;

// Host helpers shared by the stages.


void prune_shifts(const rp_ewald *ew, const double *atoms, int N, std::vector<double> &out, int &zero_idx);

// Device status words: [0] a bounded wait ran out, [1] fixed-point range overflows.
void status_clear(rp_ctx *ctx, cudaStream_t s);
void status_check(rp_ctx *ctx, cudaStream_t s);  // synchronises s

// Stage launchers (each enqueues on `stream`).
void filter_run(rp_ctx *ctx, const rp_grid *grid, const double *atoms, const int *Z, int N, const double *V_dev,
                double vdw_factor, double vdw_max, int32_t *kept_idx_dev, double *Vc_dev, int64_t capacity,
                int64_t *M_out, uint8_t *mask_dev, cudaStream_t stream);
// x, y, z and a squared radius, FP64 (32-byte aligned for one vector load)
struct alignas(32) D4 {
    double x, y, z, w;
};

// Launch parameters of the vdW mask kernel.
struct FilterParams {
    int nx, ny, nz;
    long long n_total;
    float ax[9];
    double axd[9];
    float bmin[3];
    float inv_bsize;
    int bn[3];
    float err_min;   // FP32 band around rmin^2
    float err_max;   // FP32 band around rmax^2
    int near_all;
    int A;
};

// Host half of one cube's vdW filter: the effective atoms (repeat.py:1933-1969), the
// FP32 error bands and the cell list, computed without touching the device, so that a
// batch plans its cubes on several threads and uploads every plan with one copy.
struct FilterPlan {
    FilterParams p{};
    std::vector<float4> e32;
    std::vector<D4> e64;
    std::vector<double> rmax2;
    std::vector<float> rmax2f;
    std::vector<int> boff, bidx;
    std::vector<D4> w_e64;       // working arrays of filter_plan (kept for their capacity)
    std::vector<double> w_rmax2;
    std::vector<int> w_binof, w_cur;
    size_t bytes() const;        // packed size: the arrays in order, each at a 32-byte offset
    void pack(char *dst) const;  // host image of the packed arrays
};
void filter_plan(const rp_grid *grid, const double *atoms, const int *Z, int N, double vdw_factor, double vdw_max,
                 FilterPlan &plan);
// Device half: mask, compaction and centring from a plan whose packed image is at
// packed_dev (same stream order as the copy that put it there).
void filter_launch(rp_ctx *ctx, const FilterPlan &plan, const char *packed_dev, const double *V_dev,
                   int32_t *kept_idx_dev, double *Vc_dev, long long *M_dev, uint8_t *mask_dev, cudaStream_t stream,
                   const std::string &tag, bool brick_order, double *vstats_dev);
// Many cubes at once (a pipeline group of a batch), brick order, no mask output: one launch
// per stage for up to 40 cubes.  Each item's kept count lands in *M, kept indices and
// centred ESP in its kept/Vc (room for its whole grid), (sum, max |.|) of the centred ESP in
// its vstats (2 doubles, optional).
struct FilterItem {
    const FilterPlan *plan;
    const char *packed_dev;
    const double *V;
    int32_t *kept;
    double *Vc;
    long long *M;
    double *vstats;
};
void filter_group(rp_ctx *ctx, const std::vector<FilterItem> &items, cudaStream_t stream, const std::string &tag);
// Asynchronous form: the kept count lands in *M_dev; kept_idx_dev and Vc_dev hold a
// whole grid (capacity = nx*ny*nz).  `tag` keeps the scratch of concurrent calls apart.
// brick_order: kept points in 8x4x4 brick order instead of flat order (the mixed fit
// is order-independent and culls real-space images per compact tile).
// vstats_dev (optional, 2 doubles): sum and max |.| of the centred ESP.
void filter_async(rp_ctx *ctx, const rp_grid *grid, const double *atoms, const int *Z, int N, const double *V_dev,
                  double vdw_factor, double vdw_max, int32_t *kept_idx_dev, double *Vc_dev, long long *M_dev,
                  uint8_t *mask_dev, cudaStream_t stream, const std::string &tag, bool brick_order,
                  double *vstats_dev);
// Exact Gram of a chunk of FP64 columns on the tensor cores (gram_mixed.cu): G (N x N) +=
// Phi^T Phi and r (N) += Phi^T V for Phi rows x N (row-major, ld N) and V (rows).
void gram_words_fp64(rp_ctx *ctx, const double *P, long long rows, int N, const double *V, double *G, double *r,
                     cudaStream_t stream);
// separable: the reciprocal sum by the FP64 separable transform and the Gram by
// gram_words_fp64 (the escalated fit)
// instead of the flat k-table DGEMM and DSYRK (the plain FP64 comparator)
void gram_fp64(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
               const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
               cudaStream_t stream, bool separable = false);
// vstats_dev: the filter's (sum, max |.|) of Vc (only the max is used), or nullptr to
// compute the max here.  rn (host, N) and clamp_dev (one device counter): the atoms'
// scaled vdW radii, which bound |Phi| a priori, so Phi goes straight to fixed-point
// digits in one pass; clamped values are counted in *clamp_dev (the caller then redoes
// the fit without rn).  Without them: two passes (Phi, then its centre and scale).
// d_atoms_pre / E_pre (optional): the atoms already on the device and the reciprocal rows
// already computed (recip_rows_group over a batch's pipeline group); tiles: the tile shapes.
void gram_mixed(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
                const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
                cudaStream_t stream, const double *vstats_dev = nullptr, const std::string &slot = "",
                const double *rn = nullptr, int *clamp_dev = nullptr, const double *d_atoms_pre = nullptr,
                const float2 *E_pre = nullptr, TileConfig tiles = TileConfig{});
double radius_of(int z);  // vdW radius (Bohr) of element z, the filter's table
void solve_run(rp_ctx *ctx, const double *A_dev, const double *b_dev, int N, int n_groups, const int *group_ptr,
               const int *group_idx, const double *resp_s, const double *resp_t, double qtot, double *q_dev,
               double *info, cudaStream_t stream);
// Words per system written by the bordered solve: refined residual inf-norm, min |pivot|,
// max |pivot|, singular flag, kappa = ||A||_1 ||K^-1||_1, the unknowns n+1 of the bordered
// system, FP32 refinement steps, and the factorisation path (0 FP32 in one CTA, 1 FP32
// across the GPU, 2 FP64 in one CTA, 3 FP64 across the GPU).
constexpr int kSolveInfo = 8;
// Batched constraints + bordered solves: one CTA per system, one launch.
struct SolveJob {
    const double *A, *b;
    int N, n_groups;
    const int *group_ptr, *group_idx;
    const double *resp_s, *resp_t;
    double qtot;
    double *q;
};
// fp64_first: wide systems (known ill-conditioned, e.g. an escalated fit) are factored in
// FP64 at once instead of after a stalled FP32 attempt
void solve_batch(rp_ctx *ctx, const std::vector<SolveJob> &jobs, std::vector<double> &info, cudaStream_t stream,
                 bool fp64_first = false);
// One bordered system of the solve kernel (device-side descriptor).
struct SolveDesc {
    const double *A;      // N x N input
    const double *b;      // N input
    int N;                // original atoms
    int n;                // reduced atoms
    const int *mem_ptr;   // n+1, CSR of members per reduced index
    const int *mem_idx;   // members (original atom indices)
    const double *resp_s; // n (per reduced index, already mapped) or null
    const double *resp_t; // n
    const int *map;       // N: reduced index of each original atom
    double qtot;
    double *As;           // (n+1)^2 work: bordered matrix, then LU
    double *A0;           // (n+1)^2 copy of the bordered matrix (for refinement)
    double *bs;           // n+1 rhs
    double *x;            // n+1 solution
    double *r;            // n+1 residual / correction
    int *perm;            // n+1 pivot rows
    double *q;            // N out
    double *info;         // kSolveInfo out: residual inf-norm, min|piv|, max|piv|, singular flag,
                          // kappa, unknowns n+1, refinement steps, factorisation path
    double *pre;          // null, or {flag, min|piv|, max|piv|} of a wide factorisation already in As
    int wide64;           // As holds wide FP64 factors: skip the FP32 stage and the in-CTA FP64 LU
    int host64;           // FP32 factors in the CTA, but a stalled refinement goes to the host's FP64
                          // factorisation across the GPU (pre holds its flag) instead of an in-CTA FP64 LU
    int host32;           // wide FP32 factors refined on the host path (refine_wide32): the kernel skips it
};
// Wide systems of a solve launch whose FP32 refinement may not have converged: their flags are
// on their way to pinned memory; solve_wide_fp64 (after the stream has reached them) factors
// the flagged ones again in FP64, refines them and refreshes the pinned info words.
struct SolvePending {
    bool any_wide = false;
    std::string tag;
    double *h_pre = nullptr, *h_info = nullptr, *d_info = nullptr;
    std::vector<SolveDesc> descs;
    std::vector<int> n1;
    std::vector<int> refine32;  // systems with wide FP32 factors, refined on the host path
};
// The same without waiting: returns the pinned host copy of the kSolveInfo words per job, valid
// once `stream` has reached this point.  `tag` keeps the scratch of solves in flight apart.
// With `pend`, wide systems that need FP64 factors are left for solve_wide_fp64 (the words
// are final after it); without, the call waits for them.  (Systems with overlapping symmetry
// groups are folded on the host, which waits.)
const double *solve_batch_async(rp_ctx *ctx, const std::vector<SolveJob> &jobs, cudaStream_t stream,
                                const std::string &tag, SolvePending *pend = nullptr, bool fp64_first = false);
void solve_wide_fp64(rp_ctx *ctx, SolvePending &pd, cudaStream_t stream);  // synchronises stream

// Device table builders (ewald_tables.cu).
void atom_tables_fp64(const rp_ewald *ew, const double *d_atoms, int N, double *d_B, int ldb, cudaStream_t s);
void grid_tables_fp64(const rp_ewald *ew, const int32_t *d_kept, int64_t m0, int64_t rows, double *d_T, int ldt,
                      cudaStream_t s);

// Reciprocal sum by separable lattice phases (recip_sep.cu): E[r][col][n1] for every
// grid row r = j + l*ny, col = atom (d_q == nullptr) or one charge-weighted column.
size_t recip_rows_bytes(const rp_ewald *ew, int ncols);
// `slot` keeps the scratch of fits running concurrently on different streams apart.
void recip_rows(rp_ctx *ctx, const rp_ewald *ew, const double *d_atoms, const double *d_q, int N, float2 *E,
                cudaStream_t stream, const std::string &slot = "");
// The same for many fits at once: one launch per stage for up to 64 fits (a pipeline group
// of a batch), each with its own tables, atoms and output E (recip_rows_bytes each).
struct RecipRowsJob {
    const rp_ewald *ew;
    const double *d_atoms;
    const double *d_q;
    int N;
    float2 *E;
};
void recip_rows_group(rp_ctx *ctx, const std::vector<RecipRowsJob> &jobs, cudaStream_t stream,
                      const std::string &tag);

// Shared epilogue kernels (phi_fp64.cu).
void column_sums_fp64(const double *X, int64_t rows, int cols, int ld, double *out, bool accumulate,
                      rp_ctx *ctx, cudaStream_t s);
void finish_normal_equations(const double *G, const double *r, const double *s_c, double *sumV_dev, int64_t M,
                             int N, double *A, double *b, cudaStream_t s);

inline unsigned ceil_div(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

// Records CUDA events around a stage on its stream when the ctx is timing.
struct StageTimer {
    rp_ctx *ctx;
    cudaStream_t s;
    size_t slot = (size_t)-1;
    StageTimer(rp_ctx *c, const char *name, cudaStream_t st) : ctx(c), s(st) {
        if (!ctx->timing) return;
        rp_ctx::Mark m{name, nullptr, nullptr};
        cudaEventCreate(&m.a);
        cudaEventCreate(&m.b);
        cudaEventRecord(m.a, s);
        ctx->marks.push_back(m);
        slot = ctx->marks.size() - 1;
    }
    ~StageTimer() {
        if (slot != (size_t)-1) cudaEventRecord(ctx->marks[slot].b, s);
    }
};

}  // namespace rp
