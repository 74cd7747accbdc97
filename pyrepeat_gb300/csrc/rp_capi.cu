// C ABI of librepeat_gb300 (include/repeat_gb300.h): argument checks, the
// context, and the translation of internal errors into status codes.
#include <cstring>
#include <unordered_map>

#include "common.cuh"

namespace rp {
void potential_run(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, const double *q, int N,
                   const int32_t *idx_dev, int64_t npts, double *out_dev, cudaStream_t stream);
void qeq_run(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const double *chi, const double *j_self,
             double qtot, double *q_out, double *J_out, double *info, cudaStream_t stream);
}  // namespace rp

namespace rp {
std::atomic<long long> g_launches{0};

// Raise a kernel's dynamic shared-memory limit to `bytes` when the block's static and dynamic
// shared memory together pass the 48 KB available without opting in.
void smem_optin(const void *kernel, size_t bytes) {
    int dev = 0;
    RP_CUDA(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, std::pair<size_t, size_t>> raised;  // (static, raised to)
    std::lock_guard<std::mutex> lk(mu);
    auto it = raised.find({kernel, dev});
    if (it == raised.end()) {
        cudaFuncAttributes fa;
        RP_CUDA(cudaFuncGetAttributes(&fa, kernel));
        it = raised.emplace(std::make_pair(kernel, dev), std::make_pair((size_t)fa.sharedSizeBytes, (size_t)0)).first;
    }
    if (bytes + it->second.first <= (48u << 10) || bytes <= it->second.second) return;
    RP_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    it->second.second = bytes;
}
void status_clear(rp_ctx *ctx, cudaStream_t s) {
    RP_CUDA(cudaMemsetAsync(ctx->status_words(), 0, 2 * sizeof(int), s));
}
void status_check(rp_ctx *ctx, cudaStream_t s) {
    int st[2] = {0, 0};
    RP_CUDA(cudaMemcpyAsync(st, ctx->status_words(), sizeof(st), cudaMemcpyDeviceToHost, s));
    RP_CUDA(cudaStreamSynchronize(s));
    if (st[0] != 0) fail(st[0], "a tensor-core pipeline wait ran out of time");
    if (st[1] != 0)
        fail(RP_E_STATE, std::to_string(st[1]) + " Phi values exceeded the fixed-point range of their chunk");
}
}  // namespace rp

cublasHandle_t rp_ctx::blas() {
    cublasHandle_t &h = cublas[cur_slot];
    if (!h) {
        RP_CUBLAS(cublasCreate(&h));
        RP_CUBLAS(cublasSetMathMode(h, CUBLAS_DEFAULT_MATH));  // native FP64, no emulation
    }
    return h;
}

cusolverDnHandle_t rp_ctx::solver() {
    cusolverDnHandle_t &h = cusolver[cur_slot];
    if (!h && cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) {
        h = nullptr;
        rp::fail(RP_E_CUDA, "cusolverDnCreate failed");
    }
    return h;
}

namespace {

template <class F>
int guarded(rp_ctx *ctx, F &&f) {
    try {
        if (ctx) {
            ctx->cur_slot = 0;  // calls on the caller's thread run in slot 0, default priority
            ctx->cur_prio = 0;
            RP_CUDA(cudaSetDevice(ctx->device));
        }
        f();
        if (ctx) ctx->last_error.clear();
        return RP_OK;
    } catch (const rp::Error &e) {
        if (ctx) ctx->last_error = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        if (ctx) ctx->last_error = e.what();
        return RP_E_ARG;
    }
}


}  // namespace

extern "C" {

int rp_version(void) { return 20000; }

int rp_ctx_create(int device, size_t hbm_budget, rp_ctx **out) {
    if (!out) return RP_E_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return RP_E_CUDA;
    }
    if (device < 0 || device >= n) return RP_E_ARG;
    rp_ctx *c = new rp_ctx();
    c->device = device;
    int rc = guarded(c, [&] {
        RP_CUDA(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device));
        size_t fr = 0, tot = 0;
        RP_CUDA(cudaMemGetInfo(&fr, &tot));
        c->budget = hbm_budget ? hbm_budget : (size_t)(0.9 * (double)fr);
        RP_CUDA(cudaMalloc(&c->d_status, sizeof(int) * 2 * rp::kBatchSlots));
        RP_CUDA(cudaMemset(c->d_status, 0, sizeof(int) * 2 * rp::kBatchSlots));
    });
    if (rc != RP_OK) {
        delete c;
        return rc;
    }
    *out = c;
    return RP_OK;
}

int rp_ctx_destroy(rp_ctx *ctx) {
    if (!ctx) return RP_E_ARG;
    rp::batch_server_stop(ctx);  // the batch running now finishes; queued ones are dropped
    cudaSetDevice(ctx->device);
    for (auto &kv : ctx->scratch) cudaFree(kv.second.ptr);
    for (auto &kv : ctx->host_scratch) cudaFreeHost(kv.second.ptr);
    for (cudaStream_t st : ctx->lanes) cudaStreamDestroy(st);
    for (cublasHandle_t h : ctx->cublas)
        if (h) cublasDestroy(h);
    for (cusolverDnHandle_t h : ctx->cusolver)
        if (h) cusolverDnDestroy(h);
    cudaFree(ctx->d_status);
    delete ctx;
    return RP_OK;
}

int rp_last_error(const rp_ctx *ctx, char *buf, size_t cap) {
    if (!ctx || !buf || cap == 0) return RP_E_ARG;
    size_t n = std::min(cap - 1, ctx->last_error.size());
    std::memcpy(buf, ctx->last_error.data(), n);
    buf[n] = 0;
    return RP_OK;
}

int rp_filter(rp_ctx *ctx, const rp_grid *grid, const double *atoms, const int *Z, int N, const double *V_dev,
              double vdw_factor, double vdw_max, int32_t *kept_idx_dev, double *Vc_dev, int64_t capacity,
              int64_t *M_out, uint8_t *mask_dev, rp_stream_t stream) {
    if (!ctx) return RP_E_ARG;
    return guarded(ctx, [&] {
        RP_REQUIRE(kept_idx_dev && Vc_dev, "rp_filter: null output");
        rp::filter_run(ctx, grid, atoms, Z, N, V_dev, vdw_factor, vdw_max, kept_idx_dev, Vc_dev, capacity, M_out,
                       mask_dev, (cudaStream_t)stream);
    });
}

int rp_ewald_setup(rp_ctx *ctx, const rp_grid *grid, double cutoff, int kmax, rp_ewald **out) {
    if (!ctx || !grid || !out) return RP_E_ARG;
    *out = nullptr;
    rp_ewald *ew = new rp_ewald();
    ew->device = ctx->device;
    int rc = guarded(ctx, [&] { rp::ewald_build(ew, grid, cutoff, kmax); });
    if (rc != RP_OK) {
        rp::ewald_free(ew);
        delete ew;
        return rc;
    }
    *out = ew;
    return RP_OK;
}

int rp_ewald_destroy(rp_ewald *ew) {
    if (!ew) return RP_E_ARG;
    cudaSetDevice(ew->device);
    rp::ewald_free(ew);
    delete ew;
    return RP_OK;
}

int rp_ewald_info(const rp_ewald *ew, int *K, int *S, double *alpha) {
    if (!ew) return RP_E_ARG;
    if (K) *K = ew->K;
    if (S) *S = ew->S;
    if (alpha) *alpha = ew->alpha;
    return RP_OK;
}

int rp_gram(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
            const double *Vc_dev, int64_t M, int precision, double *A_dev, double *b_dev, double *sum_phi_dev,
            rp_stream_t stream) {
    if (!ctx || !ew) return RP_E_ARG;
    return guarded(ctx, [&] {
        RP_REQUIRE(atoms && kept_idx_dev && Vc_dev && A_dev && b_dev, "rp_gram: null argument");
        RP_REQUIRE(ew->device == ctx->device, "rp_gram: ewald built on another device");
        RP_REQUIRE(precision == RP_PREC_FP64 || precision == RP_PREC_MIXED, "rp_gram: unknown precision");
        rp::status_clear(ctx, (cudaStream_t)stream);
        if (precision == RP_PREC_FP64)
            rp::gram_fp64(ctx, ew, atoms, N, kept_idx_dev, Vc_dev, M, A_dev, b_dev, sum_phi_dev, (cudaStream_t)stream);
        else
            rp::gram_mixed(ctx, ew, atoms, N, kept_idx_dev, Vc_dev, M, A_dev, b_dev, sum_phi_dev, (cudaStream_t)stream);
        rp::status_check(ctx, (cudaStream_t)stream);
    });
}

int rp_solve(rp_ctx *ctx, const double *A_dev, const double *b_dev, int N, int n_groups, const int *group_ptr,
             const int *group_idx, const double *resp_s, const double *resp_t, double qtot, double *q_dev,
             double *info, rp_stream_t stream) {
    if (!ctx) return RP_E_ARG;
    return guarded(ctx, [&] {
        rp::solve_run(ctx, A_dev, b_dev, N, n_groups, group_ptr, group_idx, resp_s, resp_t, qtot, q_dev, info,
                      (cudaStream_t)stream);
    });
}

int rp_potential(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, const double *q, int N,
                 const int32_t *idx_dev, int64_t npts, double *out_dev, rp_stream_t stream) {
    if (!ctx || !ew) return RP_E_ARG;
    return guarded(ctx, [&] {
        RP_REQUIRE(ew->device == ctx->device, "rp_potential: ewald built on another device");
        rp::potential_run(ctx, ew, atoms, q, N, idx_dev, npts, out_dev, (cudaStream_t)stream);
    });
}

int rp_qeq(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const double *chi, const double *j_self,
           double qtot, double *q, double *J, double *info, rp_stream_t stream) {
    if (!ctx || !ew) return RP_E_ARG;
    return guarded(ctx, [&] {
        RP_REQUIRE(ew->device == ctx->device, "rp_qeq: ewald built on another device");
        rp::qeq_run(ctx, ew, atoms, N, chi, j_self, qtot, q, J, info, (cudaStream_t)stream);
    });
}

}  // extern "C"

namespace rp {

// One batch of the batched fit, from its enqueue to its completion.  Everything a batch
// keeps between the two phases lives here; its device scratch, pinned staging, streams,
// status words and host object pools are those of the ctx slot it runs in.
struct BatchRun {
    int slot = 0;
    int prio = 0;  // stream priority class (rp_ctx::cur_prio) the batch runs at
    int n = 0;
    const rp_fit_desc *descs = nullptr;
    double *q_out = nullptr;
    int64_t *M_out = nullptr;
    double *info_out = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<long long> off_pts, off_n, off_nn, M;
    std::vector<rp_ewald *> ews;
    int32_t *kept = nullptr;
    double *Vc = nullptr, *A = nullptr, *b = nullptr, *q = nullptr, *vst = nullptr;
    int *clamps = nullptr;
    int ngroups = 0;
    std::vector<int> g0;
    std::vector<const double *> ginfo;  // pinned solve words of each pipeline group
    std::vector<SolvePending> gpend;    // each group's wide systems that may need FP64 factors
    int *hclamps = nullptr;             // pinned clamp counts
    double *hq = nullptr;               // pinned charges
    std::vector<cudaEvent_t> events;
    cudaEvent_t done = nullptr;         // every device step of the enqueue phase has run
    ~BatchRun() {
        for (cudaEvent_t ev : events) cudaEventDestroy(ev);
    }
    SolveJob job(int i) const {
        const rp_fit_desc &d = descs[i];
        return SolveJob{A + off_nn[i], b + off_n[i], d.N, d.n_groups, d.group_ptr, d.group_idx,
                        d.resp_s, d.resp_t, d.qtot, q + off_n[i]};
    }
};

// Enqueue phase of the batched fit (throws rp::Error): filters, Ewald tables, normal
// equations and bordered solves of every cube go to the device, with the only host waits
// on each pipeline group's kept counts; the charges, clamp counts and solve words are
// copied to pinned memory behind them and r.done is recorded.  Runs in slot ctx->cur_slot.
void batch_enqueue(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, double *q_out,
                   int64_t *M_out, double *info_out, cudaStream_t stream, BatchRun &r) {
    ctx->trace_mark("enqueue");
    r.slot = ctx->cur_slot;
    r.prio = ctx->cur_prio;
    r.n = n;
    r.descs = descs;
    r.q_out = q_out;
    r.M_out = M_out;
    r.info_out = info_out;
    r.stream = stream;
    if (n == 0) return;
    std::vector<long long> npts((size_t)n);
    r.off_pts.assign((size_t)n + 1, 0);
    r.off_n.assign((size_t)n + 1, 0);
    r.off_nn.assign((size_t)n + 1, 0);
    for (int i = 0; i < n; ++i) {
        const rp_fit_desc &d = descs[i];
        RP_REQUIRE(d.atoms && d.Z && d.N > 0, "rp_fit: null input or N <= 0");
        RP_REQUIRE(d.precision == RP_PREC_FP64 || d.precision == RP_PREC_MIXED, "rp_fit: unknown precision");
        RP_REQUIRE((V_dev && V_dev[i]) || d.V, "rp_fit: no ESP values");
        npts[i] = (long long)d.grid.n_grid[0] * d.grid.n_grid[1] * d.grid.n_grid[2];
        RP_REQUIRE(npts[i] > 0 && npts[i] < (1LL << 31), "rp_fit: bad grid");
        r.off_pts[i + 1] = r.off_pts[i] + npts[i];
        r.off_n[i + 1] = r.off_n[i] + d.N;
        r.off_nn[i + 1] = r.off_nn[i] + (long long)d.N * d.N;
    }
    const std::vector<long long> &off_pts = r.off_pts, &off_n = r.off_n, &off_nn = r.off_nn;
    // Work splits into host preparation and device stages so that the device never waits
    // on the host inside the batch, and the cubes run as a pipeline of up to four groups:
    // (1) the first group's filter plans on the host workers, one pinned upload, its grids
    // and its filter launches; (2) while they run, the Ewald tables of every cube on the
    // host workers, one pinned upload, and the reciprocal rows; then the other groups'
    // filters as in (1); (3) as each group's kept counts arrive, its normal equations go
    // to the gram streams, so later groups' filters overlap earlier groups' grams.
    constexpr int kLanes = 4;
    const int lanes = ctx->timing ? 1 : kLanes;  // stage timing: one lane, each stage alone
    auto glane = [&](int i) { return ctx->lane(i % lanes); };
    auto flane = [&](int i) { return ctx->timing ? ctx->lane(0) : ctx->lane(kLaneFilter0 + i % kLanes); };
    const int ngroups = (n >= 64 && !ctx->timing) ? 4 : 1;
    r.ngroups = ngroups;
    r.g0.assign((size_t)ngroups + 1, 0);
    std::vector<int> &g0 = r.g0;
    for (int g = 0; g <= ngroups; ++g) g0[g] = (int)((long long)n * g / ngroups);
    int32_t *kept = r.kept = ctx->buf_t<int32_t>("fit_kept", (size_t)off_pts[n]);
    double *Vc = r.Vc = ctx->buf_t<double>("fit_Vc", (size_t)off_pts[n]);
    // Grids from host memory: the filter reads a grid only at its kept points (in the
    // compaction, after the geometric mask), so a grid in page-locked host memory that the
    // device can address is read in place over the host link instead of being copied whole
    // first; any other host grid is copied to the device on the copy stream.
    std::vector<const double *> Vsrc((size_t)n, nullptr);
    bool any_copy = false;
    for (int i = 0; i < n; ++i) {
        if (V_dev && V_dev[i]) {
            Vsrc[i] = V_dev[i];
            continue;
        }
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, descs[i].V) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
            pa.devicePointer != nullptr)
            Vsrc[i] = static_cast<const double *>(pa.devicePointer);
        else
            any_copy = true;
        cudaGetLastError();  // an unregistered pointer may leave an error behind
    }
    double *Vh = any_copy ? ctx->buf_t<double>("fit_V", (size_t)off_pts[n]) : nullptr;
    long long *Md = ctx->buf_t<long long>("fit_M", (size_t)n);
    long long *Mh = static_cast<long long *>(ctx->host_buf("fit_M", sizeof(long long) * n));
    double *A = r.A = ctx->buf_t<double>("fit_A", (size_t)off_nn[n]);
    double *b = r.b = ctx->buf_t<double>("fit_b", (size_t)off_n[n]);
    r.q = ctx->buf_t<double>("fit_q", (size_t)off_n[n]);
    double *vst = r.vst = ctx->buf_t<double>("fit_vstats", 2 * (size_t)n);
    int *clamps = r.clamps = ctx->buf_t<int>("fit_clamps", (size_t)n);
    rp::status_clear(ctx, stream);
    RP_CUDA(cudaMemsetAsync(clamps, 0, sizeof(int) * n, stream));
    // events the host waits on (kept counts, the batch's end) block the waiting thread
    // instead of spinning, so a waiting host thread leaves its core to the other host work
    // of the process (the next batch's planning, the caller's threads)
    auto record = [&](cudaStream_t st, bool host_waits = false) {
        cudaEvent_t ev;
        RP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming | (host_waits ? cudaEventBlockingSync : 0)));
        r.events.push_back(ev);
        RP_CUDA(cudaEventRecord(ev, st));
        return ev;
    };
    // 1. filters, group by group: the host plans a group (its workers), packs it into the
    //    group's pinned arena and queues the upload, the grids and the filter launches, then
    //    plans the next group while the device runs this one
    auto &plan_pool = ctx->plan_pool[ctx->cur_slot];
    while ((int)plan_pool.size() < n) plan_pool.emplace_back(new rp::FilterPlan());
    auto plan = [&](int i) -> rp::FilterPlan & { return *plan_pool[(size_t)i]; };
    {
        const cudaEvent_t up = record(stream);  // every stream starts after the caller's work so far
        for (int ln = 0; ln < kLanes; ++ln) {
            RP_CUDA(cudaStreamWaitEvent(ctx->lane(ln), up, 0));
            RP_CUDA(cudaStreamWaitEvent(flane(ln), up, 0));
        }
    }
    const cudaStream_t copy_lane = ctx->lane(kLaneCopy);  // uploads: plans, grids, tables
    RP_CUDA(cudaStreamWaitEvent(copy_lane, r.events.back(), 0));
    std::vector<size_t> pl_off((size_t)n + 1, 0);
    std::vector<cudaEvent_t> kept_ready((size_t)ngroups);
    auto filter_group_g = [&](int g) {
        const int i0 = g0[g], i1 = g0[g + 1];
        ctx->parallel(i1 - i0, [&](int t) {
            const rp_fit_desc &d = descs[i0 + t];
            rp::filter_plan(&d.grid, d.atoms, d.Z, d.N, d.vdw_factor, d.vdw_max, plan(i0 + t));
        });
        ctx->trace_mark("planned group " + std::to_string(g));
        pl_off[i0] = 0;
        for (int i = i0; i < i1; ++i) pl_off[i + 1] = pl_off[i] + plan(i).bytes();
        const std::string gtag = "fit_filter#" + std::to_string(g);
        char *pl_dev = static_cast<char *>(ctx->buf(gtag, pl_off[i1]));
        char *pl_host = static_cast<char *>(ctx->host_buf(gtag, pl_off[i1]));
        ctx->parallel(i1 - i0, [&](int t) { plan(i0 + t).pack(pl_host + pl_off[i0 + t]); });
        RP_CUDA(cudaMemcpyAsync(pl_dev, pl_host, pl_off[i1], cudaMemcpyHostToDevice, copy_lane));
        for (int i = i0; i < i1; ++i)  // grids from unmapped host memory, this group's only
            if (!Vsrc[i]) {
                RP_CUDA(cudaMemcpyAsync(Vh + off_pts[i], descs[i].V, sizeof(double) * npts[i],
                                        cudaMemcpyHostToDevice, copy_lane));
                Vsrc[i] = Vh + off_pts[i];
            }
        const cudaEvent_t inputs = record(copy_lane);
        for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(flane(ln), inputs, 0));
        // the group's mixed-precision cubes in one launch per filter stage (brick order), the
        // FP64 ones (flat order, the comparator) one by one
        std::vector<rp::FilterItem> items;
        for (int i = i0; i < i1; ++i) {
            const rp_fit_desc &d = descs[i];
            const double *V = Vsrc[i];
            if (d.precision == RP_PREC_MIXED) {
                items.push_back(rp::FilterItem{&plan(i), pl_dev + pl_off[i], V, kept + off_pts[i], Vc + off_pts[i],
                                               Md + i, vst + 2 * i});
            } else {
                rp::filter_launch(ctx, plan(i), pl_dev + pl_off[i], V, kept + off_pts[i], Vc + off_pts[i], Md + i,
                                  nullptr, flane(i), "#f" + std::to_string(i % lanes), false, vst + 2 * i);
            }
        }
        rp::filter_group(ctx, items, flane(g), "#fg" + std::to_string(g));
        for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(stream, record(flane(ln)), 0));
        RP_CUDA(cudaMemcpyAsync(Mh + i0, Md + i0, sizeof(long long) * (i1 - i0), cudaMemcpyDeviceToHost, stream));
        kept_ready[g] = record(stream, true);
        ctx->trace_mark("filters queued group " + std::to_string(g));
    };
    filter_group_g(0);
    // 2. Ewald tables, written by the host workers straight into one pinned arena,
    //    uploaded with a single copy on a stream of its own.  They go up right behind the
    //    first group's grids and before the other groups' (copies from host memory are
    //    served in the order they are queued), so the first group's reciprocal rows and
    //    normal equations do not wait for the whole batch's grids to arrive.
    std::vector<size_t> ew_off((size_t)n + 1, 0);
    auto &ew_pool = ctx->ew_pool[ctx->cur_slot];
    while ((int)ew_pool.size() < n) ew_pool.emplace_back(new rp_ewald());
    r.ews.assign((size_t)n, nullptr);
    for (int i = 0; i < n; ++i) {
        size_t off9[9];
        r.ews[i] = ew_pool[(size_t)i].get();
        r.ews[i]->device = ctx->device;
        ew_off[i + 1] = ew_off[i] + rp::ewald_layout(&descs[i].grid, descs[i].kmax, off9);
    }
    // the atoms of every cube follow the tables in the same arena
    const size_t at_off = (ew_off[n] + 255) / 256 * 256;
    char *ew_dev = static_cast<char *>(ctx->buf("fit_ewald", at_off + sizeof(double) * 3 * off_n[n]));
    char *ew_host = static_cast<char *>(ctx->host_buf("fit_ewald", at_off + sizeof(double) * 3 * off_n[n]));
    double *atoms_dev = reinterpret_cast<double *>(ew_dev + at_off);
    ctx->parallel(n, [&](int i) {
        rp::ewald_build_host(r.ews[i], &descs[i].grid, descs[i].cutoff, descs[i].kmax, ew_host + ew_off[i]);
        std::copy(descs[i].atoms, descs[i].atoms + 3 * (size_t)descs[i].N,
                  reinterpret_cast<double *>(ew_host + at_off) + 3 * off_n[i]);
    });
    for (int i = 0; i < n; ++i) rp::ewald_place(r.ews[i], ew_dev + ew_off[i]);
    ctx->trace_mark("tables built");
    // the tables go up on the reciprocal rows' stream, beside the first group's grids on the
    // copy stream (with grids from host memory those are most of the batch's bytes)
    const cudaStream_t recip_lane = ctx->timing ? ctx->lane(0) : ctx->lane(kLaneRecip);
    RP_CUDA(cudaStreamWaitEvent(recip_lane, r.events.front(), 0));  // after the caller's work so far
    RP_CUDA(cudaMemcpyAsync(ew_dev, ew_host, at_off + sizeof(double) * 3 * off_n[n], cudaMemcpyHostToDevice,
                            recip_lane));
    const cudaEvent_t tables = record(recip_lane);
    for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(glane(ln), tables, 0));
    RP_CUDA(cudaStreamWaitEvent(stream, tables, 0));
    // reciprocal rows of every mixed-precision cube, a pipeline group per launch set, on that
    // stream: they need only the tables and atoms, so they run beside the filters, and each
    // group's normal equations wait for its rows
    std::vector<size_t> e_off((size_t)n + 1, 0);
    for (int i = 0; i < n; ++i)
        e_off[i + 1] = e_off[i] + (descs[i].precision == RP_PREC_MIXED
                                       ? recip_rows_bytes(r.ews[i], descs[i].N) / sizeof(float2) : 0);
    float2 *E_all = ctx->buf_t<float2>("fit_E", std::max<size_t>(e_off[n], 1));
    std::vector<cudaEvent_t> rows_ready((size_t)ngroups);
    for (int g = 0; g < ngroups; ++g) {
        std::vector<rp::RecipRowsJob> rj;
        for (int i = g0[g]; i < g0[g + 1]; ++i)
            if (descs[i].precision == RP_PREC_MIXED)
                rj.push_back(rp::RecipRowsJob{r.ews[i], atoms_dev + 3 * off_n[i], nullptr, descs[i].N,
                                              E_all + e_off[i]});
        {
            StageTimer tt(ctx, "recip_rows", recip_lane);
            rp::recip_rows_group(ctx, rj, recip_lane, "#r" + std::to_string(g));
        }
        rows_ready[g] = record(recip_lane);
    }
    for (int g = 1; g < ngroups; ++g) filter_group_g(g);
    // 3. normal equations, group by group as the kept counts arrive.  Mixed-precision fits
    //    are spread over the gram streams (each with its own scratch), so one cube's small
    //    kernels and launch gaps overlap another's; the FP64 comparator stays on the
    //    caller's stream (its cuBLAS handle is shared).  Every cube's result is independent
    //    of the stream it ran on.  A mixed fit takes the single pass (Phi straight to
    //    digits, scaled by the a-priori bounds from the scaled vdW radii); a cube whose
    //    values clamp (a cell the bound's argument does not cover) is redone at completion
    //    in two passes.
    std::vector<double> rn((size_t)off_n[n]);
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < descs[i].N; ++a)
            rn[off_n[i] + a] = descs[i].vdw_factor * rp::radius_of(descs[i].Z[a]);
    r.M.assign((size_t)n, 0);
    r.ginfo.assign((size_t)ngroups, nullptr);
    r.gpend.assign((size_t)ngroups, SolvePending{});
    for (int g = 0; g < ngroups; ++g) {
        RP_CUDA(cudaEventSynchronize(kept_ready[g]));
        ctx->trace_mark("kept counts group " + std::to_string(g));
        for (int i = g0[g]; i < g0[g + 1]; ++i) {
            r.M[i] = Mh[i];
            if (M_out) M_out[i] = r.M[i];
            RP_REQUIRE(r.M[i] > 0, "rp_fit: no grid point of cube " + std::to_string(i) + " survives the vdW filter");
        }
        for (int ln = 0; ln < lanes; ++ln) {
            RP_CUDA(cudaStreamWaitEvent(glane(ln), kept_ready[g], 0));
            RP_CUDA(cudaStreamWaitEvent(glane(ln), rows_ready[g], 0));
        }
        for (int i = g0[g]; i < g0[g + 1]; ++i) {
            const rp_fit_desc &d = descs[i];
            if (d.precision == RP_PREC_MIXED) {
                const int ln = i % lanes;
                rp::gram_mixed(ctx, r.ews[i], d.atoms, d.N, kept + off_pts[i], Vc + off_pts[i], r.M[i],
                               A + off_nn[i], b + off_n[i], nullptr, glane(ln), vst + 2 * i,
                               "#" + std::to_string(ln), rn.data() + off_n[i], clamps + i,
                               atoms_dev + 3 * off_n[i], E_all + e_off[i], ctx->tiles_for(d.N, r.M[i], d.kmax));
            } else {
                rp::gram_fp64(ctx, r.ews[i], d.atoms, d.N, kept + off_pts[i], Vc + off_pts[i], r.M[i],
                              A + off_nn[i], b + off_n[i], nullptr, stream);
            }
        }
        // 4. the group's constraint folds and bordered solves (one launch) on the caller's
        //    stream, behind its normal equations and overlapping the next group's
        for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(stream, record(glane(ln)), 0));
        std::vector<rp::SolveJob> jobs;
        for (int i = g0[g]; i < g0[g + 1]; ++i) jobs.push_back(r.job(i));
        r.ginfo[g] = rp::solve_batch_async(ctx, jobs, stream, "#g" + std::to_string(g), &r.gpend[g]);
    }
    // 5. the results to pinned memory; r.done marks the end of the device work
    r.hclamps = static_cast<int *>(ctx->host_buf("fit_clamps", sizeof(int) * n));
    RP_CUDA(cudaMemcpyAsync(r.hclamps, clamps, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
    r.hq = static_cast<double *>(ctx->host_buf("fit_qh", sizeof(double) * off_n[n]));
    RP_CUDA(cudaMemcpyAsync(r.hq, r.q, sizeof(double) * off_n[n], cudaMemcpyDeviceToHost, stream));
    r.done = record(stream, true);
}

// Completion phase (throws rp::Error): waits for r.done, refits cubes whose values clamped
// (two passes) or whose conditioning calls for FP64 (escalation), and writes the charges,
// kept counts and info words.  Runs in slot r.slot (ctx->cur_slot must be r.slot).
void batch_complete(rp_ctx *ctx, BatchRun &r) {
    const int n = r.n;
    if (n == 0) return;
    const cudaStream_t stream = r.stream;
    ctx->trace_mark("complete");
    RP_CUDA(cudaEventSynchronize(r.done));
    ctx->trace_mark("device done");
    bool changed = false;
    for (SolvePending &pd : r.gpend)  // wide systems whose FP32 refinement stalled: FP64 factors
        if (pd.any_wide) {
            rp::solve_wide_fp64(ctx, pd, stream);
            changed = true;
        }
    constexpr int W = RP_FIT_INFO_WORDS;
    std::vector<double> info((size_t)n * W, 0.0);
    // a cube's record from its solve's words (rp::kSolveInfo per system); unknowns[i] = n+1
    std::vector<double> unknowns((size_t)n, 1.0);
    auto take = [&](int i, const double *h) {
        double *o = info.data() + (size_t)W * i;
        unknowns[i] = std::max(1.0, h[5]);
        o[0] = h[0];  // refined residual
        o[1] = h[1];  // min |pivot|
        o[2] = h[2];  // max |pivot|
        o[3] = h[3];  // singular flag
        o[4] = h[4];  // kappa
        o[5] = h[7];  // factorisation path
    };
    for (int g = 0; g < r.ngroups; ++g)
        for (int i = r.g0[g]; i < r.g0[g + 1]; ++i) {
            take(i, r.ginfo[g] + (size_t)rp::kSolveInfo * (i - r.g0[g]));
            info[(size_t)W * i + 6] = r.descs[i].precision;
        }
    auto resolve = [&](const std::vector<int> &cubes, int flag, int precision) {
        std::vector<rp::SolveJob> jobs;
        for (int i : cubes) jobs.push_back(r.job(i));
        std::vector<double> rinfo;
        // an escalated cube's system is known to be beyond FP32 refinement: FP64 factors at once
        rp::solve_batch(ctx, jobs, rinfo, stream, flag == RP_FIT_ESCALATED);
        for (size_t t = 0; t < cubes.size(); ++t) {
            take(cubes[t], rinfo.data() + (size_t)rp::kSolveInfo * t);
            info[(size_t)W * cubes[t] + 6] = precision;
            info[(size_t)W * cubes[t] + 7] = (double)((int)info[(size_t)W * cubes[t] + 7] | flag);
        }
        changed = true;
    };
    // a cube whose values clamped: the two-pass fit, centred and scaled by the data, and
    // its solve again
    ctx->last_fallbacks = 0;
    std::vector<int> redo;
    for (int i = 0; i < n; ++i)
        if (r.hclamps[i] != 0) {
            ++ctx->last_fallbacks;
            redo.push_back(i);
            const rp_fit_desc &d = r.descs[i];
            rp::gram_mixed(ctx, r.ews[i], d.atoms, d.N, r.kept + r.off_pts[i], r.Vc + r.off_pts[i], r.M[i],
                           r.A + r.off_nn[i], r.b + r.off_n[i], nullptr, stream, r.vst + 2 * i, "");
        }
    if (!redo.empty()) resolve(redo, RP_FIT_TWO_PASS, RP_PREC_MIXED);
    rp::status_check(ctx, stream);
    // escalation: a mixed-precision cube whose bordered system is so ill-conditioned that
    // the Gram's rounding (~1e-7 relative) could move its charges visibly (kappa / (n+1)
    // above the ctx's limit) is fitted again in FP64 (the reciprocal sum by the FP64
    // separable transform)
    std::vector<int> esc;
    if (ctx->kappa_limit > 0.0)
        for (int i = 0; i < n; ++i)
            if (r.descs[i].precision == RP_PREC_MIXED && info[(size_t)W * i + 3] == 0.0 &&
                !(info[(size_t)W * i + 4] / unknowns[i] <= ctx->kappa_limit))
                esc.push_back(i);
    ctx->last_escalations = (int)esc.size();
    if (!esc.empty()) {
        for (int i : esc) {
            const rp_fit_desc &d = r.descs[i];
            rp::gram_fp64(ctx, r.ews[i], d.atoms, d.N, r.kept + r.off_pts[i], r.Vc + r.off_pts[i], r.M[i],
                          r.A + r.off_nn[i], r.b + r.off_n[i], nullptr, stream, true);
        }
        resolve(esc, RP_FIT_ESCALATED, RP_PREC_FP64);
    }
    if (changed) {
        RP_CUDA(cudaMemcpyAsync(r.hq, r.q, sizeof(double) * r.off_n[n], cudaMemcpyDeviceToHost, stream));
        RP_CUDA(cudaStreamSynchronize(stream));
    }
    std::copy(r.hq, r.hq + r.off_n[n], r.q_out);
    if (r.info_out) std::copy(info.begin(), info.end(), r.info_out);
    ctx->trace_mark("charges out");
    for (int i = 0; i < n; ++i)
        if (info[(size_t)W * i + 3] != 0.0)
            rp::fail(RP_E_SINGULAR, "rp_fit: bordered system of cube " + std::to_string(i) + " is singular");
}

// The batched fit on the caller's thread, in slot 0 (the pooled Ewald objects borrow the
// slot's arena: nothing to free).
void fit_batch_body(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, double *q_out,
                    int64_t *M_out, double *info_out, cudaStream_t stream) {
    ctx->cur_slot = 0;
    ctx->cur_prio = 0;
    BatchRun r;
    batch_enqueue(ctx, n, descs, V_dev, q_out, M_out, info_out, stream, r);
    batch_complete(ctx, r);
}

// Worker of the asynchronous batches.  Up to kBatchSlots batches are in flight at once, each
// in a slot of its own (scratch, pinned staging, streams, status words), so a batch
// submitted while others run starts on the device at once and overlaps them; batches are
// started in submission order and retired as they finish, in any order.
void batch_server_loop(rp_ctx *ctx) {
    BatchServer &sv = *ctx->server;
    cudaSetDevice(ctx->device);
    struct Flight {
        BatchServer::Job job;
        std::unique_ptr<BatchRun> run;
        int status = RP_OK;
        std::string msg;
    };
    std::vector<std::unique_ptr<Flight>> flights;
    bool busy[kBatchSlots] = {};
    auto failed = [](Flight &f, int code, const std::string &m) {
        if (f.status == RP_OK) {
            f.status = code;
            f.msg = m;
        }
    };
    std::unique_lock<std::mutex> lk(sv.mu);
    for (;;) {
        // 1. retire every batch whose device work has finished (or that failed to enqueue)
        bool progressed = false;
        for (size_t k = 0; k < flights.size();) {
            Flight &f = *flights[k];
            const bool ready =
                f.status != RP_OK || !f.run->done || cudaEventQuery(f.run->done) != cudaErrorNotReady;
            if (!ready) {
                ++k;
                continue;
            }
            lk.unlock();
            ctx->cur_slot = f.run->slot;
            ctx->cur_prio = f.run->prio;
            try {
                if (f.status == RP_OK) {
                    batch_complete(ctx, *f.run);
                } else {  // a failed enqueue may have left work on the slot's streams
                    for (int ln = 0; ln < kSlotLanes; ++ln) cudaStreamSynchronize(ctx->lane(ln));
                    cudaGetLastError();
                }
            } catch (const Error &e) {
                failed(f, e.code, e.msg);
            } catch (const std::exception &e) {
                failed(f, RP_E_ARG, e.what());
            }
            lk.lock();
            busy[f.run->slot] = false;
            sv.done[f.job.ticket] = {f.status, f.msg};
            sv.finished.notify_all();
            flights.erase(flights.begin() + (long)k);
            progressed = true;
        }
        if (sv.stop && flights.empty()) return;
        // 2. start the oldest queued batch in a free slot
        int free_slot = -1;
        for (int q = 0; q < kBatchSlots && free_slot < 0; ++q)
            if (!busy[q]) free_slot = q;
        if (!sv.stop && !sv.queue.empty() && free_slot >= 0) {
            std::unique_ptr<Flight> f(new Flight());
            f->job = std::move(sv.queue.front());
            sv.queue.pop_front();
            busy[free_slot] = true;
            lk.unlock();
            f->run.reset(new BatchRun());
            f->run->slot = free_slot;
            ctx->cur_slot = free_slot;
            {  // a batch of small cubes runs at the greatest stream priority (kLowPriorityWork)
                double work = 0.0;
                for (const rp_fit_desc &d : f->job.descs)
                    work = std::max(work, (double)d.grid.n_grid[0] * d.grid.n_grid[1] * d.grid.n_grid[2] * d.N);
                ctx->cur_prio = work < kLowPriorityWork ? 1 : 0;
            }
            f->run->prio = ctx->cur_prio;
            try {
                const BatchServer::Job &j = f->job;
                batch_enqueue(ctx, (int)j.descs.size(), j.descs.data(), j.has_vdev ? j.vdev.data() : nullptr,
                              j.q_out, j.M_out, j.info_out, ctx->lane(kLaneBatch), *f->run);
            } catch (const Error &e) {
                failed(*f, e.code, e.msg);
            } catch (const std::exception &e) {
                failed(*f, RP_E_ARG, e.what());
            }
            f->run->slot = free_slot;
            lk.lock();
            flights.push_back(std::move(f));
            continue;
        }
        if (progressed) continue;
        if (flights.empty())
            sv.cv.wait(lk, [&] { return sv.stop || !sv.queue.empty(); });
        else  // device work in flight: poll its events, and wake early for new submissions
            sv.cv.wait_for(lk, std::chrono::microseconds(100));
    }
}

void batch_server_stop(rp_ctx *ctx) {
    if (!ctx->server) return;
    {
        std::lock_guard<std::mutex> g(ctx->server->mu);
        ctx->server->stop = true;
    }
    ctx->server->cv.notify_all();
    if (ctx->server->th.joinable()) ctx->server->th.join();
    ctx->server.reset();
}
}  // namespace rp

extern "C" {

int rp_fit_batch(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, double *q_out,
                 int64_t *M_out, double *info_out, rp_stream_t stream) {
    if (!ctx || n < 0 || (n > 0 && (!descs || !q_out))) return RP_E_ARG;
    return guarded(ctx, [&] { rp::fit_batch_body(ctx, n, descs, V_dev, q_out, M_out, info_out, (cudaStream_t)stream); });
}

int rp_batch_submit(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, double *q_out,
                    int64_t *M_out, double *info_out, long long *ticket) {
    if (!ctx || n <= 0 || !descs || !q_out || !ticket) return RP_E_ARG;
    // no CUDA call here, and ctx->last_error is not touched: submit, poll and wait may be
    // called from different host threads (the server's lock orders them)
    {
        static std::mutex create;
        std::lock_guard<std::mutex> g(create);
        if (!ctx->server) {
            ctx->server.reset(new rp::BatchServer());
            ctx->server->th = std::thread(rp::batch_server_loop, ctx);
        }
    }
    try {
        rp::BatchServer::Job job;
        job.descs.assign(descs, descs + n);
        job.has_vdev = V_dev != nullptr;
        if (V_dev) job.vdev.assign(V_dev, V_dev + n);
        job.q_out = q_out;
        job.M_out = M_out;
        job.info_out = info_out;
        {
            std::lock_guard<std::mutex> g(ctx->server->mu);
            job.ticket = ctx->server->next++;
            *ticket = job.ticket;
            ctx->server->pending.insert(job.ticket);
            ctx->server->queue.push_back(std::move(job));
        }
        ctx->server->cv.notify_all();
        return RP_OK;
    } catch (const std::exception &) {
        return RP_E_NOMEM;
    }
}

// done = 1 once the batch has finished; *status is then its rp_fit_batch status (the
// message, if any, becomes rp_last_error) and the ticket is retired.
static int batch_result(rp_ctx *ctx, long long ticket, bool wait, int *done, int *status) {
    if (!ctx || !ctx->server) return RP_E_ARG;
    rp::BatchServer &sv = *ctx->server;
    std::unique_lock<std::mutex> lk(sv.mu);
    if (!sv.pending.count(ticket)) return RP_E_ARG;
    if (wait) sv.finished.wait(lk, [&] { return sv.done.count(ticket) > 0; });
    auto it = sv.done.find(ticket);
    if (it == sv.done.end()) {
        if (done) *done = 0;
        return RP_OK;
    }
    if (done) *done = 1;
    if (status) *status = it->second.first;
    ctx->last_error = it->second.second;
    sv.done.erase(it);
    sv.pending.erase(ticket);
    return RP_OK;
}

int rp_batch_poll(rp_ctx *ctx, long long ticket, int *done, int *status) {
    return batch_result(ctx, ticket, false, done, status);
}

int rp_batch_wait(rp_ctx *ctx, long long ticket, int *status) { return batch_result(ctx, ticket, true, nullptr, status); }

int rp_launch_count(long long *out) {
    if (!out) return RP_E_ARG;
    *out = rp::g_launches.load();
    return RP_OK;
}

int rp_autotune(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, const char *cache_path) {
    if (!ctx || n < 0 || (n > 0 && !descs)) return RP_E_ARG;
    return guarded(ctx, [&] {
        using namespace rp;
        const cudaStream_t st = ctx->lane(0);
        std::map<long long, int> first;  // bucket -> the first cube of the batch in it
        std::vector<long long> Ms((size_t)n, 0);
        long long *d_M = ctx->buf_t<long long>("tune_M", 1);
        double *d_vst = ctx->buf_t<double>("tune_vst", 2);
        int *d_clamp = ctx->buf_t<int>("tune_clamp", 1);
        // the kept points of each cube (brick order, as the batch fits them), then one cube per bucket
        std::vector<int> pick;
        for (int i = 0; i < n; ++i) {
            const rp_fit_desc &d = descs[i];
            if (d.precision != RP_PREC_MIXED) continue;
            RP_REQUIRE(d.atoms && d.Z && d.N > 0 && ((V_dev && V_dev[i]) || d.V), "rp_autotune: bad descriptor");
            const long long np = (long long)d.grid.n_grid[0] * d.grid.n_grid[1] * d.grid.n_grid[2];
            const double *V = V_dev && V_dev[i] ? V_dev[i] : nullptr;
            if (!V) {
                double *v = ctx->buf_t<double>("tune_V", (size_t)np);
                RP_CUDA(cudaMemcpyAsync(v, d.V, sizeof(double) * np, cudaMemcpyHostToDevice, st));
                V = v;
            }
            int32_t *kept = ctx->buf_t<int32_t>("tune_kept", (size_t)np);
            double *Vc = ctx->buf_t<double>("tune_Vc", (size_t)np);
            filter_async(ctx, &d.grid, d.atoms, d.Z, d.N, V, d.vdw_factor, d.vdw_max, kept, Vc, d_M, nullptr, st,
                         "#tune", true, d_vst);
            RP_CUDA(cudaMemcpyAsync(&Ms[i], d_M, sizeof(long long), cudaMemcpyDeviceToHost, st));
            RP_CUDA(cudaStreamSynchronize(st));
            const long long key = tile_key(d.N, Ms[i], d.kmax);
            if (Ms[i] > 0 && !first.count(key) && !ctx->tiles.count(key)) {
                first[key] = i;
                pick.push_back(i);
            }
        }
        std::string report;
        for (int i : pick) {
            const rp_fit_desc &d = descs[i];
            const long long np = (long long)d.grid.n_grid[0] * d.grid.n_grid[1] * d.grid.n_grid[2];
            const double *V = V_dev && V_dev[i] ? V_dev[i] : nullptr;
            if (!V) {
                double *v = ctx->buf_t<double>("tune_V", (size_t)np);
                RP_CUDA(cudaMemcpyAsync(v, d.V, sizeof(double) * np, cudaMemcpyHostToDevice, st));
                V = v;
            }
            int32_t *kept = ctx->buf_t<int32_t>("tune_kept", (size_t)np);
            double *Vc = ctx->buf_t<double>("tune_Vc", (size_t)np);
            filter_async(ctx, &d.grid, d.atoms, d.Z, d.N, V, d.vdw_factor, d.vdw_max, kept, Vc, d_M, nullptr, st,
                         "#tune", true, d_vst);
            rp_ewald ew;
            ew.device = ctx->device;
            ewald_build(&ew, &d.grid, d.cutoff, d.kmax);
            struct Free {
                rp_ewald *e;
                ~Free() { ewald_free(e); }
            } fr{&ew};
            double *d_atoms = ctx->buf_t<double>("tune_atoms", 3 * (size_t)d.N);
            RP_CUDA(cudaMemcpyAsync(d_atoms, d.atoms, sizeof(double) * 3 * d.N, cudaMemcpyHostToDevice, st));
            float2 *E = ctx->buf_t<float2>("tune_E", recip_rows_bytes(&ew, d.N) / sizeof(float2));
            recip_rows(ctx, &ew, d_atoms, nullptr, d.N, E, st, "#tune");
            std::vector<double> rn((size_t)d.N);
            for (int a = 0; a < d.N; ++a) rn[a] = d.vdw_factor * radius_of(d.Z[a]);
            double *A = ctx->buf_t<double>("tune_A", (size_t)d.N * d.N);
            double *b = ctx->buf_t<double>("tune_b", (size_t)d.N);
            cudaEvent_t e0, e1;
            RP_CUDA(cudaEventCreate(&e0));
            RP_CUDA(cudaEventCreate(&e1));
            TileConfig best{};
            float best_ms = 1e30f, default_ms = 0.f;
            for (int at : {8, 16, 32})
                for (int split : {4, 8, 16}) {
                    const TileConfig tc{at, split};
                    float ms = 1e30f;
                    for (int rep = 0; rep < 3; ++rep) {  // the first is a warm-up
                        RP_CUDA(cudaMemsetAsync(d_clamp, 0, sizeof(int), st));
                        RP_CUDA(cudaEventRecord(e0, st));
                        gram_mixed(ctx, &ew, d.atoms, d.N, kept, Vc, Ms[i], A, b, nullptr, st, d_vst, "#tune",
                                   rn.data(), d_clamp, d_atoms, E, tc);
                        RP_CUDA(cudaEventRecord(e1, st));
                        RP_CUDA(cudaEventSynchronize(e1));
                        float t = 0.f;
                        RP_CUDA(cudaEventElapsedTime(&t, e0, e1));
                        if (rep > 0) ms = std::min(ms, t);
                    }
                    if (at == 16 && split == 16) default_ms = ms;
                    if (ms < best_ms) {
                        best_ms = ms;
                        best = tc;
                    }
                }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            const long long key = tile_key(d.N, Ms[i], d.kmax);
            ctx->tiles[key] = best;
            report += std::to_string(key) + " " + std::to_string(best.phi_atoms) + " " +
                      std::to_string(best.gram_split) + " " + std::to_string(best_ms) + " " +
                      std::to_string(default_ms) + " " + std::to_string(d.N) + " " + std::to_string(Ms[i]) + "\n";
        }
        status_check(ctx, st);
        if (cache_path && *cache_path) {
            FILE *f = std::fopen(cache_path, "w");
            RP_REQUIRE(f, std::string("rp_autotune: cannot write ") + cache_path);
            std::fputs("# key phi_atoms gram_split best_ms default_ms N M\n", f);
            for (auto &kv : ctx->tiles) {
                std::string line = std::to_string(kv.first) + " " + std::to_string(kv.second.phi_atoms) + " " +
                                   std::to_string(kv.second.gram_split);
                // keep this run's timings on the buckets it measured
                const std::string tag = std::to_string(kv.first) + " ";
                size_t pos = report.find(tag);
                if (pos == 0 || (pos != std::string::npos && report[pos - 1] == '\n')) {
                    const size_t end = report.find('\n', pos);
                    line = report.substr(pos, end - pos);
                }
                std::fputs((line + "\n").c_str(), f);
            }
            std::fclose(f);
        }
    });
}

int rp_load_tiles(rp_ctx *ctx, const char *cache_path) {
    if (!ctx || !cache_path) return RP_E_ARG;
    return guarded(ctx, [&] {
        FILE *f = std::fopen(cache_path, "r");
        RP_REQUIRE(f, std::string("rp_load_tiles: cannot read ") + cache_path);
        char line[512];
        while (std::fgets(line, sizeof line, f)) {
            if (line[0] == '#') continue;
            long long key = 0;
            int at = 0, split = 0;
            if (std::sscanf(line, "%lld %d %d", &key, &at, &split) == 3 && (at == 8 || at == 16 || at == 32) &&
                split >= 1 && split <= 16)
                ctx->tiles[key] = rp::TileConfig{at, split};
        }
        std::fclose(f);
    });
}

// Diagnostics (not part of the public ABI): host timeline of the batched fit.  on != 0
// starts recording (and clears the log), 0 stops; rp_debug_trace_read writes the log as
// "label<TAB>milliseconds since the first mark" lines into buf (cap bytes, NUL-terminated).
extern "C" int rp_debug_trace(rp_ctx *ctx, int on) {
    if (!ctx) return RP_E_ARG;
    std::lock_guard<std::mutex> lk(ctx->trace_mu);
    ctx->trace = on != 0;
    if (on) ctx->trace_log.clear();
    return RP_OK;
}
extern "C" int rp_debug_trace_read(rp_ctx *ctx, char *buf, size_t cap) {
    if (!ctx || !buf || cap == 0) return RP_E_ARG;
    std::lock_guard<std::mutex> lk(ctx->trace_mu);
    std::string out;
    const double t0 = ctx->trace_log.empty() ? 0.0 : ctx->trace_log.front().second;
    char line[160];
    for (const auto &e : ctx->trace_log) {
        std::snprintf(line, sizeof(line), "%s\t%.3f\n", e.first.c_str(), e.second - t0);
        out += line;
    }
    std::snprintf(buf, cap, "%s", out.c_str());
    return RP_OK;
}

int rp_set_kappa_limit(rp_ctx *ctx, double kappa_max) {
    if (!ctx || !(kappa_max >= 0.0)) return RP_E_ARG;
    ctx->kappa_limit = kappa_max;
    return RP_OK;
}

int rp_set_timing(rp_ctx *ctx, int enable) {
    if (!ctx) return RP_E_ARG;
    ctx->timing = enable != 0;
    return RP_OK;
}

int rp_stage_times(rp_ctx *ctx, char *names, size_t names_cap, double *ms, int *count_inout) {
    if (!ctx || !count_inout) return RP_E_ARG;
    return guarded(ctx, [&] {
        std::vector<std::string> order;
        std::unordered_map<std::string, std::pair<double, int>> acc;
        for (auto &m : ctx->marks) {
            RP_CUDA(cudaEventSynchronize(m.b));
            float t = 0.f;
            RP_CUDA(cudaEventElapsedTime(&t, m.a, m.b));
            if (!acc.count(m.name)) order.push_back(m.name);
            acc[m.name].first += t;
            acc[m.name].second += 1;
            cudaEventDestroy(m.a);
            cudaEventDestroy(m.b);
        }
        ctx->marks.clear();
        std::string joined;
        int cap = *count_inout, k = 0;
        for (auto &nm : order) {
            if (k >= cap) break;
            if (ms) {
                ms[2 * k] = acc[nm].first;
                ms[2 * k + 1] = acc[nm].second;
            }
            joined += nm + "\n";
            ++k;
        }
        *count_inout = k;
        if (names && names_cap) {
            size_t n = std::min(names_cap - 1, joined.size());
            std::memcpy(names, joined.data(), n);
            names[n] = 0;
        }
    });
}

int rp_fit(rp_ctx *ctx, const rp_fit_desc *d, double *q_out, int64_t *M_out, rp_stream_t stream) {
    if (!ctx || !d || !q_out) return RP_E_ARG;
    return rp_fit_batch(ctx, 1, d, nullptr, q_out, M_out, nullptr, stream);
}

}  // extern "C"
