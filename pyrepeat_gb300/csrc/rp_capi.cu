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

void smem_optin(const void *kernel, size_t bytes) {
    if (bytes <= (48u << 10)) return;
    int dev = 0;
    RP_CUDA(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> raised;
    std::lock_guard<std::mutex> lk(mu);
    size_t &have = raised[{kernel, dev}];
    if (bytes > have) {
        RP_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        have = bytes;
    }
}
void status_clear(rp_ctx *ctx, cudaStream_t s) { RP_CUDA(cudaMemsetAsync(ctx->d_status, 0, 2 * sizeof(int), s)); }
void status_check(rp_ctx *ctx, cudaStream_t s) {
    int st[2] = {0, 0};
    RP_CUDA(cudaMemcpyAsync(st, ctx->d_status, sizeof(st), cudaMemcpyDeviceToHost, s));
    RP_CUDA(cudaStreamSynchronize(s));
    if (st[0] != 0) fail(st[0], "a tensor-core pipeline wait ran out of time");
    if (st[1] != 0)
        fail(RP_E_STATE, std::to_string(st[1]) + " Phi values exceeded the fixed-point range set on the first chunk");
}
}  // namespace rp

cublasHandle_t rp_ctx::blas() {
    if (!cublas) {
        RP_CUBLAS(cublasCreate(&cublas));
        RP_CUBLAS(cublasSetMathMode(cublas, CUBLAS_DEFAULT_MATH));  // native FP64, no emulation
    }
    return cublas;
}

namespace {

template <class F>
int guarded(rp_ctx *ctx, F &&f) {
    try {
        if (ctx) RP_CUDA(cudaSetDevice(ctx->device));
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

int rp_version(void) { return 10000; }

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
        RP_CUDA(cudaMalloc(&c->d_status, 64));
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
    if (ctx->cublas) cublasDestroy(ctx->cublas);
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
// The batched fit; throws rp::Error.  Used by rp_fit_batch (on the caller's thread) and by
// the asynchronous batch server (on its worker thread).
void fit_batch_body(rp_ctx *ctx, int n, const rp_fit_desc *descs, const double *const *V_dev, double *q_out,
                    int64_t *M_out, double *info_out, cudaStream_t stream) {
    std::vector<rp_ewald *> ews((size_t)n, nullptr);
    {
        if (n == 0) return;
        std::vector<long long> npts((size_t)n), off_pts((size_t)n + 1, 0), off_n((size_t)n + 1, 0),
            off_nn((size_t)n + 1, 0);
        for (int i = 0; i < n; ++i) {
            const rp_fit_desc &d = descs[i];
            RP_REQUIRE(d.atoms && d.Z && d.N > 0, "rp_fit: null input or N <= 0");
            RP_REQUIRE(d.precision == RP_PREC_FP64 || d.precision == RP_PREC_MIXED, "rp_fit: unknown precision");
            RP_REQUIRE((V_dev && V_dev[i]) || d.V, "rp_fit: no ESP values");
            npts[i] = (long long)d.grid.n_grid[0] * d.grid.n_grid[1] * d.grid.n_grid[2];
            RP_REQUIRE(npts[i] > 0 && npts[i] < (1LL << 31), "rp_fit: bad grid");
            off_pts[i + 1] = off_pts[i] + npts[i];
            off_n[i + 1] = off_n[i] + d.N;
            off_nn[i + 1] = off_nn[i] + (long long)d.N * d.N;
        }
        // Work splits into host preparation and device stages so that the device never waits
        // on the host inside the batch, and the cubes run as a pipeline of up to four groups:
        // (1) the filters' host halves on the host workers, one pinned upload, and the filter
        // launches of every group on their own streams; (2) while they run, the Ewald tables
        // of every cube on the host workers, one pinned upload; (3) as each group's kept
        // counts arrive, its normal equations go to the gram streams, so later groups'
        // filters overlap earlier groups' grams.
        constexpr int kLanes = 4;
        const int lanes = ctx->timing ? 1 : kLanes;  // stage timing: one lane, each stage alone
        auto glane = [&](int i) { return ctx->lane(i % lanes); };
        auto flane = [&](int i) { return ctx->timing ? ctx->lane(0) : ctx->lane(kLanes + i % kLanes); };
        const int ngroups = (n >= 64 && !ctx->timing) ? 4 : 1;
        std::vector<int> g0((size_t)ngroups + 1);
        for (int g = 0; g <= ngroups; ++g) g0[g] = (int)((long long)n * g / ngroups);
        int32_t *kept = ctx->buf_t<int32_t>("fit_kept", (size_t)off_pts[n]);
        double *Vc = ctx->buf_t<double>("fit_Vc", (size_t)off_pts[n]);
        double *Vh = nullptr;
        bool any_host = false;
        for (int i = 0; i < n; ++i) any_host |= !(V_dev && V_dev[i]);
        if (any_host) Vh = ctx->buf_t<double>("fit_V", (size_t)off_pts[n]);
        long long *Md = ctx->buf_t<long long>("fit_M", (size_t)n);
        long long *Mh = static_cast<long long *>(ctx->host_buf("fit_M", sizeof(long long) * n));
        double *A = ctx->buf_t<double>("fit_A", (size_t)off_nn[n]);
        double *b = ctx->buf_t<double>("fit_b", (size_t)off_n[n]);
        double *q = ctx->buf_t<double>("fit_q", (size_t)off_n[n]);
        double *vst = ctx->buf_t<double>("fit_vstats", 2 * (size_t)n);
        int *clamps = ctx->buf_t<int>("fit_clamps", (size_t)n);
        rp::status_clear(ctx, stream);
        RP_CUDA(cudaMemsetAsync(clamps, 0, sizeof(int) * n, stream));
        std::vector<cudaEvent_t> events;
        auto record = [&](cudaStream_t st) {
            cudaEvent_t ev;
            RP_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            events.push_back(ev);
            RP_CUDA(cudaEventRecord(ev, st));
            return ev;
        };
        struct EventGuard {  // destroyed on every exit (a recorded event may still be pending)
            std::vector<cudaEvent_t> &e;
            ~EventGuard() {
                for (cudaEvent_t ev : e) cudaEventDestroy(ev);
            }
        } guard{events};
        // 1. filters, group by group: the host plans a group (its workers), packs it into the
        //    group's pinned arena and queues the upload, the grids and the filter launches, then
        //    plans the next group while the device runs this one
        while ((int)ctx->plan_pool.size() < n) ctx->plan_pool.emplace_back(new rp::FilterPlan());
        auto plan = [&](int i) -> rp::FilterPlan & { return *ctx->plan_pool[(size_t)i]; };
        {
            const cudaEvent_t up = record(stream);  // every stream starts after the caller's work so far
            for (int ln = 0; ln < kLanes; ++ln) {
                RP_CUDA(cudaStreamWaitEvent(ctx->lane(ln), up, 0));
                RP_CUDA(cudaStreamWaitEvent(flane(ln), up, 0));
            }
        }
        const cudaStream_t copy_lane = ctx->lane(2 * kLanes);  // uploads: plans, grids, tables
        RP_CUDA(cudaStreamWaitEvent(copy_lane, events.back(), 0));
        std::vector<size_t> pl_off((size_t)n + 1, 0);
        std::vector<cudaEvent_t> kept_ready((size_t)ngroups);
        for (int g = 0; g < ngroups; ++g) {
            const int i0 = g0[g], i1 = g0[g + 1];
            ctx->parallel(i1 - i0, [&](int t) {
                const rp_fit_desc &d = descs[i0 + t];
                rp::filter_plan(&d.grid, d.atoms, d.Z, d.N, d.vdw_factor, d.vdw_max, plan(i0 + t));
            });
            pl_off[i0] = 0;
            for (int i = i0; i < i1; ++i) pl_off[i + 1] = pl_off[i] + plan(i).bytes();
            const std::string gtag = "fit_filter#" + std::to_string(g);
            char *pl_dev = static_cast<char *>(ctx->buf(gtag, pl_off[i1]));
            char *pl_host = static_cast<char *>(ctx->host_buf(gtag, pl_off[i1]));
            ctx->parallel(i1 - i0, [&](int t) { plan(i0 + t).pack(pl_host + pl_off[i0 + t]); });
            RP_CUDA(cudaMemcpyAsync(pl_dev, pl_host, pl_off[i1], cudaMemcpyHostToDevice, copy_lane));
            for (int i = i0; i < i1; ++i)  // grids from host memory, this group's only
                if (!(V_dev && V_dev[i]))
                    RP_CUDA(cudaMemcpyAsync(Vh + off_pts[i], descs[i].V, sizeof(double) * npts[i],
                                            cudaMemcpyHostToDevice, copy_lane));
            const cudaEvent_t inputs = record(copy_lane);
            for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(flane(ln), inputs, 0));
            for (int i = i0; i < i1; ++i) {
                const rp_fit_desc &d = descs[i];
                const double *V = (V_dev && V_dev[i]) ? V_dev[i] : Vh + off_pts[i];
                const int ln = i % lanes;
                rp::filter_launch(ctx, plan(i), pl_dev + pl_off[i], V, kept + off_pts[i], Vc + off_pts[i], Md + i,
                                  nullptr, flane(i), "#f" + std::to_string(ln), d.precision == RP_PREC_MIXED,
                                  vst + 2 * i);
            }
            for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(stream, record(flane(ln)), 0));
            RP_CUDA(cudaMemcpyAsync(Mh + i0, Md + i0, sizeof(long long) * (i1 - i0), cudaMemcpyDeviceToHost, stream));
            kept_ready[g] = record(stream);
        }
        // 2. Ewald tables, written by the host workers straight into one pinned arena,
        //    uploaded with a single copy on a stream of its own
        std::vector<size_t> ew_off((size_t)n + 1, 0);
        while ((int)ctx->ew_pool.size() < n) ctx->ew_pool.emplace_back(new rp_ewald());
        for (int i = 0; i < n; ++i) {
            size_t off9[9];
            ews[i] = ctx->ew_pool[(size_t)i].get();
            ews[i]->device = ctx->device;
            ew_off[i + 1] = ew_off[i] + rp::ewald_layout(&descs[i].grid, descs[i].kmax, off9);
        }
        char *ew_dev = static_cast<char *>(ctx->buf("fit_ewald", ew_off[n]));
        char *ew_host = static_cast<char *>(ctx->host_buf("fit_ewald", ew_off[n]));
        ctx->parallel(n, [&](int i) {
            rp::ewald_build_host(ews[i], &descs[i].grid, descs[i].cutoff, descs[i].kmax, ew_host + ew_off[i]);
        });
        for (int i = 0; i < n; ++i) rp::ewald_place(ews[i], ew_dev + ew_off[i]);
        RP_CUDA(cudaMemcpyAsync(ew_dev, ew_host, ew_off[n], cudaMemcpyHostToDevice, copy_lane));
        const cudaEvent_t tables = record(copy_lane);
        for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(glane(ln), tables, 0));
        RP_CUDA(cudaStreamWaitEvent(stream, tables, 0));
        // 3. normal equations, group by group as the kept counts arrive.  Mixed-precision fits
        //    are spread over the gram streams (each with its own scratch), so one cube's small
        //    kernels and launch gaps overlap another's; the FP64 comparator stays on the
        //    caller's stream (its cuBLAS handle is shared).  Every cube's result is independent
        //    of the stream it ran on.  A mixed fit takes the single pass (Phi straight to
        //    digits, scaled by the a-priori bounds from the scaled vdW radii); a cube whose
        //    values clamp (a cell the bound's argument does not cover) is redone below in
        //    two passes.
        std::vector<double> rn((size_t)off_n[n]);
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < descs[i].N; ++a)
                rn[off_n[i] + a] = descs[i].vdw_factor * rp::radius_of(descs[i].Z[a]);
        std::vector<long long> M((size_t)n);
        auto job = [&](int i) {
            const rp_fit_desc &d = descs[i];
            return rp::SolveJob{A + off_nn[i], b + off_n[i], d.N, d.n_groups, d.group_ptr, d.group_idx,
                                d.resp_s, d.resp_t, d.qtot, q + off_n[i]};
        };
        std::vector<const double *> ginfo((size_t)ngroups);
        for (int g = 0; g < ngroups; ++g) {
            RP_CUDA(cudaEventSynchronize(kept_ready[g]));
            for (int i = g0[g]; i < g0[g + 1]; ++i) {
                M[i] = Mh[i];
                if (M_out) M_out[i] = M[i];
                RP_REQUIRE(M[i] > 0, "rp_fit: no grid point of cube " + std::to_string(i) + " survives the vdW filter");
            }
            for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(glane(ln), kept_ready[g], 0));
            for (int i = g0[g]; i < g0[g + 1]; ++i) {
                const rp_fit_desc &d = descs[i];
                if (d.precision == RP_PREC_MIXED) {
                    const int ln = i % lanes;
                    rp::gram_mixed(ctx, ews[i], d.atoms, d.N, kept + off_pts[i], Vc + off_pts[i], M[i],
                                   A + off_nn[i], b + off_n[i], nullptr, glane(ln), vst + 2 * i,
                                   "#" + std::to_string(ln), rn.data() + off_n[i], clamps + i);
                } else {
                    rp::gram_fp64(ctx, ews[i], d.atoms, d.N, kept + off_pts[i], Vc + off_pts[i], M[i], A + off_nn[i],
                                  b + off_n[i], nullptr, stream);
                }
            }
            // 4. the group's constraint folds and bordered solves (one launch) on the caller's
            //    stream, behind its normal equations and overlapping the next group's
            for (int ln = 0; ln < lanes; ++ln) RP_CUDA(cudaStreamWaitEvent(stream, record(glane(ln)), 0));
            std::vector<rp::SolveJob> jobs;
            for (int i = g0[g]; i < g0[g + 1]; ++i) jobs.push_back(job(i));
            ginfo[g] = rp::solve_batch_async(ctx, jobs, stream, "#g" + std::to_string(g));
        }
        int *hclamps = static_cast<int *>(ctx->host_buf("fit_clamps", sizeof(int) * n));
        RP_CUDA(cudaMemcpyAsync(hclamps, clamps, sizeof(int) * n, cudaMemcpyDeviceToHost, stream));
        RP_CUDA(cudaStreamSynchronize(stream));
        std::vector<double> info((size_t)n * 4);
        for (int g = 0; g < ngroups; ++g)
            std::copy(ginfo[g], ginfo[g] + 4 * (size_t)(g0[g + 1] - g0[g]), info.begin() + 4 * (size_t)g0[g]);
        // 5. a cube whose values clamped: the two-pass fit, centred and scaled by the data, and
        //    its solve again
        ctx->last_fallbacks = 0;
        std::vector<int> redo;
        for (int i = 0; i < n; ++i)
            if (hclamps[i] != 0) {
                ++ctx->last_fallbacks;
                redo.push_back(i);
                const rp_fit_desc &d = descs[i];
                rp::gram_mixed(ctx, ews[i], d.atoms, d.N, kept + off_pts[i], Vc + off_pts[i], M[i], A + off_nn[i],
                               b + off_n[i], nullptr, stream, vst + 2 * i, "");
            }
        if (!redo.empty()) {
            std::vector<rp::SolveJob> jobs;
            for (int i : redo) jobs.push_back(job(i));
            std::vector<double> rinfo;
            rp::solve_batch(ctx, jobs, rinfo, stream);
            for (size_t t = 0; t < redo.size(); ++t)
                std::copy(rinfo.begin() + 4 * t, rinfo.begin() + 4 * t + 4, info.begin() + 4 * (size_t)redo[t]);
        }
        rp::status_check(ctx, stream);
        RP_CUDA(cudaMemcpyAsync(q_out, q, sizeof(double) * off_n[n], cudaMemcpyDeviceToHost, stream));
        RP_CUDA(cudaStreamSynchronize(stream));
        if (info_out) std::copy(info.begin(), info.end(), info_out);
        for (int i = 0; i < n; ++i)
            if (info[4 * (size_t)i + 3] != 0.0)
                rp::fail(RP_E_SINGULAR, "rp_fit: bordered system of cube " + std::to_string(i) + " is singular");
    }
    // the pooled Ewald objects borrow the arena: nothing to free
}

// Worker of the asynchronous batches: runs the queued batches in order on the ctx's device.
void batch_server_loop(rp_ctx *ctx) {
    BatchServer &sv = *ctx->server;
    cudaSetDevice(ctx->device);
    std::unique_lock<std::mutex> lk(sv.mu);
    for (;;) {
        sv.cv.wait(lk, [&] { return sv.stop || !sv.queue.empty(); });
        if (sv.stop) return;
        BatchServer::Job job = std::move(sv.queue.front());
        sv.queue.pop_front();
        lk.unlock();
        int status = RP_OK;
        std::string msg;
        try {
            fit_batch_body(ctx, (int)job.descs.size(), job.descs.data(), job.has_vdev ? job.vdev.data() : nullptr,
                           job.q_out, job.M_out, job.info_out, ctx->lane(2 * 4 + 1));
        } catch (const Error &e) {
            status = e.code;
            msg = e.msg;
        } catch (const std::exception &e) {
            status = RP_E_ARG;
            msg = e.what();
        }
        lk.lock();
        sv.done[job.ticket] = {status, msg};
        sv.finished.notify_all();
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
