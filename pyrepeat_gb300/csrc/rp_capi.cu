// C ABI of librepeat_gb300 (include/repeat_gb300.h): argument checks, the
// context, and the translation of internal errors into status codes.
#include <cstring>

#include "common.cuh"

namespace rp {
void ewald_build(rp_ewald *ew, const rp_grid *grid, double cutoff, int kmax);
void ewald_free(rp_ewald *ew);
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

struct DeviceBuf {  // RAII device buffer for rp_fit's own inputs/outputs
    void *p = nullptr;
    explicit DeviceBuf(size_t bytes) { RP_CUDA(cudaMalloc(&p, bytes ? bytes : 256)); }
    ~DeviceBuf() { cudaFree(p); }
    template <class T>
    T *as() { return static_cast<T *>(p); }
};

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
    cudaSetDevice(ctx->device);
    for (auto &kv : ctx->scratch) cudaFree(kv.second.ptr);
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
        if (precision == RP_PREC_FP64)
            rp::gram_fp64(ctx, ew, atoms, N, kept_idx_dev, Vc_dev, M, A_dev, b_dev, sum_phi_dev, (cudaStream_t)stream);
        else if (precision == RP_PREC_MIXED)
            rp::gram_mixed(ctx, ew, atoms, N, kept_idx_dev, Vc_dev, M, A_dev, b_dev, sum_phi_dev, (cudaStream_t)stream);
        else
            rp::fail(RP_E_ARG, "rp_gram: unknown precision");
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

int rp_fit(rp_ctx *ctx, const rp_fit_desc *d, double *q_out, int64_t *M_out, rp_stream_t stream_) {
    if (!ctx || !d || !q_out) return RP_E_ARG;
    cudaStream_t stream = (cudaStream_t)stream_;
    rp_ewald *ew = nullptr;
    int rc = guarded(ctx, [&] {
        RP_REQUIRE(d->V && d->atoms && d->Z && d->N > 0, "rp_fit: null input or N <= 0");
        const long long npts = (long long)d->grid.n_grid[0] * d->grid.n_grid[1] * d->grid.n_grid[2];
        RP_REQUIRE(npts > 0, "rp_fit: empty grid");
        const int N = d->N;
        double *V = ctx->buf_t<double>("fit_V", (size_t)npts);
        int32_t *kept = ctx->buf_t<int32_t>("fit_kept", (size_t)npts);
        double *Vc = ctx->buf_t<double>("fit_Vc", (size_t)npts);
        double *A = ctx->buf_t<double>("fit_A", (size_t)N * N);
        double *b = ctx->buf_t<double>("fit_b", (size_t)N);
        double *q = ctx->buf_t<double>("fit_q", (size_t)N);
        RP_CUDA(cudaMemcpyAsync(V, d->V, sizeof(double) * npts, cudaMemcpyHostToDevice, stream));
        int64_t M = 0;
        rp::filter_run(ctx, &d->grid, d->atoms, d->Z, N, V, d->vdw_factor, d->vdw_max, kept, Vc, npts, &M, nullptr,
                       stream);
        if (M_out) *M_out = M;
        RP_REQUIRE(M > 0, "rp_fit: no grid point survives the vdW filter");
        ew = new rp_ewald();
        ew->device = ctx->device;
        rp::ewald_build(ew, &d->grid, d->cutoff, d->kmax);
        if (d->precision == RP_PREC_MIXED)
            rp::gram_mixed(ctx, ew, d->atoms, N, kept, Vc, M, A, b, nullptr, stream);
        else
            rp::gram_fp64(ctx, ew, d->atoms, N, kept, Vc, M, A, b, nullptr, stream);
        rp::solve_run(ctx, A, b, N, d->n_groups, d->group_ptr, d->group_idx, d->resp_s, d->resp_t, d->qtot, q, nullptr,
                      stream);
        RP_CUDA(cudaMemcpyAsync(q_out, q, sizeof(double) * N, cudaMemcpyDeviceToHost, stream));
        RP_CUDA(cudaStreamSynchronize(stream));
    });
    if (ew) {
        rp::ewald_free(ew);
        delete ew;
    }
    return rc;
}

}  // extern "C"
