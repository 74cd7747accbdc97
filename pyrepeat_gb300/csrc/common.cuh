// Internal definitions shared by the translation units of librepeat_gb300.
#pragma once

#include <cuda_runtime.h>
#include <cublas_v2.h>

#include <cstdint>
#include <cstdio>
#include <string>
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

// Check a kernel launch (configuration errors surface here, not later).
#define RP_LAUNCH_CHECK() RP_CUDA(cudaGetLastError())

struct Buffer {
    void *ptr = nullptr;
    size_t bytes = 0;
};

}  // namespace rp

struct rp_ctx {
    int device = 0;
    int sm_count = 0;
    size_t budget = 0;
    size_t used = 0;
    std::string last_error;
    cublasHandle_t cublas = nullptr;
    std::unordered_map<std::string, rp::Buffer> scratch;
    int *d_status = nullptr;  // device status word for bounded waits / singular flags

    // Grow-only named scratch buffer owned by the ctx.
    void *buf(const std::string &name, size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        if (bytes == 0) bytes = 256;
        auto &b = scratch[name];
        if (b.bytes >= bytes) return b.ptr;
        if (b.ptr) {
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
    cublasHandle_t blas();
};

struct rp_ewald {
    int device = 0;
    rp_grid grid{};
    double cutoff = 20.0, alpha = 0.0, sqrt_alpha = 0.0, volume = 0.0;
    double box[9]{};
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
    // the same k-set ordered by increasing kcoef (used by the tensor-core path so
    // that small terms are accumulated before large ones)
    int *d_kidx_s = nullptr;
    double *d_kcoef_s = nullptr;
    double *d_kvec_s = nullptr;
    double2 *d_ex = nullptr;      // (kmax+1) * nx   e^{2 pi i n1 i / nx}
    double2 *d_ey = nullptr;      // (2kmax+1) * ny  e^{2 pi i n2 j / ny}, n2 offset by kmax
    double2 *d_ez = nullptr;      // (2kmax+1) * nz
};

namespace rp {

// Host helpers shared by the stages.
void prune_shifts(const rp_ewald *ew, const double *atoms, int N, std::vector<double> &out, int &zero_idx);

// Stage launchers (each enqueues on `stream`).
void filter_run(rp_ctx *ctx, const rp_grid *grid, const double *atoms, const int *Z, int N, const double *V_dev,
                double vdw_factor, double vdw_max, int32_t *kept_idx_dev, double *Vc_dev, int64_t capacity,
                int64_t *M_out, uint8_t *mask_dev, cudaStream_t stream);
void gram_fp64(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
               const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
               cudaStream_t stream);
void gram_mixed(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
                const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
                cudaStream_t stream);
void solve_run(rp_ctx *ctx, const double *A_dev, const double *b_dev, int N, int n_groups, const int *group_ptr,
               const int *group_idx, const double *resp_s, const double *resp_t, double qtot, double *q_dev,
               double *info, cudaStream_t stream);

// Device table builders (ewald_tables.cu).
void atom_tables_fp64(const rp_ewald *ew, const double *d_atoms, int N, double *d_B, int ldb, cudaStream_t s);
void grid_tables_fp64(const rp_ewald *ew, const int32_t *d_kept, int64_t m0, int64_t rows, double *d_T, int ldt,
                      cudaStream_t s);

// Shared epilogue kernels (phi_fp64.cu).
void column_sums_fp64(const double *X, int64_t rows, int cols, int ld, double *out, bool accumulate,
                      rp_ctx *ctx, cudaStream_t s);
void finish_normal_equations(const double *G, const double *r, const double *s_c, double *sumV_dev, int64_t M,
                             int N, double *A, double *b, cudaStream_t s);

inline unsigned ceil_div(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

}  // namespace rp
