// Mixed-precision Phi -> normal equations on the tensor cores (filled in below).
#include "common.cuh"

namespace rp {
void gram_mixed(rp_ctx *ctx, const rp_ewald *ew, const double *atoms, int N, const int32_t *kept_idx_dev,
                const double *Vc_dev, int64_t M, double *A_dev, double *b_dev, double *sum_phi_dev,
                cudaStream_t stream) {
    (void)ctx; (void)ew; (void)atoms; (void)N; (void)kept_idx_dev; (void)Vc_dev; (void)M; (void)A_dev; (void)b_dev;
    (void)sum_phi_dev; (void)stream;
    fail(RP_E_UNSUPPORTED, "rp_gram: mixed precision not built yet");
}
}  // namespace rp
