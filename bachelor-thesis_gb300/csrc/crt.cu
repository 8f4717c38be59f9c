// CRT (multi-modular) path -- filled in below.
#include "gbmm_internal.h"
namespace gbmm {
struct crt_cache {};
crt_cache *crt_cache_create() { return new crt_cache(); }
void crt_cache_destroy(crt_cache *c) { delete c; }
gbmm_status crt_matmul(gbmm_handle, const gbmm_mat &, const gbmm_mat &, const gbmm_mat &, int64_t, int64_t, int, int,
                       cudaStream_t) {
    return set_error(GBMM_ERR_UNSUPPORTED, "CRT path not built");
}
}  // namespace gbmm
