// batched.cu -- the batched extension path (length buckets, persistent kernel,
// graph replay).  Built out in steps; until the persistent kernel lands the
// batched path reports BWACUDA_EUNSUPPORTED rather than silently running the
// plain one.
#include "runtime.h"

namespace bwacuda {

int extend_batch_host_batched(bwacuda_ctx *, const bwacuda_ext_job *, size_t, const ExtParams &, int,
                              bwacuda_ext_result *)
{
    return BWACUDA_EUNSUPPORTED;
}

int extend_device_batched(bwacuda_ctx *, const uint8_t *, const bwacuda_dev_ext_job *, size_t,
                          const ExtParams &, bwacuda_ext_result *, cudaStream_t)
{
    return BWACUDA_EUNSUPPORTED;
}

void batched_release(bwacuda_ctx *) {}

void server_shutdown(bwacuda_ctx *) {}

}  // namespace bwacuda
