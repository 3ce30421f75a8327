// ext_persist_g1.cu -- the persistent extension bucket kernels with 1 32-job
// round per work grab (templates in ext_persist.cuh).
#include "ext_persist.cuh"

namespace bwacuda {

cudaError_t ext_persist_launch_g1(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb)
{
    return persist::ext_persist_launch_grab<1>(L, d, table, nsm, tb);
}

}  // namespace bwacuda
