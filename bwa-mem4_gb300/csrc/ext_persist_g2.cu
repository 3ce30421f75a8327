// ext_persist_g2.cu -- the persistent extension bucket kernels with 2 32-job
// rounds per work grab (templates in ext_persist.cuh).
#include "ext_persist.cuh"

namespace bwacuda {

cudaError_t ext_persist_launch_g2(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb)
{
    return persist::ext_persist_launch_grab<2>(L, d, table, nsm, tb);
}

}  // namespace bwacuda
