// ext_persist_g4.cu -- the persistent extension bucket kernels with 4 32-job
// rounds per work grab (templates in ext_persist.cuh).
#include "ext_persist.cuh"

namespace bwacuda {

cudaError_t ext_persist_launch_g4(const PersistLaunch &L, const ExtBucketDef &d, uint32_t *table, int nsm, int tb)
{
    return persist::ext_persist_launch_grab<4>(L, d, table, nsm, tb);
}

}  // namespace bwacuda
