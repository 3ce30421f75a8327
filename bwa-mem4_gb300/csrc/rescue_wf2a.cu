// rescue_wf2a.cu -- the paired register wavefront (rescue_wf2.cuh) for scorings whose two gap
// opens differ (o_del + e_del != o_ins + e_ins): F opens from M0, E from H.
#include "rescue_wf2.cuh"

namespace bwacuda {
namespace wf2 {

cudaError_t launch_asym(const RescueLaunch &Lr, int lanes, int c, int npen)
{
    return launch_shape<false>(Lr, lanes, c, npen);
}

}  // namespace wf2
}  // namespace bwacuda
