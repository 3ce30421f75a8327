// rescue_wf32.cu -- the register wavefront (rescue_wf.cuh) for 32-lane groups
// (one job per warp; padded queries up to 512 columns).
#include "rescue_wf.cuh"

namespace bwacuda {
namespace wf {

template <>
cudaError_t launch_for_qcap<32>(const RescueLaunch &Lr, int qcap)
{
    if (qcap <= 32 * 2) return launch_wf<32, 2>(Lr);
    if (qcap <= 32 * 3) return launch_wf<32, 3>(Lr);
    if (qcap <= 32 * 4) return launch_wf<32, 4>(Lr);
    if (qcap <= 32 * 5) return launch_wf<32, 5>(Lr);
    if (qcap <= 32 * 6) return launch_wf<32, 6>(Lr);
    if (qcap <= 32 * 8) return launch_wf<32, 8>(Lr);
    if (qcap <= 32 * 10) return launch_wf<32, 10>(Lr);
    if (qcap <= 32 * 12) return launch_wf<32, 12>(Lr);
    if (qcap <= 32 * 16) return launch_wf<32, 16>(Lr);
    return cudaErrorInvalidValue;
}

}  // namespace wf
}  // namespace bwacuda
