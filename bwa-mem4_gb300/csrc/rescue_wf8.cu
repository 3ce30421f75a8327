// rescue_wf8.cu -- the register wavefront (rescue_wf.cuh) for 8-lane groups
// (four jobs per warp; padded queries up to 256 columns).
#include "rescue_wf.cuh"

namespace bwacuda {
namespace wf {

template <>
cudaError_t launch_for_qcap<8>(const RescueLaunch &Lr, int qcap)
{
    if (qcap <= 8 * 4) return launch_wf<8, 4>(Lr);
    if (qcap <= 8 * 8) return launch_wf<8, 8>(Lr);
    if (qcap <= 8 * 12) return launch_wf<8, 12>(Lr);
    if (qcap <= 8 * 16) return launch_wf<8, 16>(Lr);
    if (qcap <= 8 * 20) return launch_wf<8, 20>(Lr);
    if (qcap <= 8 * 24) return launch_wf<8, 24>(Lr);
    if (qcap <= 8 * 32) return launch_wf<8, 32>(Lr);
    return cudaErrorInvalidValue;
}

}  // namespace wf
}  // namespace bwacuda
