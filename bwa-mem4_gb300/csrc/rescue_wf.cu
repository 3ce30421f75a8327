// rescue_wf.cu -- the register wavefront (rescue_wf.cuh) for 16-lane groups,
// and the dispatch over group widths.
#include "rescue_wf.cuh"

namespace bwacuda {
namespace wf {

template <>
cudaError_t launch_for_qcap<16>(const RescueLaunch &Lr, int qcap)
{
    // columns per lane for 16-lane groups
    if (qcap <= 16 * 4) return launch_wf<16, 4>(Lr);
    if (qcap <= 16 * 6) return launch_wf<16, 6>(Lr);
    if (qcap <= 16 * 8) return launch_wf<16, 8>(Lr);
    if (qcap <= 16 * 10) return launch_wf<16, 10>(Lr);
    if (qcap <= 16 * 12) return launch_wf<16, 12>(Lr);
    if (qcap <= 16 * 16) return launch_wf<16, 16>(Lr);
    if (qcap <= 16 * 20) return launch_wf<16, 20>(Lr);
    if (qcap <= 16 * 24) return launch_wf<16, 24>(Lr);
    if (qcap <= 16 * 32) return launch_wf<16, 32>(Lr);
    return cudaErrorInvalidValue;
}

}  // namespace wf

// Widest padded query the wavefront kernels take (16 or 32 lanes x 32 / 16 columns).
int rescue_wf_max_qpad() { return 512; }

// Widest padded query of `lanes`-lane groups.
static int wf_max_qpad_of(int lanes) { return lanes == 8 ? 256 : 512; }

cudaError_t rescue_wf_launch(const RescueLaunch &Lr, int qcap, int lanes)
{
    if (lanes == 8 && qcap <= wf_max_qpad_of(8)) return wf::launch_for_qcap<8>(Lr, qcap);
    if (lanes == 32) return wf::launch_for_qcap<32>(Lr, qcap);
    return wf::launch_for_qcap<16>(Lr, qcap);
}

}  // namespace bwacuda
