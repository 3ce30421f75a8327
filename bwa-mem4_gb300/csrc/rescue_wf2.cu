// rescue_wf2.cu -- launches of the paired register wavefront (rescue_wf2.cuh): two rescue jobs
// per group of 8 or 16 lanes, one in each 16-bit lane of the registers.
#include "rescue_wf2.cuh"

namespace bwacuda {

namespace {

// The matrix suits the paired wavefront when its alphabet is at most bwa's five letters and its
// N column is one value (the profile word then covers codes 0..3 and N is patched per column).
bool pair_matrix_ok(const Scoring &sc, int *npen)
{
    if (sc.m > 5) return false;
    *npen = 0;
    if (sc.m < 5) return true;
    const int8_t n0 = (int8_t)(sc.prof[0][1] & 0xffu);  // mat[0][4]
    for (int t = 1; t < 5; ++t)
        if ((int8_t)(sc.prof[t][1] & 0xffu) != n0) return false;
    *npen = n0;
    return true;
}

// Columns per lane: the smallest listed C with L * C >= need.
template <int L>
int pick_c(int need);
template <>
int pick_c<8>(int need)
{
    static const int cs[] = {4, 8, 12, 16, 20, 24, 32};
    for (int c : cs)
        if (8 * c >= need) return c;
    return 0;
}
template <>
int pick_c<16>(int need)
{
    static const int cs[] = {4, 6, 8, 10, 12, 16};
    for (int c : cs)
        if (16 * c >= need) return c;
    return 0;
}

}  // namespace

cudaError_t rescue_wf2_launch(const RescueLaunch &Lr, int qcap, int lanes, int *cols)
{
    *cols = 0;
    int npen = 0;
    if (!pair_matrix_ok(Lr.sc, &npen)) return cudaSuccess;
    // the launch's queries pad to qcap - 16 columns at most (the callers size qcap with 16 spare)
    int need = qcap - 16;
    if (need < 16) need = 16;
    if (need > 256) need = 256;
    if (lanes == 16) {
        const int c = pick_c<16>(need);
        *cols = 16 * c;
        switch (c) {
        case 4: return wf2::launch_wf2<16, 4>(Lr, npen);
        case 6: return wf2::launch_wf2<16, 6>(Lr, npen);
        case 8: return wf2::launch_wf2<16, 8>(Lr, npen);
        case 10: return wf2::launch_wf2<16, 10>(Lr, npen);
        case 12: return wf2::launch_wf2<16, 12>(Lr, npen);
        case 16: return wf2::launch_wf2<16, 16>(Lr, npen);
        default: *cols = 0; return cudaSuccess;
        }
    }
    const int c = pick_c<8>(need);
    *cols = 8 * c;
    switch (c) {
    case 4: return wf2::launch_wf2<8, 4>(Lr, npen);
    case 8: return wf2::launch_wf2<8, 8>(Lr, npen);
    case 12: return wf2::launch_wf2<8, 12>(Lr, npen);
    case 16: return wf2::launch_wf2<8, 16>(Lr, npen);
    case 20: return wf2::launch_wf2<8, 20>(Lr, npen);
    case 24: return wf2::launch_wf2<8, 24>(Lr, npen);
    case 32: return wf2::launch_wf2<8, 32>(Lr, npen);
    default: *cols = 0; return cudaSuccess;
    }
}

}  // namespace bwacuda
